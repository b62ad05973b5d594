"""The host model builds exactly the reference's tables.

Fixtures come from the reference's own ``sim_support`` (tests/golden/
make_golden.py); every table is compared bit for bit (sha256 of the bytes,
plus shape and dtype).
"""
import hashlib

import numpy as np
import pytest

from _golden import config_with_maps, experiments, tables
from taichi_sim_gb300.sim_support.simulator import Simulator
from taichi_sim_gb300.sim_support.Simulator3D import Simulator3D

NAMES = sorted(experiments())


def _build(name):
    dims, cfg = config_with_maps(name)
    cls = Simulator if dims == 2 else Simulator3D
    return cls(cfg, sim_type="viscoelastic")


@pytest.mark.parametrize("name", NAMES)
def test_tables_bit_identical(name):
    sim = _build(name)
    ref = tables(name)
    keys = sorted(k[:-4] for k in ref.files if k.endswith(".sha"))
    assert keys, "fixture holds no tables"
    bad = []
    for key in keys:
        v = np.asarray(getattr(sim, "_" + key))
        want_shape = tuple(ref[key + ".shape"].tolist())
        if v.shape != want_shape or str(v.dtype) != str(ref[key + ".dtype"]):
            bad.append(f"{key}: {v.shape}/{v.dtype} != {want_shape}/{ref[key + '.dtype']}")
            continue
        if hashlib.sha256(np.ascontiguousarray(v).tobytes()).hexdigest() != str(ref[key + ".sha"]):
            detail = ""
            if key in ref.files:
                detail = f" max|diff|={np.max(np.abs(v.astype(np.float64) - ref[key].astype(np.float64)))}"
            bad.append(f"{key}: bytes differ{detail}")
    assert not bad, "\n".join(bad)


def test_cell_scales_are_computed_once_and_follow_the_q_grids():
    """The per-cell attenuation scales a stepper uploads: the fit's formula,
    cached on the model (one computation for every shot's stepper)."""
    import numpy as np
    import sys, os
    sys.path.insert(0, os.path.dirname(__file__))
    from _cases import case_2d
    from taichi_sim_gb300.sim_support.simulator import Simulator
    sim = Simulator(case_2d(visco=1, q=(30.0, 200.0), seed=1, steps=20))
    g = sim.cell_scales()
    np.testing.assert_array_equal(g[0], sim._zener_fit.cell_scale(sim._inv_qp_grid))
    np.testing.assert_array_equal(g[1], sim._zener_fit.cell_scale(sim._inv_qs_grid))
    assert sim.cell_scales()[0] is g[0]                     # cached
    sim._inv_qp_grid = sim._inv_qp_grid * np.float32(2.0)   # a new grid object: recomputed
    np.testing.assert_array_equal(sim.cell_scales()[0], sim._zener_fit.cell_scale(sim._inv_qp_grid))
    import pytest
    with pytest.raises(ValueError):                         # in-place edits would leave the cache stale
        sim._inv_qs_grid *= np.float32(2.0)
    assert Simulator(case_2d(visco=1, steps=20)).cell_scales() is None
