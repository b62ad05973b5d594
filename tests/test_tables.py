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
