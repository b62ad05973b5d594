"""Out-of-range and unusual host tables through ts_create, against the oracle.

The reference's WGSL accessors read any out-of-range entry as 0
(shader_webgpu_viscoelastic.wgsl:18-29, 67-71, 1118-1134): a receiver point
off the grid adds nothing to its trace, and a source-map entry that names a
column outside the source term injects nothing.  A negative receiver delay
records from the first step (``it >= delay`` always holds).  The Taichi
kernel (sim_taichi_elastic.py:188-190) indexes its trace array by the
sensor map's value, so a value beyond the receiver count is undefined
behaviour there; the library ignores such entries, and the test compares
with the oracle run on the map with those entries removed.  (Non-finite
material values are rejected by ts_create before any device work: tested
in test_capi_cpu.py.)
"""
import numpy as np
import pytest

from _cases import case_2d, rel_l2
from oracle import oracle
from taichi_sim_gb300 import engine
from taichi_sim_gb300.sim_support.simulator import Simulator

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _compare(sim, family, oracle_sim=None):
    fam_oracle = {engine.TAICHI2D: oracle.TAICHI2D, engine.WGSL2D: oracle.WGSL2D}[family]
    ref = oracle.run(oracle_sim or sim, fam_oracle)
    with engine.Stepper(sim, family=family) as st:
        st.run(sim._n_steps)
        assert st.status()[2] == -1
        tr, syy = st.read("traces"), st.read("syy")
    assert np.abs(ref["sens"]).max() > 0
    assert rel_l2(syy, ref["syy"]) <= TOL
    assert rel_l2(tr, ref["sens"]) <= TOL
    return tr, ref


def test_wgsl_receiver_points_off_the_grid_read_zero():
    sim = Simulator(case_2d(visco=1, seed=21))
    nx, ny = sim.grid_shape()
    info = np.array(sim._info_rec_pt)
    rec = info[:, 2]
    info[rec == 0, 0] = -3            # receiver 0: every point left of the grid
    info[rec == 1, 1] = ny + 5        # receiver 1: below it
    info[np.flatnonzero(rec == 2)[:1], 0] = nx   # receiver 2: one point off the grid
    sim._info_rec_pt = info
    tr, ref = _compare(sim, engine.WGSL2D)
    np.testing.assert_array_equal(tr[:, :2], 0.0)
    assert np.abs(tr[:, 2]).max() > 0


def test_wgsl_source_columns_outside_the_term_inject_nothing():
    sim = Simulator(case_2d(visco=0, seed=22))
    pos = np.array(sim._pos_sources)
    nodes = np.argwhere(pos >= 0)
    assert len(nodes) > 4
    for k, (x, y) in enumerate(nodes[:4]):
        pos[x, y] = (sim._n_src + 3, -7, sim._n_src, -2)[k]
    sim._pos_sources = pos
    _compare(sim, engine.WGSL2D)


@pytest.mark.parametrize("family", [engine.TAICHI2D, engine.WGSL2D], ids=["taichi", "wgsl"])
def test_negative_delays_record_from_the_first_step(family):
    sim = Simulator(case_2d(visco=0, linear=False, seed=23, t0_rx=0.2))
    configured = int(np.min(sim._delay_recv))   # 81 steps for t0_reception = 0.2 us
    sim._delay_recv = np.full_like(np.asarray(sim._delay_recv), -4)
    tr, ref = _compare(sim, family)
    # nothing is gated: rows before the configured delay carry signal
    first = int((tr != 0).any(axis=1).argmax())
    assert configured > 40 and first < configured, (first, configured)


def test_taichi_sensor_map_values_beyond_the_receivers_are_ignored():
    sim = Simulator(case_2d(visco=0, linear=False, seed=24))
    clean = Simulator(case_2d(visco=0, linear=False, seed=24))
    pos = np.array(sim._pos_sensors)
    free = np.argwhere(pos == -1)
    # near an existing receiver, inside the normal-stress region
    x0, y0 = np.argwhere(pos >= 0)[0]
    pick = free[np.argsort(np.abs(free[:, 0] - x0) + np.abs(free[:, 1] - y0))[:3]]
    for k, (x, y) in enumerate(pick):
        pos[x, y] = sim._n_rec + k
    sim._pos_sensors = pos
    _compare(sim, engine.TAICHI2D, oracle_sim=clean)
