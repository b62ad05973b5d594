"""The persistent 2D elastic path (one cooperative launch per ts_run, the
wavefield held on chip; opt-in with TS_2D_PERSISTENT=1) against the regular
two-kernel step.

Both run the same arithmetic, expression for expression, so fields and
traces must agree bit for bit; the regular path is itself checked against
the oracle (test_gpu_parity.py, test_gpu_full_size.py).  A handle created
without TS_2D_PERSISTENT=1 takes the regular path.  The bounded wait between
thread blocks is tested by a block that never releases its step counter (a
test hook): its neighbours give up after the wait bound, the handle reports
TS_E_TIMEOUT from ts_status, and the device stays usable.
"""
import numpy as np
import pytest

from _cases import case_2d, rel_l2
from oracle import oracle
from taichi_sim_gb300 import engine, workloads
from taichi_sim_gb300.sim_support.simulator import Simulator

pytestmark = pytest.mark.gpu

NAMES = ("vx", "vy", "sxx", "syy", "sxy", "traces")

CASES = {
    "taichi_point_line": (lambda: case_2d(linear=False, seed=31), engine.TAICHI2D),
    "taichi_array_delayed": (lambda: case_2d(visco=0, t0_rx=0.2, seed=32), engine.TAICHI2D),
    "wgsl_elastic_array": (lambda: case_2d(visco=0, seed=33), engine.WGSL2D),
    "wgsl_elastic_wide": (lambda: case_2d(visco=0, linear=False, w=300, h=180, steps=400, seed=34), engine.WGSL2D),
    "taichi_elastic2d_512": (lambda: workloads.elastic2d_512(n_steps=600), engine.TAICHI2D),
}


def _run(sim, family, chunks, monkeypatch, persistent):
    monkeypatch.setenv("TS_2D_PERSISTENT", "1" if persistent else "0")
    monkeypatch.setenv("TS_TAICHI_EXACT", "1")   # the persistent kernel's form of the Taichi arithmetic
    with engine.Stepper(sim, family=family) as st:
        before = st.launch_count()
        for n in chunks:
            st.run(n)
        launches = st.launch_count() - before
        assert st.status()[2] == -1
        return {k: st.read(k) for k in NAMES}, launches


@pytest.mark.parametrize("name", sorted(CASES))
def test_persistent_equals_regular_bit_for_bit(name, monkeypatch):
    build, family = CASES[name]
    sim = Simulator(build())
    n = int(sim._n_steps)
    reg, _ = _run(sim, family, [n], monkeypatch, False)
    per, launches = _run(sim, family, [n], monkeypatch, True)
    assert launches <= 3, f"persistent path not taken ({launches} launches for {n} steps)"
    assert np.abs(reg["traces"]).max() > 0
    for k in NAMES:
        np.testing.assert_array_equal(per[k], reg[k], err_msg=k)


def test_persistent_chunks_equal_one_run(monkeypatch):
    """Steps split over many launches (each loads the slabs from and stores
    them to global memory) give the same bits as one launch."""
    sim = Simulator(case_2d(visco=0, linear=False, w=200, h=120, steps=300, seed=35))
    one, _ = _run(sim, engine.TAICHI2D, [300], monkeypatch, True)
    many, launches = _run(sim, engine.TAICHI2D, [1, 2, 37, 100, 60, 100], monkeypatch, True)
    assert launches <= 3 * 6
    for k in NAMES:
        np.testing.assert_array_equal(many[k], one[k], err_msg=k)


def test_persistent_matches_oracle(monkeypatch):
    monkeypatch.setenv("TS_2D_PERSISTENT", "1")
    sim = Simulator(case_2d(visco=0, linear=False, w=160, h=140, steps=300, seed=36))
    ref = oracle.run(sim, oracle.TAICHI2D)
    with engine.Stepper(sim, family=engine.TAICHI2D) as st:
        st.simulate()
        got = {k: st.read(k) for k in NAMES}
    for k in ("vx", "vy", "sxx", "syy", "sxy"):
        assert rel_l2(got[k], ref[k]) <= 1e-5, k
    assert rel_l2(got["traces"], ref["sens"]) <= 1e-5


def test_persistent_wait_gives_up_and_reports(monkeypatch):
    """A block that never releases its counter (a flag nothing sets): its
    neighbours stop after the wait bound (2 ms here), ts_status reports
    TS_E_TIMEOUT, and a new handle on the same device runs normally."""
    sim = Simulator(case_2d(visco=0, linear=False, w=120, h=100, steps=60, seed=37))
    monkeypatch.setenv("TS_2D_PERSISTENT", "1")
    monkeypatch.setenv("TS_PERSIST_STALL_BLOCK", "2")
    monkeypatch.setenv("TS_PERSIST_WAIT_NS", "2000000")
    with engine.Stepper(sim, family=engine.TAICHI2D) as st:
        st.run(40)
        with pytest.raises(engine.TsError, match="gave up waiting") as e:
            st.status()
        assert e.value.code == 6
        st.reset()   # clears the record; the handle keeps its test hook
    monkeypatch.delenv("TS_PERSIST_STALL_BLOCK")
    monkeypatch.delenv("TS_PERSIST_WAIT_NS")
    ref = oracle.run(sim, oracle.TAICHI2D)
    with engine.Stepper(sim, family=engine.TAICHI2D) as st:
        st.run(60)
        assert st.status()[2] == -1
        assert rel_l2(st.read("syy"), ref["syy"]) <= 1e-5
