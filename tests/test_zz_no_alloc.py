"""The allocation-free entry point agrees with the regular one.

``ts_run_noalloc_2d`` exists for callers that cannot allocate device memory
(they hand the library only buffers from their own pool); it keeps its CPML
scratch in a fixed device array inside the library.  Here the test plays
such a caller: it owns every buffer (allocated beforehand with torch), calls
the entry point through the C ABI twice in a row (steps 0..n1-1, then
n1..n1+n2-1, the second call continuing from the scratch the first left),
and compares the wavefield and traces after each call with the regular
``ts_create``/``ts_run`` path on the same experiment, within the relative-L2
tolerance of the parity tests.  Collected last, so a failure here leaves
every other test already run.
"""
import numpy as np
import pytest

from _cases import case_2d, rel_l2
from taichi_sim_gb300 import engine
from taichi_sim_gb300.sim_support.simulator import Simulator

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _device(torch, a, dtype):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


def test_noalloc_matches_regular_path_over_two_calls():
    torch = pytest.importorskip("torch")
    sim = Simulator(case_2d(visco=0, linear=False, steps=220, seed=7))
    nx, ny = sim.grid_shape()
    n1, n2 = 120, 100

    # the caller's buffers
    f32, i32 = torch.float32, torch.int32
    fields = {n: torch.zeros((nx, ny), dtype=f32, device="cuda") for n in ("vx", "vy", "sxx", "syy", "sxy")}
    mat = {n: _device(torch, getattr(sim, f"_{n}_grid_vx"), f32) for n in ("rho", "cp", "cs")}
    tabs = {}
    for ax in "xy":
        for c in "abk":
            tabs[f"{c}_{ax}"] = _device(torch, getattr(sim, f"_{c}_{ax}").ravel(), f32)
            tabs[f"{c}_{ax}h"] = _device(torch, getattr(sim, f"_{c}_{ax}_half").ravel(), f32)
    # sources: the force the WGSL kernel reads at each step, flat[k * n_src + idx]
    src = np.argwhere(sim._pos_sources >= 0)
    flat = np.asarray(sim._source_term, np.float32).ravel()
    n_rows = int(sim._n_steps)
    values = np.zeros((n_rows, len(src)), np.float32)
    for q, (x, y) in enumerate(src):
        idx = int(sim._pos_sources[x, y])
        if idx < sim._n_src:
            values[:, q] = flat[np.arange(n_rows) * sim._n_src + idx]
    src_cell = _device(torch, src[:, 0] * ny + src[:, 1], i32)
    src_value = _device(torch, values, f32)
    # receivers: one node each in this experiment
    info = np.asarray(sim._info_rec_pt)
    assert len(np.unique(info[:, 2])) == info.shape[0] == sim._n_rec
    rec_cell = _device(torch, info[:, 0] * ny + info[:, 1], i32)
    rec_first = _device(torch, np.asarray(sim._delay_recv).astype(np.int32), i32)
    traces = torch.zeros((n_rows, sim._n_rec), dtype=f32, device="cuda")
    torch.cuda.synchronize()

    a = engine.NoAlloc2DArgs()
    a.nx, a.ny, a.ord = nx, ny, sim._coefs.shape[0]
    for c in range(a.ord):
        a.coefs[c] = float(sim._coefs[c])
    a.dx, a.dy, a.dt = sim._roi.get_dx(), sim._roi.get_dz(), sim._dt
    for n, t in {**fields, **mat, **tabs}.items():
        setattr(a, n, t.data_ptr())
    a.n_src, a.src_cell, a.src_value = len(src), src_cell.data_ptr(), src_value.data_ptr()
    a.n_rec, a.rec_cell, a.rec_first_step = sim._n_rec, rec_cell.data_ptr(), rec_first.data_ptr()
    a.traces, a.n_rows = traces.data_ptr(), n_rows

    with engine.Stepper(sim, family=engine.WGSL2D, visco=False) as ref:
        for step0, n in ((0, n1), (n1, n2)):
            a.step0, a.n_steps = step0, n
            engine.run_noalloc_2d(a)
            ref.run(n)
            torch.cuda.synchronize()
            for name, t in fields.items():
                want = ref.read(name)
                got = t.cpu().numpy()
                assert np.abs(want).max() > 0, name
                assert rel_l2(got, want) <= TOL, (step0, name, rel_l2(got, want))
            want_tr = ref.read("traces")[:step0 + n]
            got_tr = traces.cpu().numpy()[:step0 + n]
            assert np.abs(want_tr).max() > 0
            assert rel_l2(got_tr, want_tr) <= TOL, (step0, rel_l2(got_tr, want_tr))


def test_noalloc_rejects_oversized_grid():
    a = engine.NoAlloc2DArgs()
    a.nx, a.ny, a.ord = 2048, 1024, 2
    with pytest.raises(RuntimeError, match="exceeds the no-allocation scratch"):
        engine.run_noalloc_2d(a)
