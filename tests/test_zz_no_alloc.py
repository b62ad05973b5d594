"""The allocation-free entry point agrees with the regular one and the oracle.

``ts_run_noalloc_2d`` exists for callers that cannot allocate device memory
(they hand the library only buffers from their own pool); it keeps its CPML
scratch in a fixed device array inside the library.  Here the test plays
such a caller: it owns every buffer (allocated beforehand with torch), calls
the entry point through the C ABI twice in a row (steps 0..n1-1, then
n1..n1+n2-1, the second call continuing from the scratch the first left),
and compares the wavefield and traces after each call with the regular
``ts_create``/``ts_run`` path on the same experiment and with the CPU oracle,
within the relative-L2 tolerance of the parity tests.  A second test hands it
source and receiver tables with cells outside the grid (ignored) and a
source split over two entries of one cell (both inject).  Collected last, so
a failure here leaves every other test already run.  (Its argument checks,
which need no GPU, are in test_capi_cpu.py.)
"""
import numpy as np
import pytest

from _cases import case_2d, rel_l2
from oracle import oracle
from taichi_sim_gb300 import engine
from taichi_sim_gb300.sim_support.simulator import Simulator

pytestmark = pytest.mark.gpu

TOL = 1e-5
FIELDS = ("vx", "vy", "sxx", "syy", "sxy")


def _device(torch, a, dtype):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


def _caller_buffers(torch, sim, src_cells=None, src_values=None, rec_cells=None):
    """Every buffer the caller owns, and the argument block that points at
    them.  Sources default to the model's (the force the WGSL kernel reads
    at each step, flat[k * n_src + idx]); receivers to its one-node ones."""
    nx, ny = sim.grid_shape()
    f32, i32 = torch.float32, torch.int32
    bufs = {n: torch.zeros((nx, ny), dtype=f32, device="cuda") for n in FIELDS}
    for n in ("rho", "cp", "cs"):
        bufs[n] = _device(torch, getattr(sim, f"_{n}_grid_vx"), f32)
    for ax in "xy":
        for c in "abk":
            bufs[f"{c}_{ax}"] = _device(torch, getattr(sim, f"_{c}_{ax}").ravel(), f32)
            bufs[f"{c}_{ax}h"] = _device(torch, getattr(sim, f"_{c}_{ax}_half").ravel(), f32)
    n_rows = int(sim._n_steps)
    if src_cells is None:
        src = np.argwhere(sim._pos_sources >= 0)
        flat = np.asarray(sim._source_term, np.float32).ravel()
        src_values = np.zeros((n_rows, len(src)), np.float32)
        for q, (x, y) in enumerate(src):
            idx = int(sim._pos_sources[x, y])
            if idx < sim._n_src:
                src_values[:, q] = flat[np.arange(n_rows) * sim._n_src + idx]
        src_cells = src[:, 0] * ny + src[:, 1]
    info = np.asarray(sim._info_rec_pt)
    assert len(np.unique(info[:, 2])) == info.shape[0] == sim._n_rec   # one node per receiver
    if rec_cells is None:
        rec_cells = info[:, 0] * ny + info[:, 1]
    n_rec = len(rec_cells)
    delay = np.asarray(sim._delay_recv).astype(np.int32).ravel()
    rec_first = np.resize(delay, n_rec)
    extra = {"src_cell": _device(torch, src_cells, i32), "src_value": _device(torch, src_values, f32),
             "rec_cell": _device(torch, rec_cells, i32), "rec_first_step": _device(torch, rec_first, i32),
             "traces": torch.zeros((n_rows, n_rec), dtype=f32, device="cuda")}
    torch.cuda.synchronize()

    a = engine.NoAlloc2DArgs()
    a.nx, a.ny, a.ord = nx, ny, sim._coefs.shape[0]
    for c in range(a.ord):
        a.coefs[c] = float(sim._coefs[c])
    a.dx, a.dy, a.dt = sim._roi.get_dx(), sim._roi.get_dz(), sim._dt
    for n, t in {**bufs, **extra}.items():
        setattr(a, n, t.data_ptr())
    a.n_src, a.n_rec, a.n_rows = len(src_cells), n_rec, n_rows
    return a, {**bufs, **extra}


def test_noalloc_matches_regular_path_over_two_calls():
    torch = pytest.importorskip("torch")
    sim = Simulator(case_2d(visco=0, linear=False, steps=220, seed=7))
    n1, n2 = 120, 100
    a, bufs = _caller_buffers(torch, sim)
    with engine.Stepper(sim, family=engine.WGSL2D, visco=False) as ref:
        for step0, n in ((0, n1), (n1, n2)):
            a.step0, a.n_steps = step0, n
            engine.run_noalloc_2d(a)
            ref.run(n)
            torch.cuda.synchronize()
            orc = oracle.run(sim, oracle.WGSL2D, n_steps=step0 + n, visco=False)
            for name in FIELDS:
                want = ref.read(name)
                got = bufs[name].cpu().numpy()
                assert np.abs(want).max() > 0, name
                assert rel_l2(got, want) <= TOL, (step0, name, rel_l2(got, want))
                assert rel_l2(got, orc[name]) <= TOL, (step0, name, "oracle", rel_l2(got, orc[name]))
            want_tr = ref.read("traces")[:step0 + n]
            got_tr = bufs["traces"].cpu().numpy()[:step0 + n]
            assert np.abs(want_tr).max() > 0
            assert rel_l2(got_tr, want_tr) <= TOL, (step0, rel_l2(got_tr, want_tr))
            assert rel_l2(got_tr, orc["sens"][:step0 + n]) <= TOL, (step0, "oracle")


def test_noalloc_ignores_cells_outside_the_grid_and_adds_duplicates():
    torch = pytest.importorskip("torch")
    sim = Simulator(case_2d(visco=0, linear=False, steps=160, seed=5))
    nx, ny = sim.grid_shape()
    n = int(sim._n_steps)

    clean, cb = _caller_buffers(torch, sim)
    clean.step0, clean.n_steps = 0, n
    engine.run_noalloc_2d(clean)
    torch.cuda.synchronize()
    want = {k: cb[k].cpu().numpy() for k in (*FIELDS, "traces")}

    # the same sources with the first one split over two entries of its cell,
    # plus entries below and beyond the grid; receivers likewise
    src_cells = cb["src_cell"].cpu().numpy()
    src_vals = cb["src_value"].cpu().numpy()
    cells = np.concatenate([[src_cells[0], -1, nx * ny], src_cells])
    vals = np.concatenate([0.5 * src_vals[:, :1], np.ones((n, 2), np.float32), src_vals], axis=1)
    vals[:, 3] *= 0.5
    rec = cb["rec_cell"].cpu().numpy()
    rec_cells = np.concatenate([rec, [-7, nx * ny + 3]])
    dirty, db = _caller_buffers(torch, sim, src_cells=cells, src_values=vals, rec_cells=rec_cells)
    dirty.step0, dirty.n_steps = 0, n
    engine.run_noalloc_2d(dirty)
    torch.cuda.synchronize()
    for k in FIELDS:
        got = db[k].cpu().numpy()
        assert rel_l2(got, want[k]) <= TOL, (k, rel_l2(got, want[k]))
    tr = db["traces"].cpu().numpy()
    assert rel_l2(tr[:, :len(rec)], want["traces"]) <= TOL
    np.testing.assert_array_equal(tr[:, len(rec):], 0.0)   # out-of-grid receivers: untouched
