"""The C-ABI library builds, loads and rejects bad input, without a GPU.

Every function declared in include/taichi_sim_gb300.h must be exported by
the shared library; ts_create validates its descriptor before touching the
device, so invalid descriptors are testable on a CPU-only machine.
"""
import ctypes
import os
import re

import numpy as np
import pytest

from taichi_sim_gb300 import engine

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "taichi_sim_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ts_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    return engine.load_library()


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 12
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_strerror_texts(lib):
    assert lib.ts_strerror(0) == b"ok"
    assert lib.ts_strerror(1) == b"invalid argument"
    assert lib.ts_strerror(99) == b"unknown error"


def _desc(**over):
    d = engine.TsDesc()
    d.abi_version = engine.ABI_VERSION
    d.family = engine.WGSL2D
    d.nx = d.ny = 32
    d.nz = 1
    d.n_steps = 10
    d.ord = 2
    for k, v in over.items():
        setattr(d, k, v)
    return d


@pytest.mark.parametrize("over,needle", [
    ({"abi_version": 99}, b"abi_version"),
    ({"family": 7}, b"family"),
    ({"ord": 1}, b"ord"),
    ({"ord": 7}, b"ord"),
    ({"nx": 3}, b"grid smaller"),
    ({"nz": 4}, b"nz must be 1"),
    ({"n_steps": 0}, b"n_steps"),
    ({}, b"missing coefficient"),
])
def test_create_rejects_bad_descriptor(lib, over, needle):
    h = ctypes.c_void_p()
    d = _desc(**over)
    rc = lib.ts_create(ctypes.byref(d), ctypes.byref(h))
    assert rc == 1, rc
    assert needle in lib.ts_last_error()
    assert h.value is None


def test_create_rejects_null(lib):
    h = ctypes.c_void_p()
    assert lib.ts_create(None, ctypes.byref(h)) == 1
    assert lib.ts_run(None, 1, None) == 1
    assert lib.ts_status(None, None, None, None) == 1
    assert lib.ts_reset(None) == 1
    lib.ts_destroy(None)  # no-op


def test_taichi_family_is_elastic_only(lib):
    keep = []

    def f(n):
        a = np.ones(n, np.float32)
        keep.append(a)
        return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))

    d = _desc(family=engine.TAICHI2D, visco=1)
    d.coefs, d.rho, d.cp, d.cs = f(2), f(32 * 32), f(32 * 32), f(32 * 32)
    for n in ("a_x", "b_x", "k_x", "a_xh", "b_xh", "k_xh", "a_y", "b_y", "k_y", "a_yh", "b_yh", "k_yh"):
        setattr(d, n, f(30))
    d.dx = d.dy = 0.1
    d.dt = 0.001
    h = ctypes.c_void_p()
    assert lib.ts_create(ctypes.byref(d), ctypes.byref(h)) == 1
    assert b"elastic only" in lib.ts_last_error()


def _batch_desc(lib, **shape):
    from taichi_sim_gb300 import batch
    batch._bind(lib)
    d = _desc(ord=2)
    phantoms = (engine.TsDesc * 1)(d)
    n_shots = (ctypes.c_int32 * 1)(4)
    tab = np.zeros(4 * 10, np.float32)
    ptrs = (ctypes.POINTER(ctypes.c_float) * 1)(tab.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    bd = batch.BatchDesc(abi_version=engine.ABI_VERSION, n_phantoms=1, phantoms=phantoms, n_shots=n_shots,
                         shot_sources=ptrs, **shape)
    return bd, (phantoms, n_shots, tab, ptrs)


@pytest.mark.parametrize("shape,needle", [
    (dict(block_cells=6), b"block_cells"),
    (dict(velocity_block_cells=2), b"block_cells"),
    (dict(nodes_per_thread=3), b"nodes_per_thread"),
    (dict(velocity_nodes_per_thread=8), b"nodes_per_thread"),
    (dict(shots_per_thread=3), b"shots_per_thread"),
])
def test_batch_create_rejects_bad_launch_shapes(lib, shape, needle):
    bd, keep = _batch_desc(lib, **shape)
    h = ctypes.c_void_p()
    assert lib.ts_batch_create(ctypes.byref(bd), ctypes.byref(h)) == 1
    assert needle in lib.ts_batch_last_error()
    assert h.value is None


def test_order4_batch_takes_the_default_shape(lib):
    bd, keep = _batch_desc(lib, velocity_nodes_per_thread=4)
    keep[0][0].ord = 4
    h = ctypes.c_void_p()
    assert lib.ts_batch_create(ctypes.byref(bd), ctypes.byref(h)) == 1
    assert b"order-4" in lib.ts_batch_last_error()


def test_adjoint_entry_points_reject_null(lib):
    from taichi_sim_gb300 import adjoint
    adjoint._bind(lib)
    assert lib.ts_adj_set_record_segments(None, 3) == 1
    assert lib.ts_adj_forward(None, None, None, None) == 1
    assert lib.ts_adj_backward(None, None, None, None) == 1


def _noalloc_args(**over):
    """A ts_noalloc2d_args that passes every check, then the overrides.  The
    pointers are host addresses the entry point never dereferences: each
    rejection happens before any CUDA call."""
    buf = np.zeros(16, np.float32)
    a = engine.NoAlloc2DArgs()
    a.nx, a.ny, a.ord = 64, 48, 2
    a.coefs[0], a.coefs[1] = 1.125, -1.0 / 24
    a.dx, a.dy, a.dt = 0.05, 0.05, 1e-3
    for n in ("vx", "vy", "sxx", "syy", "sxy", "rho", "cp", "cs", "a_x", "b_x", "k_x", "a_xh", "b_xh", "k_xh",
              "a_y", "b_y", "k_y", "a_yh", "b_yh", "k_yh", "src_cell", "src_value", "rec_cell",
              "rec_first_step", "traces"):
        setattr(a, n, buf.ctypes.data)
    a.n_src, a.n_rec, a.n_rows, a.step0, a.n_steps = 1, 1, 10, 0, 10
    for k, v in over.items():
        setattr(a, k, v)
    return a, buf


@pytest.mark.parametrize("over,needle", [
    ({"ord": 1}, "ord must be in"),
    ({"ord": 7}, "ord must be in"),
    ({"nx": 4}, "grid smaller than the stencil"),
    ({"ny": 4}, "grid smaller than the stencil"),
    ({"nx": 2048, "ny": 1024}, "exceeds the no-allocation scratch"),
    ({"vx": None}, "missing field or material"),
    ({"cs": None}, "missing field or material"),
    ({"k_yh": None}, "missing CPML table"),
    ({"step0": -1}, "steps beyond"),
    ({"n_steps": -1}, "steps beyond"),
    ({"step0": 5, "n_steps": 6}, "steps beyond"),
    ({"n_src": -1}, "bad source list"),
    ({"src_cell": None}, "bad source list"),
    ({"src_value": None}, "bad source list"),
    ({"n_rec": -2}, "bad receiver list"),
    ({"rec_first_step": None}, "bad receiver list"),
    ({"traces": None}, "bad receiver list"),
    ({"dx": 0.0}, "must be positive"),
    ({"dt": float("nan")}, "must be positive"),
])
def test_noalloc_rejects_bad_arguments(lib, over, needle):
    """Each TS_E_ARG branch of ts_run_noalloc_2d, checked before any CUDA call."""
    a, keep = _noalloc_args(**over)
    with pytest.raises(RuntimeError, match=needle):
        engine.run_noalloc_2d(a)


def test_noalloc_rejects_null_arguments(lib):
    fn = lib.ts_run_noalloc_2d
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    assert fn(None, None) == 1
    lib.ts_noalloc_last_error.restype = ctypes.c_char_p
    assert b"null arguments" in lib.ts_noalloc_last_error()


def test_noalloc_empty_lists_need_no_tables(lib):
    """n_src = n_rec = 0 needs no source or receiver table: the checks pass.
    With n_steps = 0 no kernel runs (the host pointers above are never
    handed to the device); without a GPU the call stops at the device query."""
    a, keep = _noalloc_args(n_src=0, n_rec=0, src_cell=None, src_value=None, rec_cell=None,
                            rec_first_step=None, traces=None, n_steps=0)
    try:
        engine.run_noalloc_2d(a)
    except RuntimeError as e:
        assert "invalid argument" not in str(e)


@pytest.mark.parametrize("attr,value,needle", [
    ("_rho_grid_vx", np.nan, "rho"),
    ("_cp_grid_vx", np.inf, "cp"),
    ("_cs_grid_vx", -np.inf, "cs"),
    ("_a_x", np.nan, "a_x"),
    ("_k_y_half", np.inf, "k_y_half"),
    ("_inv_qp_grid", np.nan, "g_p"),
])
def test_create_rejects_non_finite_tables(lib, attr, value, needle):
    """A NaN or Inf in the material, CPML or per-cell Q tables is refused by
    ts_create before any device work (the reference would run and fill the
    wavefield with NaN, which its stability test does not catch)."""
    import sys
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from _cases import case_2d
    from taichi_sim_gb300.sim_support.simulator import Simulator
    sim = Simulator(case_2d(visco=1, q=(30.0, 200.0), seed=1, steps=20))
    a = np.array(getattr(sim, attr), dtype=np.float32, copy=True)
    a.flat[a.size // 2] = value
    setattr(sim, attr, a)
    with pytest.raises(engine.TsError, match=f"non-finite value in {needle} at flat index"):
        engine.Stepper(sim)
