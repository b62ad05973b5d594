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
