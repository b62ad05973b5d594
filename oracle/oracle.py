"""ctypes front end of the CPU oracle: TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg use this module, and only as the checker: it restates the reference's
kernels (see ts_oracle.h for the file:line list) and is never part of the
product path.

``run(sim, family, ...)`` takes a host model built by
``taichi_sim_gb300.sim_support`` (whose tables are bit-identical to the
reference's) and runs the restated kernels from a zero state.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libts_oracle.so")

TAICHI2D, WGSL2D, WGSL3D = 0, 1, 2

_f = ctypes.POINTER(ctypes.c_float)
_i = ctypes.POINTER(ctypes.c_int32)


class Desc(ctypes.Structure):
    _fields_ = [("family", ctypes.c_int32), ("nx", ctypes.c_int32), ("ny", ctypes.c_int32),
                ("nz", ctypes.c_int32), ("n_steps", ctypes.c_int32), ("ord", ctypes.c_int32),
                ("coefs", _f), ("dx", ctypes.c_float), ("dy", ctypes.c_float), ("dz", ctypes.c_float),
                ("dt", ctypes.c_float), ("one_dx", ctypes.c_float), ("one_dy", ctypes.c_float)] + \
               [(n, _f) for n in ("a_x", "b_x", "k_x", "a_xh", "b_xh", "k_xh", "a_y", "b_y", "k_y",
                                  "a_yh", "b_yh", "k_yh", "a_z", "b_z", "k_z", "a_zh", "b_zh", "k_zh",
                                  "rho", "cp", "cs")] + \
               [("visco", ctypes.c_int32), ("n_sls", ctypes.c_int32), ("tau", _f), ("sum_alpha", _f),
                ("g_p", _f), ("g_s", _f), ("zc", _f), ("zh", _f), ("zm", _f),
                ("source_term", _f), ("src_rows", ctypes.c_int32), ("src_cols", ctypes.c_int32),
                ("n_src_el", ctypes.c_int32), ("pos_sources", _i),
                ("n_rec", ctypes.c_int32), ("n_rec_pt", ctypes.c_int32), ("pos_sensors", _i),
                ("info_rec_pt", _i), ("offset_sensors", _i), ("delay_rec", _i)]


_lib = None


def build():
    """Compile the oracle library (make in oracle/)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = ctypes.CDLL(LIB_PATH)
        for name, t in (("ts_oracle_run_f32", ctypes.c_float), ("ts_oracle_run_f64", ctypes.c_double)):
            fn = getattr(_lib, name)
            p = ctypes.POINTER(t)
            fn.argtypes = [ctypes.POINTER(Desc), ctypes.POINTER(p), ctypes.POINTER(p), p, p]
            fn.restype = ctypes.c_int
    return _lib


def _ptr(a, ctype):
    return a.ctypes.data_as(ctypes.POINTER(ctype))


def family_of(sim):
    """Which restated kernel set a model runs: Taichi semantics for the
    elastic 2D Taichi backend, WGSL semantics otherwise."""
    if sim._dims == 3:
        return WGSL3D
    return TAICHI2D if getattr(sim, "_oracle_family", None) == TAICHI2D else WGSL2D


def run(sim, family, n_steps=None, precision="f32", visco=None):
    """Run the restated reference kernels on the model's tables.

    Returns a dict with the final ``vx, vy[, vz], sxx, syy[, szz], sxy[, sxz,
    syz]`` grids, ``sens`` ``(n_steps, n_rec)`` and ``vmax2`` ``(n_steps,)``.
    """
    keep = []

    def f32(a):
        a = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
        keep.append(a)
        return _ptr(a, ctypes.c_float)

    def i32(a):
        a = np.ascontiguousarray(np.asarray(a, dtype=np.int32))
        keep.append(a)
        return _ptr(a, ctypes.c_int32)

    n_steps = sim._n_steps if n_steps is None else int(n_steps)
    d = Desc()
    d.family = family
    shape = sim.grid_shape()
    d.nx, d.ny = shape[0], shape[1]
    d.nz = shape[2] if len(shape) == 3 else 1
    d.n_steps = n_steps
    d.ord = sim._coefs.shape[0]
    d.coefs = f32(sim._coefs)
    roi = sim._roi
    if sim._dims == 2:
        d.dx, d.dy, d.dz = roi.get_dx(), roi.get_dz(), roi.get_dy()
    else:
        d.dx, d.dy, d.dz = roi.get_dx(), roi.get_dy(), roi.get_dz()
    d.dt = sim._dt
    d.one_dx, d.one_dy = sim._one_dx, sim._one_dy
    for ax in ("x", "y", "z"):
        for c in "abk":
            for suffix, tag in (("", ""), ("_half", "h")):
                name = f"_{c}_{ax}{suffix}"
                if hasattr(sim, name):
                    setattr(d, f"{c}_{ax}{tag}", f32(getattr(sim, name).flatten()))
    d.rho, d.cp, d.cs = f32(sim._rho_grid_vx), f32(sim._cp_grid_vx), f32(sim._cs_grid_vx)
    from taichi_sim_gb300.sim_support.attenuation import AttenuationCoefficients
    att = AttenuationCoefficients()
    if visco is None:
        visco = bool(sim._configs.get("simul_configs", {}).get("viscoelastic_attn", 0))
    d.visco = 1 if visco else 0
    fit = getattr(sim, "_zener_fit", None)
    d.n_sls = fit.n_sls if fit is not None else att._n_sls
    d.tau, d.sum_alpha = f32(att.tau_table()), f32(att.sum_alpha())
    if fit is not None:
        c, h, m = fit.mechanism_constants(sim._dt)
        d.zc, d.zh, d.zm = f32(c), f32(h), f32(m)
        d.g_p, d.g_s = f32(fit.cell_scale(sim._inv_qp_grid)), f32(fit.cell_scale(sim._inv_qs_grid))
    st = np.asarray(sim._source_term, dtype=np.float32)
    st2 = st[:, None] if st.ndim == 1 else st
    d.source_term = f32(st2)
    d.src_rows, d.src_cols = st2.shape
    d.n_src_el = sim._n_src
    d.pos_sources = i32(sim._pos_sources)
    d.n_rec, d.n_rec_pt = sim._n_rec, int(sim._n_pto_rec)
    d.pos_sensors = i32(sim._pos_sensors)
    d.info_rec_pt = i32(sim._info_rec_pt)
    d.offset_sensors = i32(sim._offset_sensors)
    d.delay_rec = i32(sim._delay_recv)

    real = np.float32 if precision == "f32" else np.float64
    ctype = ctypes.c_float if precision == "f32" else ctypes.c_double
    names_v = ["vx", "vy", "vz"]
    names_s = ["sxx", "syy", "szz", "sxy", "sxz", "syz"]
    fields = {n: np.zeros(shape, dtype=real) for n in names_v + names_s}
    PP = ctypes.POINTER(ctype) * 3
    PS = ctypes.POINTER(ctype) * 6
    vptr = PP(*[_ptr(fields[n], ctype) for n in names_v])
    sptr = PS(*[_ptr(fields[n], ctype) for n in names_s])
    sens = np.zeros((n_steps, max(sim._n_rec, 1)), dtype=real)
    vmax2 = np.zeros(n_steps, dtype=real)
    fn = lib().ts_oracle_run_f32 if precision == "f32" else lib().ts_oracle_run_f64
    rc = fn(ctypes.byref(d), vptr, sptr, _ptr(sens, ctype), _ptr(vmax2, ctype))
    if rc != 0:
        raise RuntimeError(f"oracle failed ({rc})")
    out = {n: fields[n] for n in names_v + names_s}
    if sim._dims == 2:
        for n in ("vz", "szz", "sxz", "syz"):
            out.pop(n)
    out["sens"] = sens[:, :sim._n_rec]
    out["vmax2"] = vmax2
    return out
