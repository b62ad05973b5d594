"""ctypes binding of the C ABI (include/taichi_sim_gb300.h) and the stepper.

:class:`Stepper` owns one ``ts_sim`` handle built from a host model
(:class:`~taichi_sim_gb300.sim_support.simulator.Simulator` or
``Simulator3D``): it passes the model's tables by pointer to ``ts_create``,
advances steps with ``ts_run``, checks stability with ``ts_status`` and reads
fields and traces back with ``ts_read``.

There is no fallback: if the CUDA library cannot be built or loaded, or no
sm_103 device is present, construction raises.
"""
import ctypes
import os
import threading

import numpy as np

from .sim_support import StabilityError, flt32
from .sim_support.attenuation import AttenuationCoefficients

TAICHI2D, WGSL2D, WGSL3D = 0, 1, 2
VX, VY, VZ, SXX, SYY, SZZ, SXY, SXZ, SYZ, TRACES = range(10)
ABI_VERSION = 2
FIELD_NAMES = {"vx": VX, "vy": VY, "vz": VZ, "sxx": SXX, "syy": SYY, "szz": SZZ, "sxy": SXY, "sxz": SXZ,
               "syz": SYZ}

_f = ctypes.POINTER(ctypes.c_float)
_i = ctypes.POINTER(ctypes.c_int32)


class TsDesc(ctypes.Structure):
    """Mirror of ``ts_desc``."""
    _fields_ = [("abi_version", ctypes.c_int32), ("family", ctypes.c_int32), ("nx", ctypes.c_int32),
                ("ny", ctypes.c_int32), ("nz", ctypes.c_int32), ("n_steps", ctypes.c_int32),
                ("ord", ctypes.c_int32), ("coefs", _f), ("dx", ctypes.c_float), ("dy", ctypes.c_float),
                ("dz", ctypes.c_float), ("dt", ctypes.c_float)] + \
               [(n, _f) for n in ("a_x", "b_x", "k_x", "a_xh", "b_xh", "k_xh", "a_y", "b_y", "k_y",
                                  "a_yh", "b_yh", "k_yh", "a_z", "b_z", "k_z", "a_zh", "b_zh", "k_zh",
                                  "rho", "cp", "cs")] + \
               [("visco", ctypes.c_int32), ("n_sls", ctypes.c_int32), ("tau", _f), ("sum_alpha", _f),
                ("g_p", _f), ("g_s", _f), ("zc", _f), ("zh", _f), ("zm", _f),
                ("source_term", _f), ("src_rows", ctypes.c_int32), ("src_cols", ctypes.c_int32),
                ("n_src_el", ctypes.c_int32), ("pos_sources", _i), ("n_rec", ctypes.c_int32),
                ("n_rec_pt", ctypes.c_int32), ("pos_sensors", _i), ("info_rec_pt", _i),
                ("offset_sensors", _i), ("delay_rec", _i)]


_lib = None
_lock = threading.Lock()


def library_path():
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "libtaichi_sim_gb300.so")


def load_library(build_if_missing=True):
    """Load (building it first if needed) the in-tree CUDA library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = library_path()
        if build_if_missing:
            from .build import build
            path = build()
        if not os.path.exists(path):
            raise RuntimeError(f"taichi_sim_gb300 CUDA library missing: {path}")
        lib = ctypes.CDLL(path)
        P = ctypes.c_void_p
        sigs = {
            "ts_create": ([ctypes.POINTER(TsDesc), ctypes.POINTER(P)], ctypes.c_int),
            "ts_run": ([P, ctypes.c_int32, P], ctypes.c_int),
            "ts_status": ([P, _i, _f, _i], ctypes.c_int),
            "ts_read": ([P, ctypes.c_int32, P, ctypes.c_size_t], ctypes.c_int),
            "ts_set_sources": ([P, _f], ctypes.c_int),
            "ts_reset": ([P], ctypes.c_int),
            "ts_reset_async": ([P, P], ctypes.c_int),
            "ts_profile_steps": ([P, ctypes.c_int32, P, _f], ctypes.c_int),
            "ts_launch_count": ([P, ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
            "ts_transfer_bytes": ([P, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)],
                                  ctypes.c_int),
            "ts_device_buffer": ([P, ctypes.c_int32, ctypes.POINTER(P), ctypes.POINTER(ctypes.c_size_t)],
                                 ctypes.c_int),
            "ts_launches_per_step": ([P, _i], ctypes.c_int),
            "ts_step_path": ([P, _i], ctypes.c_int),
            "ts_copy_field": ([P, ctypes.c_int32, P, ctypes.c_size_t, P], ctypes.c_int),
            "ts_destroy": ([P], None),
            "ts_strerror": ([ctypes.c_int], ctypes.c_char_p),
            "ts_last_error": ([], ctypes.c_char_p),
        }
        for name, (args, res) in sigs.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        _lib = lib
        return lib


class TsError(RuntimeError):
    """A C-ABI call returned an error code."""

    def __init__(self, code, where):
        lib = load_library(build_if_missing=False)
        self.code = code
        super().__init__(f"{where}: {lib.ts_strerror(code).decode()} ({lib.ts_last_error().decode()})")


def _check(code, where):
    if code != 0:
        raise TsError(code, where)


def default_family(sim, requested=None):
    if requested is not None:
        return requested
    return WGSL3D if sim._dims == 3 else WGSL2D


class Stepper:
    """One simulation resident on the GPU.

    ``family`` selects whose semantics to follow: :data:`TAICHI2D` (the
    Taichi elastic backend), :data:`WGSL2D` or :data:`WGSL3D` (the WebGPU
    viscoelastic backends).  ``visco`` defaults to the config's
    ``viscoelastic_attn``.
    """

    def __init__(self, sim, family=None, visco=None):
        self._lib = load_library()
        self.sim = sim
        self.family = default_family(sim, family)
        if (self.family == WGSL3D) != (sim._dims == 3):
            raise ValueError("family does not match the model's dimensions")
        if visco is None:
            visco = bool(sim._configs.get("simul_configs", {}).get("viscoelastic_attn", 0))
        if self.family == TAICHI2D:
            visco = False
        self.visco = visco
        self.shape = sim.grid_shape()
        self.n_rows = int(sim._n_steps)
        self.n_rec = int(sim._n_rec)
        self._keep = []
        desc = self._describe()
        h = ctypes.c_void_p()
        _check(self._lib.ts_create(ctypes.byref(desc), ctypes.byref(h)), "ts_create")
        self._h = h
        self._keep = []  # ts_create copied everything it needs
        n = ctypes.c_int32()
        _check(self._lib.ts_launches_per_step(self._h, ctypes.byref(n)), "ts_launches_per_step")
        self.launches_per_step = n.value
        _check(self._lib.ts_step_path(self._h, ctypes.byref(n)), "ts_step_path")
        # "persistent": every step of a run() in one launch, the wavefield on chip
        self.path = "persistent" if n.value == 1 else "stepped"

    # -- descriptor -----------------------------------------------------------
    def _f32(self, a):
        a = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
        self._keep.append(a)
        return a.ctypes.data_as(_f)

    def _i32(self, a):
        a = np.ascontiguousarray(np.asarray(a, dtype=np.int32))
        self._keep.append(a)
        return a.ctypes.data_as(_i)

    def _describe(self):
        sim = self.sim
        d = TsDesc()
        d.abi_version = ABI_VERSION
        d.family = self.family
        d.nx, d.ny = self.shape[0], self.shape[1]
        d.nz = self.shape[2] if len(self.shape) == 3 else 1
        d.n_steps = self.n_rows
        d.ord = sim._coefs.shape[0]
        d.coefs = self._f32(sim._coefs)
        roi = sim._roi
        if sim._dims == 2:
            d.dx, d.dy, d.dz = roi.get_dx(), roi.get_dz(), roi.get_dy()
        else:
            d.dx, d.dy, d.dz = roi.get_dx(), roi.get_dy(), roi.get_dz()
        d.dt = sim._dt
        for ax in ("x", "y", "z"):
            for c in "abk":
                for suffix, tag in (("", ""), ("_half", "h")):
                    name = f"_{c}_{ax}{suffix}"
                    if hasattr(sim, name) and (sim._dims == 3 or ax != "z"):
                        setattr(d, f"{c}_{ax}{tag}", self._f32(getattr(sim, name).flatten()))
        d.rho, d.cp, d.cs = self._f32(sim._rho_grid_vx), self._f32(sim._cp_grid_vx), self._f32(sim._cs_grid_vx)
        d.visco = 1 if self.visco else 0
        fit = getattr(sim, "_zener_fit", None)
        if self.visco:
            if fit is not None:
                c, h, m = fit.mechanism_constants(sim._dt)
                d.n_sls = fit.n_sls
                d.zc, d.zh, d.zm = self._f32(c), self._f32(h), self._f32(m)
                g_p, g_s = sim.cell_scales()
                d.g_p = self._f32(g_p)
                d.g_s = self._f32(g_s)
            else:
                att = AttenuationCoefficients()
                d.n_sls = att._n_sls
                d.tau, d.sum_alpha = self._f32(att.tau_table()), self._f32(att.sum_alpha())
        st = np.asarray(sim._source_term, dtype=np.float32)
        st2 = st[:, None] if st.ndim == 1 else st
        self._src_shape = st2.shape
        d.source_term = self._f32(st2)
        d.src_rows, d.src_cols = st2.shape
        d.n_src_el = int(sim._n_src)
        d.pos_sources = self._i32(sim._pos_sources)
        d.n_rec, d.n_rec_pt = self.n_rec, int(sim._n_pto_rec)
        d.pos_sensors = self._i32(sim._pos_sensors)
        d.info_rec_pt = self._i32(sim._info_rec_pt)
        d.offset_sensors = self._i32(sim._offset_sensors)
        d.delay_rec = self._i32(np.asarray(sim._delay_recv).reshape(-1)[:max(self.n_rec, 1)]
                                if self.n_rec else np.zeros(1, np.int32))
        return d

    # -- control --------------------------------------------------------------
    def run(self, n_steps, stream=None):
        """Enqueue ``n_steps`` steps (asynchronous)."""
        _check(self._lib.ts_run(self._h, int(n_steps), ctypes.c_void_p(stream or 0)), "ts_run")

    def status(self):
        """``(steps_done, max |v|^2 so far, first unstable step or -1)`` after a sync."""
        n, m, b = ctypes.c_int32(), ctypes.c_float(), ctypes.c_int32()
        _check(self._lib.ts_status(self._h, ctypes.byref(n), ctypes.byref(m), ctypes.byref(b)), "ts_status")
        return n.value, m.value, b.value

    def read(self, what):
        """A field (by name or ts code) as an ndarray of the grid's shape, or the traces."""
        code = FIELD_NAMES.get(what, what) if isinstance(what, str) else what
        if what == "traces" or code == TRACES:
            out = np.zeros((self.n_rows, self.n_rec), dtype=np.float32)
            code = TRACES
        else:
            out = np.zeros(self.shape, dtype=np.float32)
        _check(self._lib.ts_read(self._h, code, out.ctypes.data_as(ctypes.c_void_p), out.nbytes), "ts_read")
        return out

    def set_sources(self, source_term):
        st = np.asarray(source_term, dtype=np.float32)
        st2 = np.ascontiguousarray(st[:, None] if st.ndim == 1 else st)
        if st2.shape != self._src_shape:
            raise ValueError(f"source term shape {st2.shape} != {self._src_shape}")
        _check(self._lib.ts_set_sources(self._h, st2.ctypes.data_as(_f)), "ts_set_sources")

    def reset(self, stream=None, wait=True):
        """Zero the state; with ``wait=False`` only enqueue it on ``stream``."""
        if wait and stream is None:
            _check(self._lib.ts_reset(self._h), "ts_reset")
        else:
            _check(self._lib.ts_reset_async(self._h, ctypes.c_void_p(stream or 0)), "ts_reset_async")

    def profile_steps(self, n_steps, stream=None):
        """Mean device time (ms) of each kernel of a step over ``n_steps`` steps."""
        out = (ctypes.c_float * 2)()
        _check(self._lib.ts_profile_steps(self._h, int(n_steps), ctypes.c_void_p(stream or 0),
                                          ctypes.cast(out, _f)), "ts_profile_steps")
        return list(out)

    def transfer_bytes(self):
        """``(host->device, device->host)`` bytes copied by this handle so far."""
        a, b = ctypes.c_int64(), ctypes.c_int64()
        _check(self._lib.ts_transfer_bytes(self._h, ctypes.byref(a), ctypes.byref(b)), "ts_transfer_bytes")
        return a.value, b.value

    def launch_count(self):
        n = ctypes.c_int64()
        _check(self._lib.ts_launch_count(self._h, ctypes.byref(n)), "ts_launch_count")
        return n.value

    def device_buffer(self, what):
        code = FIELD_NAMES.get(what, what) if isinstance(what, str) else what
        p, pitch = ctypes.c_void_p(), ctypes.c_size_t()
        _check(self._lib.ts_device_buffer(self._h, code, ctypes.byref(p), ctypes.byref(pitch)), "ts_device_buffer")
        return p.value, pitch.value

    def copy_field(self, what, dst_ptr, dst_pitch=0, stream=None):
        """Enqueue a copy of a field (after the steps queued so far) to device
        or pinned host memory at ``dst_ptr`` (packed rows unless
        ``dst_pitch`` bytes); does not wait (``ts_copy_field``)."""
        code = FIELD_NAMES.get(what, what) if isinstance(what, str) else what
        _check(self._lib.ts_copy_field(self._h, code, ctypes.c_void_p(dst_ptr), int(dst_pitch),
                                       ctypes.c_void_p(stream or 0)), "ts_copy_field")

    def close(self):
        if getattr(self, "_h", None):
            self._lib.ts_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- whole run --------------------------------------------------------------
    def simulate(self, n_steps=None, check_every=None):
        """Run ``n_steps`` (default: all) steps, raising ``StabilityError`` at
        the first unstable step as the reference's loop does."""
        n_steps = self.n_rows if n_steps is None else int(n_steps)
        check_every = check_every or max(256, int(getattr(self.sim, "_it_display", 10)))
        done = 0
        while done < n_steps:
            k = min(check_every, n_steps - done)
            self.run(k)
            done += k
            _, vmax, bad = self.status()
            if bad >= 0:
                value = vmax if self.family == TAICHI2D else float(np.sqrt(np.float32(vmax)))
                raise StabilityError("Simulacao tornando-se instavel", value)
            if getattr(self.sim, "_show_debug", False):
                print(f'Time step # {done} out of {self.n_rows}')
                print(f'Max norm velocity vector V (m/s) = {np.sqrt(vmax)}')
        return done


class NoAlloc2DArgs(ctypes.Structure):
    """Mirror of ``ts_noalloc2d_args`` (see :func:`run_noalloc_2d`)."""
    _fields_ = [("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("ord", ctypes.c_int32),
                ("coefs", ctypes.c_float * 6), ("dx", ctypes.c_float), ("dy", ctypes.c_float),
                ("dt", ctypes.c_float)] + \
               [(n, ctypes.c_void_p) for n in ("vx", "vy", "sxx", "syy", "sxy", "rho", "cp", "cs",
                                                "a_x", "b_x", "k_x", "a_xh", "b_xh", "k_xh",
                                                "a_y", "b_y", "k_y", "a_yh", "b_yh", "k_yh")] + \
               [("n_src", ctypes.c_int32), ("src_cell", ctypes.c_void_p), ("src_value", ctypes.c_void_p),
                ("n_rec", ctypes.c_int32), ("rec_cell", ctypes.c_void_p), ("rec_first_step", ctypes.c_void_p),
                ("traces", ctypes.c_void_p), ("n_rows", ctypes.c_int32), ("step0", ctypes.c_int32),
                ("n_steps", ctypes.c_int32)]


def run_noalloc_2d(args, stream=None):
    """Advance an allocation-free 2D elastic simulation in caller-owned
    device buffers (``ts_run_noalloc_2d``).

    For callers that cannot allocate device memory: every buffer in ``args``
    is the caller's; the CPML memories live in the library's fixed 32 MiB
    device array (grids up to 1,048,576 nodes), shared by all calls and kept
    between them, so ``step0 == 0`` starts a simulation and later calls
    continue it; overlapping calls race.  Make the first call on a device
    before any stream capture.
    """
    lib = load_library()
    fn = lib.ts_run_noalloc_2d
    fn.argtypes = [ctypes.POINTER(NoAlloc2DArgs), ctypes.c_void_p]
    fn.restype = ctypes.c_int
    err = lib.ts_noalloc_last_error
    err.argtypes = []
    err.restype = ctypes.c_char_p
    rc = fn(ctypes.byref(args), ctypes.c_void_p(stream or 0))
    if rc != 0:
        raise RuntimeError(f"ts_run_noalloc_2d: {lib.ts_strerror(rc).decode()} ({err().decode()})")
