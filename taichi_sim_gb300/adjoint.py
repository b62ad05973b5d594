"""Gradient of a receiver-trace misfit with respect to per-cell lambda, mu
and rho: a hand-written discrete adjoint of the 2D WGSL-semantics stepper
(``ts_adj_*`` in the C ABI) behind a ``torch.autograd.Function``.

The reference simulates only (shader_webgpu_viscoelastic.wgsl:829-1072,
sim_webgpu_viscoelastic.py:469-537); this module makes that forward
differentiable without changing it:

* :meth:`AdjointProblem.node_coefficients` maps per-cell (lambda, mu, rho) to
  the per-node coefficients the kernels use, with the reference's staggered
  averaging of rho, cp and cs (shader_webgpu_viscoelastic.wgsl:863-868,
  948-950, 1020, 1032), written in torch so that autograd chains the node
  gradients back to the cells;
* :class:`TraceFunction` runs the forward on the GPU (``ts_adj_forward``)
  and, in ``backward``, the time-reversed adjoint (``ts_adj_backward``) with
  the incoming trace gradient as the adjoint source.  The forward keeps the
  state every ``checkpoint_every`` steps (default ceil(sqrt(n_steps)),
  revolve-style) and recomputes each segment before its adjoint sweep,
  except the ``record_segments`` trailing segments (default 1) whose
  features the forward pass records as it goes; ``checkpoint_every=0``
  keeps every step's features instead (no recomputation, 6 floats per node
  and step).

Shots share one problem: :meth:`AdjointProblem.set_source_term` swaps the
source table, and gradients of several shots add up in ``.grad`` as usual.
"""
import ctypes
import math

import numpy as np
import torch

from . import engine

_P = ctypes.c_void_p
_f = ctypes.POINTER(ctypes.c_float)


class AdjCoefs(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("L", "M", "Ms", "Bx", "By", "g_p", "g_s")]


class AdjGrads(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("gL", "gM", "gMs", "gBx", "gBy")]


def _bind(lib):
    if getattr(lib, "_adj_bound", False):
        return lib
    sigs = {
        "ts_adj_create": ([ctypes.POINTER(engine.TsDesc), ctypes.c_int32, ctypes.POINTER(_P)], ctypes.c_int),
        "ts_adj_pitch": ([_P, ctypes.POINTER(ctypes.c_int32)], ctypes.c_int),
        "ts_adj_set_record_segments": ([_P, ctypes.c_int32], ctypes.c_int),
        "ts_adj_set_sources": ([_P, _f], ctypes.c_int),
        "ts_adj_forward": ([_P, ctypes.POINTER(AdjCoefs), _P, _P], ctypes.c_int),
        "ts_adj_backward": ([_P, _P, ctypes.POINTER(AdjGrads), _P], ctypes.c_int),
        "ts_adj_read_field": ([_P, ctypes.c_int32, _P, ctypes.c_size_t], ctypes.c_int),
        "ts_adj_launch_count": ([_P, ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
        "ts_adj_destroy": ([_P], None),
        "ts_adj_last_error": ([], ctypes.c_char_p),
    }
    for name, (args, res) in sigs.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    lib._adj_bound = True
    return lib


def _check(lib, rc, where):
    if rc != 0:
        raise RuntimeError(f"{where}: {lib.ts_strerror(rc).decode()} ({lib.ts_adj_last_error().decode()})")


def _shift(a, dx, dy):
    """b[x, y] = a[x + dx, y + dy], zero outside the grid (the reference's
    out-of-range reads of the material grids)."""
    nx, ny = a.shape
    out = torch.zeros_like(a)
    xs, xe = max(0, -dx), min(nx, nx - dx)
    ys, ye = max(0, -dy), min(ny, ny - dy)
    if xs < xe and ys < ye:
        out[xs:xe, ys:ye] = a[xs + dx:xe + dx, ys + dy:ye + dy]
    return out


def default_checkpoint_interval(n_steps):
    return int(math.ceil(math.sqrt(n_steps)))


class AdjointProblem:
    """A 2D host model (:class:`~taichi_sim_gb300.sim_support.simulator.Simulator`)
    whose geometry, CPML, attenuation, sources and receivers are fixed and
    whose material is a differentiable input.

    ``checkpoint_every``: None = ceil(sqrt(n_steps)); 0 = keep every step's
    features (6 floats per node and step of device memory).
    ``record_segments``: trailing segments of a checkpointed run that the
    forward pass records, so that the backward pass does not recompute
    them (6 floats per node and step of each; at least 1).
    """

    def __init__(self, sim, checkpoint_every=None, visco=None, device=None, record_segments=1):
        if sim._dims != 2:
            raise ValueError("the adjoint covers 2D models")
        self._lib = _bind(engine.load_library())
        self.sim = sim
        self.device = torch.device(device or "cuda")
        dsc = engine.Stepper.__new__(engine.Stepper)
        dsc.sim = sim
        dsc.family = engine.WGSL2D
        if visco is None:
            visco = bool(sim._configs.get("simul_configs", {}).get("viscoelastic_attn", 0))
        dsc.visco = visco
        dsc.shape = sim.grid_shape()
        dsc.n_rows = int(sim._n_steps)
        dsc.n_rec = int(sim._n_rec)
        dsc._keep = []
        desc = dsc._describe()
        self._src_shape = dsc._src_shape
        self.visco = visco
        self.shape = tuple(dsc.shape)
        self.n_rows, self.n_rec = dsc.n_rows, dsc.n_rec
        self.dt = float(np.float32(sim._dt))
        if checkpoint_every is None:
            checkpoint_every = default_checkpoint_interval(self.n_rows)
        self.checkpoint_every = int(checkpoint_every)
        self._per_cell_q = getattr(sim, "_zener_fit", None) is not None and visco
        with torch.cuda.device(self.device):
            h = _P()
            _check(self._lib, self._lib.ts_adj_create(ctypes.byref(desc), self.checkpoint_every, ctypes.byref(h)),
                   "ts_adj_create")
        self._h = h
        self.record_segments = int(record_segments)
        if self.checkpoint_every > 0 and self.record_segments != 1:
            n_seg = -(-self.n_rows // self.checkpoint_every)
            _check(self._lib, self._lib.ts_adj_set_record_segments(self._h, min(self.record_segments, n_seg)),
                   "ts_adj_set_record_segments")
        p = ctypes.c_int32()
        _check(self._lib, self._lib.ts_adj_pitch(self._h, ctypes.byref(p)), "ts_adj_pitch")
        self.pitch = p.value
        self._g = None
        if self._per_cell_q:
            g_p, g_s = sim.cell_scales()
            self._g = (self._pad(torch.as_tensor(g_p, dtype=torch.float32)),
                       self._pad(torch.as_tensor(g_s, dtype=torch.float32)))
        self._token = 0          # identifies the forward the handle holds
        self._next_token = 1

    # -- material ----------------------------------------------------------------
    def material(self, dtype=torch.float32):
        """(lambda, mu, rho) per cell of the host model, on the device."""
        sim = self.sim
        rho = torch.as_tensor(np.asarray(sim._rho_grid_vx, np.float64))
        cp = torch.as_tensor(np.asarray(sim._cp_grid_vx, np.float64))
        cs = torch.as_tensor(np.asarray(sim._cs_grid_vx, np.float64))
        mu = rho * cs * cs
        lam = rho * cp * cp - 2.0 * mu
        return tuple(t.to(self.device, dtype) for t in (lam, mu, rho))

    def _pad(self, a):
        a = a.to(self.device, torch.float32)
        return torch.nn.functional.pad(a, (0, self.pitch - a.shape[1])).contiguous()

    def node_coefficients(self, lam, mu, rho):
        """Per-node (L, M, Ms, Bx, By) on the padded device layout from per-cell
        lambda, mu, rho (differentiable).  cp and cs are recovered per cell
        and averaged as the reference does (cs = 0 on either side of a
        stress node gives mu = 0 there; such cells get no mu gradient)."""
        dt = self.dt
        pos = mu > 0
        mu_safe = torch.where(pos, mu, torch.ones_like(mu))
        cs = torch.where(pos, torch.sqrt(mu_safe / rho), torch.zeros_like(mu))
        cp = torch.sqrt((lam + 2.0 * mu) / rho)
        rh = 0.5 * (_shift(rho, 1, 0) + rho)
        cph = 0.5 * (_shift(cp, 1, 0) + cp)
        c1 = _shift(cs, 1, 0)
        csl = 0.5 * (c1 + cs)
        csm = torch.where(torch.minimum(c1, cs) == 0, torch.zeros_like(csl), csl)
        L = rh * (cph * cph - 2.0 * csl * csl) * dt
        M = rh * (csm * csm) * dt
        rhy = 0.5 * (_shift(rho, 0, 1) + rho)
        s1 = _shift(cs, 0, 1)
        csh = torch.where(torch.minimum(s1, cs) == 0, torch.zeros_like(cs), 0.5 * (s1 + cs))
        Ms = rhy * (csh * csh) * dt
        rpos = rho > 0
        Bx = torch.where(rpos, dt / torch.where(rpos, rho, torch.ones_like(rho)), torch.zeros_like(rho))
        r4 = 0.25 * (rho + _shift(rho, 1, 0) + _shift(rho, 1, 1) + _shift(rho, 0, 1))
        r4pos = r4 > 0
        By = torch.where(r4pos, dt / torch.where(r4pos, r4, torch.ones_like(r4)), torch.zeros_like(r4))
        return tuple(self._pad(t) for t in (L, M, Ms, Bx, By))

    # -- shots -----------------------------------------------------------------------
    def set_source_term(self, source_term):
        """Replace the source table (``[n_steps][src_cols]``, the host model's layout)."""
        st = np.asarray(source_term, dtype=np.float32)
        st2 = np.ascontiguousarray(st[:, None] if st.ndim == 1 else st)
        if st2.shape != self._src_shape:
            raise ValueError(f"source term shape {st2.shape} != {self._src_shape}")
        _check(self._lib, self._lib.ts_adj_set_sources(self._h, st2.ctypes.data_as(_f)), "ts_adj_set_sources")
        self._token = 0

    # -- raw calls (device tensors, current stream) -------------------------------------
    def _stream(self):
        return torch.cuda.current_stream(self.device).cuda_stream

    def forward_raw(self, L, M, Ms, Bx, By):
        """Traces ``[n_steps][n_rec]`` for node coefficients on the padded layout."""
        coefs = [c.detach().to(self.device, torch.float32).contiguous() for c in (L, M, Ms, Bx, By)]
        for c in coefs:
            if tuple(c.shape) != (self.shape[0], self.pitch):
                raise ValueError(f"coefficient shape {tuple(c.shape)} != {(self.shape[0], self.pitch)}")
        c = AdjCoefs(*[t.data_ptr() for t in coefs],
                     self._g[0].data_ptr() if self._g else None, self._g[1].data_ptr() if self._g else None)
        traces = torch.empty((self.n_rows, max(self.n_rec, 1)), device=self.device, dtype=torch.float32)
        _check(self._lib, self._lib.ts_adj_forward(self._h, ctypes.byref(c), traces.data_ptr(), self._stream()),
               "ts_adj_forward")
        self._hold = coefs + [traces]   # alive until the enqueued work has run
        self._token = self._next_token
        self._next_token += 1
        return traces[:, :self.n_rec], self._token

    def backward_raw(self, residual, token=None):
        """Gradients (gL, gM, gMs, gBx, gBy) of sum(residual * traces) for the
        last forward."""
        if token is not None and token != self._token:
            raise RuntimeError("the adjoint handle no longer holds this forward (another forward or "
                               "set_source_term ran in between): call backward before the next forward")
        if self._token == 0:
            raise RuntimeError("no forward to differentiate")
        res = torch.zeros((self.n_rows, max(self.n_rec, 1)), device=self.device, dtype=torch.float32)
        res[:, :self.n_rec] = residual.to(self.device, torch.float32)
        grads = [torch.empty((self.shape[0], self.pitch), device=self.device, dtype=torch.float32)
                 for _ in range(5)]
        g = AdjGrads(*[t.data_ptr() for t in grads])
        _check(self._lib, self._lib.ts_adj_backward(self._h, res.data_ptr(), ctypes.byref(g), self._stream()),
               "ts_adj_backward")
        self._hold_b = [res]
        return tuple(grads)

    # -- differentiable calls ---------------------------------------------------------
    def traces_from_coefficients(self, L, M, Ms, Bx, By):
        return TraceFunction.apply(self, L, M, Ms, Bx, By)

    def traces(self, lam, mu, rho):
        """Receiver traces ``[n_steps][n_rec]`` (differentiable in lam, mu, rho)."""
        return self.traces_from_coefficients(*self.node_coefficients(lam, mu, rho))

    def read_field(self, name):
        """A forward field (vx, vy, sxx, syy, sxy) after the last forward, [nx][ny]."""
        out = np.zeros(self.shape, np.float32)
        _check(self._lib, self._lib.ts_adj_read_field(self._h, engine.FIELD_NAMES[name], out.ctypes.data,
                                                      out.nbytes), "ts_adj_read_field")
        return out

    def launch_count(self):
        n = ctypes.c_int64()
        _check(self._lib, self._lib.ts_adj_launch_count(self._h, ctypes.byref(n)), "ts_adj_launch_count")
        return n.value

    def close(self):
        if getattr(self, "_h", None):
            self._lib.ts_adj_destroy(self._h)
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


class TraceFunction(torch.autograd.Function):
    """traces = F(L, M, Ms, Bx, By); backward runs the adjoint on the GPU."""

    @staticmethod
    def forward(ctx, problem, L, M, Ms, Bx, By):
        traces, token = problem.forward_raw(L, M, Ms, Bx, By)
        ctx.problem, ctx.token = problem, token
        return traces.clone()

    @staticmethod
    def backward(ctx, g):
        grads = ctx.problem.backward_raw(g.contiguous(), ctx.token)
        return (None, *grads)


def l2_misfit(traces, observed):
    """0.5 * sum((traces - observed)^2), the misfit the gradient is checked on."""
    d = traces - observed
    return 0.5 * (d * d).sum()
