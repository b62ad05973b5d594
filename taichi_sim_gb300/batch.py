"""Batched shots: many shots of several phantoms in one device pass.

The reference runs one complete simulation per emission law
(``Simulator.run()`` -> ``implementation()``, sim_support/simulator.py:326-337),
re-uploading every table each time.  :class:`BatchStepper` advances every
shot of every phantom together (``ts_batch_*`` in the C ABI): per phantom
the shot index is the innermost array axis, so a warp computes 32 shots of
one grid node and the per-node coefficients are read once for all shots.

:func:`fmc_shot_sources` builds the shots of a full-matrix capture (shot e
fires element e of a linear array); :func:`focal_law_shot_sources` the shots
of emission laws (delay rows from a ``.law`` file, :func:`plane_wave_laws`
or :func:`focused_laws`); :func:`autotune` picks the launch shapes by timing
each candidate and caches the choice in ``_build/autotune.json``.
"""
import ctypes
import json
import os
import time

import numpy as np

from . import engine

_f = ctypes.POINTER(ctypes.c_float)


class BatchDesc(ctypes.Structure):
    _fields_ = [("abi_version", ctypes.c_int32), ("n_phantoms", ctypes.c_int32),
                ("phantoms", ctypes.POINTER(engine.TsDesc)), ("n_shots", ctypes.POINTER(ctypes.c_int32)),
                ("shot_sources", ctypes.POINTER(_f)), ("block_cells", ctypes.c_int32),
                ("nodes_per_thread", ctypes.c_int32), ("shots_per_thread", ctypes.c_int32),
                ("velocity_block_cells", ctypes.c_int32), ("velocity_nodes_per_thread", ctypes.c_int32)]


def _bind(lib):
    if getattr(lib, "_batch_bound", False):
        return lib
    P = ctypes.c_void_p
    sigs = {
        "ts_batch_create": ([ctypes.POINTER(BatchDesc), ctypes.POINTER(P)], ctypes.c_int),
        "ts_batch_run": ([P, ctypes.c_int32, P], ctypes.c_int),
        "ts_batch_reset": ([P, P], ctypes.c_int),
        "ts_batch_status": ([P, ctypes.POINTER(ctypes.c_int32), _f, ctypes.POINTER(ctypes.c_int32)], ctypes.c_int),
        "ts_batch_read_traces": ([P, ctypes.c_int32, P, ctypes.c_size_t], ctypes.c_int),
        "ts_batch_read_field": ([P, ctypes.c_int32, ctypes.c_int32, P, ctypes.c_size_t], ctypes.c_int),
        "ts_batch_profile_steps": ([P, ctypes.c_int32, P, _f], ctypes.c_int),
        "ts_batch_launch_count": ([P, ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
        "ts_batch_transfer_bytes": ([P, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)],
                                    ctypes.c_int),
        "ts_batch_destroy": ([P], None),
        "ts_batch_last_error": ([], ctypes.c_char_p),
    }
    for name, (args, res) in sigs.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    lib._batch_bound = True
    return lib


def _check(lib, rc, where):
    if rc != 0:
        raise RuntimeError(f"{where}: {lib.ts_strerror(rc).decode()} ({lib.ts_batch_last_error().decode()})")


def fmc_shot_sources(sim):
    """Full-matrix capture shots of a model whose first emitting probe is a
    linear array with every element emitting: shot e keeps column e of the
    source term and silences the others.  Returns ``[n_elem][n_steps][n_elem]``."""
    st = np.asarray(sim._source_term, np.float32)
    st = st[:, None] if st.ndim == 1 else st
    n_steps, n_col = st.shape
    shots = np.zeros((n_col, n_steps, n_col), np.float32)
    for e in range(n_col):
        shots[e, :, e] = st[:, e]
    return shots


def focal_law_shot_sources(sim, laws):
    """Shots of focal laws (plane-wave or focused transmissions): law k is one
    emission delay per element (the probes' ``t0_emission`` units), applied
    with ``set_t0`` as the reference's ``run()`` does
    (sim_support/simulator.py:328-333) to every emitting array (a point or
    single-element probe takes the law's first delay), and shot k's table is
    the source term built with those delays (``EmissionLaw.read_law`` gives
    such delay rows from a ``.law`` file).  The probes' delays are restored
    afterwards.  Returns ``[n_laws][n_steps][src_cols]``."""
    saved = [getattr(p, "_t0_emission", None) for p in sim._probes]
    tables = []
    try:
        for law in laws:
            row = np.atleast_1d(np.asarray(law, dtype=np.float32))
            for i in sim._emitting_probes:
                p = sim._probes[i]
                p.set_t0(row.copy() if hasattr(p, "num_elem") else np.float32(row[0]))
            st = np.asarray(sim.build_source_term(), np.float32)
            tables.append(st[:, None] if st.ndim == 1 else st)
    finally:
        for p, t0 in zip(sim._probes, saved):
            if t0 is not None:
                p.set_t0(t0)
    return np.ascontiguousarray(np.stack(tables))


def _array_element_x(sim):
    """Lateral (x) centres, mm from the ROI origin, of the elements of the
    model's first emitting linear array."""
    for i in sim._emitting_probes:
        probe = sim._probes[i]
        if hasattr(probe, "elem_list"):
            cx = float(np.asarray(probe.coord_center, np.float64).ravel()[0])
            return np.array([cx + float(e.coord_center[0]) for e in probe.elem_list], np.float64), probe
    raise ValueError("the model has no emitting linear array")


def _base_t0(probe):
    t0 = getattr(probe, "_t0_emission", None)
    return float(np.min(t0)) if t0 is not None else 0.0


def plane_wave_laws(sim, angles_deg, c=None):
    """Emission delays (one row per angle, the probes' t0_emission units)
    that steer a plane wave from the model's first emitting linear array by
    each angle (degrees from the array normal, positive towards +x), for a
    sound speed ``c`` (mm per time unit; default: the specimen's cp).  The
    earliest element of each law fires at the array's current smallest
    delay.  An extension: the reference reads and writes laws
    (sim_support/emission_law.py) but does not compute them."""
    x, probe = _array_element_x(sim)
    c = float(sim._configs["specimen_params"]["cp"] if c is None else c)
    rows = []
    for a in np.atleast_1d(angles_deg):
        d = (x - x.min()) * np.sin(np.deg2rad(float(a))) / c
        rows.append(_base_t0(probe) + d - d.min())
    return np.asarray(rows, np.float32)


def focused_laws(sim, focal_points, c=None):
    """Emission delays (one row per focal point (x, z), mm from the ROI
    origin) that focus the model's first emitting linear array at each point:
    element e fires (r_max - r_e) / c after the array's current smallest
    delay, r_e its distance to the focus (elements at the depth of the
    probe centre).  An extension, as :func:`plane_wave_laws`."""
    x, probe = _array_element_x(sim)
    c = float(sim._configs["specimen_params"]["cp"] if c is None else c)
    z0 = float(np.asarray(probe.coord_center, np.float64).ravel()[-1])
    rows = []
    for fx, fz in np.atleast_2d(np.asarray(focal_points, np.float64)):
        r = np.hypot(x - fx, fz - z0)
        rows.append(_base_t0(probe) + (r.max() - r) / c)
    return np.asarray(rows, np.float32)


def run_emission_laws(sim, laws=None, field="syy"):
    """Every emission law of a 2D model as shots of one batched launch.

    ``laws`` defaults to the model's ``.law`` file rows (``_emission_laws``,
    read in the constructor as sim_support/simulator.py:228-230 does); the
    reference instead runs ``implementation()`` once per law
    (sim_support/simulator.py:326-337).  Returns ``(traces, fields)``:
    ``[n_laws, n_steps, n_rec]`` and ``[n_laws, nx, ny]``."""
    if laws is None:
        if not hasattr(sim, "_emission_laws"):
            raise ValueError("the model has no emission laws; pass laws=")
        laws = list(sim._emission_laws)
    shots = focal_law_shot_sources(sim, laws)
    with BatchStepper([sim], [shots]) as b:
        b.run(sim._n_steps)
        _, vmax, bad = b.status()
        if bad >= 0:
            raise engine.StabilityError("Simulacao tornando-se instavel", float(np.sqrt(np.float32(vmax))))
        return b.traces(0), b.field(0, field)


class BatchStepper:
    """Every shot of several phantoms advanced together on the GPU.

    ``sims`` are 2D host models (one per phantom, WGSL semantics, sharing
    ``acc``, ``dt``, ``time_steps`` and the attenuation model); ``shot_sources[p]``
    is ``[n_shots, n_steps, src_cols]`` for phantom p.
    """

    def __init__(self, sims, shot_sources, block_cells=0, nodes_per_thread=0, shots_per_thread=0,
                 velocity_block_cells=0, velocity_nodes_per_thread=0):
        self._lib = _bind(engine.load_library())
        self.sims = list(sims)
        self.n_ph = len(self.sims)
        self._describers = [engine.Stepper.__new__(engine.Stepper) for _ in self.sims]
        descs = (engine.TsDesc * self.n_ph)()
        keep = []
        for q, (sim, dsc) in enumerate(zip(self.sims, self._describers)):
            dsc.sim = sim
            dsc.family = engine.WGSL2D
            dsc.visco = bool(sim._configs.get("simul_configs", {}).get("viscoelastic_attn", 0))
            dsc.shape = sim.grid_shape()
            dsc.n_rows = int(sim._n_steps)
            dsc.n_rec = int(sim._n_rec)
            dsc._keep = []
            descs[q] = dsc._describe()
            keep.append(dsc._keep)
        self.shot_sources = [np.ascontiguousarray(np.asarray(s, np.float32)) for s in shot_sources]
        self.n_shots = [int(s.shape[0]) for s in self.shot_sources]
        for q, s in enumerate(self.shot_sources):
            if s.shape[1:] != self._describers[q]._src_shape:
                raise ValueError(f"phantom {q}: shot table {s.shape[1:]} != source term {self._describers[q]._src_shape}")
        n_shots = (ctypes.c_int32 * self.n_ph)(*self.n_shots)
        ptrs = (_f * self.n_ph)(*[s.ctypes.data_as(_f) for s in self.shot_sources])
        bd = BatchDesc(abi_version=engine.ABI_VERSION, n_phantoms=self.n_ph, phantoms=descs, n_shots=n_shots,
                       shot_sources=ptrs, block_cells=int(block_cells), nodes_per_thread=int(nodes_per_thread),
                       shots_per_thread=int(shots_per_thread), velocity_block_cells=int(velocity_block_cells),
                       velocity_nodes_per_thread=int(velocity_nodes_per_thread))
        h = ctypes.c_void_p()
        _check(self._lib, self._lib.ts_batch_create(ctypes.byref(bd), ctypes.byref(h)), "ts_batch_create")
        self._h = h
        self.n_rows = int(self.sims[0]._n_steps)
        del keep

    def run(self, n_steps, stream=None):
        _check(self._lib, self._lib.ts_batch_run(self._h, int(n_steps), ctypes.c_void_p(stream or 0)), "ts_batch_run")

    def reset(self, stream=None):
        _check(self._lib, self._lib.ts_batch_reset(self._h, ctypes.c_void_p(stream or 0)), "ts_batch_reset")

    def status(self):
        n, m, b = ctypes.c_int32(), ctypes.c_float(), ctypes.c_int32()
        _check(self._lib, self._lib.ts_batch_status(self._h, ctypes.byref(n), ctypes.byref(m), ctypes.byref(b)),
               "ts_batch_status")
        return n.value, m.value, b.value

    def traces(self, phantom):
        """``[n_shots, n_steps, n_rec]`` traces of one phantom."""
        sim = self.sims[phantom]
        out = np.zeros((self.n_shots[phantom], self.n_rows, sim._n_rec), np.float32)
        _check(self._lib, self._lib.ts_batch_read_traces(self._h, phantom, out.ctypes.data_as(ctypes.c_void_p),
                                                         out.nbytes), "ts_batch_read_traces")
        return out

    def field(self, phantom, what="syy"):
        """``[n_shots, nx, ny]`` field of every shot of one phantom."""
        sim = self.sims[phantom]
        out = np.zeros((self.n_shots[phantom],) + tuple(sim.grid_shape()), np.float32)
        code = engine.FIELD_NAMES[what]
        _check(self._lib, self._lib.ts_batch_read_field(self._h, phantom, code, out.ctypes.data_as(ctypes.c_void_p),
                                                        out.nbytes), "ts_batch_read_field")
        return out

    def profile_steps(self, n_steps, stream=None):
        out = (ctypes.c_float * 2)()
        _check(self._lib, self._lib.ts_batch_profile_steps(self._h, int(n_steps), ctypes.c_void_p(stream or 0),
                                                           ctypes.cast(out, _f)), "ts_batch_profile_steps")
        return list(out)

    def launch_count(self):
        n = ctypes.c_int64()
        _check(self._lib, self._lib.ts_batch_launch_count(self._h, ctypes.byref(n)), "ts_batch_launch_count")
        return n.value

    def transfer_bytes(self):
        """``(host->device, device->host)`` bytes this batch has copied so far."""
        a, b = ctypes.c_int64(), ctypes.c_int64()
        _check(self._lib, self._lib.ts_batch_transfer_bytes(self._h, ctypes.byref(a), ctypes.byref(b)),
               "ts_batch_transfer_bytes")
        return a.value, b.value

    def close(self):
        if getattr(self, "_h", None):
            self._lib.ts_batch_destroy(self._h)
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


def _cache_path():
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "autotune.json")


def _key(sims, shot_sources):
    shapes = [list(s.grid_shape()) for s in sims]
    return json.dumps({"grids": shapes, "shots": [int(np.shape(x)[0]) for x in shot_sources],
                       "acc": int(sims[0]._coefs.shape[0]),
                       "visco": bool(sims[0]._configs.get("simul_configs", {}).get("viscoelastic_attn", 0))},
                      sort_keys=True)


# (block_cells, nodes_per_thread, shots_per_thread) of order-2 batches
SHAPES = tuple((cy, tx, spt) for spt in (1, 2) for cy in (4, 8) for tx in (1, 2, 4))


def pick_shapes(timings):
    """The launch shapes of the shortest step from per-shape kernel timings
    ``{"CYxTXxSPT": [stress_ms, velocity_ms]}``: per shot layout (SPT) the
    stress and velocity launches each take their fastest (CY, TX), and the
    layout with the smallest sum wins.  Returns BatchStepper keyword
    arguments."""
    best, best_ms = None, float("inf")
    for spt in sorted({int(k.split("x")[2]) for k in timings}):
        mine = {k: v for k, v in timings.items() if int(k.split("x")[2]) == spt}
        ks = min(mine, key=lambda k: mine[k][0])
        kv = min(mine, key=lambda k: mine[k][1])
        if mine[ks][0] + mine[kv][1] < best_ms:
            best_ms = mine[ks][0] + mine[kv][1]
            cs, ts_, _ = (int(v) for v in ks.split("x"))
            cv, tv, _ = (int(v) for v in kv.split("x"))
            best = {"block_cells": cs, "nodes_per_thread": ts_, "shots_per_thread": spt,
                    "velocity_block_cells": cv, "velocity_nodes_per_thread": tv}
    return best


def autotune(sims, shot_sources, candidates=SHAPES, steps=12, use_cache=True):
    """Pick the launch shapes with the shortest measured step on this GPU.

    A shape is ``(block_cells, nodes_per_thread, shots_per_thread)``: blocks
    of 32 lanes x block_cells nodes along y, nodes_per_thread nodes along x
    and shots_per_thread shots per thread.  Every candidate is timed with
    both kernels at that shape; then, per shot layout (shots_per_thread, which
    the two kernels share), the stress and the velocity launch each take
    their fastest (block_cells, nodes_per_thread), and the layout with the
    shortest step wins.  Order-4 models have the default shape only.  The
    choice is cached per problem shape.  Returns ``(shape, timings)``: shape
    is a dict of :class:`BatchStepper` keyword arguments, timings
    ``{"CYxTXxSPT": [stress_ms, velocity_ms]}`` per step."""
    key = _key(sims, shot_sources)
    path = _cache_path()
    cache = {}
    if use_cache and os.path.exists(path):
        try:
            with open(path) as f:
                cache = json.load(f)
        except (OSError, ValueError):
            cache = {}
        if key in cache and isinstance(cache[key].get("shape"), dict):
            return dict(cache[key]["shape"]), cache[key]["timings"]
    timings = {}
    if int(sims[0]._coefs.shape[0]) != 2:
        candidates = ((8, 2, 1),)
    for cy, tx, spt in candidates:
        with BatchStepper(sims, shot_sources, block_cells=cy, nodes_per_thread=tx, shots_per_thread=spt) as b:
            b.profile_steps(2)
            timings[f"{cy}x{tx}x{spt}"] = [float(v) for v in b.profile_steps(steps)]
    best = pick_shapes(timings)
    cache[key] = {"shape": best, "timings": timings, "when": time.time()}
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "w") as f:
        json.dump(cache, f, indent=1)
    return dict(best), timings
