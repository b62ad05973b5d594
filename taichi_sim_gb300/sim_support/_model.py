"""Shared set-up of the 2D and 3D host models.

Builds, from a JSON experiment description, every table the time stepper
reads.  The reference implements this twice (sim_support/simulator.py:18-318
for 2D and sim_support/Simulator3D.py:18-337 for 3D); both are restated here
once, parameterised by the number of dimensions, with the attribute names the
reference's backends read (``_nx``, ``_a_x_half``, ``_pos_sources``,
``_info_rec_pt`` ...).

Deliberate departures from the reference, each of which only affects inputs
on which the reference raises:

* ``emission_laws`` naming a ``.law`` file is read through an
  :class:`EmissionLaw` instance (the reference calls ``read_law`` unbound,
  simulator.py:230, which raises ``TypeError``).
* a 3D ``cp_map`` fills a 3D grid (Simulator3D.py:107-108 allocates a 2D one).
* ``file_config`` may also be a ``dict`` and a ``*_map`` entry an ndarray, so
  synthetic experiments need no files.

Additions (absent from the reference, inert unless configured):
``specimen_params`` ``qp``/``qs`` (+ ``qp_map``/``qs_map``) and
``simul_configs.zener_fit = {"f_min", "f_max"}`` switch the viscoelastic
stepper to per-cell quality factors fitted by :class:`ZenerFit`.
"""
import ast
import os.path

import numpy as np

from . import flt32, int32, PI, coefs_Lui, coefs_forward, CourantError
from .emission_law import EmissionLaw
from .simul_classes import (SimulationROI, SimulationProbeLinearArray, SimulationProbePoint,
                            SimulationProbeMonoCirc, SimulationProbeMatrix)

# (save_snapshots is an addition: the headless stand-in for the live view,
# which show_anim also turns on)
_CONFIG_FLAGS = ("show_anim", "show_debug", "show_figs", "plot_results", "plot_error", "plot_sensors",
                 "plot_bscan", "save_results", "save_field", "save_sensors", "save_bscan", "save_sources",
                 "source_env", "save_snapshots")


def load_config(file_config):
    """Parse an experiment description (Python-literal JSON file, or a dict)."""
    if isinstance(file_config, dict):
        return file_config
    with open(os.path.normpath(file_config), 'r') as f:
        return ast.literal_eval(f.read())


def _load_map(spec):
    if isinstance(spec, np.ndarray):
        return spec.astype(flt32)
    return np.load(os.path.normpath(spec)).astype(flt32)


class ModelBase:
    """Everything ``Simulator``/``Simulator3D`` compute before any time step."""

    _dims = 2

    def __init__(self, file_config, sim_model="split", sim_type="acoustic"):
        self._app = None
        self._device = None
        self._name = "simulator"
        self._sim_model = sim_model
        self._sim_type = sim_type
        self._configs = load_config(file_config)
        cfg = self._configs

        self._deriv_acc = cfg.get("simul_params", 2).get("acc", 2)
        table = coefs_forward if sim_model == "unsplit" else coefs_Lui
        try:
            self._coefs = np.array(table[self._deriv_acc - 2], dtype=flt32)
        except IndexError:
            print(f"Acurácia das derivadas {self._deriv_acc} não suportada. Usando o maior valor permitido (6).")
            self._coefs = np.array(table[-1], dtype=flt32)

        sp = cfg.get("simul_params", {})
        self._n_steps = sp.get("time_steps", 1000)
        self._dt = flt32(sp.get("dt", 1.0))
        self._it_display = sp.get("it_display", 10)
        self.cpml_time = sp.get("cpml_time", 1000)

        spec = cfg["specimen_params"]
        self._cp = flt32(spec.get("cp", 5.9))
        self._cs = flt32(spec.get("cs", 3.23))
        self._rho = flt32(spec.get("rho", 7800.0))
        for key in ("cp_map", "cs_map", "rho_map", "qp_map", "qs_map"):
            if key in spec:
                setattr(self, "_" + key, _load_map(spec[key]))

        pad = self._deriv_acc - 1
        roi_kw = dict(cfg["roi"], pad=pad)
        if hasattr(self, "_rho_map"):
            roi_kw["rho_map"] = self._rho_map
        self._roi = SimulationROI(**roi_kw)
        self._setup_grid()
        self._setup_materials()
        self._check_courant()
        self._setup_probes()
        self._setup_pml()
        self._setup_flags()
        self._setup_sources_receivers()
        self._setup_attenuation()
        self._app = None
        self._windows_gpu = list()

    # -- grid -----------------------------------------------------------------
    def _setup_grid(self):
        roi = self._roi
        self._nx = roi.get_nx()
        if self._dims == 2:
            # The 2D model's second axis is the ROI height (z).
            self._ny, self._nz = roi.get_nz(), roi.get_ny()
            self._dx, self._dy, self._dz = roi.get_dx(), roi.get_dz(), roi.get_dy()
        else:
            self._ny, self._nz = roi.get_ny(), roi.get_nz()
            self._dx, self._dy, self._dz = roi.get_dx(), roi.get_dy(), roi.get_dz()
        self._one_dx = flt32(1.0 / self._dx)
        self._one_dy = flt32(1.0 / self._dy)
        self._one_dz = flt32(1.0 / self._dz)

    def grid_shape(self):
        return (self._nx, self._ny) if self._dims == 2 else (self._nx, self._ny, self._nz)

    def _roi_slices(self):
        roi = self._roi
        if self._dims == 2:
            return (slice(roi.get_ix_min(), roi.get_ix_max()), slice(roi.get_iz_min(), roi.get_iz_max()))
        return (slice(roi.get_ix_min(), roi.get_ix_max()), slice(roi.get_iy_min(), roi.get_iy_max()),
                slice(roi.get_iz_min(), roi.get_iz_max()))

    def _material_grid(self, value, name):
        """Full-grid map of ``value`` with an optional ROI/full/oversized map."""
        shape = self.grid_shape()
        grid = np.ones(shape, dtype=flt32) * value
        m = getattr(self, "_" + name, None)
        if m is None:
            return grid
        if all(a < b for a, b in zip(m.shape, shape)):
            grid[self._roi_slices()] = m
        elif all(a > b for a, b in zip(m.shape, shape)):
            grid = m[tuple(slice(0, n) for n in shape)]
        elif tuple(m.shape) == tuple(shape):
            grid = m
        else:
            raise ValueError(f'{name} shape {m.shape} e incompativel com a ROI')
        return grid

    def _setup_materials(self):
        self._rho_grid_vx = self._material_grid(self._rho, "rho_map")
        # The reference overwrites the density grid in place with its
        # 2^dims-point average (the "vy" grid aliases the "vx" grid,
        # simulator.py:101-105 / Simulator3D.py:97-103): every backend then
        # reads the averaged density.  Kept, as it changes every result.
        r = self._rho_grid_vx
        self._rho_grid_vy = r
        if self._dims == 2:
            r[:-1, :-1] = flt32(0.25) * (r[:-1, :-1] + r[1:, :-1] + r[1:, 1:] + r[:-1, 1:])
        else:
            r[:-1, :-1, :-1] = flt32(0.125) * (
                r[:-1, :-1, :-1] + r[1:, :-1, :-1] + r[:-1, 1:, :-1] + r[1:, 1:, :-1] +
                r[:-1, :-1, 1:] + r[1:, :-1, 1:] + r[:-1, 1:, 1:] + r[1:, 1:, 1:])
        self._cp_grid_vx = self._material_grid(self._cp, "cp_map")
        self._cs_grid_vx = self._material_grid(self._cs, "cs_map")

    def _check_courant(self):
        cp_max = max(self._cp_grid_vx.max(), self._cp)
        inv2 = self._one_dx ** 2 + self._one_dy ** 2
        if self._dims == 3:
            inv2 = inv2 + self._one_dz ** 2
        courant = flt32(cp_max * self._dt * np.sqrt(inv2))
        self._cp_max = cp_max
        print(f'\nNumero de Courant e {courant}')
        if courant > 1.0:
            if self._dims == 2:
                raise CourantError("O passo de tempo e muito longo e a simulacao sera instavel", courant)
            raise Exception("O passo de tempo e muito longo e a simulacao sera instavel", courant)

    # -- probes -----------------------------------------------------------------
    def _setup_probes(self):
        self._probes = list()
        self._gain = flt32(0.0)
        dec = self._roi.get_dec()
        kinds = {"linear": SimulationProbeLinearArray, "point": SimulationProbePoint,
                 "mono": SimulationProbeMonoCirc, "matrix": SimulationProbeMatrix}
        self._probe_kinds = list()
        for p in self._configs["probes"]:
            kind = next((k for k in kinds if k in p), None)
            if kind is None:
                raise KeyError(f"unknown probe type in {list(p)}")
            self._probes.append(kinds[kind](**p[kind], dec=dec))
            self._probe_kinds.append(kind)
            g = getattr(self._probes[-1], "_gain", None)
            self._gain = max(self._gain, flt32(g) if g is not None else 0.0)

        stype = "2d" if self._dims == 2 else "3d"
        tx, rx, delays = list(), list(), list()
        self._n_rec = 0
        self._n_src = 0
        for pr in self._probes:
            tx += pr.get_points_roi(self._roi, simul_type=stype, dir="e")[0]
            rx += pr.get_points_roi(self._roi, simul_type=stype, dir="r")[0]
            delays += pr.get_delay_rx()
            self._n_rec += pr.receivers.count(True)
            self._n_src += pr.emitters.count(True)
        tx = np.array(tx, dtype=int32).reshape(-1, 3)
        rx = np.array(rx, dtype=int32).reshape(-1, 3)
        self._ix_src = tx[:, 0].astype(int32)
        self._ix_rec = rx[:, 0].astype(int32)
        if self._dims == 2:
            self._iy_src = tx[:, 2].astype(int32)
            self._iy_rec = rx[:, 2].astype(int32)
        else:
            self._iy_src, self._iz_src = tx[:, 1].astype(int32), tx[:, 2].astype(int32)
            self._iy_rec, self._iz_rec = rx[:, 1].astype(int32), rx[:, 2].astype(int32)
        self._n_pto_src = tx.shape[0]
        self._delay_recv = (np.array(delays) / self._dt + 1.0).astype(int32)

    def _setup_pml(self):
        # 2D uses the float32 pi constant, 3D numpy's float64 pi
        # (simulator.py:185, Simulator3D.py:188).
        pi = PI if self._dims == 2 else np.pi
        alpha_max = flt32(2.0 * pi * (self._probes[0].get_freq() / 2.0))
        self._alpha_max_pml = alpha_max
        roi, dt, cp = self._roi, self._dt, self._cp_max
        names = ("x", "y") if self._dims == 2 else ("x", "y", "z")
        roi_axes = ("x", "z") if self._dims == 2 else ("x", "y", "z")
        for k, (name, ax) in enumerate(zip(names, roi_axes)):
            if self._dims == 2:
                expand = (1,) if k == 0 else (0,)
            else:
                expand = tuple(i for i in range(3) if i != k)
            for grid, suffix in (("f", ""), ("h", "_half")):
                a, b, kk = roi.calc_pml_array(axis=ax, grid=grid, dt=dt, cp=cp, alpha_max=alpha_max)
                setattr(self, f"_a_{name}{suffix}", np.expand_dims(a.astype(flt32), axis=expand))
                setattr(self, f"_b_{name}{suffix}", np.expand_dims(b.astype(flt32), axis=expand))
                setattr(self, f"_k_{name}{suffix}", np.expand_dims(kk.astype(flt32), axis=expand))

    def _setup_flags(self):
        sc = self._configs.get("simul_configs", {})
        self._n_iter = sc.get("n_iter", 1)
        self._max_val_fields = flt32(sc.get("max_val_fields", 100.0))
        self._min_val_fields = flt32(sc.get("min_val_fields", -100.0))
        for key in _CONFIG_FLAGS:
            setattr(self, "_" + key, bool(sc.get(key, False)))
        laws = sc.get("emission_laws")
        if isinstance(laws, str) and os.path.isfile(os.path.normpath(laws)):
            self._emission_laws, _ = EmissionLaw().read_law(os.path.normpath(laws))
        rdir = sc.get("results_dir")
        if isinstance(rdir, str) and os.path.isdir(os.path.normpath(rdir)):
            self._results_dir = os.path.normpath(rdir)

    def _probe_source(self, idx, pr):
        """Source term of one probe, following the reference's dispatch.

        The 2D model's test ``"linear" or "mono" in p`` is always true, so 2D
        always calls ``get_source_term(samples, dt[, out])`` (simulator.py:248);
        the 3D model dispatches on the *last* probe's kind, the loop variable
        left over from parsing (Simulator3D.py:257-277).
        """
        kw = dict(samples=self._n_steps, dt=self._dt)
        if self._source_env:
            kw["out"] = 'e'
        if self._dims == 2:
            return pr.get_source_term(**kw)
        last = self._probe_kinds[-1]
        if last in ("linear", "mono"):
            return pr.get_source_term(**kw)
        return pr.get_source_term(**kw, ord_der=(2 if self._sim_model == "unsplit" else 1))

    def _setup_sources_receivers(self):
        stype = "2d" if self._dims == 2 else "3d"
        rec_type = "2D" if self._dims == 2 else "3d"
        terms, idx_src, idx_rec = list(), list(), list()
        self._idx_src_offset = 0
        self._idx_rec_offset = 0
        self._emitting_probes = list()
        for i, pr in enumerate(self._probes):
            st = self._probe_source(i, pr)
            _, owner = pr.get_points_roi(sim_roi=self._roi, simul_type=stype)
            if len(owner) > 0:
                terms.append(st)
                self._emitting_probes.append(i)
                idx_src += [np.array(s) + self._idx_src_offset for s in owner]
                self._idx_src_offset += len(owner)
            rec_owner = pr.get_idx_rec(sim_roi=self._roi, simul_type=rec_type)
            if len(rec_owner) > 0:
                idx_rec += [np.array(r) + self._idx_rec_offset for r in rec_owner]
                self._idx_rec_offset += len(rec_owner)
        if len(terms) == 0:
            raise ValueError("no emitting probe point lies inside the ROI")
        self._source_term = np.concatenate(terms, axis=1) if len(terms) > 1 else terms[0]

        shape = self.grid_shape()
        self._pos_sources = -np.ones(shape, dtype=int32)
        self._pos_sensors = -np.ones(shape, dtype=int32)
        if self._dims == 2:
            src_at, rec_at = (self._ix_src, self._iy_src), (self._ix_rec, self._iy_rec)
        else:
            src_at = (self._ix_src, self._iy_src, self._iz_src)
            rec_at = (self._ix_rec, self._iy_rec, self._iz_rec)
        self._pos_sources[src_at] = np.array(idx_src).astype(int32).flatten()
        self._pos_sensors[rec_at] = np.array(idx_rec).astype(int32).flatten()
        self._idx_rec = np.array(idx_rec).astype(np.int32).flatten()
        self._info_rec_pt = np.column_stack(rec_at + (self._idx_rec,)).astype(int32)
        ids = list(self._idx_rec)
        offsets = [ids[0]] + [int32(i) for i in range(1, len(ids)) if ids[i] != ids[i - 1]]
        self._offset_sensors = np.array(offsets, dtype=int32)
        self._n_pto_rec = int32(len(ids))

    def build_source_term(self):
        """The source term for the probes' current emission delays, assembled
        as the constructor assembles it (an extension: the reference builds it
        once, so a later ``set_t0`` does not reach its kernels)."""
        terms = [self._probe_source(i, self._probes[i]) for i in self._emitting_probes]
        return np.concatenate(terms, axis=1) if len(terms) > 1 else terms[0]

    def _setup_attenuation(self):
        """Per-cell quality factors (extension); ``None`` keeps global taus."""
        spec = self._configs["specimen_params"]
        fit = self._configs.get("simul_configs", {}).get("zener_fit")
        self._inv_qp_grid = self._inv_qs_grid = None
        self._zener_fit = None
        if fit is None:
            return
        from .attenuation import ZenerFit
        self._zener_fit = ZenerFit(f_min=fit.get("f_min", 2.0), f_max=fit.get("f_max", 8.0),
                                   n_sls=fit.get("n_sls", 3))
        qp = flt32(spec.get("qp", np.inf))
        qs = flt32(spec.get("qs", np.inf))
        self._qp = qp
        self._qs = qs
        self._inv_qp_grid = (1.0 / self._material_grid(qp, "qp_map").astype(np.float64)).astype(flt32)
        self._inv_qs_grid = (1.0 / self._material_grid(qs, "qs_map").astype(np.float64)).astype(flt32)
        # read-only: cell_scales() caches on the grids' identity, so a new Q
        # model must replace a grid (an in-place edit raises)
        self._inv_qp_grid.setflags(write=False)
        self._inv_qs_grid.setflags(write=False)

    def cell_scales(self):
        """Per-cell attenuation scales ``(g_p, g_s)`` of the fitted Zener
        model (float32 grids), or None without per-cell Q.  Computed once and
        kept while the 1/Q grids stay the same objects (a stepper is created
        per shot; the scales are the same for every shot).  The 1/Q grids are
        read-only: assign new arrays to change the Q model."""
        if self._zener_fit is None:
            return None
        cached = getattr(self, "_cell_scales_cache", None)
        if cached is None or cached[0] is not self._inv_qp_grid or cached[1] is not self._inv_qs_grid:
            g = (self._zener_fit.cell_scale(self._inv_qp_grid), self._zener_fit.cell_scale(self._inv_qs_grid))
            cached = (self._inv_qp_grid, self._inv_qs_grid, g)
            self._cell_scales_cache = cached
        return cached[2]
