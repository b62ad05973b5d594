"""Simulation region, CPML profiles and transducer (probe) geometry.

Mirrors sim_support/simul_classes.py of the reference.  Every table the
stepper reads (grid sizes, CPML a/b/k vectors, source wavelets, source and
receiver grid indices, reception delays) is produced here, and parity with
the reference depends on these tables being identical, so the float32 /
float64 mix of each expression follows the reference's:

* :class:`SimulationROI` - reference :30-386 (grid steps rounded to
  ``int(|log10 step|) + 2`` decimals, index ranges, nearest-grid lookup
  :301-319 and the CPML profile :321-386 after Gedney / Komatitsch-Martin).
* :class:`ElementRect`, :class:`ElementCirc` - reference :414-647.
* :class:`SimulationProbeLinearArray` - reference :650-965.
* :class:`SimulationProbePoint` - reference :967-1183.
* :class:`SimulationProbeMonoCirc` - reference :1185-1343.
* :class:`SimulationProbeMatrix` - new: a rectangular grid of one-point
  receivers (the reference's matrix array is commented out, :801-821).

Known quirks of the reference that are kept because they change tables:
in a 3D linear array the passive-axis index of each point does not include
the element's base index; ``get_idx_rec`` is called with an upper-case
``"2D"`` by the 2D model.
"""
import numpy as np
from scipy.signal import gausspulse

from . import flt32
from .gauss_wavelets import gaussian_pulse, gaussian_first_dev_pulse, gaussian_second_dev_pulse


def _rounded_step(extent, count):
    step = extent / count
    dec = int(abs(np.log10(step))) + 2
    return np.round(step, decimals=dec).astype(np.float32), dec


class SimulationROI:
    """Region of interest: ROI extent and sampling plus CPML layer widths.

    ``w`` is the x (active) axis, ``d`` the y (passive) axis and ``h`` the z
    (height) axis.  The full grid adds CPML layers and ``pad`` cells on each
    side: ``nx = w_len + len_pml_xmin + len_pml_xmax + 2 pad``.  A density
    map larger than the nominal ROI enlarges it (reference :158-190).
    """

    def __init__(self, coord_ref=np.zeros((1, 3)), height=30.0, h_len=300, width=30.0, w_len=300,
                 depth=0.0, d_len=1, len_pml_xmin=10, len_pml_xmax=10, len_pml_ymin=10, len_pml_ymax=10,
                 len_pml_zmin=10, len_pml_zmax=10, rcoef_pml=0.0001, npower_pml=2.0, k_max_pml=1.0,
                 pad=1, rho_map=None):
        if type(coord_ref) is list:
            coord_ref = np.array(coord_ref, dtype=np.float32)
        if coord_ref.shape != (1, 3):
            raise TypeError("``coord_ref`` deve ser um vetor-linha de 3 elementos [shape = (1,3)]")
        self.coord_ref = coord_ref

        self.h_step, self._dec_h = _rounded_step(height, h_len)
        self.w_step, self._dec_w = _rounded_step(width, w_len)
        if depth > 0.0 and d_len > 1:
            self.d_step, self._dec_d = _rounded_step(depth, d_len)
        else:
            # A 2D ROI reuses the x step for its (unit-length) y axis.
            self._dec_d = int(abs(np.log10(self.w_step))) + 2
            self.d_step = np.round(self.w_step, decimals=self._dec_d).astype(np.float32)

        map_w = map_h = map_d = 0
        if rho_map is not None:
            if rho_map.ndim == 1:
                map_w = rho_map.shape[0]
            elif rho_map.ndim == 2:
                map_w, map_h = rho_map.shape
            elif rho_map.ndim == 3:
                map_w, map_d, map_h = rho_map.shape

        if map_w > w_len:
            self.width, self._w_len = np.float32(map_w * self.w_step), map_w
        else:
            self.width, self._w_len = np.float32(width), w_len
        if map_h > h_len:
            self.height, self._h_len = np.float32(map_h * self.h_step), map_h
        else:
            self.height, self._h_len = np.float32(height), h_len
        if map_d > d_len:
            self.depth, self._d_len = np.float32(map_d * self.d_step), map_d
        else:
            self.depth, self._d_len = np.float32(depth), d_len

        def axis_points(origin, extent, count, dec):
            return np.linspace(origin, origin + extent, num=int(count), endpoint=False,
                               dtype=np.float32).round(decimals=dec)

        self.w_points = axis_points(coord_ref[0, 0], self.width, self._w_len, self._dec_w)
        self.d_points = axis_points(coord_ref[0, 1], self.depth, self._d_len, self._dec_d)
        self.h_points = axis_points(coord_ref[0, 2], self.height, self._h_len, self._dec_h)

        self._pml_xmin_len, self._pml_xmax_len = len_pml_xmin, len_pml_xmax
        self._pml_ymin_len, self._pml_ymax_len = len_pml_ymin, len_pml_ymax
        self._pml_zmin_len, self._pml_zmax_len = len_pml_zmin, len_pml_zmax
        self._rcoef_pml = rcoef_pml
        self._npower_pml = npower_pml
        self._k_max_pml = k_max_pml
        self._pad = pad

    def has_pml(self):
        return any((self._pml_xmin_len, self._pml_xmax_len, self._pml_ymin_len,
                    self._pml_ymax_len, self._pml_zmin_len, self._pml_zmax_len))

    def get_dx(self):
        return flt32(self.w_step)

    def get_dy(self):
        return flt32(self.d_step)

    def get_dz(self):
        return flt32(self.h_step)

    def get_nx(self):
        return self._w_len + self._pml_xmin_len + self._pml_xmax_len + 2 * self._pad

    def get_ny(self):
        return self._d_len + self._pml_ymin_len + self._pml_ymax_len + 2 * self._pad

    def get_nz(self):
        return self._h_len + self._pml_zmin_len + self._pml_zmax_len + 2 * self._pad

    def get_len_x(self):
        return self._w_len

    def get_len_y(self):
        return self._d_len

    def get_len_z(self):
        return self._h_len

    def get_ix_min(self):
        return self._pml_xmin_len + self._pad

    def get_ix_max(self):
        return self._w_len + self._pml_xmin_len + self._pad

    def get_iy_min(self):
        return self._pml_ymin_len + self._pad

    def get_iy_max(self):
        return self._d_len + self._pml_ymin_len + self._pad

    def get_iz_min(self):
        return self._pml_zmin_len + self._pad

    def get_iz_max(self):
        return self._h_len + self._pml_zmin_len + self._pad

    def get_pml_thickness_x(self):
        return (self._pml_xmin_len + self._pml_xmax_len) * self.w_step

    def get_pml_thickness_y(self):
        return (self._pml_ymin_len + self._pml_ymax_len) * self.d_step

    def get_pml_thickness_z(self):
        return (self._pml_zmin_len + self._pml_zmax_len) * self.h_step

    def get_dec(self):
        return self._dec_w, self._dec_d, self._dec_h

    @staticmethod
    def _as_point(point):
        if type(point) is list:
            point = np.array(point, dtype=np.float32)
        return point

    def is_point_in_roi(self, point):
        """True when the cartesian point (mm) lies inside the ROI box."""
        point = self._as_point(point)
        return bool(self.w_points[0] <= point[0] <= self.w_points[-1] and
                    self.d_points[0] <= point[1] <= self.d_points[-1] and
                    self.h_points[0] <= point[2] <= self.h_points[-1])

    def get_nearest_grid_idx(self, point):
        """Full-grid ``[ix, iy, iz]`` of the grid node nearest to a ROI point.

        The point is nudged by a tenth of a unit in the last kept decimal
        before rounding, so that exact half-steps resolve to the lower node
        as in the reference (:313-318).  Raises ``IndexError`` outside the ROI.
        """
        point = self._as_point(point)
        if not self.is_point_in_roi(point):
            raise IndexError(f"[{point[0]}, {point[1]}, {point[2]}] out of bounds")

        def nearest(axis_pts, value, step, dec, offset):
            target = np.round(value - step / 10.0 ** (dec - 1), decimals=dec)
            return np.absolute(axis_pts - target).argmin() + offset

        ix = nearest(self.w_points, point[0], self.w_step, self._dec_w, self._pml_xmin_len + self._pad)
        iy = nearest(self.d_points, point[1], self.d_step, self._dec_d, self._pml_ymin_len + self._pad)
        iz = nearest(self.h_points, point[2], self.h_step, self._dec_h, self._pml_zmin_len + self._pad)
        return [ix, iy, iz]

    def calc_pml_array(self, axis='x', grid='f', dt=1.0, cp=1.0, alpha_max=1.0):
        """CPML ``(a, b, k)`` vectors along one axis of the CPML+ROI span.

        Length ``n_axis - 2 pad``; ``grid='h'`` samples half a step to the
        right (staggered nodes).  Inside the layers, with normalised depth
        ``p`` in [0, 1]: ``d = d0 p^n`` with ``d0 = -(n+1) cp ln(R) / L``,
        ``k = 1 + (k_max - 1) p^n``, ``alpha = alpha_max (1 - p)``;
        ``b = exp(-(d/k + alpha) dt)`` and ``a = d (b - 1) / (k (d + k alpha))``
        where ``d > 1e-6``.  Outside the layers ``a = 0, b = 1, k = 1``, which
        makes the convolution update an identity there.
        """
        axis = axis.lower()
        if axis == 'x':
            delta, n_roi, lo, hi, dec = np.float32(self.w_step), self._w_len, self._pml_xmin_len, self._pml_xmax_len, self._dec_w
            thick = self.get_pml_thickness_x()
        elif axis == 'y':
            delta, n_roi, lo, hi, dec = np.float32(self.d_step), self._d_len, self._pml_ymin_len, self._pml_ymax_len, self._dec_d
            thick = self.get_pml_thickness_y()
        elif axis == 'z':
            delta, n_roi, lo, hi, dec = np.float32(self.h_step), self._h_len, self._pml_zmin_len, self._pml_zmax_len, self._dec_h
            thick = self.get_pml_thickness_z()
        else:
            raise IndexError(f"'axis' = {axis} not supported")
        n_span = n_roi + lo + hi
        left_edge = lo * delta
        right_edge = (lo + n_roi - 1) * delta
        left_thick = lo * delta
        right_thick = hi * delta
        d0 = flt32(-(self._npower_pml + 1.0) * cp * np.log(self._rcoef_pml) / thick)

        pos = np.round(delta * np.arange(n_span), decimals=dec).astype(np.float32)
        g = grid.lower()
        if g == 'f':
            dist_left = np.round(left_edge - pos, decimals=dec)
            dist_right = np.round(pos - right_edge, decimals=dec)
        elif g == 'h':
            dist_left = np.round(left_edge - (pos + delta / 2.0), decimals=dec).astype(np.float32)
            dist_right = np.round((pos + delta / 2.0) - right_edge, decimals=dec).astype(np.float32)
        else:
            raise IndexError(f"'grid' = {grid} not supported")

        in_left = (dist_left >= 0.0) if left_thick > 0.0 else np.zeros(dist_left.shape, dtype=bool)
        in_right = (dist_right >= 0.0) if right_thick > 0.0 else np.zeros(dist_right.shape, dtype=bool)
        in_layer = np.logical_or(in_left, in_right)
        depth = np.zeros(n_span, dtype=np.float32)
        if left_thick:
            depth[in_left] = dist_left[in_left] / left_thick
        if right_thick:
            depth[in_right] = dist_right[in_right] / right_thick
        d = (d0 * depth ** self._npower_pml).astype(np.float32)
        k = (1.0 + (self._k_max_pml - 1.0) * depth ** self._npower_pml).astype(np.float32)
        alpha = (alpha_max * (1.0 - np.where(in_layer, depth, 1.0))).astype(np.float32)
        b = np.exp(-(d / k + alpha) * dt).astype(np.float32)
        a = np.zeros(n_span, dtype=np.float32)
        sel = np.where(d > 1e-6)
        a[sel] = d[sel] * (b[sel] - 1.0) / (k[sel] * (d[sel] + k[sel] * alpha[sel]))
        return a, b, k


class SimulationProbe:
    """Base probe: centre coordinate (mm, relative to the ROI origin)."""

    def __init__(self, coord_center=np.zeros((1, 3)), dec=(2, 2, 2)):
        self.coord_center = np.array(coord_center).astype(np.float32)
        self._dec = dec


def _excitation(gain, freq, bw, t0, t, out):
    """Time derivative of a gain-scaled Gaussian pulse (the element force).

    ``np.diff(gain * pulse / dt, append=0)`` of ``scipy.signal.gausspulse``
    delayed by ``t0``, with samples below float32 epsilon flushed to zero
    (reference :456-467).
    """
    dt = t[1] - t[0]
    y_i, _, y_env = gausspulse((t - t0), fc=freq, bw=bw, retquad=True, retenv=True)
    eps = np.finfo(flt32).eps
    if out == 'e':
        y_env[np.abs(y_env) < eps] = 0.0
        sig = flt32(y_env)
    else:
        y_i[np.abs(y_i) < eps] = 0.0
        sig = flt32(y_i)
    return np.diff(gain * np.float32(sig) / dt, append=0.0).astype(flt32)


class ElementRect:
    """Rectangular element of a linear array (``dim_a`` x ``dim_p`` mm)."""

    def __init__(self, dim_a=0.5, dim_p=10.0, coord_center=np.zeros((1, 3)), freq=5., bw=0.5, gain=1.0,
                 t0=1.0, tx_en=True, rx_en=True, pulse_type="gaussian"):
        self.elem_dim_a = np.float32(dim_a)
        self.elem_dim_p = np.float32(dim_p)
        self.coord_center = coord_center.astype(np.float32)
        self.freq = np.float32(freq)
        self.bw = np.float32(bw)
        self.gain = np.float32(gain)
        self.t0 = np.float32(t0)
        self.tx_en = tx_en
        self.rx_en = rx_en
        self.pulse_type = pulse_type

    def get_element_exc_fn(self, t, out='r'):
        return _excitation(self.gain, self.freq, self.bw, self.t0, t, out)

    def get_num_points_roi(self, sim_roi=None, simul_type="2D"):
        sim_roi = SimulationROI() if sim_roi is None else sim_roi
        dec_w, dec_d, _ = sim_roi.get_dec()
        dim_p = min(self.elem_dim_p, sim_roi.depth)
        n_a = int(np.round(self.elem_dim_a / sim_roi.w_step, decimals=dec_w))
        n_p = int(np.round(dim_p / sim_roi.d_step, decimals=dec_d)) if dim_p != 0.0 else 1
        return n_a * n_p if simul_type.lower() == "3d" else n_a

    def get_points_roi(self, sim_roi=None, probe_center=np.zeros((1, 3)), simul_type="2D", dir="e"):
        """Grid indices ``[ix, iy, iz]`` of the element's active points.

        Empty when the element does not emit (``dir='e'``) or receive
        (``dir='r'``).  Points start at the node nearest the element's first
        corner and step by one node along x (and y in 3D).
        """
        sim_roi = SimulationROI() if sim_roi is None else sim_roi
        if not isinstance(dir, str):
            raise ValueError("'dir' must be a string")
        if (dir.lower() == "e" and not self.tx_en) or (dir.lower() == "r" and not self.rx_en):
            return list()
        dec_w, dec_d, _ = sim_roi.get_dec()
        dim_p = min(self.elem_dim_p, sim_roi.depth)
        n_a = int(np.round(self.elem_dim_a / sim_roi.w_step, decimals=dec_w) + 0.5)
        n_p = int(np.round(dim_p / sim_roi.d_step, decimals=dec_d) + 0.5) if dim_p != 0.0 else 1
        n_pts = n_a * n_p if simul_type.lower() == "3d" else n_a

        half_a = (self.elem_dim_a - sim_roi.w_step) / 2.0 if n_a // 2 else (self.elem_dim_a / 2.0)
        x0 = np.float32(self.coord_center[0] - half_a)
        if simul_type.lower() == "2d":
            y0 = np.float32(0.0)
        elif n_p // 2:
            y0 = np.float32(self.coord_center[1] - ((dim_p - sim_roi.d_step) / 2.0))
        else:
            y0 = np.float32(dim_p / 2.0)
        corner = np.array([x0, y0, self.coord_center[2]], np.float32) + probe_center.astype(np.float32)
        base = sim_roi.get_nearest_grid_idx(corner)
        flat_2d = simul_type == "2d"   # case-sensitive in the reference
        return [[base[0] + (p % n_a),
                 (base[1] + 0) if flat_2d else ((p // n_a) % n_p),
                 base[2]] for p in range(n_pts)]


class ElementCirc:
    """Circular element of a mono-element probe; ``radius`` in inches."""

    def __init__(self, radius=0.25, coord_center=np.zeros((3,)), freq=5., bw=0.5, gain=1.0, t0=1.0,
                 tx_en=True, rx_en=True, pulse_type="gaussian"):
        self.radius = np.float32(radius * 25.4)
        self.coord_center = coord_center.astype(np.float32)
        self.freq = np.float32(freq)
        self.bw = np.float32(bw)
        self.gain = np.float32(gain)
        self.t0 = np.float32(t0)
        self.tx_en = tx_en
        self.rx_en = rx_en
        self.pulse_type = pulse_type

    def get_element_exc_fn(self, t, out='r'):
        return _excitation(self.gain, self.freq, self.bw, self.t0, t, out)

    def _get_candidate_points(self, sim_roi, simul_type, current_center):
        """Grid nodes of the disc: a bounding square filtered by the radius."""
        simul_type = simul_type.lower()
        dec_w, dec_d, _ = sim_roi.get_dec()
        n_a = int(np.round((2.0 * self.radius) / sim_roi.w_step, decimals=dec_w))
        if simul_type == "3d":
            r_p = min(self.radius, sim_roi.depth)
            n_p = int(np.round((2.0 * r_p) / sim_roi.d_step, decimals=dec_d))
        else:
            r_p, n_p = 0.0, 1
        x_start = np.float32(current_center[0] - self.radius)
        y_start = np.float32(0.0 if simul_type == "2d" else current_center[1] - r_p)
        corner = np.array([x_start, y_start, current_center[2]], dtype=flt32)
        base = sim_roi.get_nearest_grid_idx(corner)
        pts = list()
        for jj in range(n_a):
            ddx = (jj - (n_a - 1) / 2.0) * sim_roi.w_step
            for zz in range(n_p):
                ddy = (zz - (n_p - 1) / 2.0) * sim_roi.d_step if simul_type == "3d" else 0.0
                if np.sqrt(ddx ** 2 + ddy ** 2) <= self.radius:
                    pts.append([base[0] + jj, base[1] + (0 if simul_type == "2d" else zz), base[2]])
        return pts

    def get_num_points_roi(self, sim_roi, simul_type="2D"):
        return len(self._get_candidate_points(sim_roi, simul_type, self.coord_center))

    def get_points_roi(self, sim_roi, probe_center=np.zeros((3,)), simul_type="2D", dir="e"):
        if not isinstance(dir, str):
            raise ValueError("'dir' must be a string")
        if (dir.lower() == "e" and not self.tx_en) or (dir.lower() == "r" and not self.rx_en):
            return list()
        center = self.coord_center + probe_center.astype(flt32).flatten()
        return self._get_candidate_points(sim_roi, simul_type, center)


def _flags(spec, n, what):
    """Parse an ``emitters``/``receivers`` entry: "all", "none" or a list."""
    if isinstance(spec, str) and spec == "all":
        return [True] * n
    if isinstance(spec, str) and spec == "none":
        return [False] * n
    if isinstance(spec, list):
        flags = [bool(str(el).strip().lower() == "true") for el in spec]
        return (flags + [False] * n)[:n]
    raise ValueError(f"{what} must be a string or a list of strings")


def _bool_word(word, what):
    if not isinstance(word, str):
        raise ValueError(f"{what} must be a string")
    w = word.strip().lower()
    if w not in ("true", "false"):
        raise ValueError(f"{what} must be 'True' or 'False'")
    return w == "true"


def _per_element(value, n, what):
    """Scalar or list of per-element delays, as float32 (reference :715-760)."""
    if value is None:
        return np.zeros(n, dtype=np.float32)
    if type(value) is np.float32 or type(value) is float:
        return np.ones(n, dtype=np.float32) * np.float32(value)
    if type(value) is list:
        return np.array((list(value) + [0.0] * n)[:n], dtype=np.float32)
    raise ValueError(f"{what} must be either a float [numpy.float32] or a list of floats.")


class SimulationProbeLinearArray(SimulationProbe):
    """Linear array of ``num_elem`` rectangular elements along x.

    Element ``i`` is centred at ``dim_a/2 + i pitch - ((num_elem-1) pitch +
    dim_a)/2`` relative to the probe centre, ``pitch = dim_a + inter_elem``.
    """

    def __init__(self, coord_center=np.zeros((1, 3)), dec=(2, 2, 2), num_elem=32, dim_a=0.5, dim_p=10.0,
                 inter_elem=0.1, freq=5., bw=0.5, gain=1.0, pulse_type="gaussian", id="",
                 emitters="all", receivers="all", t0_emission=None, t0_reception=None):
        super().__init__(coord_center, dec)
        self.id = id
        self.inter_elem = np.float32(inter_elem)
        self.emitters = _flags(emitters, num_elem, "emitters")
        self.receivers = _flags(receivers, num_elem, "receivers")
        self._t0_emission = _per_element(t0_emission, num_elem, "t0_emission")
        self._t0_reception = _per_element(t0_reception, num_elem, "t0_reception")
        self.pitch = np.float32(dim_a + inter_elem)
        self.num_elem = num_elem
        span_center = np.array([((num_elem - 1) * self.pitch + dim_a) / 2.0, 0.0, 0.0], dtype=np.float32)
        self.elem_list = [
            ElementRect(dim_a=dim_a, dim_p=dim_p,
                        coord_center=np.round(np.array([dim_a / 2.0 + i * self.pitch, 0.0, 0.0],
                                                       dtype=np.float32) - span_center,
                                              decimals=np.max(self._dec)),
                        freq=freq, bw=bw, gain=gain, pulse_type=pulse_type,
                        tx_en=self.emitters[i], rx_en=self.receivers[i],
                        t0=np.float32(self._t0_emission[i]))
            for i in range(num_elem)]
        self._dim_a, self._dim_p = dim_a, dim_p
        self._freq, self._bw, self._gain, self._pulse_type = freq, bw, gain, pulse_type

    def get_freq(self, mode='common'):
        if mode == 'mean':
            return np.array([e.freq for e in self.elem_list]).mean()
        if mode == 'max':
            return np.array([e.freq for e in self.elem_list]).max()
        return self._freq

    def get_points_roi(self, sim_roi=None, simul_type="2D", dir="e"):
        """``(points, element_index_per_point)``; elements outside the ROI are skipped."""
        sim_roi = SimulationROI() if sim_roi is None else sim_roi
        pts, owner = list(), list()
        for i, e in enumerate(self.elem_list):
            try:
                p = e.get_points_roi(sim_roi=sim_roi, probe_center=self.coord_center,
                                     simul_type=simul_type, dir=dir)
            except IndexError:
                continue
            pts += p
            owner += [i] * len(p)
        return pts, owner

    def get_source_term(self, samples=1000, dt=1.0, out='r'):
        """``(samples, num_elem)`` float32 force per element (zeros for non-emitters)."""
        dec = int(abs(np.log10(dt))) + 2
        t = np.round(np.arange(samples, dtype=np.float32) * dt, decimals=dec)
        term = np.zeros((samples, self.num_elem), dtype=np.float32)
        for i, e in enumerate(self.elem_list):
            if e.tx_en:
                term[:, i] = e.get_element_exc_fn(t, out)
        return term

    def get_idx_rec(self, sim_roi=None, simul_type="2D"):
        """Receiving element index of every receiver point."""
        sim_roi = SimulationROI() if sim_roi is None else sim_roi
        owner = list()
        for i, e in enumerate(self.elem_list):
            try:
                p = e.get_points_roi(sim_roi=sim_roi, probe_center=self.coord_center,
                                     simul_type=simul_type, dir='r')
            except IndexError:
                continue
            owner += [i] * len(p)
        return owner

    def get_delay_rx(self):
        return [self._t0_reception[i] for i, e in enumerate(self.elem_list) if e.rx_en]

    def set_t0(self, t0_emission=None):
        """Replace every element's emission delay (one focal law / shot)."""
        if t0_emission is None:
            self._t0_emission = np.zeros(self.num_elem, dtype=np.float32)
        elif type(t0_emission) is np.float32 or type(t0_emission) is float:
            self._t0_emission = np.ones(self.num_elem, dtype=np.float32) * np.float32(t0_emission)
        elif type(t0_emission) is list:
            self._t0_emission = np.array((list(t0_emission) + [0.0] * self.num_elem)[:self.num_elem],
                                         dtype=np.float32)
        elif type(t0_emission) is np.ndarray:
            self._t0_emission = t0_emission
        else:
            raise ValueError("t0_emission must be either a float [numpy.float32] or a list of floats.")
        for i, e in enumerate(self.elem_list):
            e.t0 = self._t0_emission[i]


class SimulationProbePoint(SimulationProbe):
    """Single-node emitter and/or receiver."""

    def __init__(self, coord_center=np.zeros((1, 3)), dec=(2, 2, 2), freq=5., bw=0.5, gain=1.0,
                 pulse_type="gaussian", id="", emitter="True", receiver="False",
                 t0_emission=None, t0_reception=None):
        super().__init__(coord_center, dec)
        self._id = id
        self.num_elem = 1
        self.emitters = [_bool_word(emitter, "emitter")]
        self.receivers = [_bool_word(receiver, "receiver")]
        self._t0_emission = np.float32(0.0 if t0_emission is None else t0_emission)
        self._t0_reception = np.float32(0.0 if t0_reception is None else t0_reception)
        self._freq, self._bw, self._gain, self._pulse_type = freq, bw, gain, pulse_type

    def get_freq(self, mode='common'):
        return self._freq

    def get_coords(self):
        return self.coord_center

    def get_points_roi(self, sim_roi=None, simul_type="2D", dir="e"):
        sim_roi = SimulationROI() if sim_roi is None else sim_roi
        if not isinstance(dir, str):
            raise ValueError("'dir' must be a string")
        if (dir.lower() == "e" and not self.emitters[0]) or (dir.lower() == "r" and not self.receivers[0]):
            return list(), list()
        y = np.float32(0.0 if simul_type.lower() == "2d" else self.coord_center[1])
        p = np.array([np.float32(self.coord_center[0]), y, np.float32(self.coord_center[2])], np.float32)
        node = sim_roi.get_nearest_grid_idx(p)
        return [[node[0], node[1], node[2]]], [0]

    def get_source_term(self, samples=1000, dt=1.0, out='r', ord_der=1):
        """``(samples,)`` float32: gain x Gaussian pulse (``ord_der`` 0), its
        first derivative (1, default) or second derivative (2)."""
        t = np.arange(samples, dtype=flt32) * dt
        sig = np.zeros(samples, dtype=flt32)
        if self.emitters[0]:
            # pulse_type "ricker" (an addition; the reference ignores
            # pulse_type) always selects the second derivative.
            if str(self._pulse_type).lower() == "ricker":
                ord_der = 2
            fn = {0: gaussian_pulse, 2: gaussian_second_dev_pulse}.get(ord_der, gaussian_first_dev_pulse)
            y_i, _, y_env = fn((t - self._t0_emission), fc=self._freq, bw=self._bw, retquad=True, retenv=True)
            eps = np.finfo(flt32).eps
            if out == 'e':
                y_env[np.abs(y_env) < eps] = 0.0
                sig = flt32(y_env)
            else:
                y_i[np.abs(y_i) < eps] = 0.0
                sig = flt32(y_i)
        return flt32(self._gain * sig)

    def get_idx_rec(self, sim_roi=None, simul_type="2D"):
        return [0] if self.receivers[0] else list()

    def get_delay_rx(self):
        return [self._t0_reception] if self.receivers[0] else list()

    def set_t0(self, t0_emission=None):
        if t0_emission is None:
            self._t0_emission = np.float32(0.0)
        elif type(t0_emission) is np.float32 or type(t0_emission) is float:
            self._t0_emission = t0_emission
        else:
            raise ValueError("t0_emission must be either a float [numpy.float32].")

    def get_receiver_points_count(self):
        return 1 if self.receivers[0] else 0


class SimulationProbeMonoCirc(SimulationProbe):
    """Mono-element probe with one circular element (radius in inches)."""

    def __init__(self, coord_center=np.zeros((1, 3)), dec=(2, 2, 2), radius=0.25, freq=5., bw=0.5,
                 gain=1.0, pulse_type="gaussian", id="", emitters="True", receivers="False",
                 t0_emission=None, t0_reception=None):
        super().__init__(coord_center, dec)
        self._id = id
        self.emitters = [_bool_word(emitters, "emitters")]
        self.receivers = [_bool_word(receivers, "receivers")]
        self._t0_reception = np.float32(t0_reception)
        self._t0_emission = np.float32(t0_emission)
        self.elem = ElementCirc(radius=radius, coord_center=np.zeros(3, dtype=np.float32), freq=freq, bw=bw,
                                gain=gain, t0=np.float32(t0_emission), tx_en=self.emitters[0],
                                rx_en=self.receivers[0], pulse_type=pulse_type)

    def get_freq(self, mode='common'):
        return self.elem.freq

    def get_coords(self):
        return self.coord_center

    def get_points_roi(self, sim_roi=None, simul_type="3D", dir="e"):
        sim_roi = SimulationROI() if sim_roi is None else sim_roi
        try:
            pts = self.elem.get_points_roi(sim_roi=sim_roi, probe_center=self.coord_center,
                                           simul_type=simul_type, dir=dir)
        except IndexError:
            return list(), list()
        return list(pts), [0] * len(pts)

    def get_source_term(self, samples=1000, dt=1.0, out='r'):
        dec = int(abs(np.log10(dt))) + 2
        t = np.round(np.arange(samples, dtype=np.float32) * dt, decimals=dec)
        term = np.zeros((samples, 1), dtype=np.float32)
        if self.elem.tx_en:
            term[:, 0] = self.elem.get_element_exc_fn(t, out)
        return term

    def get_idx_rec(self, sim_roi=None, simul_type="3D"):
        sim_roi = SimulationROI() if sim_roi is None else sim_roi
        try:
            pts = self.elem.get_points_roi(sim_roi=sim_roi, probe_center=self.coord_center,
                                           simul_type=simul_type, dir='r')
        except IndexError:
            return list()
        return [0] * len(pts)

    def get_delay_rx(self):
        return [self._t0_reception] if self.receivers[0] else list()

    def set_t0(self, t0_emission=None):
        if t0_emission is None:
            self._t0_emission = np.float32(0.0)
        elif isinstance(t0_emission, (float, int, np.number)):
            self._t0_emission = np.float32(t0_emission)
        elif isinstance(t0_emission, (list, np.ndarray)):
            self._t0_emission = np.float32(t0_emission[0])
        else:
            raise ValueError("t0_emission must be either a float [numpy.float32] or a list of floats.")
        self.elem.t0 = self._t0_emission

    def get_receiver_points_count(self, simul_type="2D", sim_roi=None):
        return len(self.get_idx_rec(sim_roi=sim_roi, simul_type=simul_type))


class SimulationProbeMatrix(SimulationProbe):
    """Receive-only matrix of ``num_x x num_y`` single-node elements.

    New (the reference's matrix array is commented out): element ``(i, j)``
    sits at ``coord_center + ((i - (num_x-1)/2) pitch_x, (j - (num_y-1)/2)
    pitch_y, 0)``, element index ``i * num_y + j``.  In 2D only the x row
    (``j`` = 0) is used.  It never emits.
    """

    def __init__(self, coord_center=np.zeros((1, 3)), dec=(2, 2, 2), num_x=8, num_y=8, pitch_x=0.1,
                 pitch_y=0.1, freq=5., id="", t0_reception=None):
        super().__init__(coord_center, dec)
        self.id = id
        self.num_x, self.num_y = int(num_x), int(num_y)
        self.pitch_x, self.pitch_y = np.float32(pitch_x), np.float32(pitch_y)
        self.num_elem = self.num_x * self.num_y
        self.emitters = [False] * self.num_elem
        self.receivers = [True] * self.num_elem
        self._t0_reception = _per_element(t0_reception, self.num_elem, "t0_reception")
        self._freq = freq

    def get_freq(self, mode='common'):
        return self._freq

    def _nodes(self, sim_roi, simul_type):
        three_d = simul_type.lower() == "3d"
        n_y = self.num_y if three_d else 1
        out = list()
        for i in range(self.num_x):
            for j in range(n_y):
                p = self.coord_center.astype(np.float32).flatten().copy()
                p[0] += np.float32((i - (self.num_x - 1) / 2.0) * self.pitch_x)
                p[1] = p[1] + np.float32((j - (self.num_y - 1) / 2.0) * self.pitch_y) if three_d else 0.0
                out.append((i * self.num_y + j, sim_roi.get_nearest_grid_idx(p)))
        return out

    def get_points_roi(self, sim_roi=None, simul_type="3D", dir="e"):
        sim_roi = SimulationROI() if sim_roi is None else sim_roi
        if dir.lower() == "e":
            return list(), list()
        nodes = self._nodes(sim_roi, simul_type)
        return [list(n) for _, n in nodes], [k for k, _ in nodes]

    def get_source_term(self, samples=1000, dt=1.0, out='r', ord_der=1):
        return np.zeros((samples, self.num_elem), dtype=np.float32)

    def get_idx_rec(self, sim_roi=None, simul_type="3D"):
        sim_roi = SimulationROI() if sim_roi is None else sim_roi
        return [k for k, _ in self._nodes(sim_roi, simul_type)]

    def get_delay_rx(self):
        return list(self._t0_reception)

    def set_t0(self, t0_emission=None):
        pass
