"""Small seeded experiments for the parity tests.

Each builder returns a config dict for the host model; sizes are chosen so
that the CPU oracle finishes in about a second.
"""
import numpy as np


def _roi(w, h, d=0, pml=8, dx=0.05, pml_z=None):
    pz = pml if pml_z is None else pml_z
    return {"coord_ref": [[0.0, 0.0, 0.0]], "height": round(h * dx, 6), "h_len": h, "width": round(w * dx, 6),
            "w_len": w, "depth": round(d * dx, 6) if d else 0.0, "d_len": d if d else 1,
            "len_pml_xmin": pml, "len_pml_xmax": pml + 1, "len_pml_ymin": pml if d else 0,
            "len_pml_ymax": pml if d else 0, "len_pml_zmin": pz, "len_pml_zmax": pz,
            "rcoef_pml": 0.001, "npower_pml": 2.0, "k_max_pml": 1.0}


def inclusions(shape, seed, n=4, background=(5.9, 3.23, 7850.0), inclusion=(1.48, 0.0, 1000.0)):
    """cp/cs/rho ROI maps: a steel block with fluid-filled elliptical holes."""
    rng = np.random.default_rng(seed)
    w, h = shape
    cp = np.full(shape, background[0], np.float32)
    cs = np.full(shape, background[1], np.float32)
    rho = np.full(shape, background[2], np.float32)
    X, Z = np.meshgrid(np.arange(w), np.arange(h), indexing="ij")
    for _ in range(n):
        cx, cz = rng.uniform(0.2 * w, 0.8 * w), rng.uniform(0.35 * h, 0.85 * h)
        a, b = rng.uniform(2, 0.12 * w), rng.uniform(2, 0.12 * h)
        th = rng.uniform(0, np.pi)
        u = (X - cx) * np.cos(th) + (Z - cz) * np.sin(th)
        v = -(X - cx) * np.sin(th) + (Z - cz) * np.cos(th)
        m = (u / a) ** 2 + (v / b) ** 2 <= 1.0
        cp[m], cs[m], rho[m] = inclusion
    return cp, cs, rho


def case_2d(w=72, h=60, steps=240, acc=2, visco=0, seed=0, maps=True, linear=True, q=None, gain=1e2, t0_rx=0.0):
    """A 2D experiment: linear array (all emit/receive) on top of a block."""
    dx = 0.05
    cfg = {
        "roi": _roi(w, h, pml=8, dx=dx),
        "probes": [],
        "simul_params": {"time_steps": steps, "dt": 2.5e-3, "acc": acc, "it_display": 50},
        "simul_configs": {"n_iter": 1, "show_anim": 0, "viscoelastic_attn": visco},
        "specimen_params": {"cp": 5.9, "cs": 3.23, "rho": 7850.0},
    }
    if linear:
        cfg["probes"].append({"linear": {"id": "p", "num_elem": 8, "dim_a": 0.15, "dim_p": 10.0,
                                         "inter_elem": 0.05, "freq": 5.0, "bw": 0.5, "gain": gain,
                                         "coord_center": [w * dx / 2, 0.0, 0.3], "emitters": "all",
                                         "t0_emission": 0.25, "receivers": "all", "t0_reception": t0_rx}})
    else:
        cfg["probes"].append({"point": {"id": "s", "emitter": "True", "receiver": "False", "freq": 5.0,
                                        "bw": 0.5, "gain": gain, "coord_center": [w * dx / 2, 0.0, 0.4],
                                        "t0_emission": 0.25}})
        cfg["probes"].append({"linear": {"id": "r", "num_elem": 16, "dim_a": 0.05, "dim_p": 0.0,
                                         "inter_elem": 0.1, "freq": 5.0, "bw": 0.5, "gain": 1.0,
                                         "coord_center": [w * dx / 2, 0.0, 0.4], "emitters": "none",
                                         "receivers": "all", "t0_reception": t0_rx}})
    if maps:
        cp, cs, rho = inclusions((w, h), seed)
        cfg["specimen_params"].update({"cp_map": cp, "cs_map": cs, "rho_map": rho})
    if q is not None:
        rng = np.random.default_rng(seed + 100)
        cfg["specimen_params"]["qp"] = 120.0
        cfg["specimen_params"]["qs"] = 80.0
        cfg["specimen_params"]["qp_map"] = rng.uniform(q[0], q[1], (w, h)).astype(np.float32)
        cfg["specimen_params"]["qs_map"] = rng.uniform(q[0], q[1], (w, h)).astype(np.float32)
        cfg["simul_configs"]["zener_fit"] = {"f_min": 2.0, "f_max": 8.0}
    return cfg


def gaussian_blobs(shape, seed, n=5, amp=0.05, sigma=(1.0, 2.0), dx=0.05, background=(5.9, 3.23, 7850.0)):
    """cp/cs/rho maps: steel with n seeded Gaussian blobs of +-amp in cp and cs
    (sigma in mm), the adjoint gradient's true model."""
    rng = np.random.default_rng(seed)
    w, h = shape
    X, Z = np.meshgrid(np.arange(w) * dx, np.arange(h) * dx, indexing="ij")
    pert = np.zeros(shape)
    for _ in range(n):
        cx, cz = rng.uniform(0.25, 0.75) * w * dx, rng.uniform(0.35, 0.8) * h * dx
        s = rng.uniform(*sigma)
        pert += rng.choice([-1.0, 1.0]) * amp * np.exp(-((X - cx) ** 2 + (Z - cz) ** 2) / (2 * s * s))
    cp = (background[0] * (1 + pert)).astype(np.float32)
    cs = (background[1] * (1 + pert)).astype(np.float32)
    rho = np.full(shape, background[2], np.float32)
    return cp, cs, rho


def case_adjoint(w=64, h=64, steps=200, acc=2, visco=1, seed=0, true_model=True, q=None, n_elem=8):
    """The adjoint cut-down: a linear array (all emit/receive) on steel with
    Gaussian blobs (true model) or plain steel (start model)."""
    cfg = case_2d(w=w, h=h, steps=steps, acc=acc, visco=visco, seed=seed, maps=False, q=q)
    cfg["probes"][0]["linear"]["num_elem"] = n_elem
    if true_model:
        cp, cs, rho = gaussian_blobs((w, h), seed, sigma=(0.15 * w * 0.05, 0.3 * w * 0.05))
        cfg["specimen_params"].update({"cp_map": cp, "cs_map": cs, "rho_map": rho})
    return cfg


def case_3d(w=30, d=26, h=34, steps=90, acc=2, visco=1, seed=0, q=None, matrix=False, probe="point"):
    """A 3D experiment: layered block, Ricker point source, receivers on top.
    ``probe="mono"``: one circular element that emits and receives
    (pulse-echo); ``probe="linear"``: a 4-element linear array, every element
    emitting and receiving."""
    dx = 0.1
    rng = np.random.default_rng(seed)
    cp = np.empty((w, d, h), np.float32)
    cs = np.empty_like(cp)
    rho = np.empty_like(cp)
    bounds = np.sort(rng.integers(4, h - 4, 3))
    props = [(2.7, 1.3, 1200.0), (4.5, 2.4, 2700.0), (6.3, 3.2, 7800.0), (5.0, 2.9, 4500.0)]
    for k, (a, b) in enumerate(zip([0, *bounds], [*bounds, h])):
        cp[:, :, a:b], cs[:, :, a:b], rho[:, :, a:b] = props[k]
    cfg = {
        "roi": _roi(w, h, d=d, pml=6, dx=dx),
        "probes": [{"point": {"id": "s", "emitter": "True", "receiver": "False", "freq": 3.0, "bw": 0.5,
                              "gain": 1e2, "pulse_type": "ricker", "coord_center": [w * dx / 2, d * dx / 2, 0.3],
                              "t0_emission": 0.3}}],
        "simul_params": {"time_steps": steps, "dt": 0.5 * dx / (6.3 * np.sqrt(3.0)), "acc": acc, "it_display": 50},
        "simul_configs": {"n_iter": 1, "show_anim": 0, "viscoelastic_attn": visco},
        "specimen_params": {"cp": 5.9, "cs": 3.23, "rho": 7850.0, "cp_map": cp, "cs_map": cs, "rho_map": rho},
    }
    if matrix:
        cfg["probes"].append({"matrix": {"id": "m", "num_x": 6, "num_y": 5, "pitch_x": 0.3, "pitch_y": 0.3,
                                         "coord_center": [w * dx / 2, d * dx / 2, 0.2]}})
    else:
        cfg["probes"].append({"point": {"id": "r", "emitter": "False", "receiver": "True",
                                        "coord_center": [w * dx / 2 + 0.5, d * dx / 2, 0.2]}})
    if probe == "mono":
        cfg["probes"] = [{"mono": {"id": "m", "radius": 0.02, "freq": 3.0, "bw": 0.5, "gain": 1e2,
                                   "pulse_type": "gaussian", "coord_center": [w * dx / 2, d * dx / 2, 0.2],
                                   "emitters": "True", "t0_emission": 0.3, "receivers": "True",
                                   "t0_reception": 0.0}}]
    elif probe == "linear":
        cfg["probes"] = [{"linear": {"id": "a", "num_elem": 4, "dim_a": 0.3, "dim_p": 0.5, "inter_elem": 0.1,
                                     "freq": 3.0, "bw": 0.5, "gain": 1e2,
                                     "coord_center": [w * dx / 2, d * dx / 2, 0.2], "emitters": "all",
                                     "receivers": "all", "t0_emission": 0.3, "t0_reception": 0.0}}]
    if q is not None:
        cfg["specimen_params"]["qp"] = 100.0
        cfg["specimen_params"]["qs"] = 60.0
        cfg["specimen_params"]["qp_map"] = rng.uniform(q[0], q[1], (w, d, h)).astype(np.float32)
        cfg["specimen_params"]["qs_map"] = rng.uniform(q[0], q[1], (w, d, h)).astype(np.float32)
        cfg["simul_configs"]["zener_fit"] = {"f_min": 2.0, "f_max": 8.0}
    return cfg


def gated_mask(sim, taichi, n_steps):
    """Trace samples a receiver does not record: rows before its first
    recorded step (WGSL semantics: row k from k = delay; Taichi: from
    k = delay - 1)."""
    n_rec = int(sim._n_rec)
    first = np.asarray(sim._delay_recv, np.int64).reshape(-1)[:n_rec] - (1 if taichi else 0)
    return np.arange(n_steps)[:, None] < first[None, :]


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / nb) if nb > 0 else float(np.linalg.norm(a - b))


def _strip_bounds(n, ord_, tabs):
    """CPML strip [0, lo) + [hi, n) of one grid axis as the library derives
    it: nodes whose CPML tables (re-indexed by node, offset ord - 1) differ
    from the identity a = 0, b = 1, 1/k = 1."""
    off = ord_ - 1
    a, b, k, ah, bh, kh = (np.asarray(t, np.float32).ravel() for t in tabs)
    nonid = np.zeros(n, bool)
    for x in range(n):
        t = x - off
        if 0 <= t < n - 2 * off:
            full = a[t] != 0 or b[t] != 1 or np.float32(1) / k[t] != 1
            half = ah[t] != 0 or bh[t] != 1 or np.float32(1) / kh[t] != 1
            nonid[x] = full or half
    lo = max([x + 1 for x in range(n // 2) if nonid[x]], default=0)
    hi = min([x for x in range(n // 2, n) if nonid[x]], default=n)
    return lo, hi


def _axis_tabs(sim, ax):
    return [getattr(sim, f"_{c}_{ax}{s}") for s in ("", "_half") for c in "abk"]


def interior_warps(sim, tx):
    """Number of warps of the single-shot step kernels that take the interior
    sweep (32 lanes along the contiguous axis, tx nodes along x per thread):
    every node of the warp inside the update regions, outside the CPML strips
    and with its window rows inside the grid (source blocks aside)."""
    shape = sim.grid_shape()
    ord_ = int(sim._coefs.shape[0])
    axes = ("x", "y") if len(shape) == 2 else ("x", "y", "z")
    bounds = [_strip_bounds(n, ord_, _axis_tabs(sim, a)) for n, a in zip(shape, axes)]
    nx, lanes_n = shape[0], shape[-1]
    lo_l, hi_l = bounds[-1]
    lane_ok = [(0 <= c < lanes_n and c >= max(ord_, lo_l) and c < min(lanes_n - ord_, hi_l))
               for c in range(((lanes_n + 31) // 32) * 32)]
    warps_lane = sum(all(lane_ok[w * 32:(w + 1) * 32]) for w in range(len(lane_ok) // 32))
    lo_x, hi_x = bounds[0]
    chunks = sum(x0 >= max(ord_, lo_x) and x0 + tx + ord_ <= nx and x0 + tx <= hi_x for x0 in range(0, nx, tx))
    rows = 1
    if len(shape) == 3:
        lo_y, hi_y = bounds[1]
        rows = sum(max(ord_, lo_y) <= y < min(shape[1] - ord_, hi_y) for y in range(shape[1]))
    return warps_lane * chunks * rows
