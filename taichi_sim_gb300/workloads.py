"""Seeded synthetic experiments with the shapes of the benchmark configurations.

No public dataset exists for this stepper; each builder returns an
experiment description (dict) for the host model, with material maps as
arrays, drawn from ``numpy.random.default_rng(seed)``:

* :func:`elastic2d_512` - 2D isotropic elastic, 512x512 grid, aluminium,
  dx = 0.05 mm, Courant 0.5, 2000 steps, 20-cell CPML (R = 1e-3), point vy
  source at grid (256, 30) with a 5 MHz Gaussian pulse of about 3 cycles,
  128 one-node receivers on row 30 (Taichi semantics).
* :func:`visco2d_1024` - 2D viscoelastic, 1024x1024 grid, steel with 8
  elliptical fluid inclusions (semi-axes 0.5-3 mm, vp 1.48, vs 0, rho
  1000), per-region Qp/Qs ~ U[50, 200], L = 3 Zener fitted over 2-8 MHz,
  4000 steps, 20-cell CPML, 5 MHz source at the top surface, 256 receivers.
* :func:`visco3d_256` - 3D viscoelastic, 256^3 grid, dx = 0.1 mm, 4
  horizontal layers (vp 2.7-6.3, vs 1.3-3.2, rho 1200-7800, Q 30-300),
  L = 3, 16-cell CPML on all faces, 1000 steps, 3 MHz Ricker point source,
  64x64 receiver plane on the top surface.

``n_steps``/``size`` arguments scale a workload down for tests.
"""
import numpy as np

# Fractional bandwidth giving a -6 dB envelope width of 3 periods:
# exp(-a (1.5 T)^2) = 1/2 with a = (pi fc bw)^2 / (4 ln 10^(6/20)).
BW_3_CYCLES = float(np.sqrt(4.0 * np.log(10 ** (6 / 20)) * np.log(2.0)) / (np.pi * 1.5))


def _roi2d(n_grid, dx, pml, acc=2):
    roi_n = n_grid - 2 * pml - 2 * (acc - 1)
    return {"coord_ref": [[0.0, 0.0, 0.0]], "height": round(roi_n * dx, 6), "h_len": roi_n,
            "width": round(roi_n * dx, 6), "w_len": roi_n, "depth": 0.0, "d_len": 1,
            "len_pml_xmin": pml, "len_pml_xmax": pml, "len_pml_ymin": 0, "len_pml_ymax": 0,
            "len_pml_zmin": pml, "len_pml_zmax": pml, "rcoef_pml": 0.001, "npower_pml": 2.0,
            "k_max_pml": 1.0}, roi_n


def courant_dt(vmax, dx, dims, courant=0.5):
    return float(courant * dx / (vmax * np.sqrt(dims)))


def elastic2d_512(n_grid=512, n_steps=2000, n_rec=128):
    dx, pml = 0.05, 20
    roi, roi_n = _roi2d(n_grid, dx, pml)
    off = pml + 1
    src_x, src_row = (n_grid // 2 - off) * dx, (30 - off) * dx
    return {
        "roi": roi,
        "probes": [
            {"point": {"id": "src", "emitter": "True", "receiver": "False", "freq": 5.0, "bw": BW_3_CYCLES,
                       "gain": 1.0, "pulse_type": "gaussian", "coord_center": [src_x, 0.0, src_row],
                       "t0_emission": 0.4}},
            {"linear": {"id": "rx", "num_elem": n_rec, "dim_a": dx, "dim_p": 0.0, "inter_elem": 2 * dx,
                        "freq": 5.0, "bw": BW_3_CYCLES, "gain": 1.0, "coord_center": [src_x, 0.0, src_row],
                        "emitters": "none", "receivers": "all", "t0_reception": 0.0}},
        ],
        "simul_params": {"time_steps": n_steps, "dt": courant_dt(6.32, dx, 2), "acc": 2, "it_display": 500},
        "simul_configs": {"n_iter": 1, "show_anim": 0, "viscoelastic_attn": 0},
        "specimen_params": {"cp": 6.32, "cs": 3.13, "rho": 2700.0},
    }


def _ellipses(shape, dx, rng, n, semi=(0.5, 3.0), z_min_mm=2.0):
    w, h = shape
    X, Z = np.meshgrid(np.arange(w) * dx, np.arange(h) * dx, indexing="ij")
    labels = np.zeros(shape, np.int32)
    for k in range(1, n + 1):
        a, b = rng.uniform(*semi, 2)
        cx = rng.uniform(0.15, 0.85) * w * dx
        height = h * dx
        cz = rng.uniform(min(z_min_mm + 3.0, 0.4 * height), max(height - 3.0, 0.6 * height))
        th = rng.uniform(0.0, np.pi)
        u = (X - cx) * np.cos(th) + (Z - cz) * np.sin(th)
        v = -(X - cx) * np.sin(th) + (Z - cz) * np.cos(th)
        labels[(u / a) ** 2 + (v / b) ** 2 <= 1.0] = k
    return labels


def visco2d_1024(n_grid=1024, n_steps=4000, n_rec=256, seed=0, n_incl=8):
    dx, pml = 0.05, 20
    roi, roi_n = _roi2d(n_grid, dx, pml)
    rng = np.random.default_rng(seed)
    labels = _ellipses((roi_n, roi_n), dx, rng, n_incl)
    cp = np.full((roi_n, roi_n), 5.9, np.float32)
    cs = np.full((roi_n, roi_n), 3.23, np.float32)
    rho = np.full((roi_n, roi_n), 7850.0, np.float32)
    incl = labels > 0
    cp[incl], cs[incl], rho[incl] = 1.48, 0.0, 1000.0
    q = rng.uniform(50.0, 200.0, (n_incl + 1, 2)).astype(np.float32)  # row 0: background
    qp, qs = q[labels, 0], q[labels, 1]
    center = roi_n * dx / 2
    pitch = min(3 * dx, (roi_n * dx - 2.0) / n_rec)
    return {
        "roi": roi,
        "probes": [
            {"point": {"id": "src", "emitter": "True", "receiver": "False", "freq": 5.0, "bw": BW_3_CYCLES,
                       "gain": 1.0, "pulse_type": "gaussian", "coord_center": [center, 0.0, 0.1],
                       "t0_emission": 0.4}},
            {"linear": {"id": "rx", "num_elem": n_rec, "dim_a": dx, "dim_p": 0.0,
                        "inter_elem": round(pitch - dx, 6), "freq": 5.0, "bw": BW_3_CYCLES, "gain": 1.0,
                        "coord_center": [center, 0.0, 0.1], "emitters": "none", "receivers": "all",
                        "t0_reception": 0.0}},
        ],
        "simul_params": {"time_steps": n_steps, "dt": courant_dt(5.9, dx, 2), "acc": 2, "it_display": 500},
        "simul_configs": {"n_iter": 1, "show_anim": 0, "viscoelastic_attn": 1,
                          "zener_fit": {"f_min": 2.0, "f_max": 8.0, "n_sls": 3}},
        "specimen_params": {"cp": 5.9, "cs": 3.23, "rho": 7850.0, "cp_map": cp, "cs_map": cs,
                            "rho_map": rho, "qp": float(q[0, 0]), "qs": float(q[0, 1]),
                            "qp_map": qp, "qs_map": qs},
    }


def visco3d_256(n_grid=256, n_steps=1000, n_rx=64, seed=0):
    dx, pml, pad = 0.1, 16, 1
    roi_n = n_grid - 2 * pml - 2 * pad
    rng = np.random.default_rng(seed)
    bounds = np.sort(rng.choice(np.arange(roi_n // 8, roi_n - roi_n // 8), 3, replace=False))
    vp = np.sort(rng.uniform(2.7, 6.3, 4))
    vp[0], vp[-1] = 2.7, 6.3
    props = np.stack([vp, vp * 0.5 + rng.uniform(-0.05, 0.05, 4).clip(-0.05, 0.05),
                      np.sort(rng.uniform(1200.0, 7800.0, 4)), rng.uniform(30.0, 300.0, 4),
                      rng.uniform(30.0, 300.0, 4)], axis=1)
    props[:, 1] = np.clip(props[:, 1], 1.3, 3.2)
    shape = (roi_n, roi_n, roi_n)
    maps = [np.empty(shape, np.float32) for _ in range(5)]
    for k, (a, b) in enumerate(zip([0, *bounds], [*bounds, roi_n])):
        for m in range(5):
            maps[m][:, :, a:b] = props[k, m]
    center = roi_n * dx / 2
    pitch = round(min(0.3, (roi_n * dx - 1.0) / n_rx), 4)
    roi = {"coord_ref": [[0.0, 0.0, 0.0]], "height": round(roi_n * dx, 6), "h_len": roi_n,
           "width": round(roi_n * dx, 6), "w_len": roi_n, "depth": round(roi_n * dx, 6), "d_len": roi_n,
           "len_pml_xmin": pml, "len_pml_xmax": pml, "len_pml_ymin": pml, "len_pml_ymax": pml,
           "len_pml_zmin": pml, "len_pml_zmax": pml, "rcoef_pml": 0.001, "npower_pml": 2.0,
           "k_max_pml": 1.0}
    return {
        "roi": roi,
        "probes": [
            {"point": {"id": "src", "emitter": "True", "receiver": "False", "freq": 3.0, "bw": 0.5,
                       "gain": 1.0, "pulse_type": "ricker", "coord_center": [center, center, 0.5],
                       "t0_emission": 0.5}},
            {"matrix": {"id": "plane", "num_x": n_rx, "num_y": n_rx, "pitch_x": pitch, "pitch_y": pitch,
                        "coord_center": [center, center, 0.2]}},
        ],
        "simul_params": {"time_steps": n_steps, "dt": courant_dt(6.3, dx, 3), "acc": 2, "it_display": 500},
        "simul_configs": {"n_iter": 1, "show_anim": 0, "viscoelastic_attn": 1,
                          "zener_fit": {"f_min": 2.0, "f_max": 8.0, "n_sls": 3}},
        "specimen_params": {"cp": float(vp[0]), "cs": float(props[0, 1]), "rho": float(props[0, 2]),
                            "cp_map": maps[0], "cs_map": maps[1], "rho_map": maps[2],
                            "qp": float(props[0, 3]), "qs": float(props[0, 4]), "qp_map": maps[3],
                            "qs_map": maps[4]},
    }


def fmc2d_phantoms(n_steps=3000, shapes=((512, 768), (768, 768), (1024, 768)), n_elem=64, seed=0,
                   dx=0.1, pml=20):
    """Full-matrix-capture phantoms: one config per grid shape (nx, ny).

    Each is a steel block with 8 seeded fluid inclusions and per-region Q
    (as :func:`visco2d_1024`) under a 64-element linear array on the top
    surface (0.5 mm elements, 0.6 mm pitch, 5 MHz pulse of about 3 cycles),
    every element emitting and receiving.  ``dx`` = 0.1 mm so the 38.3 mm
    array fits the narrowest (512-node) phantom.  Shots (one firing element
    each) come from :func:`taichi_sim_gb300.batch.fmc_shot_sources`.
    """
    cfgs = []
    for k, (nx, ny) in enumerate(shapes):
        rng = np.random.default_rng(seed + k)
        w, h = nx - 2 * pml - 2, ny - 2 * pml - 2
        labels = _ellipses((w, h), dx, rng, 8)
        cp = np.full((w, h), 5.9, np.float32)
        cs = np.full((w, h), 3.23, np.float32)
        rho = np.full((w, h), 7850.0, np.float32)
        incl = labels > 0
        cp[incl], cs[incl], rho[incl] = 1.48, 0.0, 1000.0
        q = rng.uniform(50.0, 200.0, (9, 2)).astype(np.float32)
        roi = {"coord_ref": [[0.0, 0.0, 0.0]], "height": round(h * dx, 6), "h_len": h, "width": round(w * dx, 6),
               "w_len": w, "depth": 0.0, "d_len": 1, "len_pml_xmin": pml, "len_pml_xmax": pml,
               "len_pml_ymin": 0, "len_pml_ymax": 0, "len_pml_zmin": pml, "len_pml_zmax": pml,
               "rcoef_pml": 0.001, "npower_pml": 2.0, "k_max_pml": 1.0}
        cfgs.append({
            "roi": roi,
            "probes": [{"linear": {"id": "fmc", "num_elem": n_elem, "dim_a": 0.5, "dim_p": 10.0, "inter_elem": 0.1,
                                   "freq": 5.0, "bw": BW_3_CYCLES, "gain": 1.0,
                                   "coord_center": [w * dx / 2, 0.0, 0.2], "emitters": "all",
                                   "t0_emission": 0.4, "receivers": "all", "t0_reception": 0.0}}],
            "simul_params": {"time_steps": n_steps, "dt": courant_dt(5.9, dx, 2), "acc": 2, "it_display": 500},
            "simul_configs": {"n_iter": 1, "show_anim": 0, "viscoelastic_attn": 1,
                              "zener_fit": {"f_min": 2.0, "f_max": 8.0, "n_sls": 3}},
            "specimen_params": {"cp": 5.9, "cs": 3.23, "rho": 7850.0, "cp_map": cp, "cs_map": cs, "rho_map": rho,
                                "qp": float(q[0, 0]), "qs": float(q[0, 1]), "qp_map": q[labels, 0],
                                "qs_map": q[labels, 1]},
        })
    return cfgs


def adjoint2d_512x1024(n_steps=3000, shape=(512, 1024), n_elem=16, n_rec=256, seed=0, true_model=True,
                       n_blobs=5, dx=0.05, pml=20):
    """The adjoint-gradient experiment: a 512 x 1024 grid (x across, y in
    depth), dx = 0.05 mm, 20-cell CPML; true model = steel with n_blobs
    seeded Gaussian blobs of +-5 % in vp and vs (sigma 1-2 mm), start model
    = plain steel (``true_model=False``); viscoelastic with the reference's
    fixed relaxation times (L = 3, no per-cell Q); a 16-element linear array
    (0.5 mm elements, 0.6 mm pitch, 5 MHz pulse of about 3 cycles) on the top
    surface, shot e firing element e (shots from
    :func:`taichi_sim_gb300.batch.fmc_shot_sources`), and 256 one-node
    receivers at 1.5 dx pitch under it; 3000 steps."""
    nx, ny = shape
    w, h = nx - 2 * pml - 2, ny - 2 * pml - 2
    rng = np.random.default_rng(seed)
    cp = np.full((w, h), 5.9, np.float32)
    cs = np.full((w, h), 3.23, np.float32)
    rho = np.full((w, h), 7850.0, np.float32)
    if true_model:
        X, Z = np.meshgrid(np.arange(w) * dx, np.arange(h) * dx, indexing="ij")
        pert = np.zeros((w, h))
        for _ in range(n_blobs):
            cx, cz = rng.uniform(0.2, 0.8) * w * dx, rng.uniform(0.15, 0.7) * h * dx
            s = rng.uniform(1.0, 2.0)
            pert += rng.choice([-1.0, 1.0]) * 0.05 * np.exp(-((X - cx) ** 2 + (Z - cz) ** 2) / (2 * s * s))
        cp = (cp * (1 + pert)).astype(np.float32)
        cs = (cs * (1 + pert)).astype(np.float32)
    roi = {"coord_ref": [[0.0, 0.0, 0.0]], "height": round(h * dx, 6), "h_len": h, "width": round(w * dx, 6),
           "w_len": w, "depth": 0.0, "d_len": 1, "len_pml_xmin": pml, "len_pml_xmax": pml,
           "len_pml_ymin": 0, "len_pml_ymax": 0, "len_pml_zmin": pml, "len_pml_zmax": pml,
           "rcoef_pml": 0.001, "npower_pml": 2.0, "k_max_pml": 1.0}
    center = w * dx / 2
    return {
        "roi": roi,
        "probes": [
            {"linear": {"id": "tx", "num_elem": n_elem, "dim_a": 0.5, "dim_p": 10.0, "inter_elem": 0.1,
                        "freq": 5.0, "bw": BW_3_CYCLES, "gain": 1.0, "coord_center": [center, 0.0, 0.2],
                        "emitters": "all", "t0_emission": 0.4, "receivers": "none", "t0_reception": 0.0}},
            {"linear": {"id": "rx", "num_elem": n_rec, "dim_a": dx, "dim_p": 0.0, "inter_elem": 0.5 * dx,
                        "freq": 5.0, "bw": BW_3_CYCLES, "gain": 1.0, "coord_center": [center, 0.0, 0.3],
                        "emitters": "none", "receivers": "all", "t0_reception": 0.0}},
        ],
        "simul_params": {"time_steps": n_steps, "dt": courant_dt(5.9 * 1.06, dx, 2), "acc": 2, "it_display": 500},
        "simul_configs": {"n_iter": 1, "show_anim": 0, "viscoelastic_attn": 1},
        "specimen_params": {"cp": 5.9, "cs": 3.23, "rho": 7850.0, "cp_map": cp, "cs_map": cs, "rho_map": rho},
    }


WORKLOADS = {"elastic2d": elastic2d_512, "visco2d": visco2d_1024, "visco3d": visco3d_256}

# Algorithmic bytes per cell-update (float32): every per-cell state array
# read and written once per step, per-cell material (and Q) read once, CPML
# memories counted on strip cells only (dead arrays, sources and receivers
# excluded).  Fixed by the benchmark definition.
B_ALG = {"elastic2d": 57.0, "visco2d": 134.5, "visco3d": 254.0}
