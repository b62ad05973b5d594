"""Generate the golden fixtures under tests/golden/ from the reference project.

Run where a checkout of the reference project is available (read-only is
enough), naming it with ``--ref`` or the ``TAICHI_SIM_REF`` environment
variable::

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py --ref <checkout>

What it writes (all small, compressed):

* ``tables_<name>.npz`` - the host tables the reference's own ``sim_support``
  builds for each experiment below (CPML vectors, source terms, source and
  receiver maps, delays, material grids).  Large arrays are stored as a
  sha256 of their bytes plus shape/dtype; small ones verbatim.  The GUI
  modules the reference imports at module level (matplotlib, pyqtgraph,
  PyQt6) are replaced by empty stubs; ``show_anim`` is forced off.
* ``inputs_pedro.npz`` - the cp/cs/rho maps of ``pedro/teste_pedro.json``.
* ``bscan_teste_aco.npz`` - the reference's only known-answer result,
  ``pedro/results/result_teste_aco.npy``: the Taichi elastic B-scan of
  ``pedro/teste_pedro.json`` (10000 steps, 64 receivers).
* ``experiments.json`` - the experiment descriptions used, with map paths
  rewritten to keys of the inputs files.
"""
import argparse
import ast
import hashlib
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SMALL = 1 << 16  # arrays with at most this many elements are stored verbatim


def stub_gui():
    class _Stub:
        def __init__(self, *a, **k):
            pass

        def __getattr__(self, name):
            return _Stub()

        def __call__(self, *a, **k):
            return _Stub()

    class _Any(types.ModuleType):
        __all__ = []

        def __getattr__(self, name):
            if name.startswith("__"):
                raise AttributeError(name)
            return _Stub

    for name in ("matplotlib", "matplotlib.pyplot", "pyqtgraph", "pyqtgraph.widgets",
                 "pyqtgraph.widgets.RawImageWidget", "PyQt6", "PyQt6.QtWidgets", "PyQt6.QtCore",
                 "PyQt6.QtGui"):
        sys.modules[name] = _Any(name)
    # The live-view window module subclasses Qt widgets at import time.
    qt_window = types.ModuleType("sim_support.windows_qt")
    qt_window.Window = _Stub
    sys.modules["sim_support.windows_qt"] = qt_window


def digest(a):
    a = np.ascontiguousarray(a)
    return hashlib.sha256(a.tobytes()).hexdigest()


TABLE_ATTRS = ["_nx", "_ny", "_nz", "_dt", "_dx", "_dy", "_dz", "_coefs", "_n_steps", "_n_src", "_n_rec",
               "_n_pto_src", "_n_pto_rec", "_idx_rec_offset", "_idx_src_offset", "_delay_recv",
               "_info_rec_pt", "_offset_sensors", "_source_term", "_pos_sources", "_pos_sensors",
               "_rho_grid_vx", "_cp_grid_vx", "_cs_grid_vx", "_ix_src", "_iy_src", "_ix_rec", "_iy_rec",
               "_idx_rec", "_gain"]
PML = [f"_{c}_{ax}{h}" for ax in "xyz" for c in "abk" for h in ("", "_half")]


def snapshot(sim):
    out = dict()
    for name in TABLE_ATTRS + PML + ["_iz_src", "_iz_rec"]:
        if not hasattr(sim, name):
            continue
        v = np.asarray(getattr(sim, name))
        key = name.lstrip("_")
        out[f"{key}.shape"] = np.array(v.shape, dtype=np.int64)
        out[f"{key}.dtype"] = np.array(str(v.dtype))
        out[f"{key}.sha"] = np.array(digest(v))
        if v.size <= SMALL:
            out[key] = v
    return out


EXPERIMENTS = {
    # name: (config path relative to the reference, dims, overrides)
    "teste_pedro": ("pedro/teste_pedro.json", 2, {}),
    "ponto": ("ensaios/ponto/ponto.json", 2, {}),
    "tat_cfg3": ("ensaios/ensaio_tat/bloquinho_tat_cfg3.json", 2, {}),
    "bloquinho": ("ensaios/bloquinho/bloquinho.json", 2, {}),
    "mono_aco": ("ensaios/ensaio_mono/aco_cfg.json", 3, {}),
}


def synthetic_point_line(n=128):
    """A config-1-like 2D experiment: point vy source + line of 1-node receivers."""
    return {
        "roi": {"coord_ref": [[0.0, 0.0, 0.0]], "height": 23.5, "h_len": 470, "width": 23.5, "w_len": 470,
                "depth": 0.0, "d_len": 1, "len_pml_xmin": 20, "len_pml_xmax": 20, "len_pml_ymin": 0,
                "len_pml_ymax": 0, "len_pml_zmin": 20, "len_pml_zmax": 20, "rcoef_pml": 0.001,
                "npower_pml": 2.0, "k_max_pml": 1.0},
        "probes": [
            {"point": {"id": "src", "emitter": "True", "receiver": "False", "freq": 5.0, "bw": 0.5,
                       "gain": 1.0, "pulse_type": "gaussian", "coord_center": [11.75, 0.0, 0.45],
                       "t0_emission": 0.3}},
            {"linear": {"id": "rx", "num_elem": n, "dim_a": 0.05, "dim_p": 0.0, "inter_elem": 0.1,
                        "freq": 5.0, "bw": 0.5, "gain": 1.0, "coord_center": [11.75, 0.0, 0.45],
                        "emitters": "none", "receivers": "all", "t0_reception": 0.0}},
        ],
        "simul_params": {"time_steps": 300, "dt": 2.797e-3, "acc": 2, "it_display": 100},
        "simul_configs": {"n_iter": 1, "show_anim": 0, "viscoelastic_attn": 0},
        "specimen_params": {"cp": 6.32, "cs": 3.13, "rho": 2700.0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("TAICHI_SIM_REF"),
                    help="checkout of the reference project (or set TAICHI_SIM_REF)")
    args = ap.parse_args()
    if not args.ref:
        ap.error("name the reference checkout with --ref or TAICHI_SIM_REF")
    ref = os.path.abspath(args.ref)
    stub_gui()
    sys.path.insert(0, ref)
    os.chdir(ref)
    from sim_support.simulator import Simulator
    from sim_support.Simulator3D import Simulator3D

    experiments = dict()
    for name, (path, dims, _) in EXPERIMENTS.items():
        with open(path) as f:
            cfg = ast.literal_eval(f.read())
        cfg["simul_configs"]["show_anim"] = 0
        tmp = os.path.join("/tmp", f"_golden_{name}.json")
        with open(tmp, "w") as f:
            f.write(repr(cfg))
        sim = (Simulator if dims == 2 else Simulator3D)(tmp, sim_type="viscoelastic")
        np.savez_compressed(os.path.join(HERE, f"tables_{name}.npz"), **snapshot(sim))
        experiments[name] = {"dims": dims, "config": cfg, "source": path}
        print("tables", name, sim._nx, sim._ny, getattr(sim, "_nz", None))

    syn = synthetic_point_line()
    tmp = "/tmp/_golden_point_line.json"
    with open(tmp, "w") as f:
        f.write(repr(syn))
    sim = Simulator(tmp, sim_type="elastic")
    np.savez_compressed(os.path.join(HERE, "tables_point_line.npz"), **snapshot(sim))
    experiments["point_line"] = {"dims": 2, "config": syn, "source": "synthetic"}

    maps = {n: np.load(f"pedro/bloquinho_pedro/{n}_aco.npy") for n in ("cp", "cs", "rho")}
    np.savez_compressed(os.path.join(HERE, "inputs_pedro.npz"), **maps)
    for key, label in (("ponto", None), ("bloquinho", "bloq"), ("tat_cfg3", "tat")):
        spec = experiments[key]["config"]["specimen_params"]
        arrays = {k: np.load(v) for k, v in spec.items() if k.endswith("_map")}
        if arrays:
            np.savez_compressed(os.path.join(HERE, f"inputs_{key}.npz"), **arrays)
    bscan = np.load("pedro/results/result_teste_aco.npy")
    np.savez_compressed(os.path.join(HERE, "bscan_teste_aco.npz"), bscan=bscan,
                        sha=np.array(digest(bscan)))
    with open(os.path.join(HERE, "experiments.json"), "w") as f:
        json.dump(experiments, f, indent=1)


if __name__ == "__main__":
    main()
