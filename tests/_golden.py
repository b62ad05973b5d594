"""Loaders for the committed golden fixtures (tests/golden/)."""
import copy
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def experiments():
    with open(os.path.join(GOLDEN, "experiments.json")) as f:
        return json.load(f)


def config_with_maps(name):
    """The experiment's config with every ``*_map`` path replaced by its array."""
    exp = experiments()[name]
    cfg = copy.deepcopy(exp["config"])
    path = os.path.join(GOLDEN, f"inputs_{name}.npz")
    spec = cfg["specimen_params"]
    if name == "teste_pedro":
        maps = np.load(os.path.join(GOLDEN, "inputs_pedro.npz"))
        for k in ("cp", "cs", "rho"):
            spec[f"{k}_map"] = maps[k]
    elif os.path.exists(path):
        maps = np.load(path)
        for k in list(spec):
            if k.endswith("_map"):
                spec[k] = maps[k]
    cfg["simul_configs"]["show_anim"] = 0
    return exp["dims"], cfg


def tables(name):
    return np.load(os.path.join(GOLDEN, f"tables_{name}.npz"))


def golden_bscan():
    return np.load(os.path.join(GOLDEN, "bscan_teste_aco.npz"))["bscan"]
