"""Drop-in alias of :mod:`taichi_sim_gb300.sim_support.emission_law`."""
from taichi_sim_gb300.sim_support.emission_law import *  # noqa: F401,F403
from taichi_sim_gb300.sim_support import emission_law as _impl

globals().update({k: v for k, v in vars(_impl).items() if not k.startswith("__")})
