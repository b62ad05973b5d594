"""Drop-in alias of :mod:`taichi_sim_gb300.sim_support.gauss_wavelets`."""
from taichi_sim_gb300.sim_support.gauss_wavelets import *  # noqa: F401,F403
from taichi_sim_gb300.sim_support import gauss_wavelets as _impl

globals().update({k: v for k, v in vars(_impl).items() if not k.startswith("__")})
