"""Drop-in alias package: ``import sim_support`` resolves to
:mod:`taichi_sim_gb300.sim_support`, so code written against the reference's
``sim_support`` (``from sim_support.simulator import Simulator`` ...) runs
unchanged on the GB300 stepper."""
from taichi_sim_gb300.sim_support import *  # noqa: F401,F403
from taichi_sim_gb300.sim_support import (flt32, int32, PI, DEGREES_TO_RADIANS, ZERO, STABILITY_THRESHOLD,  # noqa: F401
                                          HUGEVAL, coefs_Lui, coefs_forward, CourantError, StabilityError)
