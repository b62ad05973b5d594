"""Host-side model of the staggered-grid (visco)elastic stepper.

Mirrors the public surface of the reference project's ``sim_support`` package
(``sim_support/__init__.py``): scalar types, module constants, the staggered
finite-difference coefficient tables and the two exceptions raised by the
time loop.  The CUDA engine in :mod:`taichi_sim_gb300.engine` consumes the
tables that :class:`~taichi_sim_gb300.sim_support.simulator.Simulator` builds.
"""
import numpy as np

flt32 = np.float32
int32 = np.int32

PI = flt32(np.pi)
DEGREES_TO_RADIANS = flt32(PI / 180.0)
ZERO = flt32(0.0)
# A squared velocity norm above this marks a run as unstable
# (sim_support/__init__.py:16 in the reference).
STABILITY_THRESHOLD = flt32(1.0e38)
HUGEVAL = flt32(1.0e30)

# Staggered-grid first-derivative weights of Lui & Sen (2009),
# doi:10.1111/j.1365-246X.2009.04305.x.  Row ``acc - 2`` holds ``acc``
# weights; the published values must be identical to the reference's table
# (sim_support/__init__.py:20-28) for the stencils to agree.
coefs_Lui = [
    [9.0 / 8.0, -1.0 / 24.0],
    [75.0 / 64.0, -25.0 / 384.0, 3.0 / 640.0],
    [1225.0 / 1024.0, -245.0 / 3072.0, 49.0 / 5120.0, -5.0 / 7168.0],
    [19845.0 / 16384.0, -735.0 / 8192.0, 567.0 / 40960.0, -405.0 / 229376.0,
     35.0 / 294912.0],
    [160083.0 / 131072.0, -12705.0 / 131072.0, 22869.0 / 1310720.0,
     -5445.0 / 1835008.0, 847.0 / 2359296.0, -63.0 / 2883584.0],
]

# Forward (non-staggered) first-derivative weights used by the "unsplit"
# model family (sim_support/__init__.py:32-42); the mirrored backward weights
# are these reversed with the sign flipped.
coefs_forward = [
    [-2.0 / 6.0, -3.0 / 6.0, 6.0 / 6.0, -1.0 / 6.0],
    [3.0 / 60.0, -30.0 / 60.0, -20.0 / 60.0, 60.0 / 60.0, -15.0 / 60.0, 2.0 / 60.0],
    [-4.0 / 420.0, 42.0 / 420.0, -252.0 / 420.0, -105.0 / 420.0, 420.0 / 420.0,
     -126.0 / 420.0, 28.0 / 420.0, -3.0 / 420.0],
    [5.0 / 2520.0, -60.0 / 2520.0, 360.0 / 2520.0, -1680.0 / 2520.0, -504.0 / 2520.0,
     2520.0 / 2520.0, -840.0 / 2520.0, 240.0 / 2520.0, -45.0 / 2520.0, 4.0 / 2520.0],
    [-12.0 / 27720.0, 165.0 / 27720.0, -1100.0 / 27720.0, 4950.0 / 27720.0,
     -19800.0 / 27720.0, -4620.0 / 27720.0, 27720.0 / 27720.0, -9900.0 / 27720.0,
     3300.0 / 27720.0, -825.0 / 27720.0, 132.0 / 27720.0, -10.0 / 27720.0],
]


class CourantError(ValueError):
    """The time step breaks the CFL bound (Courant number above 1).

    Same constructor and ``str`` form as the reference
    (sim_support/__init__.py:48-61): ``CourantError(message, value)``.
    """

    def __init__(self, mensagem, valor):
        super().__init__(mensagem)
        self.valor = valor

    def __str__(self):
        return f"{super().__str__()} [Valor: {self.valor}]"


class StabilityError(ValueError):
    """The wavefield is blowing up (velocity norm above the threshold).

    Same constructor and ``str`` form as the reference
    (sim_support/__init__.py:65-76): ``StabilityError(message, value)``.
    """

    def __init__(self, mensagem, valor):
        super().__init__(mensagem)
        self.valor = valor

    def __str__(self):
        return f"{super().__str__()} [Valor: {self.valor}]"


__all__ = ['flt32', 'int32', 'PI', 'DEGREES_TO_RADIANS', 'ZERO',
           'STABILITY_THRESHOLD', 'HUGEVAL', 'coefs_Lui', 'coefs_forward',
           'CourantError', 'StabilityError']
