"""Zener (standard linear solid) attenuation constants.

:class:`AttenuationCoefficients` mirrors sim_support/attenuation.py:8-30 of the
reference: three mechanisms with fixed relaxation times for the P ("kappa")
and S moduli, and the sums ``sum(tau_eps / tau_sigma)`` that normalise the
memory-variable source terms.  The twelve relaxation times are data the
reference hard-codes; they are reproduced verbatim because the viscoelastic
stepper's output depends on them bit for bit.

:class:`ZenerFit` is new (the reference has no per-cell quality factor): it
fits L relaxation mechanisms to a constant-Q target over a frequency band,
so that a per-cell ``Q`` map can drive the same memory-variable recurrence.
With a spatially constant Q it reduces to the global-tau form.
"""
import numpy as np


class AttenuationCoefficients:
    """Global L=3 Zener relaxation times (units as in the reference)."""

    def __init__(self):
        self._n_sls = 3
        self._kappa_coeffs = (
            np.array([1.1063680886151313E-007, 3.1856366036932041E-008, 9.2197868528094345E-009],
                     dtype=np.float32),
            np.array([1.1026580338785149E-007, 3.1830988624149110E-008, 9.1888147513272412E-009],
                     dtype=np.float32),
        )
        self._non_kappa_coeffs = (
            np.array([1.6007136049523215E-007, 3.1849176860846836E-008, 6.3419851645615403E-009],
                     dtype=np.float32),
            np.array([1.5988027842097575E-007, 3.1825778973240451E-008, 6.3344086277835006E-009],
                     dtype=np.float32),
        )
        self._tau_epsilon_p, self._tau_sigma_p = self._kappa_coeffs
        self._tau_epsilon_s, self._tau_sigma_s = self._non_kappa_coeffs
        ratio_p = self._tau_epsilon_p / self._tau_sigma_p
        ratio_s = self._tau_epsilon_s / self._tau_sigma_s
        # Python's sum over float32 elements: ((0 + r0) + r1) + r2 in float32.
        self._sum_alpha_p = sum(ratio_p)
        self._sum_alpha_s = sum(ratio_s)

    def tau_table(self):
        """``(4, n_sls)`` float32: tau_eps_p, tau_sigma_p, tau_eps_s, tau_sigma_s."""
        return np.array([self._tau_epsilon_p, self._tau_sigma_p,
                         self._tau_epsilon_s, self._tau_sigma_s], dtype=np.float32)

    def sum_alpha(self):
        """``(2,)`` float32: sum of tau_eps/tau_sigma for P and for S."""
        return np.array([self._sum_alpha_p, self._sum_alpha_s], dtype=np.float32)


class ZenerFit:
    """Constant-Q fit of ``n_sls`` Zener mechanisms over ``[f_min, f_max]``.

    The relaxation frequencies are log-spaced over the band,
    ``tau_sigma_l = 1 / (2 pi f_l)`` (time unit = 1 / frequency unit, i.e. us
    for MHz).  In the low-loss approximation the inverse quality factor of the
    generalised body is ``Q^-1(w) = sum_l y_l w tau_l / (1 + w^2 tau_l^2)``;
    the unit weights ``y_l`` are the least-squares solution of
    ``Q^-1(w) = 1`` on 64 log-spaced frequencies, so a cell with quality
    factor Q uses ``y_l / Q`` and ``tau_eps_l = tau_sigma_l (1 + y_l / Q)``.

    Plugged into the reference's memory-variable update (deltat_phi =
    dt (1 - tau_eps/tau_sigma) / tau_sigma / sum(tau_eps/tau_sigma)), each
    mechanism's source weight factors into a per-mechanism constant times a
    per-cell scale: ``phi_l = c_l * g`` with ``c_l = -dt y_l / tau_sigma_l``
    and ``g = (1/Q) / (n_sls + (1/Q) sum(y))``.
    """

    def __init__(self, f_min=2.0, f_max=8.0, n_sls=3, n_fit=64):
        if not (f_max > f_min > 0):
            raise ValueError("need 0 < f_min < f_max")
        self.n_sls = int(n_sls)
        f_l = np.geomspace(f_min, f_max, self.n_sls) if self.n_sls > 1 else np.array([np.sqrt(f_min * f_max)])
        self.tau_sigma = 1.0 / (2.0 * np.pi * f_l)
        w = 2.0 * np.pi * np.geomspace(f_min, f_max, n_fit)
        wt = w[:, None] * self.tau_sigma[None, :]
        basis = wt / (1.0 + wt * wt)
        self.y_unit, *_ = np.linalg.lstsq(basis, np.ones(n_fit), rcond=None)
        self._basis_w = w

    def inverse_q(self, q, f):
        """Model ``Q^-1`` at frequencies ``f`` for a quality factor ``q``."""
        wt = 2.0 * np.pi * np.asarray(f, dtype=np.float64)[:, None] * self.tau_sigma[None, :]
        return (wt / (1.0 + wt * wt)) @ (self.y_unit / q)

    def mechanism_constants(self, dt):
        """Per-mechanism float32 constants ``(c, h, m)`` for a time step ``dt``.

        ``h = dt / (2 tau_sigma)`` and ``m = 1 / (1 + h)`` as in the
        reference's recurrence; ``c`` multiplies the per-cell scale ``g``.
        """
        dt = float(dt)
        c = (-dt * self.y_unit / self.tau_sigma).astype(np.float32)
        h = (0.5 * dt / self.tau_sigma).astype(np.float32)
        m = (1.0 / (1.0 + h.astype(np.float64))).astype(np.float32)
        return c, h, m

    def cell_scale(self, inv_q):
        """Per-cell float32 scale ``g = (1/Q) / (n_sls + (1/Q) sum(y))``."""
        inv_q = np.asarray(inv_q, dtype=np.float64)
        return (inv_q / (self.n_sls + inv_q * float(np.sum(self.y_unit)))).astype(np.float32)
