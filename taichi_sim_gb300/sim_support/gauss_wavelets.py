"""Gaussian-modulated sinusoid wavelets used as source terms.

Mirrors sim_support/gauss_wavelets.py of the reference:

* :func:`gaussian_pulse` is ``scipy.signal.gausspulse`` itself (reference
  :6-7; the reference pins scipy 1.16.1, whose published algorithm is the one
  called here).
* :func:`gaussian_first_dev_pulse` is the time derivative of the
  Gaussian envelope times the carrier (reference :10-103).
* :func:`gaussian_second_dev_pulse` is the Ricker-like second derivative
  (reference :106-200).

The envelope constant follows scipy's definition: the spectrum falls by
``bwr`` dB at ``fc * (1 +- bw / 2)``, which gives
``a = -(pi fc bw)^2 / (4 ln(10^(bwr/20)))``.  The arithmetic is written in
the same operand order and with the same float32/float64 mix as the
reference so that the source tables agree bit for bit.
"""
import numpy as np
from scipy.signal import gausspulse

from . import PI


def gaussian_pulse(*args, **kwargs):
    """``scipy.signal.gausspulse`` (Gaussian-modulated cosine)."""
    return gausspulse(*args, **kwargs)


def _envelope_rate(fc, bw, bwr):
    if fc < 0:
        raise ValueError(f"Center frequency (fc={fc:.2f}) must be >=0.")
    if bw <= 0:
        raise ValueError(f"Fractional bandwidth (bw={bw:.2f}) must be > 0.")
    if bwr >= 0:
        raise ValueError(f"Reference level for bandwidth (bwr={bwr:.2f}) must be < 0 dB")
    level = pow(10.0, bwr / 20.0)
    return -(PI * fc * bw) ** 2 / (4.0 * np.log(level))


def _cutoff(a, tpr):
    if tpr >= 0:
        raise ValueError("Reference level for time cutoff must be < 0 dB")
    return np.sqrt(-np.log(pow(10.0, tpr / 20.0)) / a)


def _select(y_i, y_q, y_env, retquad, retenv):
    if retquad and retenv:
        return y_i, y_q, y_env
    if retquad:
        return y_i, y_q
    if retenv:
        return y_i, y_env
    return y_i


def gaussian_first_dev_pulse(t, fc=1000, bw=0.5, bwr=-6, tpr=-60, retquad=False, retenv=False):
    """First time-derivative of ``exp(-a t^2) cos(2 pi fc t)``.

    Returns the in-phase part, and optionally the quadrature part and the
    (signed) envelope derivative, as ``scipy.signal.gausspulse`` does.
    ``t='cutoff'`` returns the time where the envelope falls to ``tpr`` dB.
    """
    a = _envelope_rate(fc, bw, bwr)
    if isinstance(t, str):
        if t == 'cutoff':
            return _cutoff(a, tpr)
        raise ValueError("If `t` is a string, it must be 'cutoff'")
    g = np.exp(-a * t * t)
    env = -2 * g * (a * t)
    phase = 2 * PI * fc * t
    y_i = -2 * g * (a * t * np.cos(phase) + PI * fc * np.sin(phase))
    y_q = env * np.sin(2 * PI * fc * t)
    return _select(y_i, y_q, env, retquad, retenv)


def gaussian_second_dev_pulse(t, fc=1000, bw=0.5, bwr=-6, tpr=-60, retquad=False, retenv=False):
    """Second time-derivative of ``exp(-a t^2) cos(2 pi fc t)`` (Ricker-like).

    Same return conventions as :func:`gaussian_first_dev_pulse`.
    """
    a = _envelope_rate(fc, bw, bwr)
    if isinstance(t, str):
        if t == 'cutoff':
            return _cutoff(a, tpr)
        raise ValueError("If `t` is a string, it must be 'cutoff'")
    g = np.exp(-a * t * t)
    env = 2.0 * a * g * (2.0 * a * t ** 2 - 1.0)
    y_i = g * ((2.0 * a * (2.0 * a * t ** 2 - 1.0) - 4.0 * (PI * fc) ** 2) * np.cos(2 * PI * fc * t) +
               8.0 * PI * a * fc * t * np.sin(2 * PI * fc * t))
    y_q = env * np.sin(2 * PI * fc * t)
    return _select(y_i, y_q, env, retquad, retenv)
