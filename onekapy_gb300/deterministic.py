"""Drop-in deterministic capture zone of oneka/deterministic.py:65-235.

The mean of every distribution (compute_variate_mean), the fit's mean
coefficients (coef = coef_ev) and one realization of the same GPU pipeline.
"""
from __future__ import annotations

from . import _capi as C
from .stochastic import create_stochastic_capturezone


def create_deterministic_capturezone(
        target, npaths, duration,
        base, c_dist, p_dist, t_dist,
        stochastic_wells, observations,
        spacing, umbra, confined,
        tol, maxstep, *, precision=C.FP64, window=None):
    """Deterministic capture zone of the target well (oneka/deterministic.py:65-235)."""
    return create_stochastic_capturezone(
        target, npaths, duration, 1, base, c_dist, p_dist, t_dist, stochastic_wells, observations,
        spacing, umbra, confined, tol, maxstep, precision=precision, window=window,
        mode=C.MODE_MEAN)
