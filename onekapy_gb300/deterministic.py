"""Drop-in deterministic capture zone of oneka/deterministic.py:65-235.

The mean of every distribution (compute_variate_mean), the fit's mean
coefficients (coef = coef_ev) and one realization of the same GPU pipeline.
"""
from __future__ import annotations

import logging

from . import _capi as C
from .stochastic import create_stochastic_capturezone

log = logging.getLogger("Oneka")


def create_deterministic_capturezone(
        target, npaths, duration,
        base, c_dist, p_dist, t_dist,
        stochastic_wells, observations,
        spacing, umbra, confined,
        tol, maxstep, *, precision=C.FP64, window=None):
    """Deterministic capture zone of the target well (oneka/deterministic.py:65-235)."""
    pfield = create_stochastic_capturezone(
        target, npaths, duration, 1, base, c_dist, p_dist, t_dist, stochastic_wells, observations,
        spacing, umbra, confined, tol, maxstep, precision=precision, window=window,
        mode=C.MODE_MEAN)
    if log.isEnabledFor(logging.INFO):
        # the reference's parameter block (oneka/deterministic.py:186-205)
        coef = pfield.realizations.coef.cpu().numpy()[0]
        K, n, _ = pfield.realizations.aquifer.cpu().numpy()[0]
        log.info("\n")
        log.info("Deterministic Capture Zone Parameters: ")
        log.info("base         = %.2f", base)
        log.info("conductivity = %.2f", K)
        log.info("porosity     = %.2f", n)
        log.info("recharge     = %+.4e", -2 * (coef[0] + coef[1]))
        log.info("\n")
        log.info("Conic Discharge Potential Coefficients: ")
        for name, v in zip("ABCDEF", coef):
            log.info("%s = %+.4e", name, v)
    return pfield
