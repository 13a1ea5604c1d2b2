"""Probability outputs of a chronicled run as device tensors (no plotting).

  probability          pgrid / total_weight                 (oneka/visualize.py:230)
  smoothed_probability gaussian_filter(Z, smooth, mode='constant', cval=0)
                                                            (oneka/visualize.py:232-233)
  impact_curve         probabilities sorted in decreasing order against
                       cumulative area                      (oneka/visualize.py:382-385)
  decile_table         Pr(capture) exceeds p -> area        (oneka/oneka.py:278-288)

Smoothing runs the oneka_gaussian_filter kernel; the impact curve comes from
the oneka_count_histogram kernel over the int32 visit counts (every
probability is count / R, so the sorted curve is a cumulative histogram).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _capi as C

ACRE_M2 = 4046.86          # m^2 per acre, as the reference reports areas


class CaptureZoneError(Exception):
    """Empty capture zone (oneka/visualize.py:224-226)."""


def _pgrid(pfield) -> torch.Tensor:
    """The field's weighted counts as a device tensor (a field held on the
    host, such as one loaded from an archive, is copied to the device)."""
    dev = getattr(pfield, "pgrid_device", None)
    if dev is not None:
        return dev
    return torch.as_tensor(np.asarray(pfield.pgrid, dtype=np.float64), device=C.device())


def probability(pfield) -> torch.Tensor:
    """pgrid / total_weight as an IEEE division per cell, as NumPy computes it
    (a tensor divided by a Python scalar would be multiplied by the
    reciprocal instead, which differs in the last bit)."""
    if pfield.total_weight <= 0:
        raise CaptureZoneError("Empty capture zone")
    pg = _pgrid(pfield)
    return torch.div(pg, torch.full_like(pg, float(pfield.total_weight)))


def gaussian_weights(sigma: float, truncate: float = 4.0) -> np.ndarray:
    """The 1-D Gaussian weights scipy.ndimage uses for this sigma (radius
    int(truncate * sigma + 0.5), normalized to sum 1)."""
    radius = int(truncate * float(sigma) + 0.5)
    x = np.arange(-radius, radius + 1)
    phi = np.exp(-0.5 / (float(sigma) * float(sigma)) * x ** 2)
    return phi / phi.sum()


def smoothed_probability(pfield, smooth) -> torch.Tensor:
    Z = probability(pfield).contiguous()
    if not smooth > 0:
        return Z
    w = torch.as_tensor(gaussian_weights(smooth), device=Z.device)
    out = torch.empty_like(Z)
    tmp = torch.empty_like(Z)
    C.check(C.load().oneka_gaussian_filter(C.ptr(Z), C.ptr(out), C.ptr(tmp), Z.shape[0], Z.shape[1],
                                           C.ptr(w), (w.numel() - 1) // 2, C.stream_ptr()))
    return out


def _integer_counts(pfield):
    counts = getattr(pfield, "counts", None)
    if counts is not None:
        return counts
    pg = _pgrid(pfield)
    if float(pfield.total_weight).is_integer() and bool((pg == torch.round(pg)).all()):
        return pg.to(torch.int32)
    return None


def impact_curve(spacing, pfield):
    """(pr, area): probabilities in decreasing order and the cumulative area
    [m^2] whose probability of capture is at least pr (visualize.py:382-385)."""
    if pfield.total_weight <= 0:
        raise CaptureZoneError("Empty capture zone")
    counts = _integer_counts(pfield)
    n = int(_pgrid(pfield).numel())
    if counts is not None and float(pfield.total_weight) == float(int(pfield.total_weight)):
        R = int(pfield.total_weight)
        nb = int(max(R, int(counts.max().item())) + 1)
        hist = torch.zeros(nb, dtype=torch.int64, device=counts.device)
        c = counts.contiguous()
        C.check(C.load().oneka_count_histogram(C.ptr(c), c.numel(), nb, C.ptr(hist), C.stream_ptr()))
        h = hist.cpu().numpy()
        values = np.arange(nb - 1, -1, -1, dtype=np.float64) / float(pfield.total_weight)
        pr = np.repeat(values, h[::-1])
    else:   # non-integer weights: sort the probabilities on the device
        pr = torch.sort(probability(pfield).reshape(-1), descending=True).values.cpu().numpy()
    area = (np.arange(n) + 1) * spacing ** 2
    return pr, area


def decile_table(pr, area):
    """[(p, pr[i], area_m2, area_acres)] for p = 0.05 .. 0.95 (oneka/oneka.py:278-288)."""
    rows = []
    for p in np.linspace(0.05, 0.95, 19):
        i = int(np.argmax(pr <= p))
        rows.append((float(p), float(pr[i]), float(area[i]), float(area[i] / ACRE_M2)))
    return rows
