"""Drop-in stochastic capture zone of oneka/stochastic.py:76-376 on the GPU.

``create_stochastic_capturezone`` keeps the reference's signature and returns
a ``ProbabilityField``.  Every realization is drawn, fitted and MVN-drawn by
``oneka_realize`` (Philox counter streams instead of NumPy's global RNG, so a
run is reproducible from ``seed``), then all particles of all realizations
are tracked and chronicled by ``oneka_track``.

By default the result replays the reference's auto-expanding grid exactly (a
first pass records every trace's bounding box).  Passing ``window=half_width``
instead fixes the grid to the square of that half width around the target
well, the fast path for large runs: traces leaving it are clipped.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _capi as C
from . import engine as E
from .engine import DistributionError, Lognormal
from .probabilityfield import ProbabilityField
from .model import RangeError


def _check_status(real: E.Realizations):
    st = real.status.cpu().numpy()
    if np.any(st == C.REAL_RANGE):
        raise RangeError("model.fit_coeficient: elevation < base")
    if np.any(st == C.REAL_NOT_SPD):
        raise np.linalg.LinAlgError("normal equations are not positive definite")


def create_stochastic_capturezone(
        target, npaths, duration, nrealizations,
        base, c_dist, p_dist, t_dist,
        stochastic_wells, observations,
        spacing, umbra, confined,
        tol, maxstep, *, seed=0, precision=C.FP64, window=None, chunk=4096,
        mode=C.MODE_STOCHASTIC):
    """Stochastic capture zone of the target well (oneka/stochastic.py:76-270)."""
    dev = C.device()
    site = E.Site(stochastic_wells, observations, base, target=target, c_dist=c_dist, p_dist=p_dist,
                  t_dist=t_dist, device=dev)
    real = E.realize(site, nrealizations, seed=seed, mode=mode)
    _check_status(real)
    opts = E.TrackOptions(duration=duration, tol=tol, maxstep=maxstep, umbra=umbra,
                          confined=confined, precision=precision)
    release = torch.as_tensor(site.release(npaths), device=dev)
    if precision == C.FP32 and nrealizations >= 256:
        opts = E.autotune(site, real, release, opts, E.Grid.window(site.xt, site.yt, spacing,
                                                                   window or 2000.0))
    pfield = ProbabilityField(spacing, spacing, site.xt, site.yt)
    if window is not None:
        grid = E.Grid.window(site.xt, site.yt, spacing, window)
        pfield.expand(grid.xmin + 0.5 * spacing, grid.xmin + (grid.ncols - 1.5) * spacing,
                      grid.ymin + 0.5 * spacing, grid.ymin + (grid.nrows - 1.5) * spacing)
        frames = None
    else:
        # pass 1: bounding boxes in the reference's order (realization, then path)
        bbs = []
        for a in range(0, nrealizations, chunk):
            sub = real.slice(a, min(nrealizations, a + chunk))
            out = E.TrackOutputs.alloc(sub.n, npaths, dev, endpoint=False, bbox=True, stats=False)
            E.track(site, sub, release, opts, E.Grid(0.0, 0.0, 1.0, 1.0, 1, 1), outputs=out)
            bbs.append(out.bbox.reshape(-1, 4).cpu().numpy())
        bb = np.concatenate(bbs) if bbs else np.zeros((0, 4))
        g0 = (pfield.xmin, pfield.xmax, pfield.ymin, pfield.ymax)
        _, frames_np = E.replay_expand(None, None, spacing, spacing, bb, grid0=g0)
        if bb.shape[0]:
            pfield.expand(bb[:, 0].min(), bb[:, 1].max(), bb[:, 2].min(), bb[:, 3].max())
        frames = frames_np
        grid = pfield._grid()
    counts = torch.zeros((grid.nrows, grid.ncols), dtype=torch.int32, device=dev)
    registered = torch.zeros(1, dtype=torch.int64, device=dev)
    for a in range(0, nrealizations, chunk):
        b = min(nrealizations, a + chunk)
        fr = None
        if frames is not None and npaths > 0:
            fr = torch.frombuffer(bytearray(frames[a * npaths:b * npaths].tobytes()),
                                  dtype=torch.uint8).to(dev)
        E.track(site, real.slice(a, b), release, opts, grid, counts=counts, registered=registered,
                frames=fr)
    pfield.counts = counts
    pfield.pgrid = counts.to(torch.float64)
    pfield.total_weight = float(registered.item())
    pfield.realizations = real
    return pfield


def generate_random_variate(arg):
    """A variate from a constant, uniform or triangular distribution
    (oneka/stochastic.py:274-306), drawn from NumPy's global generator on the
    host like the reference.  The GPU path draws its own (Philox) variates."""
    if type(arg) is not tuple:
        value = arg
    elif len(arg) == 2:
        value = np.random.uniform(arg[0], arg[1])
    elif len(arg) == 3:
        value = np.random.triangular(arg[0], arg[1], arg[2])
    else:
        raise DistributionError('<arg> must be a scalar, pair, or triple.')
    return value


def compute_variate_mean(arg):
    """Mean of a constant, uniform or triangular distribution (oneka/stochastic.py:310-342)."""
    if isinstance(arg, Lognormal):
        return float(np.exp(arg.mu + 0.5 * arg.sigma**2))
    if type(arg) is not tuple:
        value = arg
    elif len(arg) == 2:
        value = (arg[0] + arg[1]) / 2.0
    elif len(arg) == 3:
        value = (arg[0] + arg[1] + arg[2]) / 3.0
    else:
        raise DistributionError('<arg> must be a scalar, pair, or triple.')
    return value


def isdistribution(arg, lb, ub):
    """Do the arguments define a valid distribution? (oneka/stochastic.py:345-376)"""
    if isinstance(arg, int) or isinstance(arg, float):
        return lb <= arg <= ub
    if isinstance(arg, tuple) or isinstance(arg, list):
        if len(arg) == 2:
            return lb <= arg[0] <= arg[1] <= ub
        elif len(arg) == 3:
            return lb <= arg[0] <= arg[1] <= arg[2] <= ub
    return False
