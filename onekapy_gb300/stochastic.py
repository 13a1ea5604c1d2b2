"""Drop-in stochastic capture zone of oneka/stochastic.py:76-376 on the GPU.

``create_stochastic_capturezone`` keeps the reference's signature and returns
a ``ProbabilityField``.  Every realization is drawn, fitted and MVN-drawn by
``oneka_realize`` (Philox counter streams instead of NumPy's global RNG, so a
run is reproducible from ``seed``), then all particles of all realizations
are tracked and chronicled by ``oneka_track``.

By default the result replays the reference's auto-expanding grid exactly (a
first pass records every trace's bounding box).  Passing ``window=half_width``
instead fixes the grid to the square of that half width around the target
well, the fast path for large runs: traces leaving it are clipped (counted
in ``pfield.traces_leaving_grid``).

A fixed-window run can be checkpointed: ``checkpoint=path`` saves the counts
after every chunk of realizations and resumes from a saved state of the same
inputs; ``max_chunks`` stops after that many chunks (``pfield.complete`` is
then False) so that a later call continues the run.  The resumed counts equal
those of an uninterrupted run.
"""
from __future__ import annotations

import logging

import numpy as np
import torch

from . import _capi as C
from . import checkpoint as CK
from . import engine as E
from .engine import DistributionError, Lognormal
from .probabilityfield import ProbabilityField
from .model import RangeError


log = logging.getLogger("Oneka")


def _log_realizations(real: E.Realizations, base: float):
    """The reference's per-realization log lines (oneka/stochastic.py:243-250),
    written only when the "Oneka" logger takes INFO (one copy to the host)."""
    if not log.isEnabledFor(logging.INFO) or real.coef_ev is None:
        return
    coef = real.coef.cpu().numpy()
    ev = real.coef_ev.cpu().numpy()
    aq = real.aquifer.cpu().numpy()
    for i in range(real.n):
        K, n, H = aq[i]
        c, e = coef[i], ev[i]
        log.info("Realization #%d: %.2f, %.2f, %.2f, %.2f, %.4e", i, base, K, n, H, 2 * (c[0] + c[1]))
        log.info("    coef ev:  (%+.4e, %+.4e, %+.4e, %+.4e, %+.4e, %+.4e)", *e)
        log.info("    coef rng: (%+.4e, %+.4e, %+.4e, %+.4e, %+.4e, %+.4e)", *c)


# Geometry a fresh field reaches when expanded to a fixed window: the
# expansion replays the reference's repeated += / -= one node at a time (a
# host loop), so the outcome is kept per (spacing, target, window grid).
_window_fields: dict = {}


def _window_field(spacing, xt, yt, grid: E.Grid) -> ProbabilityField:
    pfield = ProbabilityField(spacing, spacing, xt, yt)
    key = (float(spacing), float(xt), float(yt), grid.xmin, grid.ymin, grid.nrows, grid.ncols)
    geo = _window_fields.get(key)
    if geo is None:
        pfield.expand(grid.xmin + 0.5 * spacing, grid.xmin + (grid.ncols - 1.5) * spacing,
                      grid.ymin + 0.5 * spacing, grid.ymin + (grid.nrows - 1.5) * spacing)
        _window_fields[key] = (pfield.xmin, pfield.xmax, pfield.ymin, pfield.ymax, pfield.nrows, pfield.ncols)
    else:
        pfield.xmin, pfield.xmax, pfield.ymin, pfield.ymax, pfield.nrows, pfield.ncols = geo
        pfield._alloc()
    return pfield


def _check_status(real: E.Realizations):
    st = real.status.cpu().numpy()
    if np.any(st == C.REAL_RANGE):
        raise RangeError("model.fit_coeficient: elevation < base")
    if np.any(st == C.REAL_NOT_SPD):
        raise np.linalg.LinAlgError("normal equations are not positive definite")
    if np.any(st == C.REAL_NOT_FINITE):
        raise np.linalg.LinAlgError("the regional-flow fit is not finite (an observation on a well? "
                                    "utilities.filter_obs removes observations within a buffer of the wells)")


def create_stochastic_capturezone(
        target, npaths, duration, nrealizations,
        base, c_dist, p_dist, t_dist,
        stochastic_wells, observations,
        spacing, umbra, confined,
        tol, maxstep, *, seed=0, precision=C.FP64, window=None, chunk=4096,
        mode=C.MODE_STOCHASTIC, checkpoint=None, max_chunks=None):
    """Stochastic capture zone of the target well (oneka/stochastic.py:76-270)."""
    if checkpoint is not None and window is None:
        raise ValueError("checkpoint needs a fixed window (the auto-expanding grid is known only at the end)")
    dev = C.device()
    site = E.Site(stochastic_wells, observations, base, target=target, c_dist=c_dist, p_dist=p_dist,
                  t_dist=t_dist, device=dev)
    real = E.realize(site, nrealizations, seed=seed, mode=mode)
    _check_status(real)
    if mode == C.MODE_STOCHASTIC:
        _log_realizations(real, base)
    opts = E.TrackOptions(duration=duration, tol=tol, maxstep=maxstep, umbra=umbra,
                          confined=confined, precision=precision)
    release = torch.as_tensor(site.release(npaths), device=dev)
    if precision == C.FP32 and nrealizations >= 256:
        opts = E.autotune(site, real, release, opts, E.Grid.window(site.xt, site.yt, spacing,
                                                                   window or 2000.0))
    if window is not None:
        grid = E.Grid.window(site.xt, site.yt, spacing, window)
        pfield = _window_field(spacing, site.xt, site.yt, grid)
        frames = None
    else:
        pfield = ProbabilityField(spacing, spacing, site.xt, site.yt)
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
    state = None
    first = 0
    counts = torch.zeros((grid.nrows, grid.ncols), dtype=torch.int32, device=dev)
    registered = torch.zeros(1, dtype=torch.int64, device=dev)
    if checkpoint is not None:
        sig = CK.signature(target=target, npaths=npaths, duration=duration, nrealizations=nrealizations,
                           base=base, c_dist=c_dist, p_dist=p_dist, t_dist=t_dist,
                           stochastic_wells=stochastic_wells, observations=observations, spacing=spacing,
                           umbra=umbra, confined=confined, tol=tol, maxstep=maxstep, seed=seed,
                           precision=precision, window=window, mode=mode)
        state = CK.open_state(checkpoint, sig, (grid.nrows, grid.ncols), nrealizations)
        counts.copy_(torch.from_numpy(state.counts))
        registered.fill_(state.registered)
        first = state.next_realization
    counters = torch.zeros(E.COUNTERS, dtype=torch.int64, device=dev)
    if state is not None:          # the resumed run's counters continue the saved ones
        counters.copy_(torch.from_numpy(state.counters))
    out = E.TrackOutputs(counters=counters)
    done_chunks = 0
    a = first
    while a < nrealizations and (max_chunks is None or done_chunks < max_chunks):
        b = min(nrealizations, a + chunk)
        fr = None
        if frames is not None and npaths > 0:
            fr = torch.frombuffer(bytearray(frames[a * npaths:b * npaths].tobytes()),
                                  dtype=torch.uint8).to(dev)
        E.track(site, real.slice(a, b), release, opts, grid, counts=counts, registered=registered,
                frames=fr, outputs=out)
        a = b
        done_chunks += 1
        if state is not None:
            state.counts = counts.cpu().numpy()
            state.registered = int(registered.item())
            state.counters = counters.cpu().numpy()
            state.next_realization = a
            state.save(checkpoint)
    pfield.counts = counts
    pfield.pgrid = counts.to(torch.float64)
    pfield.total_weight = float(registered.item())
    pfield.realizations = real
    pfield.complete = a >= nrealizations
    c = counters.cpu().tolist()
    pfield.trace_counters = dict(zip(E.COUNTER_NAMES[:7], c[:7]))
    pfield.traces_leaving_grid = int(c[6])
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
