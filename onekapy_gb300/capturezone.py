"""Drop-in capture zone functions of oneka/capturezone.py:51-253 on the GPU.

``feval`` must be a Model-backed velocity function (``model.ModelFeval``,
what ``Model``-based callers build): the whole Dormand-Prince trace runs in
the ``oneka_track`` kernel, so an arbitrary Python callable cannot be
evaluated there and is rejected with TypeError.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _capi as C
from . import engine as E
from .model import Model, ModelFeval

DEFAULT_MAX_VERTICES_PROBE = 0


def _model_of(feval):
    if isinstance(feval, ModelFeval):
        return feval.model, feval.confined
    raise TypeError("feval must be a Model-backed velocity function (onekapy_gb300.model.ModelFeval); "
                    "arbitrary Python callables cannot run on the GPU tracker")


def _device_model(model: Model, dev):
    wells = [(float(w[0]), float(w[1]), float(w[2]), float(w[3])) for w in model.wells]
    site = E.Site(wells, np.zeros((0, 4)), model.base, target=0, xo=model.xo, yo=model.yo, device=dev)
    real = E.Realizations.given(np.asarray(model.coef, dtype=np.float64).reshape(1, 6),
                                np.array([[w[3] for w in wells]]),
                                np.array([[model.conductivity, model.porosity, model.thickness]]), dev)
    return site, real


def compute_backtrace(xs, ys, duration, tol, maxstep, feval, *, precision=C.FP64, max_attempts=0):
    """One Dormand-Prince backtrace (oneka/capturezone.py:127-253).

    Returns the list of vertices [(xs, ys), (x1, y1), ...].  A dry cell ends
    the trace early, as in the reference."""
    model, confined = _model_of(feval)
    dev = C.device()
    site, real = _device_model(model, dev)
    opts = E.TrackOptions(duration=duration, tol=tol, maxstep=maxstep, umbra=0.0, confined=confined,
                          precision=precision, max_attempts=max_attempts)
    grid = E.Grid(0.0, 0.0, 1.0, 1.0, 1, 1)
    rel = np.array([[float(xs), float(ys)]])
    probe = E.TrackOutputs.alloc(1, 1, dev, endpoint=False)
    E.track(site, real, rel, opts, grid, outputs=probe)
    nv = int(probe.nvertices.item())
    out = E.TrackOutputs.alloc(1, 1, dev, endpoint=False, max_vertices=max(nv, 1))
    E.track(site, real, rel, opts, grid, outputs=out)
    v = out.vertices[0, 0, :nv].cpu().numpy()
    return [(float(a), float(b)) for a, b in v]


def compute_capturezone(xtarget, ytarget, rtarget, npaths, duration, pfield, umbra, weight, tol,
                        maxstep, feval, *, precision=C.FP64, max_attempts=0):
    """Capture zone of the target well (oneka/capturezone.py:51-123).

    The traces are rasterized into ``pfield`` as the reference does, including
    the grid growth it performs trace by trace: a first pass records each
    trace's bounding box, the expand sequence is replayed to give every trace
    the grid it would have met, and a second pass chronicles the traces.
    """
    model, confined = _model_of(feval)
    dev = C.device()
    site, real = _device_model(model, dev)
    rel = E.release_ring(xtarget, ytarget, rtarget, npaths)
    opts = E.TrackOptions(duration=duration, tol=tol, maxstep=maxstep, umbra=umbra, confined=confined,
                          precision=precision, max_attempts=max_attempts)
    if npaths > 0:
        first = E.TrackOutputs.alloc(1, npaths, dev, endpoint=False, bbox=True, stats=False)
        E.track(site, real, rel, opts, E.Grid(0.0, 0.0, 1.0, 1.0, 1, 1), outputs=first)
        bb = first.bbox.reshape(-1, 4).cpu().numpy()
        if pfield.nrows == 0:
            # the reference's first expand on an empty field (probabilityfield.py:205-220)
            pfield.expand(bb[0, 0], bb[0, 1], bb[0, 2], bb[0, 3])
        g0 = (pfield.xmin, pfield.xmax, pfield.ymin, pfield.ymax)
        (xmin, ymin, nrows, ncols, xmax, ymax), frames = E.replay_expand(
            None, None, pfield.deltax, pfield.deltay, bb, grid0=g0)
        pfield.expand(bb[:, 0].min(), bb[:, 1].max(), bb[:, 2].min(), bb[:, 3].max())
        assert (pfield.nrows, pfield.ncols) == (nrows, ncols)
        fr = torch.frombuffer(bytearray(frames.tobytes()), dtype=torch.uint8).to(dev)
        E.track(site, real, rel, opts, pfield._grid(), frames=fr, mark_only=pfield.mask)
    pfield.register(weight)
