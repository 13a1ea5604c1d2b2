"""Shared helpers of the GPU parity tests: run a golden case through the C ABI."""
import numpy as np
import torch

from onekapy_gb300 import _capi as C
from onekapy_gb300 import engine as E


def golden_site(d, dev):
    wells = [(float(w[0]), float(w[1]), float(w[2]), 0.0) for w in d["wells"]]
    return E.Site(wells, d["obs"], float(d["base"]), target=0, device=dev)


def golden_real(d, dev):
    aq = np.stack([d["K"], d["n"], d["H"]], axis=1)
    return E.Realizations.given(d["coef"], d["q"], aq, dev)


def golden_grid(d, key="grid"):
    g = d[key]
    return E.Grid(float(g[0]), float(g[1]), float(g[2]), float(g[3]), int(g[4]), int(g[5]))


def golden_opts(d, precision, head64=False):
    return E.TrackOptions(duration=float(d["duration"]), tol=float(d["tol"]), maxstep=float(d["maxstep"]),
                          umbra=float(d["umbra"]), confined=bool(d["confined"]), precision=precision,
                          head64=head64)


def run_golden(d, precision, max_vertices=None, slots=None, head64=False, release_shift=None):
    dev = C.device()
    site = golden_site(d, dev)
    real = golden_real(d, dev)
    grid = golden_grid(d)
    nreal, npaths = d["nvertices"].shape
    mv = d["vertices"].shape[2] if max_vertices is None else max_vertices
    out = E.TrackOutputs.alloc(nreal, npaths, dev, bbox=True, max_vertices=mv)
    counts = torch.zeros((grid.nrows, grid.ncols), dtype=torch.int32, device=dev)
    reg = torch.zeros(1, dtype=torch.int64, device=dev)
    release = d["release"] if release_shift is None else d["release"] + np.asarray(release_shift)
    E.track(site, real, torch.as_tensor(release, device=dev), golden_opts(d, precision, head64), grid,
            counts=counts, registered=reg, outputs=out, slots=slots)
    torch.cuda.synchronize()
    return dict(counts=counts.cpu().numpy(), registered=int(reg.item()),
                vertices=out.vertices.cpu().numpy(), nvertices=out.nvertices.cpu().numpy(),
                naccept=out.naccept.cpu().numpy(), nattempt=out.nattempt.cpu().numpy(),
                status=out.status.cpu().numpy(), endpoint=out.endpoint.cpu().numpy(),
                bbox=out.bbox.cpu().numpy())
