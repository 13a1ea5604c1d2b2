"""GPU: one batched launch over uneven sites equals one oneka_track per site."""
import pytest
import torch

pytestmark = pytest.mark.gpu

from onekapy_gb300 import _capi as C  # noqa: E402
from onekapy_gb300 import engine as E  # noqa: E402
from onekapy_gb300 import sites as S  # noqa: E402


def _jobs(specs, npaths_cap=96, nreal_cap=40):
    dev = C.device()
    jobs = []
    for k, spec in enumerate(specs):
        site = E.Site(spec.wells, spec.observations, spec.base, c_dist=spec.c_dist, p_dist=spec.p_dist,
                      t_dist=spec.t_dist, device=dev)
        nreal = min(spec.nreal, nreal_cap)
        real = E.realize(site, nreal, seed=500 + k)
        half = min(spec.half, 1500.0)
        grid = E.Grid.window(site.xt, site.yt, spec.spacing, half)
        npaths = min(spec.npaths, npaths_cap)
        opts = E.TrackOptions(duration=min(spec.duration, 5 * 365.25), tol=spec.tol, maxstep=spec.maxstep,
                              umbra=spec.umbra, confined=spec.confined, precision=C.FP32)
        jobs.append(E.TrackJob(site, real, torch.as_tensor(site.release(npaths), device=dev), opts, grid,
                               torch.zeros((grid.nrows, grid.ncols), dtype=torch.int32, device=dev),
                               torch.zeros(1, dtype=torch.int64, device=dev)))
    return jobs


def test_batched_equals_per_site_calls():
    specs = S.config3(nsites=6) + [S.config2(nreal=30, npaths=64), S.config4(nreal=20, npaths=64)]
    jobs = _jobs(specs)
    E.track_batched(jobs)
    torch.cuda.synchronize()
    for j in jobs:
        counts = torch.zeros_like(j.counts)
        reg = torch.zeros(1, dtype=torch.int64, device=counts.device)
        E.track(j.site, j.real, j.release, j.opts, j.grid, counts=counts, registered=reg)
        torch.cuda.synchronize()
        assert int(reg.item()) == int(j.registered.item()) == j.real.n - int((j.real.status != 0).sum())
        assert torch.equal(counts, j.counts), int((counts != j.counts).sum())
        assert int(j.counts.sum()) > 0


def test_batched_small_scratch_runs_in_waves():
    """A scratch too small for all slots at once: several waves, same counts."""
    specs = S.config3(nsites=3)
    a = _jobs(specs)
    b = _jobs(specs)
    E.track_batched(a)
    slot = max(j.grid.slot_bytes() for j in b)
    scratch = torch.zeros(5 * slot + 1024, dtype=torch.uint8, device=C.device())
    E.track_batched(b, scratch=scratch)
    torch.cuda.synchronize()
    for x, y in zip(a, b):
        assert torch.equal(x.counts, y.counts)
    assert int(scratch.count_nonzero()) == 0      # the scratch is left zero
