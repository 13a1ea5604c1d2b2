"""oneka_track_noalloc: the chronicle without caller-provided scratch.

Some callers of this library cannot allocate device memory: a plugin whose
host process owns and divides up all device memory, or a binding that can
only hand over buffers the host already has.  oneka_track_noalloc serves
them: it takes its realization slots from a fixed 32 MiB array inside the
library instead of a caller's scratch buffer.  These tests call it through
the C ABI, twice in a row on the same inputs, and require each result to
equal oneka_track with caller scratch (visit counts are integers: equal
means bit-identical).  The file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest
import torch

from conftest import golden
from gpu_helpers import golden_grid, golden_opts, golden_real, golden_site

pytestmark = pytest.mark.gpu

from onekapy_gb300 import _capi as C  # noqa: E402
from onekapy_gb300 import engine as E  # noqa: E402
from onekapy_gb300 import sites as S  # noqa: E402


def _run(entry, site, real, release, opts, grid):
    L = C.load()
    dev = site.device
    counts = torch.zeros((grid.nrows, grid.ncols), dtype=torch.int32, device=dev)
    reg = torch.zeros(1, dtype=torch.int64, device=dev)
    common = [ctypes.byref(site.c()), ctypes.byref(real.c()), real.n, C.ptr(release), release.shape[0],
              ctypes.byref(opts.c()), ctypes.byref(grid.c()), None, C.ptr(counts), C.ptr(reg), None]
    if entry == "noalloc":
        rc = L.oneka_track_noalloc(*common, C.stream_ptr())
    else:
        scratch = torch.zeros(grid.slot_bytes() * real.n, dtype=torch.uint8, device=dev)
        rc = L.oneka_track(*common, C.ptr(scratch), scratch.numel(), C.stream_ptr())
    C.check(rc)
    torch.cuda.synchronize()
    return counts.cpu().numpy(), int(reg.item())


def _check_twice(site, real, release, opts, grid):
    want, want_reg = _run("track", site, real, release, opts, grid)
    assert want.sum() > 0
    for _ in range(2):
        got, got_reg = _run("noalloc", site, real, release, opts, grid)
        assert got_reg == want_reg
        assert np.array_equal(got, want), f"{int((got != want).sum())} nodes differ"


def test_noalloc_matches_track_on_reference_case():
    """FP64, the confined golden case (its counts also equal the reference's)."""
    d = golden("track_confined_u10.npz")
    dev = C.device()
    release = torch.as_tensor(d["release"], device=dev)
    _check_twice(golden_site(d, dev), golden_real(d, dev), release, golden_opts(d, C.FP64), golden_grid(d))
    got, _ = _run("noalloc", golden_site(d, dev), golden_real(d, dev), release, golden_opts(d, C.FP64),
                  golden_grid(d))
    assert np.array_equal(got, d["counts"])


def test_noalloc_matches_track_over_several_launches():
    """FP32 on the 1601 x 1601 grid: 150 realizations need two passes over the 32 MiB array."""
    spec = S.config2(nreal=150, npaths=32)
    dev = C.device()
    site = E.Site(spec.wells, spec.observations, spec.base, c_dist=spec.c_dist, p_dist=spec.p_dist,
                  t_dist=spec.t_dist, device=dev)
    real = E.realize(site, spec.nreal, seed=99)
    grid = E.Grid.window(site.xt, site.yt, spec.spacing, spec.half)
    assert grid.slot_bytes() * spec.nreal > C.NOALLOC_SCRATCH_BYTES
    opts = E.TrackOptions(duration=spec.duration, tol=spec.tol, maxstep=spec.maxstep, umbra=spec.umbra,
                          confined=spec.confined, precision=C.FP32)
    _check_twice(site, real, torch.as_tensor(site.release(spec.npaths), device=dev), opts, grid)


def test_noalloc_allocates_no_device_memory():
    """The defining property: after a first call on the device (which loads
    the library's module and with it the fixed array), further calls leave
    the device's free memory and torch's allocations unchanged."""
    spec = S.config1()
    dev = C.device()
    site = E.Site(spec.wells, spec.observations, spec.base, c_dist=spec.c_dist, p_dist=spec.p_dist,
                  t_dist=spec.t_dist, device=dev)
    real = E.realize(site, 8, seed=7)
    grid = E.Grid.window(site.xt, site.yt, spec.spacing, spec.half)
    opts = E.TrackOptions(duration=spec.duration, tol=spec.tol, maxstep=spec.maxstep, umbra=spec.umbra,
                          confined=spec.confined, precision=C.FP32)
    release = torch.as_tensor(site.release(24), device=dev)
    counts = torch.zeros((grid.nrows, grid.ncols), dtype=torch.int32, device=dev)
    reg = torch.zeros(1, dtype=torch.int64, device=dev)
    args = [ctypes.byref(site.c()), ctypes.byref(real.c()), real.n, C.ptr(release), release.shape[0],
            ctypes.byref(opts.c()), ctypes.byref(grid.c()), None, C.ptr(counts), C.ptr(reg), None,
            C.stream_ptr()]
    L = C.load()
    C.check(L.oneka_track_noalloc(*args))         # the warm-up call a host makes at its own set-up
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    torch0 = torch.cuda.memory_allocated()
    for _ in range(2):
        C.check(L.oneka_track_noalloc(*args))
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert torch.cuda.memory_allocated() == torch0
    assert free1 == free0, (free0, free1)
    assert int(reg.item()) == 3 * 8 and int(counts.sum().item()) > 0


def test_noalloc_rejects_a_grid_beyond_its_array():
    d = golden("track_confined_u10.npz")
    dev = C.device()
    site, real = golden_site(d, dev), golden_real(d, dev)
    big = E.Grid(-40000.0, -40000.0, 2.0, 2.0, 40001, 40001)   # 200 MB per realization slot
    counts = torch.zeros(1, dtype=torch.int32, device=dev)
    release = torch.as_tensor(d["release"], device=dev)
    L = C.load()
    rc = L.oneka_track_noalloc(ctypes.byref(site.c()), ctypes.byref(real.c()), real.n, C.ptr(release),
                               release.shape[0], ctypes.byref(golden_opts(d, C.FP64).c()),
                               ctypes.byref(big.c()), None, C.ptr(counts), None, None, C.stream_ptr())
    assert rc == C.ONEKA_ERR_SCRATCH
    assert b"fixed scratch" in L.oneka_last_error()
