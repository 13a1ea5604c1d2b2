"""Device-resident engine for the per-realization hot path.

A site lives on the GPU as tensors; realizations are drawn and fitted by
``oneka_realize`` and tracked/chronicled by ``oneka_track``.  The classes here
are what the reference-compatible modules (``stochastic``, ``capturezone``,
``deterministic``) and ``bench.py`` drive.

Reference map (paths within OnekaPy):
  oneka/stochastic.py:224-241    draws, fit, MVN draw          -> realize() (oneka_realize)
  oneka/capturezone.py:51-253    backtrace + chronicle         -> track() (oneka_track), track_batched()
  oneka/stochastic.py:274-306    distributions                 -> dist()
  oneka/capturezone.py:110-115   release ring                  -> release_ring()
  oneka/probabilityfield.py:125-261  grid geometry             -> Grid, replay_expand()
"""
from __future__ import annotations

import ctypes
import dataclasses
import functools
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _capi as C

F64 = torch.float64
I32 = torch.int32


# ---------------------------------------------------------------------------
# distributions
# ---------------------------------------------------------------------------
class DistributionError(Exception):
    """Invalid distribution (oneka/stochastic.py:70-72)."""


@dataclass(frozen=True)
class Lognormal:
    """exp(N(mu, sigma)): the lognormal conductivity of the synthetic sites (extension)."""
    mu: float
    sigma: float


def dist(arg) -> C.OnekaDist:
    """scalar -> constant, (min, max) -> uniform, (min, mode, max) -> triangular
    (oneka/stochastic.py:297-304); ``Lognormal`` -> lognormal."""
    if isinstance(arg, Lognormal):
        return C.OnekaDist(C.DIST_LOGNORMAL, 0, float(arg.mu), float(arg.sigma), 0.0)
    if type(arg) is not tuple:
        return C.OnekaDist(C.DIST_CONST, 0, float(arg), 0.0, 0.0)
    if len(arg) == 2:
        return C.OnekaDist(C.DIST_UNIFORM, 0, float(arg[0]), float(arg[1]), 0.0)
    if len(arg) == 3:
        return C.OnekaDist(C.DIST_TRIANGULAR, 0, float(arg[0]), float(arg[1]), float(arg[2]))
    raise DistributionError("<arg> must be a scalar, pair, or triple.")


# ---------------------------------------------------------------------------
# geometry
# ---------------------------------------------------------------------------
@dataclass
class Grid:
    """Node grid: node (i, j) at (xmin + j*dx, ymin + i*dy)."""
    xmin: float
    ymin: float
    dx: float
    dy: float
    nrows: int
    ncols: int

    def c(self) -> C.OnekaGrid:
        return C.OnekaGrid(float(self.xmin), float(self.ymin), float(self.dx), float(self.dy),
                           int(self.nrows), int(self.ncols))

    @property
    def words_per_row(self) -> int:
        return (self.ncols + 31) // 32

    def slot_bytes(self) -> int:
        return int(C.load().oneka_track_scratch_bytes(ctypes.byref(self.c()), 1))

    @staticmethod
    def window(xo, yo, spacing, half_x, half_y=None) -> "Grid":
        """The grid ProbabilityField(spacing, spacing, xo, yo) grows to when
        expanded to [xo - half_x, xo + half_x] x [yo - half_y, yo + half_y]
        (the repeated += / -= of oneka/probabilityfield.py:229-245, so node
        coordinates equal the reference's).  The replay is a host loop of a
        few thousand steps, so results are cached per argument tuple."""
        half_y = half_x if half_y is None else half_y
        return dataclasses.replace(_window_grid(float(xo), float(yo), float(spacing), float(half_x),
                                                float(half_y)))


@functools.lru_cache(maxsize=256)
def _window_grid(xo, yo, spacing, half_x, half_y) -> Grid:
    (xmin, ymin, nrows, ncols, _, _), _ = replay_expand(
        xo, yo, spacing, spacing,
        np.array([[xo - half_x + 0.5 * spacing, xo + half_x - 0.5 * spacing,
                   yo - half_y + 0.5 * spacing, yo + half_y - 0.5 * spacing]]))
    return Grid(xmin, ymin, spacing, spacing, nrows, ncols)


FRAME_DTYPE = np.dtype([("xmin", "<f8"), ("ymin", "<f8"), ("coff", "<i4"), ("roff", "<i4"),
                        ("ncols", "<i4"), ("nrows", "<i4")])


def _grow_sequence(start, step, limit, upward):
    """Values start, start -/+ step, ... (rounded at every step, as the
    reference's repeated subtraction) until one passes `limit` strictly."""
    seq = [start]
    v = start
    if upward:
        while limit >= v:
            v = v + step
            seq.append(v)
    else:
        while limit <= v:
            v = v - step
            seq.append(v)
    return np.array(seq, dtype=np.float64)


def replay_expand(xo, yo, dx, dy, bboxes, grid0=None):
    """Replay ProbabilityField.expand (oneka/probabilityfield.py:222-261) for
    traces rasterized in order, starting from the 3x3 grid around (xo, yo)
    (or `grid0` = (xmin, xmax, ymin, ymax) of an existing grid).

    bboxes: [n, 4] (xmin, xmax, ymin, ymax) per trace.  Returns the final
    (xmin, ymin, nrows, ncols, xmax, ymax) and a FRAME_DTYPE record per trace:
    the grid origin the reference held when it rasterized that trace and its
    offset in the final grid.  Vectorised: each bound moves along the fixed
    sequence of repeated additions, so its position after trace k is set by
    the running extreme of the requests.
    """
    bb = np.asarray(bboxes, dtype=np.float64).reshape(-1, 4)
    if grid0 is None:
        x0, x1, y0, y1 = xo - dx, xo + dx, yo - dy, yo + dy
    else:
        x0, x1, y0, y1 = grid0
    ncols0 = int(round((x1 - x0) / dx)) + 1
    nrows0 = int(round((y1 - y0) / dy)) + 1
    if bb.shape[0] == 0:
        return (x0, y0, nrows0, ncols0, x1, y1), np.zeros(0, FRAME_DTYPE)
    if np.any(bb[:, 0] > bb[:, 1]) or np.any(bb[:, 2] > bb[:, 3]):
        raise ValueError("bbox with min > max")
    lo_x = np.minimum.accumulate(bb[:, 0])
    hi_x = np.maximum.accumulate(bb[:, 1])
    lo_y = np.minimum.accumulate(bb[:, 2])
    hi_y = np.maximum.accumulate(bb[:, 3])
    sx0 = _grow_sequence(x0, dx, lo_x[-1], upward=False)
    sx1 = _grow_sequence(x1, dx, hi_x[-1], upward=True)
    sy0 = _grow_sequence(y0, dy, lo_y[-1], upward=False)
    sy1 = _grow_sequence(y1, dy, hi_y[-1], upward=True)
    # steps taken = number of sequence values the running request reaches
    # (loop runs while request <= xmin, i.e. stops at the first value < request)
    kx0 = np.searchsorted(-sx0, -lo_x, side="right")
    kx1 = np.searchsorted(sx1, hi_x, side="right")
    ky0 = np.searchsorted(-sy0, -lo_y, side="right")
    ky1 = np.searchsorted(sy1, hi_y, side="right")
    fx, fy = kx0[-1], ky0[-1]
    ncols = ncols0 + int(kx0[-1]) + int(kx1[-1])
    nrows = nrows0 + int(ky0[-1]) + int(ky1[-1])
    frames = np.zeros(bb.shape[0], FRAME_DTYPE)
    frames["xmin"] = sx0[kx0]
    frames["ymin"] = sy0[ky0]
    frames["coff"] = fx - kx0
    frames["roff"] = fy - ky0
    frames["ncols"] = ncols0 + kx0 + kx1
    frames["nrows"] = nrows0 + ky0 + ky1
    return (float(sx0[fx]), float(sy0[fy]), nrows, ncols, float(sx1[kx1[-1]]),
            float(sy1[ky1[-1]])), frames


_rings: dict = {}


def release_ring(xtarget, ytarget, rtarget, npaths) -> np.ndarray:
    """Release points of compute_capturezone (oneka/capturezone.py:110-115),
    evaluated element by element with NumPy exactly as the reference does
    (NumPy's scalar cos/sin; its vectorized ones may round differently).
    Rings are cached per (target, radius, npaths); a copy is returned."""
    key = (float(xtarget), float(ytarget), float(rtarget), int(npaths))
    ring = _rings.get(key)
    if ring is None:
        STEPAWAY = 1.0
        ring = np.empty((npaths, 2), dtype=np.float64)
        for i, theta in enumerate(np.linspace(0, 2 * np.pi, npaths + 1)[0:-1]):
            ring[i, 0] = (rtarget + STEPAWAY) * np.cos(theta) + xtarget
            ring[i, 1] = (rtarget + STEPAWAY) * np.sin(theta) + ytarget
        if len(_rings) > 64:
            _rings.clear()
        _rings[key] = ring
    return ring.copy()


# ---------------------------------------------------------------------------
# site and realizations on the device
# ---------------------------------------------------------------------------
class Site:
    """A site on the device: wells (list order), observations, distributions."""

    def __init__(self, wells, observations, base, target=0, c_dist=10.0, p_dist=0.25, t_dist=10.0,
                 xo=None, yo=None, device=None):
        self.device = device or C.device()
        self.well_list = [tuple(w) for w in wells]
        self.nwells = len(self.well_list)
        if self.nwells < 1:
            raise ValueError("a site needs at least one well")
        self.target = int(target)
        xt, yt, rt = self.well_list[self.target][0:3]
        self.xt, self.yt, self.rt = float(xt), float(yt), float(rt)
        self.xo = self.xt if xo is None else float(xo)
        self.yo = self.yt if yo is None else float(yo)
        self.base = float(base)
        self.wells = torch.tensor([[float(w[0]), float(w[1]), float(w[2])] for w in self.well_list],
                                  dtype=F64, device=self.device)
        obs = np.asarray(observations, dtype=np.float64).reshape(-1, 4)
        self.nobs = obs.shape[0]
        self.obs = torch.tensor(obs, dtype=F64, device=self.device)
        qd = [dist(w[3]) if len(w) > 3 else dist(0.0) for w in self.well_list]
        arr = (C.OnekaDist * self.nwells)(*qd)
        self.qdist = torch.frombuffer(bytearray(bytes(arr)), dtype=torch.uint8).to(self.device)
        self.adist = (C.OnekaDist * 3)(dist(c_dist), dist(p_dist), dist(t_dist))
        self.logr2 = None
        if self.nobs:
            self.logr2 = torch.empty((self.nobs, self.nwells), dtype=F64, device=self.device)
            C.check(C.load().oneka_site_logr2(ctypes.byref(self.c()), C.ptr(self.logr2),
                                              C.stream_ptr()))

    def c(self) -> C.OnekaSite:
        return C.OnekaSite(self.nwells, self.nobs, self.target, 0, self.base, self.xo, self.yo,
                           C.ptr(self.wells), C.ptr(self.obs) if self.nobs else None)

    def release(self, npaths) -> np.ndarray:
        return release_ring(self.xt, self.yt, self.rt, npaths)


@dataclass
class Realizations:
    coef: torch.Tensor
    q: torch.Tensor
    aquifer: torch.Tensor
    status: torch.Tensor
    coef_ev: torch.Tensor | None = None
    coef_cov: torch.Tensor | None = None

    @property
    def n(self) -> int:
        return self.coef.shape[0]

    @staticmethod
    def empty(n, nwells, device, with_fit=True) -> "Realizations":
        return Realizations(
            coef=torch.empty((n, 6), dtype=F64, device=device),
            q=torch.empty((n, nwells), dtype=F64, device=device),
            aquifer=torch.empty((n, 3), dtype=F64, device=device),
            status=torch.zeros((n,), dtype=I32, device=device),
            coef_ev=torch.empty((n, 6), dtype=F64, device=device) if with_fit else None,
            coef_cov=torch.empty((n, 36), dtype=F64, device=device) if with_fit else None)

    @staticmethod
    def given(coef, q, aquifer, device) -> "Realizations":
        coef = torch.as_tensor(np.asarray(coef, dtype=np.float64).reshape(-1, 6), device=device)
        n = coef.shape[0]
        return Realizations(
            coef=coef.contiguous(),
            q=torch.as_tensor(np.asarray(q, dtype=np.float64).reshape(n, -1), device=device).contiguous(),
            aquifer=torch.as_tensor(np.asarray(aquifer, dtype=np.float64).reshape(n, 3),
                                    device=device).contiguous(),
            status=torch.zeros((n,), dtype=I32, device=device))

    def slice(self, a, b) -> "Realizations":
        sl = lambda t: None if t is None else t[a:b]
        return Realizations(self.coef[a:b], self.q[a:b], self.aquifer[a:b], self.status[a:b],
                            sl(self.coef_ev), sl(self.coef_cov))

    def c(self) -> C.OnekaRealizations:
        return C.OnekaRealizations(C.ptr(self.coef), C.ptr(self.coef_ev), C.ptr(self.coef_cov),
                                   C.ptr(self.q), C.ptr(self.aquifer), C.ptr(self.status))


def realize(site: Site, nreal: int, seed: int = 0, first: int = 0, mode: int = C.MODE_STOCHASTIC,
            out: Realizations | None = None, stream=None) -> Realizations:
    """Draw, fit and MVN-draw realizations [first, first + nreal) (oneka_realize)."""
    if out is None:
        out = Realizations.empty(nreal, site.nwells, site.device)
    co = out.c()
    C.check(C.load().oneka_realize(ctypes.byref(site.c()), C.ptr(site.qdist), site.adist,
                                   C.ptr(site.logr2), int(seed) & 0xFFFFFFFFFFFFFFFF,
                                   int(first), int(nreal), int(mode), ctypes.byref(co),
                                   C.stream_ptr(stream)))
    return out


@dataclass
class TrackOptions:
    duration: float
    tol: float = 1.0
    maxstep: float = 10.0
    umbra: float = 10.0
    confined: bool = True
    precision: int = C.FP64
    max_attempts: int = 0
    block: int = 0
    window_kb: int = 0
    occupancy: int = 0
    head64: bool = False

    def c(self) -> C.OnekaTrackOpts:
        return C.OnekaTrackOpts(float(self.duration), float(self.tol), float(self.maxstep),
                                float(self.umbra), int(bool(self.confined)), int(self.precision),
                                int(self.max_attempts), int(self.block), int(self.window_kb),
                                int(self.occupancy), int(bool(self.head64)))


# A launch of this many realization slots or more registers its counts column
# by column (two kernels: the sums, then the slot headers cleared); fewer, one
# block per slot (csrc/chronicle.cu, kColumnsMinSlots).
REGISTER_COLUMNS_MIN_SLOTS = 4096

# OnekaTrackOut.counters: attempts, accepted steps, node tests, word ORs, DRY
# traces, STEP_LIMIT traces, traces that left the grid, (reserved)
COUNTERS = 8
COUNTER_NAMES = ("step_attempts", "accepted_steps", "chronicle_node_tests", "chronicle_word_ors", "dry_traces",
                 "step_limit_traces", "traces_leaving_grid", "reserved")


@dataclass
class TrackOutputs:
    """Per-particle outputs [nreal, npaths] (any subset)."""
    endpoint: torch.Tensor | None = None
    bbox: torch.Tensor | None = None
    naccept: torch.Tensor | None = None
    nattempt: torch.Tensor | None = None
    status: torch.Tensor | None = None
    vertices: torch.Tensor | None = None
    nvertices: torch.Tensor | None = None
    counters: torch.Tensor | None = None

    @staticmethod
    def alloc(nreal, npaths, device, *, endpoint=True, bbox=False, stats=True, max_vertices=0,
              counters=False):
        shp = (nreal, npaths)
        return TrackOutputs(
            endpoint=torch.empty(shp + (2,), dtype=F64, device=device) if endpoint else None,
            bbox=torch.empty(shp + (4,), dtype=F64, device=device) if bbox else None,
            naccept=torch.zeros(shp, dtype=I32, device=device) if stats else None,
            nattempt=torch.zeros(shp, dtype=I32, device=device) if stats else None,
            status=torch.zeros(shp, dtype=I32, device=device) if stats else None,
            vertices=(torch.full(shp + (max_vertices, 2), float("nan"), dtype=F64, device=device)
                      if max_vertices else None),
            nvertices=torch.zeros(shp, dtype=I32, device=device) if (stats or max_vertices) else None,
            counters=torch.zeros(COUNTERS, dtype=torch.int64, device=device) if counters else None)

    def c(self) -> C.OnekaTrackOut:
        mv = 0 if self.vertices is None else int(self.vertices.shape[2])
        return C.OnekaTrackOut(C.ptr(self.endpoint), C.ptr(self.bbox), C.ptr(self.naccept),
                               C.ptr(self.nattempt), C.ptr(self.status), C.ptr(self.vertices),
                               C.ptr(self.nvertices), mv, 0, C.ptr(self.counters))


_scratch: dict = {}


def scratch_buffer(nbytes: int, device) -> torch.Tensor:
    """A cached device buffer for the chronicle's realization slots."""
    key = (str(device),)
    buf = _scratch.get(key)
    if buf is None or buf.numel() < nbytes:
        # oneka_track wants zeroed slots and leaves them zeroed
        buf = torch.zeros(max(nbytes, 16), dtype=torch.uint8, device=device)
        _scratch[key] = buf
    return buf


def track(site: Site, real: Realizations, release, opts: TrackOptions, grid: Grid,
          counts: torch.Tensor | None = None, registered: torch.Tensor | None = None,
          frames: torch.Tensor | None = None, outputs: TrackOutputs | None = None,
          slots: int | None = None, scratch: torch.Tensor | None = None, stream=None,
          mark_only: torch.Tensor | None = None):
    """oneka_track: backtrack ``npaths`` particles per realization and
    chronicle them into ``counts`` (int32 [nrows, ncols])."""
    L = C.load()
    if not isinstance(release, torch.Tensor):
        release = torch.as_tensor(np.asarray(release, dtype=np.float64).reshape(-1, 2),
                                  device=site.device)
    release = release.contiguous()
    npaths = release.shape[0]
    g = grid.c()
    sbytes = 0
    sptr = None
    if mark_only is not None:
        sptr = C.ptr(mark_only)
        sbytes = mark_only.numel() * mark_only.element_size()
    elif counts is not None:
        slot_b = grid.slot_bytes()
        if scratch is None:
            nslots = slots or max(1, min(real.n, (4 << 30) // slot_b))
            scratch = scratch_buffer(nslots * slot_b, site.device)
        sptr = C.ptr(scratch)
        sbytes = scratch.numel() * scratch.element_size()
    rc = L.oneka_track(ctypes.byref(site.c()), ctypes.byref(real.c()), real.n, C.ptr(release), npaths,
                       ctypes.byref(opts.c()), ctypes.byref(g), C.ptr(frames), C.ptr(counts),
                       C.ptr(registered), ctypes.byref(outputs.c()) if outputs else None, sptr,
                       sbytes, C.stream_ptr(stream))
    C.check(rc)


# ---------------------------------------------------------------------------
# autotuner: block shape, occupancy and chronicle window of the FP32 tracker
# ---------------------------------------------------------------------------
TUNE_CANDIDATES = [(256, 2, 32), (256, 3, 32), (256, 4, 32), (256, 4, 16), (128, 4, 32), (128, 6, 16),
                   (128, 6, 32), (128, 8, 16), (64, 8, 16)]
_tuned: dict = {}


def pick_fastest(n: int, time_one, repeats: int) -> tuple[int, list]:
    """Index of the fastest of `n` candidates and each one's best time.
    `time_one(i)` runs candidate i once and returns its duration.  The
    candidates take turns: round 0 runs each once untimed (warm-up), then
    `repeats` timed rounds run each once again, so a drift of the clock
    during the tuning affects every candidate alike."""
    best = [float("inf")] * n
    for rnd in range(repeats + 1):
        for i in range(n):
            t = time_one(i)
            if rnd > 0:
                best[i] = min(best[i], t)
    return min(range(n), key=lambda i: best[i]), best


def site_signature(site: Site, grid: Grid, opts: TrackOptions, npaths: int) -> tuple:
    return (site.nwells, bool(opts.confined), int(opts.precision), grid.nrows, grid.ncols, int(npaths))


def autotune(site: Site, real: Realizations, release, opts: TrackOptions, grid: Grid, *, sample=256,
             candidates=TUNE_CANDIDATES, repeats=3, verbose=False) -> TrackOptions:
    """Time the tracker's launch variants on a sample of the realizations and
    return `opts` with the fastest (block, occupancy, window_kb).  The
    candidates take turns (one launch each per round, the first round
    untimed), so a drift of the clock over the tuning hits them alike; each
    keeps its best round.  Results are cached per site shape for the
    process."""
    key = site_signature(site, grid, opts, len(release))
    if key in _tuned:
        b, o, w = _tuned[key]
        return TrackOptions(**{**opts.__dict__, "block": b, "occupancy": o, "window_kb": w})
    n = max(1, min(sample, real.n))
    sub = real.slice(0, n)
    counts = torch.zeros((grid.nrows, grid.ncols), dtype=torch.int32, device=site.device)
    scratch = scratch_buffer(grid.slot_bytes() * n, site.device)
    trials = [TrackOptions(**{**opts.__dict__, "block": b, "occupancy": o, "window_kb": w})
              for (b, o, w) in candidates]

    def time_one(i):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        track(site, sub, release, trials[i], grid, counts=counts, scratch=scratch)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    i_best, best_times = pick_fastest(len(trials), time_one, repeats)
    if verbose:
        for (b, o, w), t in zip(candidates, best_times):
            print(f"autotune block={b} occupancy={o} window_kb={w}: {t:.3f} ms")
    best = tuple(candidates[i_best])
    _tuned[key] = best
    return TrackOptions(**{**opts.__dict__, "block": best[0], "occupancy": best[1], "window_kb": best[2]})


# ---------------------------------------------------------------------------
# many sites in one launch
# ---------------------------------------------------------------------------
@dataclass
class TrackJob:
    """One site of a batched launch (oneka_track_batched)."""
    site: Site
    real: Realizations
    release: torch.Tensor
    opts: TrackOptions
    grid: Grid
    counts: torch.Tensor
    registered: torch.Tensor | None = None
    outputs: TrackOutputs | None = None


def batched_scratch_bytes(jobs) -> int:
    arr, _keep = _job_array(jobs)
    return int(C.load().oneka_track_batched_scratch_bytes(arr, len(jobs)))


def _job_array(jobs):
    keep = []
    arr = (C.OnekaTrackJob * max(1, len(jobs)))()
    for i, j in enumerate(jobs):
        site_c, real_c, opts_c, grid_c = j.site.c(), j.real.c(), j.opts.c(), j.grid.c()
        out_c = j.outputs.c() if j.outputs is not None else None
        keep += [site_c, real_c, opts_c, grid_c, out_c]
        arr[i] = C.OnekaTrackJob(ctypes.pointer(site_c), ctypes.pointer(real_c), j.real.n,
                                 int(j.release.shape[0]), C.ptr(j.release), ctypes.pointer(opts_c),
                                 ctypes.pointer(grid_c), C.ptr(j.counts), C.ptr(j.registered),
                                 ctypes.pointer(out_c) if out_c is not None else None)
    return arr, keep


def track_batched(jobs, scratch: torch.Tensor | None = None, stream=None) -> None:
    """Track and chronicle every realization of every job in batched launches
    (FP32 build; the first job's block/occupancy apply to all)."""
    if not jobs:
        return
    arr, keep = _job_array(jobs)
    if scratch is None:
        need = int(C.load().oneka_track_batched_scratch_bytes(arr, len(jobs)))
        scratch = scratch_buffer(min(need, 16 << 30) + 256, jobs[0].site.device)
    base = C.ptr(scratch)
    pad = (-base) % 256
    C.check(C.load().oneka_track_batched(arr, len(jobs), base + pad, scratch.numel() - pad,
                                         C.stream_ptr(stream)))

