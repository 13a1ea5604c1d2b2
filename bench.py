#!/usr/bin/env python
"""Benchmark of the per-realization hot path on the 10,000-realization site.

Workload (one "step"): the mixed-aquifer site with 1 target + 10 neighbour
wells and 60 observations; 10,000 realizations x 1,000 particles, 20-year
backtrack, adaptive Dormand-Prince step (tol 1 m, maxstep 10 m), chronicled
on a 5 m grid over 8 km x 8 km (1601 x 1601 int32 counts).  A step draws and
fits every realization (oneka_realize, FP64) and tracks + chronicles every
particle (oneka_track, FP32 fast build), with all inputs resident in HBM.

Printed (one JSON line on rank 0): realizations/s (value), particle-steps/s,
the plain FP64 GPU tracker on a sample of the same realizations, the FP32
build's L-inf capture-probability error against it, the end-to-end rate
through the public API with host buffers, the roofline of the tracking
kernel against the measured FP32 FMA peak, and the oracle CPU port timed on
this host's cores.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Other workloads (one JSON line each; the default line above is the headline):

    --workload config3   64 uneven sites (2-200 wells, 1k-20k realizations,
                         360/1024/4096 paths, 5-50 years, 256^2-1024^2 grids) in
                         one batched launch sequence replayed as a CUDA graph,
                         against one oneka_track call per site.
    --workload config4   unconfined stress site (31 wells, water table 0.5-3 m
                         above the base near the target, 5,000 x 2,048, 25 years):
                         the FP32 build timed, and its per-cell capture-probability
                         errors and endpoint drift against the all-FP64 run.
    --workload config5   the learned surrogate on the fixed 31-well site: 200,000
                         tracker-chronicled training pairs, MLP 39 -> 3 x 512 GELU ->
                         256 x 256 logits trained with the project's kernels, then
                         100,000 fresh realizations screened with 5 % judges,
                         against tracking all of them.
"""
from __future__ import annotations

import argparse
import json
import os
import shutil
import signal
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "realizations/s & particle-steps/s on 1 GB300 vs plain FP64; L∞ capture-prob err"
UNIT = "realizations/s"
SEED = 20261203
E2E_CALLS = 3           # timed public-API calls averaged into e2e
TUNE_SAMPLE = 2048      # realizations the autotuner times each launch shape on (several waves)
SURROGATE_TOLERANCE = 0.01   # judge L-inf bar of the screened field: the tracker's own accuracy bar
# DRAM bytes per realization of the tracking launch on this site, from one ncu
# capture of a 1,000-realization launch (dram__bytes_read.sum 15.56 MB +
# dram__bytes_write.sum 0.07 MB).
TRACK32_DRAM_BYTES_PER_REALIZATION = (15.555072e6 + 0.069888e6) / 1000


def args_():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nreal", type=int, default=10000)
    ap.add_argument("--npaths", type=int, default=1000)
    ap.add_argument("--fp64-sample", type=int, default=None,
                    help="realizations of the FP64 comparison (default: all)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="config2", choices=["config2", "config3", "config4", "config5"])
    ap.add_argument("--fraction", type=float, default=1.0,
                    help="config3/config5: fraction of the realization counts run")
    ap.add_argument("--epochs", type=int, default=6, help="config5: training epochs")
    return ap.parse_args()


def workload_config(spec, a, world):
    return {"workload": "config2-mixed-11wells: 10k realizations x 1k paths, 20 y, 5 m grid 8x8 km",
            "nreal_per_gpu": spec.nreal, "npaths": spec.npaths, "nwells": len(spec.wells),
            "nobs": len(spec.observations), "grid": "1601x1601", "duration_d": spec.duration,
            "tol_m": spec.tol, "maxstep_m": spec.maxstep, "umbra_m": spec.umbra, "seed": SEED,
            "parallelism": f"realization shards x{world}",
            "l2": "512 MB buffer written between timed steps"}


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 50 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        if not shutil.which("nvidia-smi"):
            return
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        self.out = open(self.path, "w")
        self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                      "-i", str(self.index), "-lms", "50"], stdout=self.out,
                                     stderr=subprocess.DEVNULL)

    def stop(self):
        if self.proc is None:
            return None
        self.proc.send_signal(signal.SIGTERM)
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.out.close()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------------------
def cpu_oracle_rate(spec, site_np, nreal, nthreads, seed=7):
    """The oracle CPU port (C, OpenMP) on `nreal` realizations at full npaths:
    realization draw + NumPy fit + MVN draw on the host, then tracking."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from onekapy_gb300.engine import Lognormal, Grid, release_ring
    oracle.build()
    rng = np.random.default_rng(seed)

    def draw(d):
        if isinstance(d, Lognormal):
            return float(np.exp(d.mu + d.sigma * rng.normal()))
        if type(d) is not tuple:
            return float(d)
        return float(rng.uniform(*d)) if len(d) == 2 else float(rng.triangular(*d))

    t0 = time.perf_counter()
    coefs, qs, aqs = [], [], []
    for _ in range(nreal):
        wl = [(w[0], w[1], w[2], draw(w[3])) for w in spec.wells]
        K, n, H = draw(spec.c_dist), draw(spec.p_dist), draw(spec.t_dist)
        ev, cov = oracle.fit(spec.observations, wl, spec.base, K, H, 0.0, 0.0)
        coefs.append(rng.multivariate_normal(ev.reshape(6), cov))
        qs.append([w[3] for w in wl])
        aqs.append([K, n, H])
    g = Grid.window(0.0, 0.0, spec.spacing, spec.half)
    r = oracle.track(np.array([w[:2] for w in spec.wells]), np.array(coefs), np.array(qs), np.array(aqs),
                     release_ring(0.0, 0.0, spec.wells[0][2], spec.npaths),
                     (g.xmin, g.ymin, g.dx, g.dy, g.nrows, g.ncols), duration=spec.duration,
                     tol=spec.tol, maxstep=spec.maxstep, umbra=spec.umbra, confined=spec.confined,
                     nthreads=nthreads)
    dt = time.perf_counter() - t0
    return nreal / dt, float(r["naccept"].sum()) / dt, dt


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# ---------------------------------------------------------------------------
def run_reference(a):
    """The reference arm: the oracle CPU port of the path on all host threads."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from onekapy_gb300 import sites as S
    spec = S.config2(nreal=a.nreal, npaths=a.npaths)
    threads = host_threads()
    sample = 30 * max(4, threads)
    for _ in range(a.warmup):
        cpu_oracle_rate(spec, None, max(2, threads // 4), threads)
    rates, steps_rates, total = [], [], 0.0
    for k in range(a.steps):
        r, sr, dt = cpu_oracle_rate(spec, None, sample, threads, seed=100 + k)
        rates.append(r)
        steps_rates.append(sr)
        total += dt
    v = float(np.mean(rates))
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": 1e3 * total / a.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference", "particle_steps_per_s": float(np.mean(steps_rates)),
            "config": workload_config(spec, a, 1) | {"sample_realizations_per_step": sample},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{sample} realizations x {spec.npaths} paths of the workload per "
                                       "step (host draw + NumPy fit + C/OpenMP tracking)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ---------------------------------------------------------------------------
def run_ours(a):
    import torch
    import torch.distributed as dist

    from onekapy_gb300 import _capi as C
    from onekapy_gb300 import engine as E
    from onekapy_gb300 import sites as S
    from onekapy_gb300 import build as B

    B.build()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = C.device()
    spec = S.config2(nreal=a.nreal, npaths=a.npaths)
    R, P = spec.nreal, spec.npaths
    first = rank * R
    site = E.Site(spec.wells, spec.observations, spec.base, c_dist=spec.c_dist, p_dist=spec.p_dist,
                  t_dist=spec.t_dist, device=dev)
    grid = E.Grid.window(site.xt, site.yt, spec.spacing, spec.half)
    release = torch.as_tensor(site.release(P), device=dev)
    real = E.Realizations.empty(R, site.nwells, dev, with_fit=False)
    counts = torch.zeros((grid.nrows, grid.ncols), dtype=torch.int32, device=dev)
    reg = torch.zeros(1, dtype=torch.int64, device=dev)
    scratch = torch.zeros(grid.slot_bytes() * R, dtype=torch.uint8, device=dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    mk = lambda prec: E.TrackOptions(duration=spec.duration, tol=spec.tol, maxstep=spec.maxstep,
                                     umbra=spec.umbra, confined=spec.confined, precision=prec)
    o32, o64 = mk(C.FP32), mk(C.FP64)
    stream = torch.cuda.current_stream()
    # block shape / occupancy / chronicle window picked on a sample (setup, untimed)
    E.realize(site, R, seed=SEED, first=first, out=real)
    o32 = E.autotune(site, real, release, o32, grid, sample=min(R, TUNE_SAMPLE))

    def step(opts, n, ev=None, outputs=None):
        counts.zero_()
        reg.zero_()
        sub = real.slice(0, n)
        if ev:
            ev[0].record(stream)
        E.realize(site, n, seed=SEED, first=first, out=sub)
        if ev:
            ev[1].record(stream)
        E.track(site, sub, release, opts, grid, counts=counts, registered=reg, scratch=scratch,
                outputs=outputs)
        if ev:
            ev[2].record(stream)

    # warm-up, then one untimed pass with the work counters
    for _ in range(a.warmup):
        step(o32, R)
    torch.cuda.synchronize()
    cnt = E.TrackOutputs(counters=torch.zeros(E.COUNTERS, dtype=torch.int64, device=dev))
    step(o32, R, outputs=cnt)
    torch.cuda.synchronize()
    counters = [int(v) for v in cnt.counters.cpu().tolist()]
    attempts, accepts, ntests, natoms = counters[:4]
    counts32_full = counts.clone()

    # timed region
    sampler = ClockSampler(local)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    sampler.start()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(a.steps)]
    for k in range(a.steps):
        flush.fill_(k & 0xFF)
        step(o32, R, ev=evs[k])
    torch.cuda.synchronize()
    clocks = sampler.stop()
    step_ms = [e[0].elapsed_time(e[2]) for e in evs]
    track_ms = [e[1].elapsed_time(e[2]) for e in evs]
    realize_ms = [e[0].elapsed_time(e[1]) for e in evs]
    t_step = float(np.sum(step_ms)) / 1e3
    if world > 1:
        t = torch.tensor([t_step], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_step = float(t.item())
    ms_per_step = 1e3 * t_step / a.steps
    value = world * R * a.steps / t_step
    if world > 1:   # integer sum of the ranks' count grids (after the timed region)
        from onekapy_gb300.shard import reduce_counts
        reduce_counts(counts, reg)
    psteps = world * accepts * a.steps / t_step

    line = None
    if rank == 0:
        # the plain FP64 GPU tracker on every realization of the step (timed like a step) ...
        n64 = min(a.fp64_sample or R, R)
        step(o64, min(8, n64))
        torch.cuda.synchronize()
        e64 = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        step(o64, n64, ev=e64)
        torch.cuda.synchronize()
        fp64_rate = n64 / (e64[0].elapsed_time(e64[2]) / 1e3)
        # ... and the FP32 build against it, realization by realization and trace by trace
        cmps, grids = fp32_vs_fp64(site, real.slice(0, n64), release, {"fp32": o32}, o64, grid, spec.spacing)
        cmp = cmps["fp32"]
        if n64 == R:
            assert torch.equal(grids["fp32"], counts32_full), "mark-only counts differ from the step's counts"

        # end to end through the public API with host buffers
        from onekapy_gb300.stochastic import create_stochastic_capturezone
        e2e_n = R

        # the reference's caller reads pf.pgrid, a host float64 array (copied back from the device)
        def e2e_once():
            pf = create_stochastic_capturezone(0, P, spec.duration, e2e_n, spec.base, spec.c_dist,
                                               spec.p_dist, spec.t_dist, spec.wells, spec.observations,
                                               spec.spacing, spec.umbra, spec.confined, spec.tol,
                                               spec.maxstep, seed=SEED, precision=C.FP32,
                                               window=spec.half, chunk=R)
            return pf.pgrid, pf

        e2e_once()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(E2E_CALLS):
            host_pgrid, pf = e2e_once()
        t_e2e = (time.perf_counter() - t0) / E2E_CALLS
        h2d = (len(spec.wells) * (3 * 8 + 32) + len(spec.observations) * 32 + P * 16)
        d2h = host_pgrid.nbytes + e2e_n * 4 + 8
        assert np.array_equal(host_pgrid, counts32_full.cpu().numpy().astype(np.float64)), \
            "public API and engine disagree"

        # roofline of the tracking kernel: algorithmic FP32 flops per launch
        flops = algorithmic_flops(len(spec.wells), spec.confined, attempts, ntests)
        t_track = float(np.mean(track_ms)) / 1e3
        peak = ctypes_peak(C, fp64=False)
        achieved = flops / t_track / 1e12

        cpu = None
        if world == 1 and not a.no_cpu_baseline:
            th = host_threads()
            ns = 30 * max(4, th)      # about 2 s wall on 16 threads: about 30 s of CPU work
            rate, srate, dt = cpu_oracle_rate(spec, None, ns, th)
            cpu = {"value": rate, "unit": UNIT, "cores": th, "kind": "port",
                   "sample": f"{ns} realizations x {P} paths of the workload ({dt:.1f} s wall; "
                             "host draw + NumPy fit + C/OpenMP tracking)",
                   "particle_steps_per_s": srate}
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
                "warmup": a.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": workload_config(spec, a, world),
                "particle_steps_per_s": psteps,
                "step_breakdown_ms": {"realize_fp64": float(np.mean(realize_ms)),
                                      "track_chronicle_fp32": float(np.mean(track_ms))},
                "fp64_gpu": {"realizations_per_s": fp64_rate, "realizations": n64,
                             "speedup_fp32_over_fp64": value / world / fp64_rate},
                "fp32_vs_fp64": cmp,
                "work_per_step": dict(zip(E.COUNTER_NAMES[:7], counters[:7])),
                "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak / 1e12,
                             "unit": "TFLOP/s", "frac": achieved / (peak / 1e12),
                             "traffic": TRACK32_DRAM_BYTES_PER_REALIZATION * R,
                             "traffic_source": "ncu dram__bytes_read+write of a 1000-realization launch, "
                                               "scaled by realizations",
                             "kernel": "track32_kernel; time includes the register pass (1.5 % of "
                                       "the 10,000-realization step), traffic is the tracker's",
                             "peak_source": "measured FP32 FMA loop on this GPU (oneka_fma_peak)"},
                "roofline_hbm": _hbm_roofline(TRACK32_DRAM_BYTES_PER_REALIZATION * R, t_track),
                "e2e": {"value": e2e_n / t_e2e, "unit": UNIT, "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": d2h},
                "tracker_launch": {"block": o32.block, "occupancy": o32.occupancy,
                                   "window_kb": o32.window_kb, "chosen_by": f"autotune on {min(R, TUNE_SAMPLE)} realizations"},
                # per step: realize, track, and the register pass (column by
                # column from 4,096 slots: two kernels, the second clearing
                # the slot headers)
                "gpu_launches": (2 + (2 if R >= E.REGISTER_COLUMNS_MIN_SLOTS else 1)) * a.steps,
                "clocks": clocks,
                "cpu_baseline": cpu}
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    if line is not None:
        print(json.dumps(line))


def popcount32(x):
    """Set bits of each int32 word (SWAR, on the device; wraps like C)."""
    x = x - ((x >> 1) & 0x55555555)
    x = (x & 0x33333333) + ((x >> 2) & 0x33333333)
    x = (x + (x >> 4)) & 0x0F0F0F0F
    return (x * 0x01010101) >> 24


# A trace is well conditioned when its FP64 endpoint moves less than this many
# cells as its release point moves 1 nm (an amplification below 5,000).
WELL_CONDITIONED_CELLS = 1e-6


def fp32_vs_fp64(site, real, release, variants, o64, grid, spacing, chunk=1000, conditioning=True):
    """FP32 builds (`variants`: name -> options) against the FP64 build on
    every realization of `real` and every trace, outside any timed region.
    All run in mark-only mode (realization k's traces ORed into its own
    bitmask), so the comparison is per realization: the visited-node sets of
    the two builds are XORed and counted.  The count grids are the bitmasks
    summed over realizations.

    Per variant: the capture-probability L-inf (resolution 1/R), the summed
    count difference over the FP64 counts, the fraction of per-realization
    node visits that differ (popcount of the XOR over the FP64 popcount; its
    largest value in any one realization too), the endpoint drift in cells
    over every trace that ended normally in both builds, and how many traces
    took the same numbers of attempted and accepted steps.  Also returns the
    count grids of each variant.

    With `conditioning`, the FP64 build also runs with the release ring moved
    by 1 nm and by 100 nm, and each trace's conditioning is how far its FP64
    endpoint moves (cells).  Reported: the fraction of well-conditioned
    traces (1 nm moves the endpoint less than WELL_CONDITIONED_CELLS), the
    FP32 drift over them (the 1e-3 cell bar), and for every trace the ratio
    of its FP32 drift to its FP64 endpoint's movement under 100 nm."""
    import torch
    from onekapy_gb300 import _capi as C
    from onekapy_gb300 import engine as E
    dev = site.device
    R, P = real.n, release.shape[0]
    slot_words = grid.slot_bytes() // 4
    mwords = grid.nrows * grid.words_per_row
    names = list(variants) + ["fp64"]
    cnt = {k: torch.zeros((grid.nrows, grid.words_per_row * 32), dtype=torch.int64, device=dev) for k in names}
    acc = {k: {"xor": 0, "ref": 0, "worst": 0.0, "drift": [], "same": 0, "status": 0, "s1": [], "s100": []}
           for k in variants}
    shifted = {1e-9: release + torch.tensor([1e-9, 0.0], dtype=release.dtype, device=release.device),
               1e-7: release + torch.tensor([1e-7, 0.0], dtype=release.dtype, device=release.device)}
    for a in range(0, R, chunk):
        b = min(R, a + chunk)
        sub = real.slice(a, b)
        masks, outs = {}, {}
        for name in names:
            o = o64 if name == "fp64" else variants[name]
            masks[name] = torch.zeros((b - a, slot_words), dtype=torch.int32, device=dev)
            outs[name] = E.TrackOutputs.alloc(b - a, P, dev, endpoint=True, stats=True)
            E.track(site, sub, release, o, grid, mark_only=masks[name], outputs=outs[name])
            v = masks[name][:, :mwords].view(b - a, grid.nrows, grid.words_per_row)
            for bit in range(32):
                cnt[name][:, bit::32] += ((v >> bit) & 1).sum(dim=0)
        m64, o64_ = masks["fp64"][:, :mwords], outs["fp64"]
        r = popcount32(m64).sum(dim=1)
        sens = {}
        if conditioning:
            for dlt, rel in shifted.items():
                od = E.TrackOutputs.alloc(b - a, P, dev, endpoint=True, stats=False)
                E.track(site, sub, rel, o64, grid, outputs=od)
                sens[dlt] = (od.endpoint - o64_.endpoint).norm(dim=-1) / spacing
        for name in variants:
            A, o = acc[name], outs[name]
            x = popcount32(masks[name][:, :mwords] ^ m64).sum(dim=1)
            A["xor"] += int(x.sum().item())
            A["ref"] += int(r.sum().item())
            A["worst"] = max(A["worst"], float((x.double() / r.clamp(min=1).double()).max().item()))
            ok = (o.status == C.TRACE_OK) & (o64_.status == C.TRACE_OK)
            A["status"] += int((o.status == o64_.status).sum().item())
            A["drift"].append(((o.endpoint - o64_.endpoint).norm(dim=-1) / spacing)[ok].float())
            if conditioning:
                A["s1"].append(sens[1e-9][ok].float())
                A["s100"].append(sens[1e-7][ok].float())
            A["same"] += int(((o.naccept == o64_.naccept) & (o.nattempt == o64_.nattempt)).sum().item())
        del masks, outs
    c64 = cnt["fp64"][:, :grid.ncols]
    res, grids = {}, {}
    for name in variants:
        A = acc[name]
        c = cnt[name][:, :grid.ncols]
        dr = torch.cat(A["drift"]) if A["drift"] else torch.zeros(0, device=dev)
        # torch.quantile takes at most 2^24 elements: quantiles of the sorted drift by index
        srt = torch.sort(dr).values
        q = [float(srt[min(srt.numel() - 1, int(round(f * (srt.numel() - 1))))].item()) for f in (0.5, 0.99, 0.999)] \
            if srt.numel() else [0.0] * 3
        res[name] = {
            "realizations": R, "traces": R * P,
            "linf_capture_probability": float((c - c64).abs().max().item()) / R,
            "linf_resolution": 1.0 / R,
            "cells_above_0.01": int(((c - c64).abs().double() / R > 0.01).sum().item()),
            "sum_abs_count_diff_over_sum64": float((c - c64).abs().sum().item()) / max(1, int(c64.sum().item())),
            "mismatched_visit_fraction": A["xor"] / max(1, A["ref"]),
            "mismatched_visit_fraction_worst_realization": A["worst"],
            "fp64_visits": A["ref"],
            "endpoint_drift_cells": {"p50": q[0], "p99": q[1], "p999": q[2],
                                     "max": float(dr.max().item()) if dr.numel() else 0.0,
                                     "traces_over_1e-3": int((dr > 1e-3).sum().item()),
                                     "traces_over_1e-2": int((dr > 1e-2).sum().item()),
                                     "traces_compared": int(dr.numel())},
            "status_agreement": A["status"] / (R * P),
            "traces_with_same_step_counts": A["same"] / (R * P)}
        if conditioning and dr.numel():
            s1 = torch.cat(A["s1"])
            s100 = torch.cat(A["s100"])
            well = s1 <= WELL_CONDITIONED_CELLS
            dw = dr[well]
            res[name]["conditioning"] = {
                "well_conditioned_fraction": float(well.double().mean().item()),
                "well_conditioned_definition": "FP64 endpoint moves < 1e-6 cell under a 1 nm release shift",
                "drift_max_well_conditioned_cells": float(dw.max().item()) if dw.numel() else 0.0,
                "well_conditioned_over_1e-3": int((dw > 1e-3).sum().item()),
                "ill_conditioned_traces": int((~well).sum().item()),
                "ill_conditioned_over_1e-3": int((dr[~well] > 1e-3).sum().item()),
                "max_ratio_drift_to_fp64_shift_100nm": float((dr / s100.clamp(min=1e-30))[~well].max().item())
                if bool((~well).any()) else 0.0,
                "traces_outside_bar": int((dr > torch.clamp(20.0 * s100, min=1e-3)).sum().item())}
        grids[name] = c.to(torch.int32)
    grids["fp64"] = c64.to(torch.int32)
    return res, grids


def _hbm_roofline(dram_bytes, seconds):
    """The tracking step against HBM: its measured DRAM traffic over the
    measured copy bandwidth (it is not memory-bound; this shows by how much)."""
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak, src = 6800.0, "fallback 6.8 TB/s"
    if os.path.exists(peaks_path):
        peak, src = float(json.load(open(peaks_path))["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs of measured"
    achieved = dram_bytes / seconds / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": dram_bytes, "peak_source": src}


def ctypes_peak(C, fp64):
    import ctypes
    import torch
    v = ctypes.c_double(0.0)
    C.check(C.load().oneka_fma_peak(1 if fp64 else 0, ctypes.byref(v), C.stream_ptr()))
    torch.cuda.synchronize()
    return v.value


# ---------------------------------------------------------------------------
# other workloads
# ---------------------------------------------------------------------------
def _setup():
    import torch
    from onekapy_gb300 import _capi as C
    from onekapy_gb300 import build as B
    B.build()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    return C.device()


def _site(spec, dev):
    from onekapy_gb300 import engine as E
    return E.Site(spec.wells, spec.observations, spec.base, c_dist=spec.c_dist, p_dist=spec.p_dist,
                  t_dist=spec.t_dist, device=dev)


def _opts(spec, precision):
    from onekapy_gb300 import engine as E
    return E.TrackOptions(duration=spec.duration, tol=spec.tol, maxstep=spec.maxstep, umbra=spec.umbra,
                          confined=spec.confined, precision=precision)


def algorithmic_flops(nwells, confined, attempts, node_tests):
    """FP32 flops of the tracking kernel's work: attempts x (6 F_v + 150) plus
    12 per chronicle node test; F_v = 10 N_w + 12 (confined), 16 N_w + 24
    (general)."""
    fv = 10 * nwells + 12 + (0 if confined else 6 * nwells + 12)
    return attempts * (6 * fv + 150) + 12 * node_tests


def fp32_roofline(flops, seconds, kernel):
    import torch
    from onekapy_gb300 import _capi as C
    peak = ctypes_peak(C, fp64=False)
    torch.cuda.synchronize()
    achieved = flops / seconds / 1e12
    return {"bound": "fp32", "achieved": achieved, "peak": peak / 1e12, "unit": "TFLOP/s",
            "frac": achieved / (peak / 1e12), "traffic": None, "kernel": kernel,
            "peak_source": "measured FP32 FMA loop on this GPU (oneka_fma_peak)"}


def _line(a, value, unit, metric, config, dtype="f32", **extra):
    return {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": a.steps,
            "warmup": a.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": dtype, "data": "synthetic", "config": config} | extra


def _timed(fn, a, stream, flush):
    """W untimed calls, then K calls timed with events, L2 flushed between."""
    import torch
    for _ in range(a.warmup):
        fn()
    torch.cuda.synchronize()
    sampler = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    sampler.start()
    ms = []
    for k in range(a.steps):
        flush.fill_(k & 0xFF)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    return ms, sampler.stop()


def run_config3(a):
    """64 uneven sites: realize + batched tracking of every site, captured
    once as a CUDA graph and replayed per step; one oneka_track call per site
    (the unbatched form) timed beside it; both must give the same counts."""
    import torch
    from onekapy_gb300 import _capi as C
    from onekapy_gb300 import engine as E
    from onekapy_gb300 import sites as S
    dev = _setup()
    specs = S.config3()
    jobs = []
    for k, spec in enumerate(specs):
        site = _site(spec, dev)
        n = max(1, int(round(spec.nreal * a.fraction)))
        real = E.Realizations.empty(n, site.nwells, dev, with_fit=False)
        E.realize(site, n, seed=SEED + k, out=real)
        grid = E.Grid.window(site.xt, site.yt, spec.spacing, spec.half)
        jobs.append(E.TrackJob(site, real, torch.as_tensor(site.release(spec.npaths), device=dev),
                               _opts(spec, C.FP32), grid,
                               torch.zeros((grid.nrows, grid.ncols), dtype=torch.int32, device=dev),
                               torch.zeros(1, dtype=torch.int64, device=dev)))
    tot_real = sum(j.real.n for j in jobs)
    tot_part = sum(j.real.n * j.release.shape[0] for j in jobs)
    # launch shape: autotuned on the site with the most particle work (setup, untimed)
    big = max(jobs, key=lambda j: j.real.n * j.release.shape[0] * j.opts.duration)
    tuned = E.autotune(big.site, big.real, big.release, big.opts, big.grid, sample=min(big.real.n, 1024))
    for j in jobs:
        j.opts = E.TrackOptions(**{**j.opts.__dict__, "block": tuned.block, "occupancy": tuned.occupancy,
                                   "window_kb": tuned.window_kb})
    need = E.batched_scratch_bytes(jobs)
    scratch = torch.zeros(min(need, 32 << 30) + 256, dtype=torch.uint8, device=dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)

    def body():
        for k, j in enumerate(jobs):
            j.counts.zero_()
            j.registered.zero_()
            E.realize(j.site, j.real.n, seed=SEED + k, out=j.real)
        E.track_batched(jobs, scratch=scratch)

    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        body()                                     # warm every kernel before capture
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        body()
    stream = torch.cuda.current_stream()
    ms, clocks = _timed(graph.replay, a, stream, flush)
    batched = [j.counts.clone() for j in jobs]
    # work counters (untimed pass)
    for j in jobs:
        j.outputs = E.TrackOutputs(counters=torch.zeros(E.COUNTERS, dtype=torch.int64, device=dev))
    body()
    torch.cuda.synchronize()
    accepts = sum(int(j.outputs.counters[1].item()) for j in jobs)
    attempts = sum(int(j.outputs.counters[0].item()) for j in jobs)
    flops = sum(algorithmic_flops(j.site.nwells, j.opts.confined, int(j.outputs.counters[0].item()),
                                  int(j.outputs.counters[2].item())) for j in jobs)
    for j in jobs:
        j.outputs = None
    # one call per site (realize + oneka_track), same realizations
    def per_site():
        for k, j in enumerate(jobs):
            j.counts.zero_()
            j.registered.zero_()
            E.realize(j.site, j.real.n, seed=SEED + k, out=j.real)
            E.track(j.site, j.real, j.release, j.opts, j.grid, counts=j.counts, registered=j.registered,
                    scratch=scratch)
    a1 = argparse.Namespace(**{**a.__dict__, "warmup": 1, "steps": 1})
    ms_site, _ = _timed(per_site, a1, stream, flush)
    same = all(torch.equal(b, j.counts) for b, j in zip(batched, jobs))
    t = float(np.mean(ms)) / 1e3
    cfg = {"workload": f"config3-64-uneven-sites: {tot_real} realizations, {tot_part} particles "
                       f"(fraction {a.fraction} of each site's realizations)",
           "sites": len(jobs), "realizations": tot_real, "particles": tot_part,
           "l2": "512 MB buffer written between timed steps", "graph": "realize + batched track, one replay"}
    line = _line(a, tot_real / t, UNIT, METRIC + " (64 uneven sites, batched)", cfg,
                 ms_per_step=1e3 * t, particle_steps_per_s=accepts / t, particles_per_s=tot_part / t,
                 work_per_step={"step_attempts": attempts, "accepted_steps": accepts},
                 roofline=fp32_roofline(flops, t, "track32_batch_kernel (+ register_batch_kernel, realize); "
                                                  "per-site F_v by well count"),
                 per_site_calls={"ms_per_step": ms_site[0], "realizations_per_s": tot_real / (ms_site[0] / 1e3),
                                 "batched_speedup": ms_site[0] / (1e3 * t)},
                 counts_equal_batched_vs_per_site=bool(same),
                 tracker_launch={"block": tuned.block, "occupancy": tuned.occupancy,
                                 "window_kb": tuned.window_kb},
                 clocks=clocks)
    print(json.dumps(line))


def run_config4(a):
    """Unconfined stress site: FP32 build timed; per-cell capture-probability
    error and endpoint drift of the FP32 build against the all-FP64 run of the
    same realizations."""
    import torch
    from onekapy_gb300 import _capi as C
    from onekapy_gb300 import engine as E
    from onekapy_gb300 import sites as S
    dev = _setup()
    spec = S.config4()
    site = _site(spec, dev)
    R, P = spec.nreal, spec.npaths
    grid = E.Grid.window(site.xt, site.yt, spec.spacing, spec.half)
    release = torch.as_tensor(site.release(P), device=dev)
    real = E.Realizations.empty(R, site.nwells, dev, with_fit=False)
    E.realize(site, R, seed=SEED, out=real)
    o32 = E.autotune(site, real, release, _opts(spec, C.FP32), grid, sample=min(R, 1024))
    o64 = _opts(spec, C.FP64)
    counts = torch.zeros((grid.nrows, grid.ncols), dtype=torch.int32, device=dev)
    scratch = torch.zeros(grid.slot_bytes() * R, dtype=torch.uint8, device=dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()

    def step32():
        counts.zero_()
        E.realize(site, R, seed=SEED, out=real)
        E.track(site, real, release, o32, grid, counts=counts, scratch=scratch)

    ms, clocks = _timed(step32, a, stream, flush)
    t = float(np.mean(ms)) / 1e3
    o32h = E.TrackOptions(**{**o32.__dict__, "head64": True})
    # speeds: the FP32 build with the FP64 head inversion on every realization, the FP64 build on a
    # sample (its rate; about 100 realizations/s here)
    secs, outs = {}, {}
    for name, o, n in (("fp32", o32, R), ("fp32_head64", o32h, R), ("fp64", o64, min(R, 1000))):
        c = torch.zeros_like(counts)
        out = E.TrackOutputs(counters=torch.zeros(E.COUNTERS, dtype=torch.int64, device=dev))
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        E.track(site, real.slice(0, n), release, o, grid, counts=c, scratch=scratch, outputs=out)
        e1.record()
        torch.cuda.synchronize()
        secs[name] = (e0.elapsed_time(e1) / 1e3, n)
        outs[name] = out
    # errors against the FP64 build on every realization and trace
    n64 = min(a.fp64_sample or R, R)
    cmps, _ = fp32_vs_fp64(site, real.slice(0, n64), release, {"fp32": o32, "fp32_head64": o32h}, o64, grid,
                           spec.spacing)
    cnt32 = outs["fp32"].counters
    steps = int(cnt32[1].item())
    flops = algorithmic_flops(site.nwells, spec.confined, int(cnt32[0].item()), int(cnt32[2].item()))
    fp64_rate = secs["fp64"][1] / secs["fp64"][0]
    cfg = {"workload": "config4-unconfined-31wells: 5000 realizations x 2048 paths, 25 y, 5 m grid 8x8 km",
           "nreal": R, "npaths": P, "fp64_realizations_compared": n64,
           "l2": "512 MB buffer written between timed steps"}
    line = _line(a, R / t, UNIT, METRIC + " (unconfined stress)", cfg, ms_per_step=1e3 * t,
                 particle_steps_per_s=steps / t,
                 roofline=fp32_roofline(flops, t, "track32_kernel (+ register_counts, realize)"),
                 fp64_gpu={"realizations_per_s": fp64_rate, "timed_realizations": secs["fp64"][1],
                           "speedup_fp32_over_fp64": (R / t) / fp64_rate},
                 fp32_vs_fp64=cmps["fp32"],
                 fp32_head64={"note": "general path with heads within 1 % of the aquifer top re-inverted in FP64",
                              "seconds_all_realizations": secs["fp32_head64"][0],
                              "seconds_fp32_all_realizations": secs["fp32"][0],
                              "vs_fp64": cmps["fp32_head64"]},
                 tracker_launch={"block": o32.block, "occupancy": o32.occupancy, "window_kb": o32.window_kb},
                 clocks=clocks)
    print(json.dumps(line))


def run_config5(a):
    """The learned surrogate: train on tracker-chronicled masks, then screen
    fresh realizations with judges; compare with tracking all of them."""
    import math
    import torch
    from onekapy_gb300 import _capi as C
    from onekapy_gb300 import engine as E
    from onekapy_gb300 import sites as S
    from onekapy_gb300 import surrogate as SG
    dev = _setup()
    spec = S.config5()
    site = _site(spec, dev)
    ntrain = int(round(200000 * a.fraction))
    nscreen = int(round(100000 * a.fraction))
    side = 256
    grid = E.Grid(site.xt - 0.5 * (side - 1) * spec.spacing, site.yt - 0.5 * (side - 1) * spec.spacing,
                  spec.spacing, spec.spacing, side, side)
    release = torch.as_tensor(site.release(spec.npaths), device=dev)
    opts = E.autotune(site, E.realize(site, 1024, seed=1), release, _opts(spec, C.FP32), grid, sample=1024)
    stream = torch.cuda.current_stream()
    # training pairs: realizations and their chronicle masks
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    train_real = E.realize(site, ntrain, seed=SEED)
    masks, slot_words = SG.chronicle_masks(site, train_real, release, opts, grid)
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    feats = SG.Features(train_real, site.nwells)
    X = feats(train_real)
    visit_rate = float(torch.count_nonzero(masks[:, :grid.nrows * grid.words_per_row]).item())
    model = SG.MLP([64, 512, 512, 512, side * side], dev, seed=5, out_bias=math.log(0.02 / 0.98))
    t0 = time.perf_counter()
    losses = SG.train(model, X, masks, slot_words, grid.words_per_row, side, epochs=a.epochs, batch=512,
                      lr=1.5e-3, lr_final=1e-4)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    nsteps = a.epochs * (ntrain // 512)
    flops_step = 3 * 2 * 512 * sum(i * o for i, o in zip(model.dims[:-1], model.dims[1:]))
    del masks
    # GEMM roofline: the last layer's forward GEMM of a 512-realization batch
    xb = X[:512]
    h = model._hidden(xb)
    L = model.layers[-1]
    logits = torch.empty((512, side * side), dtype=torch.float32, device=dev)
    gm = lambda: SG.gemm(h, True, L.wb, True, logits, 512, side * side, 512, bias=L.b)
    for _ in range(3):
        gm()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(20):
        gm()
    e1.record()
    torch.cuda.synchronize()
    t_gemm = e0.elapsed_time(e1) / 1e3 / 20
    gemm_tf = 2 * 512 * side * side * 512 / t_gemm / 1e12
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {"bf16_tflops": 1900.0}
    # screening of fresh realizations, end to end (draw + judges + surrogate)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    fresh = E.Realizations.empty(nscreen, site.nwells, dev, with_fit=False)
    results = []

    def screen_once():
        E.realize(site, nscreen, seed=SEED + 1, out=fresh)
        results.append(SG.screen(model, feats, site, fresh, release, opts, grid, judge_fraction=0.05,
                                 tolerance=SURROGATE_TOLERANCE))

    ms, clocks = _timed(screen_once, a, stream, flush)
    res = results[-1]
    # tracking every fresh realization (the method without the surrogate)
    counts = torch.zeros((side, side), dtype=torch.int32, device=dev)

    def track_all():
        counts.zero_()
        E.realize(site, nscreen, seed=SEED + 1, out=fresh)
        E.track(site, fresh, release, opts, grid, counts=counts)

    a1 = argparse.Namespace(**{**a.__dict__, "warmup": 1, "steps": 2})
    ms_all, _ = _timed(track_all, a1, stream, flush)
    full = counts.double() / nscreen
    err = (res.field - full).abs()
    t = float(np.mean(ms)) / 1e3
    t_all = float(np.mean(ms_all)) / 1e3
    cfg = {"workload": f"config5-surrogate-31wells: train {ntrain} pairs, screen {nscreen} realizations "
                       f"(5 % judges), 1000 paths, 20 y, 256x256 grid at 20 m",
           "mlp": "39 (padded 64) -> 512 -> 512 -> 512 GELU -> 65536 logits, BF16 with FP32 master weights",
           "l2": "512 MB buffer written between timed steps"}
    line = _line(a, nscreen / t, UNIT, METRIC + " (surrogate-screened)", cfg, dtype="bf16",
                 ms_per_step=1e3 * t,
                 track_all={"ms_per_step": 1e3 * t_all, "realizations_per_s": nscreen / t_all},
                 speedup_over_track_all=t_all / t,
                 judges={"n": res.n_judges, "linf": res.judge_linf, "mean_abs": res.judge_l1,
                         "tolerance": SURROGATE_TOLERANCE, "accepted": res.accepted},
                 field_vs_track_all={"linf": float(err.max().item()), "mean_abs": float(err.mean().item())},
                 screen_breakdown_ms={"judges_tracked": 1e3 * res.seconds_judges,
                                      "surrogate": 1e3 * res.seconds_surrogate},
                 training={"pairs": ntrain, "chronicle_seconds": t_data, "epochs": a.epochs, "steps": nsteps,
                           "seconds": t_train, "achieved_tflops": flops_step * nsteps / t_train / 1e12,
                           "loss_first": losses[0], "loss_last": losses[-1],
                           "visited_word_fraction": visit_rate / (ntrain * grid.nrows * grid.words_per_row)},
                 roofline={"bound": "tensor",
                           "kernel": ("gemm_tc_kernel (tcgen05, TMEM accumulators, TMA; last layer 512 x 65536 x 512, "
                                      "FP32 logits)" if SG.gemm_path(True, True, 512) else
                                      "gemm_bf16_kernel (mma.sync; last layer 512 x 65536 x 512)"),
                           "achieved": gemm_tf, "peak": peaks["bf16_tflops"], "unit": "TFLOP/s",
                           "frac": gemm_tf / peaks["bf16_tflops"], "traffic": None,
                           "peak_source": "MEASURED_PEAKS.json bf16_tflops (cuBLAS burst) of measured"},
                 clocks=clocks)
    print(json.dumps(line))


if __name__ == "__main__":
    a = args_()
    if a.impl == "reference":
        run_reference(a)
    elif a.workload == "config3":
        run_config3(a)
    elif a.workload == "config4":
        run_config4(a)
    elif a.workload == "config5":
        run_config5(a)
    else:
        run_ours(a)
