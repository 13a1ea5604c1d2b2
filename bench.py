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
# DRAM bytes per realization of the tracking launch on this site, from one ncu
# capture of a 1,000-realization launch (15.62 MB; profiles/).
TRACK32_DRAM_BYTES_PER_REALIZATION = 15.62e6 / 1000


def args_():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nreal", type=int, default=10000)
    ap.add_argument("--npaths", type=int, default=1000)
    ap.add_argument("--fp64-sample", type=int, default=200)
    ap.add_argument("--no-cpu-baseline", action="store_true")
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
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

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
                                      "-i", str(self.index), "-lms", "200"], stdout=self.out,
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
    sample = 10 * max(4, threads)
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
    o32 = E.autotune(site, real, release, o32, grid, sample=min(R, 1024))

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
    cnt = E.TrackOutputs(counters=torch.zeros(4, dtype=torch.int64, device=dev))
    step(o32, R, outputs=cnt)
    torch.cuda.synchronize()
    attempts, accepts, ntests, natoms = (int(v) for v in cnt.counters.cpu().tolist())
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
        # plain FP64 GPU tracker and the FP32 build on the same sample of realizations
        n64 = min(a.fp64_sample, R)
        step(o64, min(8, n64))
        torch.cuda.synchronize()
        e64 = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        step(o64, n64, ev=e64)
        torch.cuda.synchronize()
        c64 = counts.clone()
        fp64_rate = n64 / (e64[0].elapsed_time(e64[2]) / 1e3)
        step(o32, n64)
        torch.cuda.synchronize()
        c32 = counts.clone()
        linf = float((c32 - c64).abs().max().item()) / n64
        mism = float(((c32 > 0) != (c64 > 0)).sum().item()) / max(1, int((c64 > 0).sum().item()))

        # end to end through the public API with host buffers
        from onekapy_gb300.stochastic import create_stochastic_capturezone
        e2e_n = R

        def e2e_once():
            pf = create_stochastic_capturezone(0, P, spec.duration, e2e_n, spec.base, spec.c_dist,
                                               spec.p_dist, spec.t_dist, spec.wells, spec.observations,
                                               spec.spacing, spec.umbra, spec.confined, spec.tol,
                                               spec.maxstep, seed=SEED, precision=C.FP32,
                                               window=spec.half, chunk=R)
            return pf.pgrid.cpu().numpy(), pf

        e2e_once()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        host_pgrid, pf = e2e_once()
        t_e2e = time.perf_counter() - t0
        h2d = (len(spec.wells) * (3 * 8 + 32) + len(spec.observations) * 32 + P * 16)
        d2h = host_pgrid.nbytes + e2e_n * 4 + 8
        assert np.array_equal(host_pgrid, counts32_full.cpu().numpy().astype(np.float64)), \
            "public API and engine disagree"

        # roofline of the tracking kernel: algorithmic FP32 flops per launch
        nw = len(spec.wells)
        fv = 10 * nw + 12 + (0 if spec.confined else 6 * nw + 12)
        flops = attempts * (6 * fv + 150) + 12 * ntests
        t_track = float(np.mean(track_ms)) / 1e3
        peak = ctypes_peak(C, fp64=False)
        achieved = flops / t_track / 1e12

        cpu = None
        if world == 1 and not a.no_cpu_baseline:
            th = host_threads()
            ns = 10 * max(4, th)      # about 1-2 s wall on 16 threads: 15-30 s of CPU work
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
                "fp64_gpu": {"realizations_per_s": fp64_rate, "sample_realizations": n64,
                             "speedup_fp32_over_fp64": value / world / fp64_rate},
                "fp32_vs_fp64": {"linf_capture_probability": linf, "mismatched_visited_fraction": mism,
                                 "sample_realizations": n64},
                "work_per_step": {"step_attempts": attempts, "accepted_steps": accepts,
                                  "chronicle_node_tests": ntests, "chronicle_word_atomics": natoms},
                "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak / 1e12,
                             "unit": "TFLOP/s", "frac": achieved / (peak / 1e12),
                             "traffic": TRACK32_DRAM_BYTES_PER_REALIZATION * R,
                             "traffic_source": "ncu dram__bytes_read+write of a 1000-realization launch, "
                                               "scaled by realizations (profiles/track32_config2_1000real_full.md)",
                             "kernel": "track32_kernel (+ register_counts_kernel)",
                             "peak_source": "measured FP32 FMA loop on this GPU (oneka_fma_peak)"},
                "e2e": {"value": e2e_n / t_e2e, "unit": UNIT, "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": d2h},
                "tracker_launch": {"block": o32.block, "occupancy": o32.occupancy,
                                   "window_kb": o32.window_kb, "chosen_by": "autotune on 1024 realizations"},
                "gpu_launches": 3 * a.steps,
                "clocks": clocks,
                "cpu_baseline": cpu}
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    if line is not None:
        print(json.dumps(line))


def ctypes_peak(C, fp64):
    import ctypes
    import torch
    v = ctypes.c_double(0.0)
    C.check(C.load().oneka_fma_peak(1 if fp64 else 0, ctypes.byref(v), C.stream_ptr()))
    torch.cuda.synchronize()
    return v.value


if __name__ == "__main__":
    a = args_()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)
