"""Seeded synthetic sites with the shapes of the benchmark configurations.

No public dataset is involved; every site is generated from a fixed seed
(site seed = 1000 + configuration number).  Shapes follow the workload
definitions:

  config 1  confined, 1 target + 3 neighbour wells within 2 km, 25 observations
            in a 3 km square, 100 realizations x 100 paths, 10 years, 10 m grid
            over 4 km x 4 km.
  config 2  mixed (top 30 m, heads straddling it), 1 + 10 wells within 5 km,
            60 observations, 10,000 realizations x 1,000 paths, 20 years,
            5 m grid over 8 km x 8 km.
  config 3  64 uneven sites (2-200 neighbour wells, 20-200 observations,
            1,000-20,000 realizations, 360/1024/4096 paths, 5-50 years,
            256^2-1024^2 grids at 5-20 m).
  config 4  unconfined, water table 0.5-3 m above the base near the target,
            target Q ~ U(1000, 3000), 30 neighbour wells, 5,000 x 2,048, 25 years.
  config 5  the surrogate's fixed site: 1 + 30 wells, mixed aquifer (top 30 m),
            20 m grid of 256 x 256 nodes; 39 varying parameters per
            realization (A..F, 31 discharges, K, porosity).

Heads of the confined/mixed sites come from a seeded quadratic head surface
(A, B ~ 1e-7, C ~ 1e-8, D, E ~ 1e-3) plus N(0, sigma) noise; the unconfined
site's heads come from a seeded unconfined potential that includes the wells.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .engine import Lognormal

DAY_PER_YEAR = 365.25


@dataclass
class SiteSpec:
    name: str
    wells: list            # (x, y, rw, qdist) in list order; the target first
    observations: list     # (x, y, z_ev, z_std)
    base: float
    c_dist: object
    p_dist: object
    t_dist: object
    confined: bool
    duration: float        # [d]
    npaths: int
    nreal: int
    spacing: float
    umbra: float
    half: float            # half width of the grid window [m]
    tol: float = 1.0
    maxstep: float = 10.0
    target: int = 0
    extra: dict = field(default_factory=dict)


def _neighbours(rng, n, radius, q):
    out = []
    for _ in range(n):
        r = radius * np.sqrt(rng.uniform(0.05, 1.0))
        a = rng.uniform(0.0, 2.0 * np.pi)
        out.append((float(np.round(r * np.cos(a), 2)), float(np.round(r * np.sin(a), 2)), 0.25, q))
    return out


def _quadratic_heads(rng, n, half, F, sigma, scale=1.0):
    A = scale * rng.uniform(0.5, 1.5) * 1e-7
    B = scale * rng.uniform(0.5, 1.5) * 1e-7
    Cc = scale * rng.uniform(-1.0, 1.0) * 1e-8
    ang = rng.uniform(0.0, 2.0 * np.pi)
    D = 1e-3 * np.cos(ang)
    E = 1e-3 * np.sin(ang)
    obs = []
    for _ in range(n):
        x = float(np.round(rng.uniform(-half, half), 2))
        y = float(np.round(rng.uniform(-half, half), 2))
        z = A * x * x + B * y * y + Cc * x * y + D * x + E * y + F + rng.normal(0.0, sigma)
        obs.append((x, y, float(z), sigma))
    return obs


def config1(seed: int = 1001) -> SiteSpec:
    rng = np.random.default_rng(seed)
    wells = [(0.0, 0.0, 0.25, (400.0, 600.0))] + _neighbours(rng, 3, 2000.0, (100.0, 500.0))
    obs = _quadratic_heads(rng, 25, 1500.0, 500.0, 0.1)
    return SiteSpec("config1-confined-4wells", wells, obs, 0.0, Lognormal(np.log(10.0), 0.3),
                    (0.2, 0.3), (20.0, 30.0), True, 10 * DAY_PER_YEAR, 100, 100, 10.0, 10.0, 2000.0)


def config2(seed: int = 1002, nreal: int = 10000, npaths: int = 1000) -> SiteSpec:
    rng = np.random.default_rng(seed)
    wells = [(0.0, 0.0, 0.25, (400.0, 600.0))] + _neighbours(rng, 10, 5000.0, (100.0, 500.0))
    obs = _quadratic_heads(rng, 60, 3000.0, 30.0, 0.1)
    return SiteSpec("config2-mixed-11wells", wells, obs, 0.0, Lognormal(np.log(10.0), 0.3),
                    (0.2, 0.3), 30.0, False, 20 * DAY_PER_YEAR, npaths, nreal, 5.0, 10.0, 4000.0)


def config4(seed: int = 1004, nreal: int = 5000, npaths: int = 2048) -> SiteSpec:
    rng = np.random.default_rng(seed)
    nb = _neighbours(rng, 30, 3000.0, (50.0, 150.0))
    qn = [0.5 * (w[3][0] + w[3][1]) for w in nb]
    K0 = 30.0

    def head(x, y):
        phi = 2.0e-3 * K0 * 10.0 * x + 1.0e-3 * K0 * 10.0 * y - 30.0
        for (xw, yw, qq) in [(0.0, 0.0, 2000.0)] + [(w[0], w[1], q) for w, q in zip(nb, qn)]:
            phi += qq / (4 * np.pi) * np.log((x - xw) ** 2 + (y - yw) ** 2 + 1e-6)
        return float(np.sqrt(2.0 * max(phi, 1.0) / K0))

    obs = []
    for _ in range(60):
        x = float(np.round(rng.uniform(-2000, 2000), 2))
        y = float(np.round(rng.uniform(-2000, 2000), 2))
        if min(np.hypot(x - w[0], y - w[1]) for w in [(0.0, 0.0)] + nb) < 100.0:
            continue
        obs.append((x, y, head(x, y) + float(rng.normal(0, 0.05)), 0.05))
    wells = [(0.0, 0.0, 0.25, (1000.0, 3000.0))] + nb
    return SiteSpec("config4-unconfined-31wells", wells, obs, 0.0, (25.0, 35.0), (0.2, 0.3), 20.0,
                    False, 25 * DAY_PER_YEAR, npaths, nreal, 5.0, 10.0, 4000.0)


def config3(seed: int = 1003, nsites: int = 64):
    """64 uneven sites; returns a list of SiteSpec."""
    rng = np.random.default_rng(seed)
    sites = []
    for k in range(nsites):
        nnb = int(np.round(np.exp(rng.uniform(np.log(2), np.log(200)))))
        nobs = int(rng.integers(20, 201))
        nreal = int(np.round(np.exp(rng.uniform(np.log(1000), np.log(20000)))))
        npaths = int(rng.choice([360, 1024, 4096]))
        years = float(rng.uniform(5, 50))
        side = int(rng.choice([256, 512, 768, 1024]))
        spacing = float(rng.choice([5.0, 10.0, 20.0]))
        wells = [(0.0, 0.0, 0.25, (300.0, 800.0))] + _neighbours(rng, nnb, 0.5 * side * spacing,
                                                                 (50.0, 400.0))
        obs = _quadratic_heads(rng, nobs, 0.4 * side * spacing, 200.0, 0.1)
        sites.append(SiteSpec(f"config3-site{k:02d}", wells, obs, 0.0, Lognormal(np.log(10.0), 0.3),
                              (0.2, 0.3), (20.0, 30.0), True, years * DAY_PER_YEAR, npaths, nreal,
                              spacing, 2 * spacing, 0.5 * (side - 1) * spacing))
    return sites


def config5(seed: int = 1005, nreal: int = 200000, npaths: int = 1000) -> SiteSpec:
    """The surrogate's fixed 31-well site (config-2 style, 20 m grid of 256 x 256)."""
    rng = np.random.default_rng(seed)
    wells = [(0.0, 0.0, 0.25, (400.0, 600.0))] + _neighbours(rng, 30, 5000.0, (100.0, 500.0))
    obs = _quadratic_heads(rng, 60, 3000.0, 30.0, 0.1)
    return SiteSpec("config5-surrogate-31wells", wells, obs, 0.0, Lognormal(np.log(10.0), 0.3),
                    (0.2, 0.3), 30.0, False, 20 * DAY_PER_YEAR, npaths, nreal, 20.0, 20.0,
                    0.5 * 255 * 20.0)

