"""Generate the golden fixtures under tests/golden/ by running the OnekaPy reference.

This script is the only committed file that reads the reference tree.  It runs
in the development container, where the reference sources are mounted; the
fixtures it writes travel with the repository, and the tests compare against
them.  It never touches the product package.

    ONEKA_REFERENCE=<path of the OnekaPy checkout> python tests/golden/make_golden.py
    python tests/golden/make_golden.py --reference <path of the OnekaPy checkout>

What it records (all FP64, as the reference computes):

* ``track_<case>.npz``: a small synthetic site, per-realization parameters
  (K, n, H, discharges, fitted coef_ev / coef_cov and the drawn coef),
  the release ring, the pre-expanded grid, the reference's chronicle counts
  (``compute_capturezone`` + ``register``), and every particle's vertices from
  ``compute_backtrace``.
* ``expand_<case>.npz``: the same with the reference's auto-expanding grid
  (no pre-expansion), for the frame replay.
* ``fit_cases.npz``: ``Model.fit_regional_flow`` on synthetic observation sets.
* ``raster_cases.npz``: ``ProbabilityField.rasterize`` on random polylines.
* ``expand_geometry.npz``: ``ProbabilityField.expand`` geometry sequences.
* ``site_<name>.npz``: the reference's own site files (``data/<name>.py``) run
  through its top-level sequence: ``filter_obs`` with the site's buffer
  (oneka/oneka.py:254), then the deterministic driver
  (``create_deterministic_capturezone``, oneka/deterministic.py:65-235): the
  site's inputs (distributions, mean wells and aquifer, raw and filtered
  observations), the fitted coef_ev / coef_cov, and the auto-expanded grid's
  geometry and counts.

Synthetic sites are seeded.  The site fixtures hold the numbers of the
reference's site files as inputs next to its outputs on them.

    python tests/golden/make_golden.py --only sites     # just the site fixtures
    python tests/golden/make_golden.py --only stats     # just summary_statistics.npz
    python tests/golden/make_golden.py --only archive   # just archive_reference.bz2
    python tests/golden/make_golden.py --only fitrows   # just fit_rows_cases.npz

* ``fit_rows_cases.npz``: the reference's ``Model.construct_fit`` rows WA, Wb
  and ``Model.compute_fit`` solution on the inputs of ``fit_cases.npz``.

* ``archive_reference.bz2`` (+ ``archive_reference.npz``, the field it holds):
  an archive written by the reference's own ``dump_oneka``
  (oneka/archive.py:46-82) of a reference ProbabilityField with registered
  weights and a pending registration grid.  The same run checks the other
  direction: an archive written by ``onekapy_gb300.archive.dump_oneka`` is
  opened by the reference's ``load_oneka`` (oneka/archive.py:85-89) and
  yields the reference's class with the same attributes.
"""
from __future__ import annotations

import argparse
import os
import platform
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def import_reference(path):
    # Compile the reference from its .py sources into a private cache; the
    # bytecode shipped inside the reference tree is never read.
    sys.pycache_prefix = os.path.join(tempfile.gettempdir(), "oneka_ref_pycache")
    sys.dont_write_bytecode = False
    sys.path.insert(0, path)
    np.float = float        # removed from NumPy >= 1.24; the reference still names it
    from oneka import capturezone, model, probabilityfield
    return model, capturezone, probabilityfield


SITE_FILES = ["basic", "basic_deterministic", "barnesville", "carlos", "long_prairie", "paynesville", "perham"]


def _dist_row(d):
    """A distribution as [kind, a, b, c]: kind 0 constant, 2 uniform (a, b), 3 triangular."""
    if type(d) is not tuple:
        return [0.0, float(d), 0.0, 0.0]
    if len(d) == 2:
        return [2.0, float(d[0]), float(d[1]), 0.0]
    return [3.0, float(d[0]), float(d[1]), float(d[2])]


def make_site_goldens(out, meta, names=None):
    """The reference's deterministic capture zone of each of its site files."""
    import importlib
    import time
    from oneka import deterministic, model, stochastic, utilities
    for name in names or SITE_FILES:
        site = importlib.import_module(f"data.{name}")
        t0 = time.time()
        # as the reference's top-level driver does (oneka/oneka.py:254): drop
        # observations within the buffer of any well, then the capture zone
        obs = utilities.filter_obs(site.OBSERVATIONS, site.WELLS, site.BUFFER)
        pf = deterministic.create_deterministic_capturezone(
            site.TARGET, site.NPATHS, site.DURATION, site.BASE, site.C_DIST, site.P_DIST, site.T_DIST,
            site.WELLS, obs, site.SPACING, site.UMBRA, site.CONFINED, site.TOL, site.MAXSTEP)
        # the driver's own fit, repeated to record its coefficients
        mean = stochastic.compute_variate_mean
        wells = [[w[0], w[1], w[2], mean(w[3])] for w in site.WELLS]
        K, n, H = mean(site.C_DIST), mean(site.P_DIST), mean(site.T_DIST)
        xt, yt, rt = site.WELLS[site.TARGET][0:3]
        mo = model.Model(site.BASE, K, n, H, wells)
        ev, cov = mo.fit_regional_flow(obs, xt, yt)
        np.savez_compressed(
            os.path.join(out, f"site_{name}.npz"),
            wells=np.array(wells, dtype=np.float64), qdist=np.array([_dist_row(w[3]) for w in site.WELLS]),
            obs_raw=np.array(site.OBSERVATIONS, dtype=np.float64), buffer=float(site.BUFFER),
            obs=np.array([tuple(float(v) for v in o) for o in obs], dtype=np.float64),
            c_dist=np.array(_dist_row(site.C_DIST)), p_dist=np.array(_dist_row(site.P_DIST)),
            t_dist=np.array(_dist_row(site.T_DIST)), base=float(site.BASE), K=float(K), n=float(n), H=float(H),
            coef_ev=np.reshape(ev, 6), coef_cov=np.reshape(cov, 36), target=int(site.TARGET),
            xt=float(xt), yt=float(yt), rt=float(rt), npaths=int(site.NPATHS), duration=float(site.DURATION),
            spacing=float(site.SPACING), umbra=float(site.UMBRA), confined=bool(site.CONFINED),
            tol=float(site.TOL), maxstep=float(site.MAXSTEP), pgrid=pf.pgrid, xmin=pf.xmin, ymin=pf.ymin,
            xmax=pf.xmax, ymax=pf.ymax, nrows=pf.nrows, ncols=pf.ncols, total_weight=pf.total_weight, **meta)
        print(f"site_{name}: {len(wells)} wells, {len(obs)} of {len(site.OBSERVATIONS)} obs, grid {pf.nrows}x{pf.ncols}, "
              f"{int(np.count_nonzero(pf.pgrid))} visited nodes, {time.time() - t0:.1f} s", flush=True)


def make_stats_goldens(out, meta):
    """utilities.summary_statistics on the retained observations of each site
    file, as the reference's driver logs them (oneka/oneka.py:258-259), and
    on a synthetic table with NaNs and mixed formats."""
    import importlib
    from oneka import utilities
    cases = []
    for name in SITE_FILES:
        site = importlib.import_module(f"data.{name}")
        obs = utilities.filter_obs(site.OBSERVATIONS, site.WELLS, site.BUFFER)
        cases.append((np.array(obs, dtype=np.float64), ["Easting", "Northing", "Head", "Stdev"],
                      ["12.2f", "12.2f", "12.2f", "12.2f"], "Retained Observations"))
    rng = np.random.default_rng(5)
    v = rng.normal(size=(40, 3)) * [1.0, 100.0, 1e-3]
    v[[3, 17], 1] = np.nan
    cases.append((v, ["a", "bb", "c"], ["8.3f", "10.1f", "11.3e"], "Mixed formats"))
    fields = {}
    for i, (vals, names, fmts, title) in enumerate(cases):
        fields[f"values_{i}"] = vals
        fields[f"names_{i}"] = np.array(names)
        fields[f"formats_{i}"] = np.array(fmts)
        fields[f"title_{i}"] = np.array(title)
        fields[f"text_{i}"] = np.array(utilities.summary_statistics([tuple(r) for r in vals], names, fmts,
                                                                    title).getvalue())
    np.savez_compressed(os.path.join(out, "summary_statistics.npz"), ncases=len(cases), **fields, **meta)
    print(f"summary_statistics.npz: {len(cases)} cases")


def import_reference_utilities():
    from oneka import utilities
    return utilities


def make_site(rng, *, nnb, radius, nobs, obs_half, head_fn, sigma, q_target, q_nb, rw=0.25):
    wells = [(0.0, 0.0, rw, q_target)]
    for _ in range(nnb):
        r = radius * np.sqrt(rng.uniform(0.15, 1.0))
        a = rng.uniform(0, 2 * np.pi)
        wells.append((float(np.round(r * np.cos(a), 1)), float(np.round(r * np.sin(a), 1)), rw,
                      q_nb))
    obs = []
    for _ in range(nobs):
        x = float(np.round(rng.uniform(-obs_half, obs_half), 1))
        y = float(np.round(rng.uniform(-obs_half, obs_half), 1))
        z = head_fn(x, y) + rng.normal(0, sigma)
        obs.append((x, y, float(z), sigma))
    return wells, obs


def draw_realizations(M, rng, wells_st, obs, base, kdist, ndist, hdist, nreal):
    """Per-realization draw, fit and MVN draw, using the reference's own fit."""
    K, n, H, Q, EV, COV, COEF = [], [], [], [], [], [], []
    for _ in range(nreal):
        wells = [(w[0], w[1], w[2], float(rng.uniform(*w[3]))) for w in wells_st]
        k = float(kdist(rng))
        nn = float(ndist(rng))
        h = float(hdist(rng))
        mo = M.Model(base, k, nn, h, wells)
        ev, cov = mo.fit_regional_flow(obs, wells[0][0], wells[0][1])
        ev = np.reshape(ev, [6, ])
        coef = rng.multivariate_normal(ev, cov)
        K.append(k); n.append(nn); H.append(h); Q.append([w[3] for w in wells])
        EV.append(ev); COV.append(cov); COEF.append(coef)
    return dict(K=np.array(K), n=np.array(n), H=np.array(H), q=np.array(Q), coef_ev=np.array(EV),
                coef_cov=np.array(COV), coef=np.array(COEF))


def release(xt, yt, rt, npaths):
    pts = []
    for theta in np.linspace(0, 2 * np.pi, npaths + 1)[0:-1]:
        pts.append(((rt + 1.0) * np.cos(theta) + xt, (rt + 1.0) * np.sin(theta) + yt))
    return np.array(pts, dtype=np.float64)


def run_track_case(M, C, PF, name, *, wells, obs, base, real, npaths, duration, tol, maxstep,
                   spacing, umbra, confined, half, preexpand=True, max_vertices_store=None):
    xt, yt, rt = wells[0][0], wells[0][1], wells[0][2]
    pf = PF.ProbabilityField(spacing, spacing, xt, yt)
    if preexpand:
        pf.expand(xt - half + 0.5 * spacing, xt + half - 0.5 * spacing,
                  yt - half + 0.5 * spacing, yt + half - 0.5 * spacing)
    xmin0, ymin0, nr0, nc0 = pf.xmin, pf.ymin, pf.nrows, pf.ncols
    nreal = len(real["K"])
    verts, nverts = [], []
    for r in range(nreal):
        wl = [(w[0], w[1], w[2], real["q"][r][i]) for i, w in enumerate(wells)]
        mo = M.Model(base, real["K"][r], real["n"][r], real["H"][r], wl, xt, yt, real["coef"][r])
        if confined:
            def feval(xy, mo=mo):
                Vx, Vy = mo.compute_velocity_confined(xy[0], xy[1])
                return np.array([-Vx, -Vy])
        else:
            def feval(xy, mo=mo):
                Vx, Vy = mo.compute_velocity(xy[0], xy[1])
                return np.array([-Vx, -Vy])
        C.compute_capturezone(xt, yt, rt, npaths, duration, pf, umbra, 1.0, tol, maxstep, feval)
        for (xs, ys) in release(xt, yt, rt, npaths):
            v = C.compute_backtrace(xs, ys, duration, tol, maxstep, feval)
            verts.append(np.array([(float(a[0]), float(a[1])) for a in v], dtype=np.float64))
            nverts.append(len(v))
    maxv = max(nverts)
    V = np.full((len(verts), maxv, 2), np.nan)
    for i, v in enumerate(verts):
        V[i, :len(v)] = v
    out = dict(
        wells=np.array([w[:3] for w in wells], dtype=np.float64), obs=np.array(obs, dtype=np.float64),
        base=base, npaths=npaths, duration=duration, tol=tol, maxstep=maxstep, spacing=spacing,
        umbra=umbra, confined=int(confined), release=release(xt, yt, rt, npaths),
        grid0=np.array([xmin0, ymin0, spacing, spacing, nr0, nc0], dtype=np.float64),
        grid=np.array([pf.xmin, pf.ymin, pf.deltax, pf.deltay, pf.nrows, pf.ncols], dtype=np.float64),
        counts=pf.pgrid.astype(np.int32), total_weight=pf.total_weight,
        vertices=V.reshape(nreal, npaths, maxv, 2), nvertices=np.array(nverts).reshape(nreal, npaths),
        **{k: np.asarray(v) for k, v in real.items()})
    assert np.all(pf.pgrid == np.round(pf.pgrid))
    return out


def make_archive_goldens(out, meta, PF):
    """An archive written by the reference, and the check that the reference
    reads one written by this package."""
    import glob
    import shutil
    from oneka import archive as RA
    pf = PF.ProbabilityField(10.0, 10.0, 0.0, 0.0)
    rr = np.random.default_rng(5)
    for k, w in enumerate([1.0, 1.0, 0.5, 2.0]):
        pts = rr.uniform(-150, 150, size=2) + np.cumsum(rr.normal(0, 20, size=(12, 2)), axis=0)
        pf.rasterize(list(pts[:, 0]), list(pts[:, 1]), 15.0)
        pf.register(w)
    pts = np.cumsum(rr.normal(0, 20, size=(6, 2)), axis=0)
    pf.rasterize(list(pts[:, 0]), list(pts[:, 1]), 12.0)     # pending: rgrid set, not registered
    args = ("archive-golden", 12.5, 0, 24, 3652.5, 4, 0.0, (5.0, 10.0), 0.25, (20.0, 25.0, 30.0),
            [(0.0, 0.0, 0.25, (400.0, 600.0))], [(100.0, 50.0, 30.0, 0.1)], 100.0, 10.0, 15.0, 2.0,
            True, 1.0, 10.0)
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as td:
        os.chdir(td)
        try:
            RA.dump_oneka(*args, pf)
        finally:
            os.chdir(cwd)
        written = glob.glob(os.path.join(td, "*Oneka*.bz2")) + glob.glob(os.path.join(td, "logs", "Oneka*.bz2"))
        assert len(written) == 1, written
        shutil.copyfile(written[0], os.path.join(out, "archive_reference.bz2"))
    np.savez_compressed(os.path.join(out, "archive_reference.npz"), pgrid=pf.pgrid, rgrid=pf.rgrid,
                        geometry=np.array([pf.deltax, pf.deltay, pf.nrows, pf.ncols, pf.xmin, pf.xmax,
                                           pf.ymin, pf.ymax, pf.total_weight]), **meta)
    # the other direction: this package's archive, read by the reference
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from onekapy_gb300 import archive as OA
    from onekapy_gb300.probabilityfield import ProbabilityField as OurPF
    ours = OurPF.__new__(OurPF)
    ours.__setstate__(dict(pf.__dict__))
    with tempfile.TemporaryDirectory() as td:
        fn = OA.dump_oneka(*args, ours, filename=os.path.join(td, "ours.bz2"))
        d = RA.load_oneka(fn)
    got = d["pfield"]
    assert type(got) is PF.ProbabilityField, type(got)
    for k in ("deltax", "deltay", "nrows", "ncols", "xmin", "xmax", "ymin", "ymax", "total_weight"):
        assert getattr(got, k) == getattr(pf, k), k
    assert got.pgrid.dtype == np.float64 and np.array_equal(got.pgrid, pf.pgrid)
    assert got.rgrid.dtype == bool and np.array_equal(got.rgrid, pf.rgrid)
    print("archive: reference archive written; this package's archive read by the reference's load_oneka")


def make_fit_rows_goldens(out, meta, M):
    """construct_fit (WA, Wb) and compute_fit (ev, cov) of the reference on the fit cases' inputs."""
    d = np.load(os.path.join(out, "fit_cases.npz"))
    rows = {}
    for i in range(int(d["ncases"])):
        wq = [tuple(float(v) for v in r) for r in d[f"wells_{i}"]]
        ob = [tuple(float(v) for v in r) for r in d[f"obs_{i}"]]
        mo = M.Model(float(d[f"base_{i}"]), float(d[f"K_{i}"]), 0.25, float(d[f"H_{i}"]), wq)
        WA, Wb = mo.construct_fit(ob, wq[0][0], wq[0][1])
        ev, cov = M.Model.compute_fit(WA, Wb)
        rows.update({f"WA_{i}": WA, f"Wb_{i}": Wb, f"ev_{i}": ev, f"cov_{i}": cov, f"xo_{i}": wq[0][0],
                     f"yo_{i}": wq[0][1]})
    np.savez_compressed(os.path.join(out, "fit_rows_cases.npz"), ncases=int(d["ncases"]), **rows, **meta)
    print("fit rows: construct_fit and compute_fit of", int(d["ncases"]), "cases")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("ONEKA_REFERENCE"),
                    help="OnekaPy checkout (default: $ONEKA_REFERENCE)")
    ap.add_argument("--out", default=HERE)
    ap.add_argument("--only", choices=["sites", "stats", "archive", "fitrows"], default=None)
    ap.add_argument("--site", action="append", default=None, help="with --only sites: these site files only")
    args = ap.parse_args()
    if not args.reference:
        ap.error("give --reference or set ONEKA_REFERENCE to the OnekaPy checkout")
    M, C, PF = import_reference(args.reference)
    meta = dict(numpy=np.__version__, python=platform.python_version(), machine=platform.machine())
    print("reference imported;", meta)
    if args.only == "stats":
        make_stats_goldens(args.out, meta)
        return
    if args.only == "archive":
        make_archive_goldens(args.out, meta, PF)
        return
    if args.only == "fitrows":
        make_fit_rows_goldens(args.out, meta, M)
        return
    make_site_goldens(args.out, meta, args.site)
    if args.only == "sites":
        return
    make_stats_goldens(args.out, meta)
    make_archive_goldens(args.out, meta, PF)

    rng = np.random.default_rng(20260101)
    day = 365.25

    # ---- confined, C1-like: heads from a quadratic read as head, F = 500 m.
    A, B, Cc, D, E = 1.0e-7, 0.8e-7, 1.0e-8, 1.2e-3, -0.7e-3
    hf = lambda x, y: A * x * x + B * y * y + Cc * x * y + D * x + E * y + 500.0
    wells, obs = make_site(rng, nnb=3, radius=2000.0, nobs=25, obs_half=1500.0, head_fn=hf,
                           sigma=0.1, q_target=(400.0, 600.0), q_nb=(100.0, 500.0))
    real = draw_realizations(M, rng, wells, obs, 0.0,
                             lambda g: np.exp(np.log(10.0) + 0.3 * g.normal()),
                             lambda g: g.uniform(0.2, 0.3), lambda g: g.uniform(20, 30), 3)
    cases = {}
    cases["confined_u10"] = run_track_case(
        M, C, PF, "confined_u10", wells=wells, obs=obs, base=0.0, real=real, npaths=24,
        duration=10 * day, tol=1, maxstep=10, spacing=10, umbra=10, confined=True, half=2000.0)
    cases["confined_u20"] = run_track_case(
        M, C, PF, "confined_u20", wells=wells, obs=obs, base=0.0, real=real, npaths=16,
        duration=10 * day, tol=1, maxstep=20, spacing=10, umbra=20, confined=True, half=2000.0)

    # ---- mixed: top 30 m, heads straddling the top (general head path).
    hf2 = lambda x, y: 2e-7 * x * x + 1e-7 * y * y + 1.5e-3 * x - 0.8e-3 * y + 30.5
    wells2, obs2 = make_site(rng, nnb=5, radius=2500.0, nobs=40, obs_half=2500.0, head_fn=hf2,
                             sigma=0.1, q_target=(400.0, 600.0), q_nb=(100.0, 400.0))
    real2 = draw_realizations(M, rng, wells2, obs2, 0.0,
                              lambda g: np.exp(np.log(10.0) + 0.3 * g.normal()),
                              lambda g: g.uniform(0.2, 0.3), lambda g: 30.0, 2)
    cases["mixed_general"] = run_track_case(
        M, C, PF, "mixed_general", wells=wells2, obs=obs2, base=0.0, real=real2, npaths=16,
        duration=5 * day, tol=1, maxstep=10, spacing=5, umbra=10, confined=False, half=1500.0)

    # ---- thin unconfined: water table 1-3 m above base, strong pumping: dry cells.
    # Heads come from a true unconfined potential that includes the wells, so
    # the water table sits 1-3 m above base next to the target well.
    nb3 = [(700.0, -400.0, 100.0), (-900.0, 300.0, 80.0), (200.0, 1100.0, 120.0),
           (-500.0, -1000.0, 60.0)]

    def hf3(x, y, K0=30.0):
        phi = 2.0e-3 * 30.0 * x + 1.0e-3 * 30.0 * y - 20.0
        for (xw, yw, qq) in [(0.0, 0.0, 2000.0)] + nb3:
            phi += qq / (4 * np.pi) * np.log((x - xw) ** 2 + (y - yw) ** 2 + 1e-9)
        return float(np.sqrt(2.0 * max(phi, 1.0) / K0))
    wells3, obs3 = make_site(rng, nnb=0, radius=0.0, nobs=30, obs_half=1200.0, head_fn=hf3,
                             sigma=0.05, q_target=(1800.0, 2200.0), q_nb=None)
    wells3 += [(xw, yw, 0.25, (0.8 * qq, 1.2 * qq)) for (xw, yw, qq) in nb3]
    real3 = draw_realizations(M, rng, wells3, obs3, 0.0,
                              lambda g: g.uniform(25.0, 35.0),
                              lambda g: g.uniform(0.2, 0.3), lambda g: 20.0, 4)
    cases["unconfined_thin"] = run_track_case(
        M, C, PF, "unconfined_thin", wells=wells3, obs=obs3, base=0.0, real=real3, npaths=16,
        duration=2 * day, tol=1, maxstep=10, spacing=5, umbra=10, confined=False, half=1000.0)

    # ---- the same site with F lowered: some realizations are dry at the ring.
    real3d = {k: np.array(v, copy=True) for k, v in real3.items()}
    real3d["coef"][:, 5] -= 450.0
    cases["unconfined_dryshift"] = run_track_case(
        M, C, PF, "unconfined_dryshift", wells=wells3, obs=obs3, base=0.0, real=real3d,
        npaths=16, duration=2 * day, tol=1, maxstep=10, spacing=5, umbra=10, confined=False,
        half=1000.0)
    # ---- forward tracking (negative duration) into the pumping well: partial dry traces.
    cases["forward_dry"] = run_track_case(
        M, C, PF, "forward_dry", wells=wells3, obs=obs3, base=0.0, real=real3, npaths=16,
        duration=-20.0, tol=1, maxstep=10, spacing=5, umbra=10, confined=False, half=1000.0)

    # ---- auto-expanding grid (no pre-expansion): the reference grows its grid.
    cases["expanding_u20"] = run_track_case(
        M, C, PF, "expanding_u20", wells=wells, obs=obs, base=0.0,
        real={k: v[:2] for k, v in real.items()}, npaths=12, duration=5 * day, tol=1,
        maxstep=20, spacing=10, umbra=20, confined=True, half=0.0, preexpand=False)

    for name, d in cases.items():
        np.savez_compressed(os.path.join(args.out, f"track_{name}.npz"), **d, **meta)
        print(name, "registered", d["total_weight"], "nonzero", int((d["counts"] > 0).sum()),
              "max vertices", d["vertices"].shape[2], "grid", d["grid"])

    # ---- forward and backward single traces via compute_backtrace.
    mo = M.Model(0.0, 10.0, 0.25, 25.0, [(0.0, 0.0, 0.25, 500.0), (300.0, -200.0, 0.25, 200.0)],
                 0.0, 0.0, real["coef"][0])
    feval = lambda xy: -np.array(mo.compute_velocity_confined(xy[0], xy[1]))
    tr = []
    for (xs, ys, dur) in [(40.0, 10.0, -20.0), (-60.0, 35.0, -45.0), (20.0, -15.0, 400.0)]:
        v = C.compute_backtrace(xs, ys, dur, 1, 5, feval)
        tr.append(np.array([(float(a[0]), float(a[1])) for a in v]))
    maxv = max(len(v) for v in tr)
    TV = np.full((len(tr), maxv, 2), np.nan)
    for i, v in enumerate(tr):
        TV[i, :len(v)] = v
    np.savez_compressed(os.path.join(args.out, "backtrace_cases.npz"), vertices=TV,
                        nvertices=np.array([len(v) for v in tr]), coef=real["coef"][0],
                        starts=np.array([(40.0, 10.0, -20.0), (-60.0, 35.0, -45.0), (20.0, -15.0, 400.0)]),
                        **meta)

    # ---- fits: confined, mixed and unconfined observation sets.
    fit_rows = []
    for (wl, ob, base, K, H) in [(wells, obs, 0.0, 12.0, 25.0), (wells2, obs2, 0.0, 9.0, 30.0),
                                 (wells3, obs3, 0.0, 30.0, 20.0)]:
        wq = [(w[0], w[1], w[2], 0.5 * (w[3][0] + w[3][1])) for w in wl]
        mo = M.Model(base, K, 0.25, H, wq)
        ev, cov = mo.fit_regional_flow(ob, wq[0][0], wq[0][1])
        fit_rows.append(dict(wells=np.array(wq), obs=np.array(ob), base=base, K=K, H=H,
                             ev=np.reshape(ev, [6]), cov=cov))
    np.savez_compressed(os.path.join(args.out, "fit_cases.npz"),
                        **{f"{k}_{i}": v for i, d in enumerate(fit_rows) for k, v in d.items()},
                        ncases=len(fit_rows), **meta)
    make_fit_rows_goldens(args.out, meta, M)

    # ---- rasterize: random polylines on a fixed window (incl. zero-length and off-grid).
    rr = np.random.default_rng(7)
    polys, grids, rgrids = [], [], []
    for k in range(12):
        sp = [2.0, 5.0, 10.0, 2.5][k % 4]
        um = sp * [1.0, 2.0, 1.5][k % 3]
        pf = PF.ProbabilityField(sp, sp, 0.0, 0.0)
        pf.expand(-300.0, 300.0, -200.0, 250.0)
        n = int(rr.integers(1, 40))
        start = rr.uniform(-250, 250, size=2)
        steps = rr.normal(0, 8.0, size=(n - 1, 2))
        if k % 5 == 0 and n > 3:
            steps[1] = 0.0                      # zero-length segment
        if k % 4 == 3:
            start = np.array([290.0, -190.0])   # runs off the grid edge
        pts = np.vstack([start, start + np.cumsum(steps, axis=0)]) if n > 1 else start[None, :]
        pf.rasterize(list(pts[:, 0]), list(pts[:, 1]), um)
        polys.append(np.pad(pts, ((0, 40 - len(pts)), (0, 0)), constant_values=np.nan))
        grids.append([pf.xmin, pf.ymin, pf.deltax, pf.deltay, pf.nrows, pf.ncols, um, len(pts)])
        rgrids.append(np.packbits(pf.rgrid.reshape(-1)))
    np.savez_compressed(os.path.join(args.out, "raster_cases.npz"), polys=np.array(polys),
                        grids=np.array(grids), **{f"rgrid_{i}": g for i, g in enumerate(rgrids)},
                        **meta)

    # ---- expand geometry sequences.
    seqs = []
    for (dx, xo, yo, boxes) in [(1.0, 100.0, 50.0, [(100.0, 200.0, 50.0, 100.0), (150.0, 175.0, 75.0, 100.0)]),
                                (2.5, 0.3, -7.1, [(-40.2, 13.3, -9.0, 40.7), (-80.0, -79.0, 100.0, 101.0)]),
                                (0.7, 1234.567, 89.01, [(1200.0, 1300.0, 50.0, 60.0)])]:
        pf = PF.ProbabilityField(dx, dx, xo, yo)
        geo = []
        for b in boxes:
            pf.expand(*b)
            geo.append([pf.xmin, pf.xmax, pf.ymin, pf.ymax, pf.nrows, pf.ncols])
        seqs.append(dict(dx=dx, xo=xo, yo=yo, boxes=np.array(boxes), geo=np.array(geo)))
    np.savez_compressed(os.path.join(args.out, "expand_geometry.npz"),
                        **{f"{k}_{i}": v for i, d in enumerate(seqs) for k, v in d.items()},
                        ncases=len(seqs), **meta)
    # ---- filter_obs: buffer removals and runs of consecutive near-duplicates.
    U = import_reference_utilities()
    fr = np.random.default_rng(11)
    fcases = []
    for k in range(4):
        wl = [(float(x), float(y), 0.25, 500.0) for x, y in fr.uniform(-1000, 1000, size=(3 + k, 2))]
        ob = []
        for _ in range(30):
            x, y = fr.uniform(-1200, 1200, size=2)
            ob.append((float(x), float(y), float(fr.uniform(90, 110)), float(fr.choice([0.1, 0.5, 2.0]))))
            if fr.uniform() < 0.3:      # a near-duplicate right after it
                ob.append((float(x + fr.uniform(-0.6, 0.6)), float(y + fr.uniform(-0.6, 0.6)),
                           float(fr.uniform(90, 110)), float(fr.choice([0.1, 0.5]))))
        ob.append((wl[0][0] + 50.0, wl[0][1], 100.0, 1.0))   # inside the buffer of a well
        buf = [100.0, 60.0, 0.0, 250.0][k]
        res = U.filter_obs(ob, wl, buf)
        fcases.append(dict(wells=np.array(wl), obs=np.array(ob), buffer=buf,
                           retained=np.array([tuple(float(v) for v in r) for r in res])))
    np.savez_compressed(os.path.join(args.out, "filter_obs_cases.npz"),
                        **{f"{k}_{i}": v for i, d in enumerate(fcases) for k, v in d.items()},
                        ncases=len(fcases), **meta)
    print("done")


if __name__ == "__main__":
    main()
