"""GPU parity: the CUDA path (through the C ABI) against the reference goldens and the oracle.

Bars:
  * FP64 build: visit counts bit-exact; vertices equal to the reference's
    (bit-exact except where libm pow/log and CUDA pow/log round a step
    factor or a logarithm differently, then within 1e-9 relative).
  * FP32 build, on every trace: the endpoint within 1e-3 of the cell size of
    the FP64 build's wherever the FP64 trace is well conditioned (its
    endpoint moves less than 1e-6 cell when the release point moves 1 nm),
    and within 20 times the FP64 endpoint's own movement under a 100 nm
    release displacement everywhere; capture-probability L-inf <= 0.01.
"""
import numpy as np
import pytest
import torch

import known_answers as KA
from conftest import TRACK_CASES, golden
from gpu_helpers import golden_grid, golden_opts, golden_real, golden_site, run_golden

pytestmark = pytest.mark.gpu

from onekapy_gb300 import _capi as C  # noqa: E402
from onekapy_gb300 import engine as E  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _lib():
    C.load()
    C.device()


def _vertex_agreement(got_v, got_n, d):
    nv = d["nvertices"]
    assert np.array_equal(got_n, nv), "vertex counts differ from the reference"
    mv = d["vertices"].shape[2]
    mask = np.arange(mv)[None, None, :] < nv[:, :, None]
    g = got_v[:, :, :mv][mask]
    w = d["vertices"][mask]
    same_trace = [np.array_equal(got_v[i, j, :nv[i, j]], d["vertices"][i, j, :nv[i, j]])
                  for i in range(nv.shape[0]) for j in range(nv.shape[1])]
    return g, w, float(np.mean(same_trace))


# Fraction of traces whose every vertex is bit-identical to the reference's.
# The rest differ by ulps after a step factor pow(x, 0.2), a log or an x**2
# that glibc rounds differently from a correctly rounded result.
MIN_IDENTICAL = {"confined_u10": 0.95, "confined_u20": 0.95, "mixed_general": 0.75,
                 "unconfined_thin": 0.75, "unconfined_dryshift": 0.75}


@pytest.mark.parametrize("case", TRACK_CASES)
def test_fp64_counts_bit_exact_vs_reference(case):
    d = golden(f"track_{case}.npz")
    r = run_golden(d, C.FP64)
    assert r["registered"] == int(d["total_weight"])
    assert np.array_equal(r["counts"], d["counts"]), \
        f"{case}: {(r['counts'] != d['counts']).sum()} nodes differ"
    if case == "forward_dry":
        # forward traces run into the pumping well's singularity, where ulp
        # differences grow until the dry cell is met at a different step;
        # the dry status itself and the chronicle agree
        assert np.all(r["status"] == C.TRACE_DRY)
        return
    g, w, frac = _vertex_agreement(r["vertices"], r["nvertices"], d)
    assert np.allclose(g, w, rtol=1e-9, atol=1e-9)
    assert frac >= MIN_IDENTICAL[case], f"only {frac:.3f} of traces bit-identical"


@pytest.mark.parametrize("case,head64", [("confined_u10", False), ("mixed_general", False),
                                         ("unconfined_thin", False), ("mixed_general", True),
                                         ("unconfined_thin", True)])
def test_fp32_drift_and_probability(case, head64):
    """FP32 build against the FP64 parity build on the reference goldens; with
    head64 the general path re-inverts heads near the aquifer top in FP64."""
    d = golden(f"track_{case}.npz")
    r64 = run_golden(d, C.FP64)
    r32 = run_golden(d, C.FP32, head64=head64)
    s1 = run_golden(d, C.FP64, release_shift=[1e-9, 0.0])
    s100 = run_golden(d, C.FP64, release_shift=[1e-7, 0.0])
    ok = (r32["status"] == C.TRACE_OK) & (r64["status"] == C.TRACE_OK)
    assert np.array_equal(r32["status"], r64["status"])
    cell = float(d["spacing"])
    drift = np.linalg.norm(r32["endpoint"] - r64["endpoint"], axis=-1)[ok] / cell
    sens1 = np.linalg.norm(s1["endpoint"] - r64["endpoint"], axis=-1)[ok] / cell
    sens100 = np.linalg.norm(s100["endpoint"] - r64["endpoint"], axis=-1)[ok] / cell
    well = sens1 <= 1e-6
    assert well.mean() >= 0.95
    assert drift[well].max() <= 1e-3, drift[well].max()
    assert np.all(drift <= np.maximum(1e-3, 20.0 * sens100))
    R = int(d["total_weight"])
    linf = np.abs(r32["counts"] - r64["counts"]).max() / R
    assert linf <= 0.01 + 1.0 / R  # at most one realization flips any node at this tiny R
    mism = (r32["counts"] != r64["counts"]).sum() / max(1, (r64["counts"] > 0).sum())
    assert mism <= 0.02, mism


def test_fp64_expanding_grid_replay_matches_reference():
    """compute_capturezone-style replay of the reference's growing grid."""
    d = golden("track_expanding_u20.npz")
    dev = C.device()
    site, real = golden_site(d, dev), golden_real(d, dev)
    nreal, npaths = d["nvertices"].shape
    opts = golden_opts(d, C.FP64)
    rel = torch.as_tensor(d["release"], device=dev)
    first = E.TrackOutputs.alloc(nreal, npaths, dev, bbox=True, stats=False, endpoint=False)
    E.track(site, real, rel, opts, E.Grid(0.0, 0.0, 1.0, 1.0, 1, 1), outputs=first)
    g0 = d["grid0"]
    (xmin, ymin, nrows, ncols, _, _), frames = E.replay_expand(
        float(d["wells"][0, 0]), float(d["wells"][0, 1]), float(g0[2]), float(g0[3]),
        first.bbox.reshape(-1, 4).cpu().numpy())
    grid = E.Grid(xmin, ymin, float(g0[2]), float(g0[3]), nrows, ncols)
    assert (xmin, ymin, nrows, ncols) == (d["grid"][0], d["grid"][1], d["grid"][4], d["grid"][5])
    counts = torch.zeros((nrows, ncols), dtype=torch.int32, device=dev)
    fr = torch.frombuffer(bytearray(frames.tobytes()), dtype=torch.uint8).to(dev)
    E.track(site, real, rel, opts, grid, counts=counts, frames=fr)
    assert np.array_equal(counts.cpu().numpy(), d["counts"])


def test_wave_size_invariance():
    """Counts are integer sums: any number of realization slots per wave gives the same grid."""
    d = golden("track_confined_u10.npz")
    a = run_golden(d, C.FP64, slots=1)
    b = run_golden(d, C.FP64, slots=3)
    assert np.array_equal(a["counts"], b["counts"])
    assert np.array_equal(a["counts"], d["counts"])


def test_attempt_cap_and_skipped_realizations():
    d = golden("track_confined_u10.npz")
    dev = C.device()
    site, real = golden_site(d, dev), golden_real(d, dev)
    real.status[1] = C.REAL_NOT_SPD
    opts = golden_opts(d, C.FP64)
    opts.max_attempts = 5
    grid = golden_grid(d)
    nreal, npaths = d["nvertices"].shape
    out = E.TrackOutputs.alloc(nreal, npaths, dev)
    counts = torch.zeros((grid.nrows, grid.ncols), dtype=torch.int32, device=dev)
    reg = torch.zeros(1, dtype=torch.int64, device=dev)
    E.track(site, real, torch.as_tensor(d["release"], device=dev), opts, grid, counts=counts,
            registered=reg, outputs=out)
    st = out.status.cpu().numpy()
    assert int(reg.item()) == nreal - 1
    assert np.all(st[1] == C.TRACE_SKIPPED)
    assert np.all(st[[0, 2]] == C.TRACE_STEP_LIMIT)
    assert np.all(out.nattempt.cpu().numpy()[[0, 2]] == 5)


def test_model_known_answers_gpu():
    from onekapy_gb300.model import Model
    m = KA.MODEL
    mo = Model(m["base"], m["conductivity"], m["porosity"], m["thickness"], m["wells"], m["xo"],
               m["yo"], m["coef"])
    assert np.isclose(mo.compute_potential(*KA.POTENTIAL[0]), KA.POTENTIAL[1], rtol=KA.RTOL)
    assert np.isclose(mo.compute_head(*KA.HEAD[0]), KA.HEAD[1], rtol=KA.RTOL)
    assert np.allclose(mo.compute_discharge(*KA.DISCHARGE[0]), KA.DISCHARGE[1], rtol=KA.RTOL)
    for (pt, v) in KA.VELOCITY:
        assert np.allclose(mo.compute_velocity(*pt), v, rtol=KA.RTOL)


def test_model_evaluate_matches_oracle(oracle_mod):
    from onekapy_gb300.model import Model
    d = golden("track_mixed_general.npz")
    wells = [(w[0], w[1], w[2], q) for w, q in zip(d["wells"], d["q"][0])]
    mo = Model(0.0, d["K"][0], d["n"][0], d["H"][0], wells, 0.0, 0.0, d["coef"][0])
    pts = np.random.default_rng(3).uniform(-1500, 1500, size=(500, 2))
    got = mo.evaluate(pts)
    want = oracle_mod.evaluate(d["wells"][:, :2], d["q"][0], 0.0, d["K"][0], d["n"][0], d["H"][0],
                               0.0, 0.0, d["coef"][0], pts)
    for k in ("potential", "discharge", "head", "velocity"):
        assert np.allclose(got[k], want[k], rtol=1e-13, atol=0), k
    assert np.array_equal(got["status"], want["status"])


def test_fit_known_answer_gpu():
    from onekapy_gb300.model import Model
    m = KA.MODEL
    mo = Model(m["base"], m["conductivity"], m["porosity"], m["thickness"], m["wells"])
    ev, cov = mo.fit_regional_flow(KA.FIT_OBS, *KA.FIT_ORIGIN)
    assert np.allclose(ev.reshape(6), KA.FIT_EV, rtol=KA.FIT_RTOL)
    assert np.allclose(cov, KA.FIT_COV, rtol=KA.FIT_RTOL)


def test_fit_matches_reference_goldens():
    from onekapy_gb300.model import Model
    d = golden("fit_cases.npz")
    for i in range(int(d["ncases"])):
        w = [tuple(r) for r in d[f"wells_{i}"]]
        mo = Model(float(d[f"base_{i}"]), float(d[f"K_{i}"]), 0.25, float(d[f"H_{i}"]), w)
        ev, cov = mo.fit_regional_flow([tuple(r) for r in d[f"obs_{i}"]], w[0][0], w[0][1])
        assert np.allclose(ev.reshape(6), d[f"ev_{i}"], rtol=1e-8, atol=0), i
        assert np.allclose(cov, d[f"cov_{i}"], rtol=1e-8, atol=0), i


def test_construct_fit_and_compute_fit_match_reference():
    """Model.construct_fit runs oneka_fit_rows and Model.compute_fit runs
    oneka_fit_solve (FP64 on the device); both against the reference's own
    construct_fit / compute_fit outputs on the same inputs."""
    from onekapy_gb300.model import Model, RangeError
    d = golden("fit_rows_cases.npz")
    for i in range(int(d["ncases"])):
        w = [tuple(r) for r in golden("fit_cases.npz")[f"wells_{i}"]]
        f = golden("fit_cases.npz")
        mo = Model(float(f[f"base_{i}"]), float(f[f"K_{i}"]), 0.25, float(f[f"H_{i}"]), w)
        obs = [tuple(r) for r in f[f"obs_{i}"]]
        WA, Wb = mo.construct_fit(obs, float(d[f"xo_{i}"]), float(d[f"yo_{i}"]))
        assert isinstance(WA, np.ndarray) and WA.shape == d[f"WA_{i}"].shape and Wb.shape == d[f"Wb_{i}"].shape
        assert np.allclose(WA, d[f"WA_{i}"], rtol=1e-14, atol=0), i
        assert np.allclose(Wb, d[f"Wb_{i}"], rtol=1e-12, atol=1e-12), i
        ev, cov = Model.compute_fit(d[f"WA_{i}"], d[f"Wb_{i}"])
        assert ev.shape == (6, 1) and cov.shape == (6, 6)
        assert np.allclose(ev, d[f"ev_{i}"], rtol=1e-8, atol=0), i
        assert np.allclose(cov, d[f"cov_{i}"], rtol=1e-8, atol=0), i
    # an observed head at the base raises like the reference's construct_fit
    with pytest.raises(RangeError):
        mo.construct_fit([(10.0, 20.0, mo.base, 0.1)] + obs, 0.0, 0.0)
    # a rank-deficient problem raises LinAlgError
    with pytest.raises(np.linalg.LinAlgError):
        Model.compute_fit(np.ones((10, 6)), np.ones((10, 1)))


def test_realize_draws_match_philox_restatement(oracle_mod):
    """Integer Philox streams and uniform/triangular variates are bit-exact;
    lognormal (log/cos/exp) within 1e-14 relative."""
    dev = C.device()
    wells = [(0.0, 0.0, 0.25, (400.0, 600.0)), (500.0, 100.0, 0.25, (100.0, 200.0, 500.0)),
             (-300.0, 700.0, 0.25, 250.0)]
    obs = [(x, y, 500.0 + 0.001 * x, 0.1) for x in (-900.0, -100.0, 700.0) for y in (-800.0, 50.0, 900.0)]
    site = E.Site(wells, obs, 0.0, c_dist=E.Lognormal(np.log(10.0), 0.3), p_dist=(0.2, 0.3),
                  t_dist=(20.0, 25.0, 30.0), device=dev)
    seed, first, n = 123456789, 1000, 64
    real = E.realize(site, n, seed=seed, first=first)
    q = real.q.cpu().numpy()
    aq = real.aquifer.cpu().numpy()
    kinds = [(1, 400.0, 600.0, 0.0), (2, 100.0, 200.0, 500.0), (0, 250.0, 0.0, 0.0)]
    for r in range(n):
        for w, (k, a, b, c) in enumerate(kinds):
            u0, u1 = oracle_mod.philox_uniforms(seed, first + r, w)
            assert q[r, w] == oracle_mod.variate(k, a, b, c, u0, u1)
        u0, u1 = oracle_mod.philox_uniforms(seed, first + r, 3)
        assert np.isclose(aq[r, 0], oracle_mod.variate(3, np.log(10.0), 0.3, 0, u0, u1), rtol=1e-14)
        u0, u1 = oracle_mod.philox_uniforms(seed, first + r, 4)
        assert aq[r, 1] == oracle_mod.variate(1, 0.2, 0.3, 0, u0, u1)
        u0, u1 = oracle_mod.philox_uniforms(seed, first + r, 5)
        assert aq[r, 2] == oracle_mod.variate(2, 20.0, 25.0, 30.0, u0, u1)
    # the fit of each drawn realization equals the NumPy restatement
    ev = real.coef_ev.cpu().numpy()
    cov = real.coef_cov.cpu().numpy().reshape(n, 6, 6)
    for r in range(0, n, 7):
        wl = [(w[0], w[1], w[2], q[r, i]) for i, w in enumerate(wells)]
        e, c = oracle_mod.fit(obs, wl, 0.0, aq[r, 0], aq[r, 2], 0.0, 0.0)
        assert np.allclose(ev[r], e.reshape(6), rtol=1e-8, atol=1e-12 * np.abs(e).max())
        assert np.allclose(cov[r], c, rtol=1e-7, atol=1e-12 * np.abs(c).max())
    # shard invariance: drawing [first+10, first+20) alone gives the same realizations
    part = E.realize(site, 10, seed=seed, first=first + 10)
    assert torch.equal(part.coef, real.coef[10:20])


@pytest.mark.parametrize("kind", ["uniform", "triangular", "lognormal"])
def test_variates_match_numpy_distributions(kind):
    """The realization draws (row a1) against the reference's generators:
    10^6 Philox variates from oneka_realize, as well discharges of a
    1,000-well site over 1,000 realizations, against 10^6 draws of NumPy's
    legacy generator (np.random.uniform / np.random.triangular, the calls of
    oneka/stochastic.py:297-304, and np.random.lognormal for the lognormal
    extension).  Bars: mean within 0.2 % and variance within 1 % of NumPy's
    and of the exact values (about 7 and 3.7 standard errors at n = 10^6); Kolmogorov-Smirnov D below 2.5 sqrt(2/n) = 0.0035 between
    the two samples and below 2.5 / sqrt(n) = 0.0025 against the exact CDF
    (n = 10^6; two samples of one distribution exceed these with probability
    about 10^-5)."""
    stats = pytest.importorskip("scipy.stats")
    dev = C.device()
    nw, nr = 1000, 1000
    if kind == "uniform":
        d, ref = (400.0, 600.0), np.random.RandomState(11).uniform(400.0, 600.0, nw * nr)
        cdf = stats.uniform(400.0, 200.0).cdf
        mean, var = 500.0, 200.0 ** 2 / 12
    elif kind == "triangular":
        d, ref = (100.0, 200.0, 500.0), np.random.RandomState(12).triangular(100.0, 200.0, 500.0, nw * nr)
        cdf = stats.triang(c=0.25, loc=100.0, scale=400.0).cdf
        mean = 800.0 / 3
        var = (100.0 ** 2 + 200.0 ** 2 + 500.0 ** 2 - 100.0 * 200.0 - 100.0 * 500.0 - 200.0 * 500.0) / 18
    else:
        d, ref = E.Lognormal(np.log(10.0), 0.3), np.random.RandomState(13).lognormal(np.log(10.0), 0.3, nw * nr)
        cdf = stats.lognorm(s=0.3, scale=10.0).cdf
        mean = 10.0 * np.exp(0.045)
        var = (np.exp(0.09) - 1) * np.exp(2 * np.log(10.0) + 0.09)
    wells = [(float(i), 0.0, 0.25, d) for i in range(nw)]
    site = E.Site(wells, np.zeros((0, 4)), 0.0, device=dev)
    real = E.realize(site, nr, seed=977)
    got = real.q.cpu().numpy().reshape(-1)
    assert got.size == nw * nr and np.all(np.isfinite(got))
    for m, v in ((got.mean(), got.var()), (ref.mean(), ref.var())):
        assert abs(m - mean) <= 0.002 * mean and abs(v - var) <= 0.01 * var, (kind, m, v, mean, var)
    assert abs(got.mean() - ref.mean()) <= 0.002 * mean and abs(got.var() - ref.var()) <= 0.01 * var
    assert stats.ks_2samp(got, ref).statistic < 0.0035, kind
    assert stats.kstest(got, cdf).statistic < 0.0025, kind


def test_mvn_draw_statistics():
    """A..F draws have the fitted mean and covariance (stochastic.py:240-241)."""
    dev = C.device()
    wells = [(0.0, 0.0, 0.25, 500.0)]
    rng = np.random.default_rng(5)
    obs = [(float(x), float(y), 500.0 + 1e-3 * x - 5e-4 * y + 1e-7 * x * x, 0.1)
           for x, y in rng.uniform(-1500, 1500, size=(25, 2))]
    site = E.Site(wells, obs, 0.0, c_dist=10.0, p_dist=0.25, t_dist=25.0, device=dev)
    n = 40000
    real = E.realize(site, n, seed=7)
    coef = real.coef.cpu().numpy()
    ev = real.coef_ev.cpu().numpy()[0]
    cov = real.coef_cov.cpu().numpy()[0].reshape(6, 6)
    sd = np.sqrt(np.diag(cov))
    z = (coef.mean(0) - ev) / (sd / np.sqrt(n))
    assert np.all(np.abs(z) < 5), z
    emp = np.cov(coef.T)
    corr_emp = emp / np.outer(np.sqrt(np.diag(emp)), np.sqrt(np.diag(emp)))
    corr = cov / np.outer(sd, sd)
    assert np.allclose(np.sqrt(np.diag(emp)) / sd, 1, atol=0.03)
    assert np.allclose(corr_emp, corr, atol=0.03)


def test_rasterize_and_register_match_reference():
    from onekapy_gb300.probabilityfield import ProbabilityField
    d = golden("raster_cases.npz")
    for i, (poly, g) in enumerate(zip(d["polys"], d["grids"])):
        xmin, ymin, dx, dy, nrows, ncols, umbra, npts = g
        pf = ProbabilityField(dx, dy, 0.0, 0.0)
        pf.expand(-300.0, 300.0, -200.0, 250.0)
        pts = poly[:int(npts)]
        pf.rasterize(list(pts[:, 0]), list(pts[:, 1]), umbra)
        assert (pf.xmin, pf.ymin, pf.nrows, pf.ncols) == (xmin, ymin, int(nrows), int(ncols))
        want = np.unpackbits(d[f"rgrid_{i}"])[: int(nrows) * int(ncols)].reshape(int(nrows), int(ncols))
        assert np.array_equal(pf.rgrid, want.astype(bool)), i
        pf.register(0.5)
        assert np.array_equal(pf.pgrid, 0.5 * want)
        assert not pf.rgrid.any()


def test_distancesquared_known_answer_gpu():
    from onekapy_gb300.probabilityfield import ProbabilityField
    args, want = KA.DISTANCESQUARED
    assert np.isclose(ProbabilityField.distancesquared(*args), want, atol=1e-9)


def test_expand_known_answer_gpu():
    from onekapy_gb300.probabilityfield import ProbabilityField, RangeError
    with pytest.raises(RangeError):
        ProbabilityField(0, 0)
    pf = ProbabilityField(1, 1)
    with pytest.raises(RangeError):
        pf.expand(1, 0, 1, 0)
    pf.expand(*KA.EXPAND_REQUEST)
    r = KA.EXPAND_RESULT
    assert (pf.nrows, pf.ncols) == (r["nrows"], r["ncols"])
    assert np.isclose(pf.xmin, r["xmin"]) and np.isclose(pf.xmax, r["xmax"])
    assert np.isclose(pf.ymin, r["ymin"]) and np.isclose(pf.ymax, r["ymax"])
    pf.expand(*KA.EXPAND_SECOND)
    assert (pf.nrows, pf.ncols) == (r["nrows"], r["ncols"])


@pytest.mark.parametrize("precision", [C.FP64, C.FP32])
def test_trace_counters_match_per_particle_outputs(precision):
    """OnekaTrackOut.counters against the per-particle outputs of the same
    launch: attempts, accepted steps, DRY and STEP_LIMIT traces, and the traces
    whose bounding box reaches the grid's outer nodes (a window smaller than
    the traces, so that some are clipped)."""
    d = golden("track_unconfined_dryshift.npz")
    dev = C.device()
    site = golden_site(d, dev)
    real = golden_real(d, dev)
    g0 = golden_grid(d)
    grid = E.Grid(site.xt - 2 * g0.dx, site.yt - 2 * g0.dy, g0.dx, g0.dy, 5, 5)   # 5 x 5 nodes
    nreal, npaths = d["nvertices"].shape
    out = E.TrackOutputs.alloc(nreal, npaths, dev, bbox=True, counters=True)
    counts = torch.zeros((grid.nrows, grid.ncols), dtype=torch.int32, device=dev)
    E.track(site, real, torch.as_tensor(d["release"], device=dev), golden_opts(d, precision), grid,
            counts=counts, outputs=out)
    torch.cuda.synchronize()
    c = out.counters.cpu().numpy()
    st = out.status.cpu().numpy()
    assert c[0] == int(out.nattempt.sum().item())
    assert c[1] == int(out.naccept.sum().item())
    assert c[4] == int((st == C.TRACE_DRY).sum()) and c[4] > 0
    assert c[5] == int((st == C.TRACE_STEP_LIMIT).sum())
    bb = out.bbox.cpu().numpy().reshape(-1, 4)
    xmax = grid.xmin + (grid.ncols - 1) * grid.dx
    ymax = grid.ymin + (grid.nrows - 1) * grid.dy
    left = (bb[:, 0] <= grid.xmin) | (bb[:, 1] >= xmax) | (bb[:, 2] <= grid.ymin) | (bb[:, 3] >= ymax)
    assert c[6] == int(left.sum()) and c[6] > 0
    assert c[7] == 0
