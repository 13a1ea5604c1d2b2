"""GPU: the reference-compatible API and full-size workloads against the oracle."""
import numpy as np
import pytest
import torch

from conftest import golden

pytestmark = pytest.mark.gpu

from onekapy_gb300 import _capi as C  # noqa: E402
from onekapy_gb300 import engine as E  # noqa: E402
from onekapy_gb300 import sites as S  # noqa: E402


def _oracle_counts(oracle_mod, site, real, spec, grid, frames=None, nthreads=0):
    wells = site.wells.cpu().numpy()[:, :2]
    return oracle_mod.track(wells, real.coef.cpu().numpy(), real.q.cpu().numpy(),
                            real.aquifer.cpu().numpy(), site.release(spec.npaths),
                            (grid.xmin, grid.ymin, grid.dx, grid.dy, grid.nrows, grid.ncols),
                            duration=spec.duration, tol=spec.tol, maxstep=spec.maxstep,
                            umbra=spec.umbra, confined=spec.confined, base=spec.base,
                            xo=site.xo, yo=site.yo, frames=frames, nthreads=nthreads)


def _gpu_counts(site, real, spec, grid, precision, outputs=None, head64=False):
    dev = site.device
    counts = torch.zeros((grid.nrows, grid.ncols), dtype=torch.int32, device=dev)
    reg = torch.zeros(1, dtype=torch.int64, device=dev)
    opts = E.TrackOptions(duration=spec.duration, tol=spec.tol, maxstep=spec.maxstep, umbra=spec.umbra,
                          confined=spec.confined, precision=precision, head64=head64)
    E.track(site, real, torch.as_tensor(site.release(spec.npaths), device=dev), opts, grid,
            counts=counts, registered=reg, outputs=outputs)
    torch.cuda.synchronize()
    return counts.cpu().numpy(), int(reg.item())


def _site(spec):
    return E.Site(spec.wells, spec.observations, spec.base, target=spec.target, c_dist=spec.c_dist,
                  p_dist=spec.p_dist, t_dist=spec.t_dist, device=C.device())


def test_compute_backtrace_matches_reference():
    from onekapy_gb300.capturezone import compute_backtrace
    from onekapy_gb300.model import Model, make_feval
    d = golden("backtrace_cases.npz")
    mo = Model(0.0, 10.0, 0.25, 25.0, [(0.0, 0.0, 0.25, 500.0), (300.0, -200.0, 0.25, 200.0)],
               0.0, 0.0, d["coef"])
    feval = make_feval(mo, confined=True)
    for k, (xs, ys, dur) in enumerate(d["starts"]):
        v = np.array(compute_backtrace(xs, ys, dur, 1, 5, feval))
        n = int(d["nvertices"][k])
        assert v.shape == (n, 2)
        assert np.allclose(v, d["vertices"][k, :n], rtol=1e-12, atol=1e-9)


def test_compute_backtrace_rejects_python_feval():
    from onekapy_gb300.capturezone import compute_backtrace
    with pytest.raises(TypeError):
        compute_backtrace(0.0, 0.0, 10.0, 1, 5, lambda xy: np.zeros(2))


def test_compute_capturezone_dropin_on_growing_grid():
    """ProbabilityField starting at 3x3 around the target grows as in the reference."""
    from onekapy_gb300.capturezone import compute_capturezone
    from onekapy_gb300.model import Model, make_feval
    from onekapy_gb300.probabilityfield import ProbabilityField
    d = golden("track_expanding_u20.npz")
    xt, yt, rt = d["wells"][0]
    pf = ProbabilityField(float(d["spacing"]), float(d["spacing"]), xt, yt)
    for r in range(d["coef"].shape[0]):
        wl = [(w[0], w[1], w[2], q) for w, q in zip(d["wells"], d["q"][r])]
        mo = Model(float(d["base"]), d["K"][r], d["n"][r], d["H"][r], wl, xt, yt, d["coef"][r])
        compute_capturezone(xt, yt, rt, int(d["npaths"]), float(d["duration"]), pf, float(d["umbra"]),
                            1.0, float(d["tol"]), float(d["maxstep"]), make_feval(mo, bool(d["confined"])))
    assert (pf.xmin, pf.ymin, pf.nrows, pf.ncols) == (d["grid"][0], d["grid"][1], d["grid"][4], d["grid"][5])
    assert pf.total_weight == d["total_weight"]
    assert np.array_equal(pf.pgrid, d["counts"].astype(np.float64))


def test_config1_full_fp64_bit_exact_vs_oracle(oracle_mod):
    """Config 1 in full (100 realizations x 100 paths) on the fixed 4 km window."""
    spec = S.config1()
    site = _site(spec)
    real = E.realize(site, spec.nreal, seed=1001)
    assert int((real.status != 0).sum()) == 0
    grid = E.Grid.window(site.xt, site.yt, spec.spacing, spec.half)
    got, reg = _gpu_counts(site, real, spec, grid, C.FP64)
    want = _oracle_counts(oracle_mod, site, real, spec, grid)
    assert reg == spec.nreal == want["registered"]
    assert np.array_equal(got, want["counts"]), f"{(got != want['counts']).sum()} nodes differ"
    got32, _ = _gpu_counts(site, real, spec, grid, C.FP32)
    linf = np.abs(got32 - got).max() / spec.nreal
    assert linf <= 0.01, linf


@pytest.mark.parametrize("ncols,window_kb", [(64, 0), (65, 0), (64, -1), (65, -1)])
def test_fp32_chronicle_at_the_grid_edges(ncols, window_kb):
    """A 61 x ncols window about the target that every trace leaves on all
    sides: the FP32 chronicle marks nothing outside the grid (no bit past a
    row's last column, no word outside its realization's slot), its node sets
    differ from the FP64 build's only at umbra-boundary ties, and the
    registered counts are the masks' sums.  window_kb 0 runs the rows through
    the shared-memory window (it covers this grid), -1 straight to the slot;
    ncols 64 has no padding bits (a stray mark lands on a neighbouring row's
    node), 65 has 31 (an odd right clamp)."""
    spec = S.config2(nreal=48, npaths=512)
    site = _site(spec)
    real = E.realize(site, spec.nreal, seed=2025)
    sp = spec.spacing
    nrows = 61
    grid = E.Grid(site.xt - 30.3 * sp, site.yt - 30.6 * sp, sp, sp, nrows, ncols)
    dev = site.device
    rel = torch.as_tensor(site.release(spec.npaths), device=dev)
    words = grid.slot_bytes() // 4
    wpr = grid.words_per_row
    masks = {}
    for prec in (C.FP32, C.FP64):
        opts = E.TrackOptions(duration=spec.duration, tol=spec.tol, maxstep=spec.maxstep, umbra=spec.umbra,
                              confined=spec.confined, precision=prec, window_kb=window_kb)
        buf = torch.zeros((real.n + 2, words), dtype=torch.int32, device=dev)   # a guard slot either side
        out = E.TrackOutputs(counters=torch.zeros(E.COUNTERS, dtype=torch.int64, device=dev))
        E.track(site, real, rel, opts, grid, mark_only=buf[1:-1], outputs=out)
        b = buf.cpu().numpy().view(np.uint32)
        assert not b[0].any() and not b[-1].any(), "a mark outside the realizations' slots"
        m = b[1:-1, :nrows * wpr].reshape(real.n, nrows, wpr)
        assert not b[1:-1, nrows * wpr:words - 4].any(), "a mark in the slot's padding words"
        if ncols % 32:
            assert not (m[:, :, -1] >> (ncols % 32)).any(), "a mark past the last column"
        masks[prec] = m
        assert int(out.counters[6].item()) > 0          # traces left the grid
    bits = lambda a: np.unpackbits(a.view(np.uint8), bitorder="little").reshape(real.n, nrows, -1)[:, :, :ncols]
    v32, v64 = bits(masks[C.FP32]), bits(masks[C.FP64])
    assert v64.sum() > 0
    mismatch = (v32 != v64).sum() / v64.sum()
    assert mismatch <= 1e-4, mismatch
    # registration: the counts are the masks' sums, nothing written past the grid
    counts = torch.zeros((nrows + 1, ncols), dtype=torch.int32, device=dev)
    opts = E.TrackOptions(duration=spec.duration, tol=spec.tol, maxstep=spec.maxstep, umbra=spec.umbra,
                          confined=spec.confined, precision=C.FP32, window_kb=window_kb)
    E.track(site, real, rel, opts, grid, counts=counts[:nrows])
    c = counts.cpu().numpy()
    assert not c[nrows].any()
    assert np.array_equal(c[:nrows], v32.sum(axis=0))


@pytest.mark.parametrize("precision", [C.FP32, C.FP64])
def test_register_column_pass_equals_mask_sums(precision):
    """Launches of 4,096 slots or more register column by column (bit-sliced
    sums over slot ranges); their counts equal the per-realization masks of a
    mark-only run summed on the host, and the slots are left cleared (a
    second launch on the same scratch gives the same counts)."""
    spec = S.config2(nreal=4500, npaths=64)
    site = _site(spec)
    real = E.realize(site, spec.nreal, seed=4242)
    dev = site.device
    sp = spec.spacing
    grid = E.Grid(site.xt - 100.2 * sp, site.yt - 99.7 * sp, sp, sp, 201, 201)
    rel = torch.as_tensor(site.release(spec.npaths), device=dev)
    opts = E.TrackOptions(duration=spec.duration, tol=spec.tol, maxstep=spec.maxstep, umbra=spec.umbra,
                          confined=spec.confined, precision=precision)
    words = grid.slot_bytes() // 4
    masks = torch.zeros((real.n, words), dtype=torch.int32, device=dev)
    E.track(site, real, rel, opts, grid, mark_only=masks)
    m = masks.cpu().numpy().view(np.uint32)[:, :grid.nrows * grid.words_per_row]
    bits = np.unpackbits(m.view(np.uint8), bitorder="little").reshape(real.n, grid.nrows, -1)[:, :, :grid.ncols]
    want = bits.sum(axis=0, dtype=np.int64)
    scratch = torch.zeros(grid.slot_bytes() * real.n, dtype=torch.uint8, device=dev)
    for _ in range(2):
        counts = torch.zeros((grid.nrows, grid.ncols), dtype=torch.int32, device=dev)
        E.track(site, real, rel, opts, grid, counts=counts, scratch=scratch)
        torch.cuda.synchronize()
        assert np.array_equal(counts.cpu().numpy(), want)
    assert not scratch.any().item()


def _track(site, real, spec, grid, precision, release=None, head64=False):
    """One oneka_track call: host counts, registered count, and per-trace
    endpoint / naccept / nattempt / status."""
    dev = site.device
    rel = site.release(spec.npaths) if release is None else release
    out = E.TrackOutputs.alloc(real.n, spec.npaths, dev)
    counts = torch.zeros((grid.nrows, grid.ncols), dtype=torch.int32, device=dev)
    reg = torch.zeros(1, dtype=torch.int64, device=dev)
    opts = E.TrackOptions(duration=spec.duration, tol=spec.tol, maxstep=spec.maxstep, umbra=spec.umbra,
                          confined=spec.confined, precision=precision, head64=head64)
    E.track(site, real, torch.as_tensor(rel, device=dev), opts, grid, counts=counts, registered=reg, outputs=out)
    torch.cuda.synchronize()
    return counts.cpu().numpy(), int(reg.item()), {k: getattr(out, k).cpu().numpy()
                                                   for k in ("endpoint", "naccept", "nattempt", "status")}


# The FP32 build's endpoint bar, trace by trace.  A trace is well conditioned
# when its FP64 endpoint moves less than WELL_CONDITIONED_CELLS (cells) as its
# release point moves 1 nm (an amplification below 5,000).  Every well-
# conditioned trace must end within 1e-3 cell of the FP64 build.  The others
# pass a neighbour well's stagnation zone, where the FP64 trace itself moves
# by the FP32 build's error under a displacement of about a micrometre: each
# must end within 20 times the distance its FP64 endpoint moves when the
# release point moves 100 nm (measured on 4.1 M traces of the unconfined
# stress site: at most 14 times).
WELL_CONDITIONED_CELLS = 1e-6


def _fp32_bars(site, real, spec, grid, c64, o64, ill_fraction_max, ntrace_real=None):
    """The FP32 build against the FP64 build's counts c64 and outputs o64 on
    `real`: L-inf over all realizations, the per-trace bars on the first
    ntrace_real realizations (default all)."""
    R = real.n
    n = R if ntrace_real is None else min(R, ntrace_real)
    c32, _, o32 = _track(site, real, spec, grid, C.FP32)
    linf = np.abs(c32.astype(np.int64) - c64).max() / R
    assert linf <= 0.01, linf
    rel = site.release(spec.npaths)
    sub = real.slice(0, n)
    _, _, o1 = _track(site, sub, spec, grid, C.FP64, release=rel + np.array([1e-9, 0.0]))
    _, _, o100 = _track(site, sub, spec, grid, C.FP64, release=rel + np.array([1e-7, 0.0]))
    o32 = {k: v[:n] for k, v in o32.items()}
    o64 = {k: v[:n] for k, v in o64.items()}
    ok = (o32["status"] == C.TRACE_OK) & (o64["status"] == C.TRACE_OK)
    assert np.array_equal(o32["status"], o64["status"])
    cell = spec.spacing
    drift = np.linalg.norm(o32["endpoint"] - o64["endpoint"], axis=-1)[ok] / cell
    sens1 = np.linalg.norm(o1["endpoint"] - o64["endpoint"], axis=-1)[ok] / cell
    sens100 = np.linalg.norm(o100["endpoint"] - o64["endpoint"], axis=-1)[ok] / cell
    well = sens1 <= WELL_CONDITIONED_CELLS
    assert drift[well].max() <= 1e-3, drift[well].max()
    assert np.all(drift <= np.maximum(1e-3, 20.0 * sens100)), np.max(drift / np.maximum(sens100, 1e-30))
    assert (~well).mean() <= ill_fraction_max, (~well).mean()
    return drift, well


def test_config2_200x1000_fp64_bit_exact_fp32_every_trace(oracle_mod):
    """Config 2 site (mixed aquifer, general head path), 200 realizations x
    1,000 paths: FP64 counts, registrations and step counts equal the
    oracle's; the FP32 build within the bars on every trace, L-inf <= 0.01."""
    spec = S.config2(nreal=200, npaths=1000)
    site = _site(spec)
    real = E.realize(site, spec.nreal, seed=1002)
    grid = E.Grid.window(site.xt, site.yt, spec.spacing, spec.half)
    got, reg, o64 = _track(site, real, spec, grid, C.FP64)
    want = _oracle_counts(oracle_mod, site, real, spec, grid)
    assert reg == want["registered"] == spec.nreal
    assert np.array_equal(o64["naccept"], want["naccept"])
    assert np.array_equal(got, want["counts"]), f"{(got != want['counts']).sum()} nodes differ"
    drift, well = _fp32_bars(site, real, spec, grid, got, o64, ill_fraction_max=0.001)
    assert drift.max() <= 1e-3, drift.max()          # every trace of this site is within the bar


def test_config4_100x2048_fp64_bit_exact_fp32_every_trace(oracle_mod):
    """Config 4 (thin unconfined, 31 wells), 100 realizations x 2,048 paths:
    FP64 against the oracle, and the FP32 build (with and without the FP64
    head inversion near the aquifer top) within the bars on every trace."""
    spec = S.config4(nreal=100, npaths=2048)
    site = _site(spec)
    real = E.realize(site, spec.nreal, seed=1004)
    ok = real.status.cpu().numpy() == 0
    grid = E.Grid.window(site.xt, site.yt, spec.spacing, spec.half)
    got, reg, o64 = _track(site, real, spec, grid, C.FP64)
    want = _oracle_counts(oracle_mod, site, real, spec, grid)
    assert reg == int(ok.sum()) == want["registered"]
    assert np.array_equal(o64["naccept"], want["naccept"])
    assert np.array_equal(got, want["counts"]), f"{(got != want['counts']).sum()} nodes differ"
    _fp32_bars(site, real, spec, grid, got, o64, ill_fraction_max=0.02)
    c32h, _, _ = _track(site, real, spec, grid, C.FP32, head64=True)
    assert np.abs(c32h.astype(np.int64) - got).max() / max(reg, 1) <= 0.01


# Four of the 64 batched sites: the most wells (192) with 4,096 paths over
# 49 years, 175 wells on a 768^2 grid at 5 m, the fewest wells (2), and a
# 360-path site with 148 wells.
CONFIG3_SITES = [43, 59, 23, 14]


@pytest.mark.parametrize("k", CONFIG3_SITES)
def test_config3_sites_fp64_bit_exact_and_fp32(oracle_mod, k):
    """Config 3 sites: FP64 counts of 4 realizations equal the oracle's; the
    FP32 build against FP64 on 200 realizations: L-inf <= 0.01 and the
    per-trace bars."""
    spec = S.config3()[k]
    site = _site(spec)
    grid = E.Grid.window(site.xt, site.yt, spec.spacing, spec.half)
    small = E.realize(site, 4, seed=3000 + k)
    got, reg, o64 = _track(site, small, spec, grid, C.FP64)
    want = _oracle_counts(oracle_mod, site, small, spec, grid)
    assert reg == want["registered"]
    assert np.array_equal(o64["naccept"], want["naccept"])
    assert np.array_equal(got, want["counts"]), f"site {k}: {(got != want['counts']).sum()} nodes differ"
    real = E.realize(site, 200, seed=3000 + k)
    c64, _, o64 = _track(site, real, spec, grid, C.FP64)
    _fp32_bars(site, real, spec, grid, c64, o64, ill_fraction_max=0.02, ntrace_real=40)


def test_create_stochastic_capturezone_dropin(oracle_mod):
    """The reference-signature driver: GPU draws, auto-expanding grid replay, oracle check."""
    from onekapy_gb300.stochastic import create_stochastic_capturezone
    spec = S.config1()
    pf = create_stochastic_capturezone(0, 24, spec.duration, 6, spec.base, spec.c_dist, spec.p_dist,
                                       spec.t_dist, spec.wells, spec.observations, spec.spacing,
                                       2 * spec.spacing, True, spec.tol, spec.maxstep, seed=11)
    real = pf.realizations
    site = _site(spec)
    assert pf.total_weight == 6.0
    # the oracle replays the same expand sequence from the bounding boxes it computes itself
    first = oracle_mod.track(site.wells.cpu().numpy()[:, :2], real.coef.cpu().numpy(),
                             real.q.cpu().numpy(), real.aquifer.cpu().numpy(), site.release(24),
                             (site.xt - 10, site.yt - 10, 10.0, 10.0, 3, 3), duration=spec.duration,
                             tol=1, maxstep=10, umbra=20, confined=True, want_counts=False,
                             xo=site.xo, yo=site.yo)
    (xmin, ymin, nrows, ncols, _, _), frames = oracle_mod.replay_expand(
        site.xt, site.yt, 10.0, 10.0, first["bbox"].reshape(-1, 4))
    assert (pf.xmin, pf.ymin, pf.nrows, pf.ncols) == (xmin, ymin, nrows, ncols)
    want = oracle_mod.track(site.wells.cpu().numpy()[:, :2], real.coef.cpu().numpy(),
                            real.q.cpu().numpy(), real.aquifer.cpu().numpy(), site.release(24),
                            (xmin, ymin, 10.0, 10.0, nrows, ncols), duration=spec.duration, tol=1,
                            maxstep=10, umbra=20, confined=True, frames=frames, xo=site.xo, yo=site.yo)
    assert np.array_equal(pf.pgrid, want["counts"].astype(np.float64))


def test_returned_field_runs_the_reference_callers_unchanged(oracle_mod):
    """create_stochastic_capturezone returns a field on which the reference's
    own caller code runs as written: Z = pf.pgrid/pf.total_weight
    (oneka/visualize.py:230), the impact curve's sort (visualize.py:382-384)
    and the decile loop (oneka/oneka.py:278-288); each gives the values that
    the oracle's counts give."""
    from onekapy_gb300.stochastic import create_stochastic_capturezone
    spec = S.config1()
    pf = create_stochastic_capturezone(0, 32, spec.duration, 10, spec.base, spec.c_dist, spec.p_dist,
                                       spec.t_dist, spec.wells, spec.observations, spec.spacing, spec.umbra,
                                       True, spec.tol, spec.maxstep, seed=21, window=spec.half)
    site = _site(spec)
    spec32 = S.config1()
    spec32.npaths = 32
    grid = E.Grid(pf.xmin, pf.ymin, pf.deltax, pf.deltay, pf.nrows, pf.ncols)
    want = _oracle_counts(oracle_mod, site, pf.realizations, spec32, grid)["counts"].astype(np.float64)
    assert isinstance(pf.pgrid, np.ndarray) and pf.pgrid.dtype == np.float64
    assert isinstance(pf.rgrid, np.ndarray) and pf.rgrid.dtype == bool
    spacing = spec.spacing
    # oneka/visualize.py:230
    Z = pf.pgrid/pf.total_weight
    assert np.array_equal(Z, want / 10.0)
    # oneka/visualize.py:382-384
    pr = np.flip(np.sort(pf.pgrid/pf.total_weight, axis=None))
    n = pr.shape[0]
    area = (np.arange(n)+1)*spacing**2
    pr_want = np.flip(np.sort(want / 10.0, axis=None))
    assert np.array_equal(pr, pr_want)
    # oneka/oneka.py:278-288
    rows, rows_want = [], []
    for p in np.linspace(0.05, 0.95, 19):
        i = np.argmax(pr <= p)
        rows.append('{0:8.3f} {1:16,.0f} {2:16,.2f}'.format(pr[i], area[i], area[i] / 4046.86))
        j = np.argmax(pr_want <= p)
        rows_want.append('{0:8.3f} {1:16,.0f} {2:16,.2f}'.format(pr_want[j], area[j], area[j] / 4046.86))
    assert rows == rows_want
    from onekapy_gb300.outputs import decile_table, impact_curve
    pr2, area2 = impact_curve(spacing, pf)
    assert np.array_equal(pr2, pr) and np.array_equal(area2, area)
    assert [r[1] for r in decile_table(pr2, area2)] == [float(pr[np.argmax(pr <= p)])
                                                       for p in np.linspace(0.05, 0.95, 19)]


def test_deterministic_capturezone_runs():
    from onekapy_gb300.deterministic import create_deterministic_capturezone
    spec = S.config1()
    pf = create_deterministic_capturezone(0, 16, spec.duration, spec.base, spec.c_dist, spec.p_dist,
                                          spec.t_dist, spec.wells, spec.observations, spec.spacing,
                                          spec.umbra, True, spec.tol, spec.maxstep, window=spec.half)
    assert pf.total_weight == 1.0
    p = pf.probability()
    assert float(p.max()) == 1.0 and float(p.min()) == 0.0


def test_checkpoint_resume_equals_uninterrupted_run(tmp_path):
    """A fixed-window run stopped after one chunk and resumed from its
    checkpoint gives the counts of the uninterrupted run."""
    from onekapy_gb300.stochastic import create_stochastic_capturezone
    spec = S.config1()
    args = (0, 48, spec.duration, 12, spec.base, spec.c_dist, spec.p_dist, spec.t_dist, spec.wells,
            spec.observations, spec.spacing, spec.umbra, True, spec.tol, spec.maxstep)
    kw = dict(seed=5, precision=C.FP32, window=600.0, chunk=5)
    full = create_stochastic_capturezone(*args, **kw)
    assert full.complete and full.total_weight == 12.0
    path = str(tmp_path / "run.npz")
    part = create_stochastic_capturezone(*args, **kw, checkpoint=path, max_chunks=1)
    assert not part.complete and part.total_weight == 5.0
    rest = create_stochastic_capturezone(*args, **kw, checkpoint=path)
    assert rest.complete and rest.total_weight == 12.0
    assert torch.equal(rest.counts, full.counts)
    assert rest.trace_counters == full.trace_counters        # the counters resume too
    done = create_stochastic_capturezone(*args, **kw, checkpoint=path)     # nothing left to do
    assert done.complete and torch.equal(done.counts, full.counts)
    with pytest.raises(ValueError, match="different inputs"):
        create_stochastic_capturezone(*args, **{**kw, "seed": 6}, checkpoint=path)
    assert full.traces_leaving_grid >= 0 and full.trace_counters["accepted_steps"] > 0


def test_drivers_write_the_reference_log_lines(caplog):
    """With the "Oneka" logger at INFO, the stochastic driver writes the
    reference's three lines per realization and the deterministic driver its
    parameter block; the logged values are the realizations' own."""
    import logging
    from onekapy_gb300.deterministic import create_deterministic_capturezone
    from onekapy_gb300.stochastic import create_stochastic_capturezone
    spec = S.config1()
    args = (spec.base, spec.c_dist, spec.p_dist, spec.t_dist, spec.wells, spec.observations, spec.spacing,
            spec.umbra, True, spec.tol, spec.maxstep)
    with caplog.at_level(logging.INFO, logger="Oneka"):
        pf = create_stochastic_capturezone(0, 16, spec.duration, 3, *args, seed=3, window=300.0)
    lines = [r.getMessage() for r in caplog.records if r.name == "Oneka"]
    assert len(lines) == 9 and lines[0].startswith("Realization #0: ")
    c = pf.realizations.coef.cpu().numpy()[2]
    assert lines[8] == "    coef rng: (" + ", ".join(f"{v:+.4e}" for v in c) + ")"
    caplog.clear()
    with caplog.at_level(logging.INFO, logger="Oneka"):
        pf = create_deterministic_capturezone(0, 16, spec.duration, *args)
    lines = [r.getMessage() for r in caplog.records if r.name == "Oneka"]
    assert "Deterministic Capture Zone Parameters: " in lines
    assert lines[-1] == f"F = {pf.realizations.coef.cpu().numpy()[0][5]:+.4e}"
    assert not any(l.startswith("Realization #") for l in lines)
