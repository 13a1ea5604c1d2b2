"""GPU: the reference's own site files (data/*.py) through its top-level
sequence (filter_obs, then the deterministic driver), against the fixtures
of tests/golden/site_<name>.npz."""
import glob
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from onekapy_gb300 import _capi as C  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
SITES = sorted(os.path.basename(p)[5:-4] for p in glob.glob(os.path.join(HERE, "golden", "site_*.npz")))


def _load(name):
    return np.load(os.path.join(HERE, "golden", f"site_{name}.npz"))


def _dist(row):
    kind, a, b, c = (float(v) for v in row)
    return a if kind == 0 else ((a, b) if kind == 2 else (a, b, c))


@pytest.mark.parametrize("name", SITES)
def test_site_capturezone_bit_exact_with_reference_coefficients(name):
    """compute_capturezone with the reference's own fitted coefficients and
    mean parameters reproduces its auto-expanded grid and counts exactly."""
    from onekapy_gb300.capturezone import compute_capturezone
    from onekapy_gb300.model import Model, make_feval
    from onekapy_gb300.probabilityfield import ProbabilityField
    d = _load(name)
    xt, yt, rt = float(d["xt"]), float(d["yt"]), float(d["rt"])
    pf = ProbabilityField(float(d["spacing"]), float(d["spacing"]), xt, yt)
    wells = [tuple(float(v) for v in w) for w in d["wells"]]
    mo = Model(float(d["base"]), float(d["K"]), float(d["n"]), float(d["H"]), wells, xt, yt, d["coef_ev"])
    compute_capturezone(xt, yt, rt, int(d["npaths"]), float(d["duration"]), pf, float(d["umbra"]), 1.0,
                        float(d["tol"]), float(d["maxstep"]), make_feval(mo, bool(d["confined"])))
    assert (pf.xmin, pf.ymin, pf.nrows, pf.ncols) == (float(d["xmin"]), float(d["ymin"]), int(d["nrows"]),
                                                      int(d["ncols"]))
    got = pf.pgrid
    want = d["pgrid"]
    assert np.array_equal(got, want), f"{int((got != want).sum())} of {want.size} nodes differ"


@pytest.mark.parametrize("name", SITES)
def test_site_deterministic_dropin(name):
    """The drop-in sequence (filter_obs, then the deterministic driver: GPU
    means, GPU fit, GPU tracking) on the reference's site file: the same
    observations survive the filter, the fit agrees with the reference's
    lstsq/inv, and the capture zone with its counts."""
    from onekapy_gb300.deterministic import create_deterministic_capturezone
    from onekapy_gb300.utilities import filter_obs
    d = _load(name)
    wells = [(float(w[0]), float(w[1]), float(w[2]), _dist(q)) for w, q in zip(d["wells"], d["qdist"])]
    raw = [tuple(float(v) for v in o) for o in d["obs_raw"]]
    obs = filter_obs(raw, wells, float(d["buffer"]))
    assert np.array_equal(np.array(obs, dtype=np.float64).reshape(-1, 4), d["obs"])
    pf = create_deterministic_capturezone(int(d["target"]), int(d["npaths"]), float(d["duration"]),
                                          float(d["base"]), _dist(d["c_dist"]), _dist(d["p_dist"]),
                                          _dist(d["t_dist"]), wells, obs, float(d["spacing"]),
                                          float(d["umbra"]), bool(d["confined"]), float(d["tol"]),
                                          float(d["maxstep"]))
    real = pf.realizations
    ev = real.coef.cpu().numpy()[0]
    assert np.allclose(ev, d["coef_ev"], rtol=1e-8, atol=1e-12 * np.abs(d["coef_ev"]).max())
    assert pf.total_weight == float(d["total_weight"])
    got = pf.pgrid
    want = d["pgrid"]
    if got.shape == want.shape and (pf.xmin, pf.ymin) == (float(d["xmin"]), float(d["ymin"])):
        differ = int((got != want).sum())
    else:
        differ = -1
    print(f"site {name}: coef_ev max rel diff {np.max(np.abs(ev - d['coef_ev']) / np.abs(d['coef_ev'])):.2e}, "
          f"{differ} of {int((want > 0).sum())} visited nodes differ")
    # the fit differs from lstsq in the last bits, so a node lying on the
    # umbra boundary may flip; the grid and nearly every node agree
    assert differ >= 0 and differ <= max(2, 0.001 * int((want > 0).sum())), differ


def test_unfiltered_site_with_observation_on_a_well_raises():
    """long_prairie without filter_obs has an observation on a well: the fit
    takes log 0 and is not finite.  The reference's backtrace would then run
    forever on NaN velocities; here the realization is flagged and the driver
    raises at once."""
    from onekapy_gb300 import engine as E
    from onekapy_gb300.deterministic import create_deterministic_capturezone
    d = _load("long_prairie")
    wells = [(float(w[0]), float(w[1]), float(w[2]), _dist(q)) for w, q in zip(d["wells"], d["qdist"])]
    raw = [tuple(float(v) for v in o) for o in d["obs_raw"]]
    assert any((o[0], o[1]) == (w[0], w[1]) for o in raw for w in wells)
    with pytest.raises(np.linalg.LinAlgError, match="not finite"):
        create_deterministic_capturezone(int(d["target"]), int(d["npaths"]), float(d["duration"]),
                                         float(d["base"]), _dist(d["c_dist"]), _dist(d["p_dist"]),
                                         _dist(d["t_dist"]), wells, raw, float(d["spacing"]),
                                         float(d["umbra"]), bool(d["confined"]), float(d["tol"]),
                                         float(d["maxstep"]))
    site = E.Site(wells, raw, float(d["base"]), c_dist=_dist(d["c_dist"]), p_dist=_dist(d["p_dist"]),
                  t_dist=_dist(d["t_dist"]), device=C.device())
    real = E.realize(site, 4, seed=1)
    assert (real.status.cpu().numpy() == C.REAL_NOT_FINITE).all()


@pytest.mark.parametrize("name", SITES)
def test_site_capturezone_fp32_close_to_reference(name):
    """The FP32 build on the reference's sites (its coefficients, the
    reference's auto-expanded grid): nearly every node agrees with the
    reference's counts; a node on the umbra boundary may flip."""
    from onekapy_gb300.capturezone import compute_capturezone
    from onekapy_gb300.model import Model, make_feval
    from onekapy_gb300.probabilityfield import ProbabilityField
    d = _load(name)
    xt, yt, rt = float(d["xt"]), float(d["yt"]), float(d["rt"])
    pf = ProbabilityField(float(d["spacing"]), float(d["spacing"]), xt, yt)
    wells = [tuple(float(v) for v in w) for w in d["wells"]]
    mo = Model(float(d["base"]), float(d["K"]), float(d["n"]), float(d["H"]), wells, xt, yt, d["coef_ev"])
    compute_capturezone(xt, yt, rt, int(d["npaths"]), float(d["duration"]), pf, float(d["umbra"]), 1.0,
                        float(d["tol"]), float(d["maxstep"]), make_feval(mo, bool(d["confined"])),
                        precision=C.FP32)
    want = d["pgrid"]
    got = pf.pgrid
    assert got.shape == want.shape
    differ = int((got != want).sum())
    visited = int((want > 0).sum())
    print(f"site {name} FP32: {differ} of {visited} visited nodes differ")
    assert differ <= max(2, 0.001 * visited), differ
