"""Pin the CPU oracle against the reference: its own known answers and the
golden fixtures made by running it (tests/golden/make_golden.py)."""
import platform

import numpy as np
import pytest

import known_answers as KA
from conftest import TRACK_CASES, golden


def _grid(d, key="grid"):
    g = d[key]
    return (float(g[0]), float(g[1]), float(g[2]), float(g[3]), int(g[4]), int(g[5]))


def _aquifer(d):
    return np.stack([d["K"], d["n"], d["H"]], axis=1)


def test_known_answers_model(oracle_mod):
    m = KA.MODEL
    wells = np.array([w[:2] for w in m["wells"]])
    q = np.array([w[3] for w in m["wells"]])
    pts = [KA.POTENTIAL[0], KA.DISCHARGE[0], KA.VELOCITY[0][0], KA.VELOCITY[1][0]]
    r = oracle_mod.evaluate(wells, q, m["base"], m["conductivity"], m["porosity"], m["thickness"],
                            m["xo"], m["yo"], m["coef"], pts, confined=False)
    assert np.isclose(r["potential"][0], KA.POTENTIAL[1], rtol=KA.RTOL)
    assert np.isclose(r["head"][0], KA.HEAD[1], rtol=KA.RTOL)
    assert np.allclose(r["discharge"][1], KA.DISCHARGE[1], rtol=KA.RTOL)
    assert np.allclose(r["velocity"][2], KA.VELOCITY[0][1], rtol=KA.RTOL)
    assert np.allclose(r["velocity"][3], KA.VELOCITY[1][1], rtol=KA.RTOL)


def test_known_answer_fit(oracle_mod):
    m = KA.MODEL
    ev, cov = oracle_mod.fit(KA.FIT_OBS, m["wells"], m["base"], m["conductivity"], m["thickness"],
                             *KA.FIT_ORIGIN)
    assert np.allclose(ev.reshape(6), KA.FIT_EV, rtol=KA.FIT_RTOL)
    assert np.allclose(cov, KA.FIT_COV, rtol=KA.FIT_RTOL)


def test_known_answer_distancesquared(oracle_mod):
    args, want = KA.DISTANCESQUARED
    assert np.isclose(oracle_mod.distancesquared(*args), want, atol=1e-9)


def test_known_answer_expand(oracle_mod):
    # ProbabilityField(1, 1) starts empty in the reference; its first expand
    # places (xmin, ymin) one node in from the corner (probabilityfield.py:205-213).
    x0, x1, y0, y1 = KA.EXPAND_REQUEST
    xmin, ymin = x0 - 1.0, y0 - 1.0
    import math
    ncols = max(3, math.ceil((x1 - xmin) / 1.0) + 2)
    nrows = max(3, math.ceil((y1 - ymin) / 1.0) + 2)
    assert (nrows, ncols) == (KA.EXPAND_RESULT["nrows"], KA.EXPAND_RESULT["ncols"])
    assert xmin + (ncols - 1) == KA.EXPAND_RESULT["xmax"]


@pytest.mark.parametrize("case", TRACK_CASES)
def test_oracle_track_matches_reference(oracle_mod, case):
    d = golden(f"track_{case}.npz")
    maxv = d["vertices"].shape[2]
    r = oracle_mod.track(d["wells"][:, :2], d["coef"], d["q"], _aquifer(d), d["release"], _grid(d),
                         duration=float(d["duration"]), tol=float(d["tol"]),
                         maxstep=float(d["maxstep"]), umbra=float(d["umbra"]),
                         confined=bool(d["confined"]), base=float(d["base"]),
                         xo=float(d["wells"][0, 0]), yo=float(d["wells"][0, 1]),
                         want_vertices=True, max_vertices=maxv)
    assert r["registered"] == int(d["total_weight"])
    assert np.array_equal(r["counts"], d["counts"]), "visit counts differ from the reference"
    assert np.array_equal(r["nvertices"], d["nvertices"])
    nv = d["nvertices"]
    mask = np.arange(maxv)[None, None, :] < nv[:, :, None]
    got = r["vertices"][mask]
    want = d["vertices"][mask]
    if platform.machine() == str(d["machine"]):
        assert np.array_equal(got, want), "vertices not bit-identical on the fixture's machine"
    else:
        assert np.allclose(got, want, rtol=1e-12, atol=1e-9)


def test_oracle_expanding_grid_replay(oracle_mod):
    """The frame replay reproduces the reference's auto-expanding grid."""
    d = golden("track_expanding_u20.npz")
    g0 = d["grid0"]
    common = dict(duration=float(d["duration"]), tol=float(d["tol"]), maxstep=float(d["maxstep"]),
                  umbra=float(d["umbra"]), confined=bool(d["confined"]), base=float(d["base"]),
                  xo=float(d["wells"][0, 0]), yo=float(d["wells"][0, 1]))
    first = oracle_mod.track(d["wells"][:, :2], d["coef"], d["q"], _aquifer(d), d["release"],
                             (g0[0], g0[1], g0[2], g0[3], int(g0[4]), int(g0[5])),
                             want_counts=False, **common)
    bb = first["bbox"].reshape(-1, 4)
    (xmin, ymin, nrows, ncols, xmax, ymax), frames = oracle_mod.replay_expand(
        float(d["wells"][0, 0]), float(d["wells"][0, 1]), float(g0[2]), float(g0[3]), bb)
    assert (xmin, ymin, nrows, ncols) == (d["grid"][0], d["grid"][1], d["grid"][4], d["grid"][5])
    r = oracle_mod.track(d["wells"][:, :2], d["coef"], d["q"], _aquifer(d), d["release"],
                         (xmin, ymin, g0[2], g0[3], nrows, ncols), frames=frames, **common)
    assert np.array_equal(r["counts"], d["counts"])
    # Without the replay (one fixed frame) the counts differ at the edges: the
    # reference clipped early traces to its smaller grid.
    r2 = oracle_mod.track(d["wells"][:, :2], d["coef"], d["q"], _aquifer(d), d["release"],
                          (xmin, ymin, g0[2], g0[3], nrows, ncols), **common)
    assert r2["counts"].sum() >= r["counts"].sum()


def test_oracle_rasterize_matches_reference(oracle_mod):
    d = golden("raster_cases.npz")
    for i, (poly, g) in enumerate(zip(d["polys"], d["grids"])):
        xmin, ymin, dx, dy, nrows, ncols, umbra, npts = g
        pts = poly[:int(npts)]
        got = oracle_mod.rasterize((xmin, ymin, dx, dy, int(nrows), int(ncols)), pts, umbra)
        want = np.unpackbits(d[f"rgrid_{i}"])[: int(nrows) * int(ncols)].reshape(int(nrows), int(ncols))
        assert np.array_equal(got, want), f"raster case {i}"


def test_oracle_expand_geometry(oracle_mod):
    d = golden("expand_geometry.npz")
    for i in range(int(d["ncases"])):
        dx, xo, yo = float(d[f"dx_{i}"]), float(d[f"xo_{i}"]), float(d[f"yo_{i}"])
        boxes = d[f"boxes_{i}"]
        for k in range(len(boxes)):
            (xmin, ymin, nrows, ncols, xmax, ymax), _ = oracle_mod.replay_expand(xo, yo, dx, dx, boxes[:k + 1])
            want = d[f"geo_{i}"][k]
            assert (xmin, xmax, ymin, ymax, nrows, ncols) == tuple(want[:4]) + (int(want[4]), int(want[5]))


def test_oracle_fit_matches_reference(oracle_mod):
    d = golden("fit_cases.npz")
    for i in range(int(d["ncases"])):
        w = [tuple(r) for r in d[f"wells_{i}"]]
        ob = [tuple(r) for r in d[f"obs_{i}"]]
        ev, cov = oracle_mod.fit(ob, w, float(d[f"base_{i}"]), float(d[f"K_{i}"]), float(d[f"H_{i}"]),
                                 w[0][0], w[0][1])
        assert np.allclose(ev.reshape(6), d[f"ev_{i}"], rtol=1e-12, atol=0)
        assert np.allclose(cov, d[f"cov_{i}"], rtol=1e-12, atol=0)


def test_oracle_attempt_cap(oracle_mod):
    """A capped particle reports STEP_LIMIT instead of spinning (the reference has no cap)."""
    d = golden("track_confined_u10.npz")
    r = oracle_mod.track(d["wells"][:, :2], d["coef"][:1], d["q"][:1], _aquifer(d)[:1],
                         d["release"][:4], _grid(d), duration=float(d["duration"]),
                         tol=1.0, maxstep=10.0, umbra=10.0, confined=True,
                         xo=0.0, yo=0.0, max_attempts=5)
    assert np.all(r["status"] == oracle_mod.ORC_STEP_LIMIT)
    assert np.all(r["nattempt"] == 5)
