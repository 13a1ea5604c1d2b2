"""Host-side next-row pieces: filter_obs against the reference's own output,
the archive format, and the decile table logic."""
import os
import tempfile

import numpy as np

from conftest import golden


def test_filter_obs_matches_reference():
    from onekapy_gb300.utilities import filter_obs
    d = golden("filter_obs_cases.npz")
    for i in range(int(d["ncases"])):
        obs = [tuple(float(v) for v in r) for r in d[f"obs_{i}"]]
        wells = [tuple(float(v) for v in r) for r in d[f"wells_{i}"]]
        got = np.array([tuple(float(v) for v in r) for r in filter_obs(obs, wells, float(d[f"buffer_{i}"]))])
        want = d[f"retained_{i}"]
        assert got.shape == want.shape, i
        assert np.array_equal(got, want), i


def test_archive_round_trip_with_reference_keys():
    from onekapy_gb300 import archive
    with tempfile.TemporaryDirectory() as td:
        fn = archive.dump_oneka("p", 1.5, 0, 100, 3652.5, 10, 0.0, (1, 2), 0.2, 25.0,
                                [(0.0, 0.0, 0.25, 500.0)], [(1.0, 2.0, 30.0, 0.1)], 100, 10, 20, 4,
                                True, 1, 10, {"stand-in": "pfield"}, directory=td)
        assert os.path.basename(fn).startswith("Oneka") and fn.endswith(".bz2")
        d = archive.load_oneka(fn)
    assert tuple(d.keys()) == archive.KEYS
    assert d["c_dist"] == (1, 2) and d["pfield"] == {"stand-in": "pfield"}


def test_archive_written_by_the_reference_loads():
    """tests/golden/archive_reference.bz2 was written by the reference's own
    dump_oneka (oneka/archive.py:46-82); load_oneka returns this package's
    ProbabilityField with the reference's attributes and arrays."""
    from onekapy_gb300 import archive
    from onekapy_gb300.probabilityfield import ProbabilityField
    d = archive.load_oneka(os.path.join(os.path.dirname(__file__), "golden", "archive_reference.bz2"))
    assert tuple(d.keys()) == archive.KEYS
    assert d["projectname"] == "archive-golden" and d["t_dist"] == (20.0, 25.0, 30.0)
    want = golden("archive_reference.npz")
    pf = d["pfield"]
    assert isinstance(pf, ProbabilityField)
    g = want["geometry"]
    assert (pf.deltax, pf.deltay, pf.nrows, pf.ncols, pf.xmin, pf.xmax, pf.ymin, pf.ymax,
            pf.total_weight) == tuple(g[:2]) + (int(g[2]), int(g[3])) + tuple(g[4:])
    assert isinstance(pf.pgrid, np.ndarray) and pf.pgrid.dtype == np.float64
    assert np.array_equal(pf.pgrid, want["pgrid"])
    assert np.array_equal(pf.rgrid, want["rgrid"]) and pf.rgrid.any()


def test_archive_pickles_the_reference_class(monkeypatch):
    """dump_oneka writes pfield as oneka.probabilityfield.ProbabilityField, so
    the reference's load_oneka (a plain pickle.load) rebuilds its own class:
    here a stand-in module with a plain class, as the reference defines it
    (no __setstate__), plays the reference."""
    import bz2
    import pickle
    import sys
    import types
    from onekapy_gb300 import archive
    from onekapy_gb300.probabilityfield import ProbabilityField
    want = golden("archive_reference.npz")
    g = want["geometry"]
    ours = ProbabilityField.__new__(ProbabilityField)
    ours.__setstate__(dict(deltax=g[0], deltay=g[1], nrows=int(g[2]), ncols=int(g[3]), xmin=g[4], xmax=g[5],
                           ymin=g[6], ymax=g[7], total_weight=g[8], pgrid=want["pgrid"], rgrid=want["rgrid"]))
    with tempfile.TemporaryDirectory() as td:
        fn = archive.dump_oneka("p", 1.5, 0, 100, 3652.5, 10, 0.0, (1, 2), 0.2, 25.0, [], [], 100, 10, 20, 4,
                                True, 1, 10, ours, filename=os.path.join(td, "a.bz2"))
        raw = bz2.BZ2File(fn).read()
        assert b"oneka.probabilityfield" in raw and b"onekapy_gb300" not in raw and b"torch" not in raw
        assert "oneka" not in sys.modules          # the stand-in lived only while the file was written

        class RefPF:                                # the reference's class: plain attributes
            pass
        RefPF.__module__, RefPF.__qualname__, RefPF.__name__ = "oneka.probabilityfield", "ProbabilityField", \
            "ProbabilityField"
        pkg, mod = types.ModuleType("oneka"), types.ModuleType("oneka.probabilityfield")
        pkg.__path__ = []
        mod.ProbabilityField = RefPF
        pkg.probabilityfield = mod
        monkeypatch.setitem(sys.modules, "oneka", pkg)
        monkeypatch.setitem(sys.modules, "oneka.probabilityfield", mod)
        with bz2.BZ2File(fn, "r") as fp:           # oneka/archive.py:85-89
            d = pickle.load(fp)
    pf = d["pfield"]
    assert type(pf) is RefPF
    assert (pf.nrows, pf.ncols, pf.xmin, pf.total_weight) == (int(g[2]), int(g[3]), g[4], g[8])
    assert pf.pgrid.dtype == np.float64 and np.array_equal(pf.pgrid, want["pgrid"])
    assert pf.rgrid.dtype == bool and np.array_equal(pf.rgrid, want["rgrid"])


def test_decile_table_logic():
    from onekapy_gb300.outputs import decile_table
    pr = np.flip(np.sort(np.array([0.0, 0.0, 0.1, 0.5, 0.5, 1.0, 0.96])))
    area = (np.arange(pr.size) + 1) * 100.0
    rows = decile_table(pr, area)
    assert len(rows) == 19
    for p, v, a, acres in rows:
        i = int(np.argmax(pr <= p))
        assert v == pr[i] and a == area[i] and np.isclose(acres, area[i] / 4046.86)


def test_summary_statistics_matches_reference_text():
    """utilities.summary_statistics reproduces the reference's table text on
    the retained observations of its site files and on a table with NaNs."""
    from onekapy_gb300.utilities import summary_statistics
    d = golden("summary_statistics.npz")
    for i in range(int(d["ncases"])):
        vals = [tuple(r) for r in d[f"values_{i}"]]
        got = summary_statistics(vals, list(d[f"names_{i}"]), list(d[f"formats_{i}"]),
                                 str(d[f"title_{i}"])).getvalue()
        assert got == str(d[f"text_{i}"]), i
