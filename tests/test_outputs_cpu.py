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
