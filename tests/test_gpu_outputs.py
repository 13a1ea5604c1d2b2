"""GPU: probability outputs (smoothing, impact curve) and archives of a real field."""
import os
import tempfile

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

from onekapy_gb300 import _capi as C  # noqa: E402
from onekapy_gb300 import sites as S  # noqa: E402


@pytest.fixture(scope="module")
def pfield():
    from onekapy_gb300.stochastic import create_stochastic_capturezone
    spec = S.config1()
    return create_stochastic_capturezone(0, 48, spec.duration, 40, spec.base, spec.c_dist, spec.p_dist,
                                         spec.t_dist, spec.wells, spec.observations, spec.spacing,
                                         spec.umbra, True, spec.tol, spec.maxstep, seed=5, window=spec.half,
                                         precision=C.FP32)


def test_smoothing_matches_scipy(pfield):
    scipy_ndimage = pytest.importorskip("scipy.ndimage")
    from onekapy_gb300.outputs import probability, smoothed_probability
    Z = pfield.pgrid / pfield.total_weight
    for smooth in (1.0, 4.0, 2.5):
        got = smoothed_probability(pfield, smooth).cpu().numpy()
        want = scipy_ndimage.gaussian_filter(Z, smooth, mode="constant", cval=0.0)
        assert np.allclose(got, want, rtol=1e-12, atol=1e-15), smooth
    assert np.array_equal(smoothed_probability(pfield, 0).cpu().numpy(), Z)


def test_impact_curve_matches_sorted_probabilities(pfield):
    from onekapy_gb300.outputs import decile_table, impact_curve
    pr, area = impact_curve(10.0, pfield)
    Z = pfield.pgrid / pfield.total_weight
    want = np.flip(np.sort(Z, axis=None))          # oneka/visualize.py:382
    from onekapy_gb300.outputs import probability
    assert np.array_equal(probability(pfield).cpu().numpy(), Z)
    assert np.array_equal(pr, want)
    assert np.array_equal(area, (np.arange(Z.size) + 1) * 10.0 ** 2)
    rows = decile_table(pr, area)
    assert rows[0][1] <= 0.05 + 1e-12 or rows[0][1] == pr[np.argmax(pr <= 0.05)]


def test_archive_of_a_gpu_field_round_trips(pfield):
    from onekapy_gb300 import archive
    with tempfile.TemporaryDirectory() as td:
        fn = archive.dump_oneka("c1", 0.0, 0, 48, 3652.5, 40, 0.0, 1, 2, 3, [], [], 100, 10, 10, 0, True, 1,
                                10, pfield, filename=os.path.join(td, "x.bz2"))
        d = archive.load_oneka(fn)
    pf2 = d["pfield"]
    assert (pf2.nrows, pf2.ncols, pf2.xmin, pf2.total_weight) == (pfield.nrows, pfield.ncols, pfield.xmin,
                                                                  pfield.total_weight)
    assert np.array_equal(pf2.pgrid, pfield.pgrid) and isinstance(pf2.pgrid, np.ndarray)
