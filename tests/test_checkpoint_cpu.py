"""Checkpoint state files (host only): round trip, signatures, mismatches."""
import os

import numpy as np
import pytest

from onekapy_gb300 import checkpoint as CK
from onekapy_gb300.engine import Lognormal


def _inputs(**over):
    base = dict(target=0, npaths=100, duration=3652.5, nrealizations=40, base=0.0,
                c_dist=Lognormal(np.log(10.0), 0.3), p_dist=(0.2, 0.3), t_dist=(20.0, 30.0),
                stochastic_wells=[(0.0, 0.0, 0.25, (400.0, 600.0)), (100.0, 50.0, 0.25, 300.0)],
                observations=[(10.0, 20.0, 500.0, 0.1)], spacing=10.0, umbra=10.0, confined=True, tol=1.0,
                maxstep=10.0, seed=7, precision=1, window=500.0, mode=0)
    base.update(over)
    return base


def test_signature_is_stable_and_sensitive():
    a = CK.signature(**_inputs())
    assert a == CK.signature(**_inputs())
    assert a != CK.signature(**_inputs(seed=8))
    assert a != CK.signature(**_inputs(p_dist=(0.2, 0.31)))
    assert a != CK.signature(**_inputs(c_dist=Lognormal(np.log(10.0), 0.31)))
    assert a != CK.signature(**_inputs(nrealizations=41))


def test_state_round_trip_and_atomic_write(tmp_path):
    path = str(tmp_path / "run.npz")
    st = CK.RunState("abc", np.arange(12, dtype=np.int32).reshape(3, 4), 5, 8, 40,
                     np.array([100, 90, 7, 6, 1, 0, 2, 0], dtype=np.int64))
    st.save(path)
    assert sorted(os.listdir(tmp_path)) == ["run.npz"]          # no temporary left behind
    got = CK.RunState.load(path)
    assert got.signature == "abc" and got.registered == 5 and got.next_realization == 8
    assert got.nrealizations == 40 and not got.complete
    assert got.counts.dtype == np.int32 and np.array_equal(got.counts, st.counts)
    assert got.counters.dtype == np.int64 and np.array_equal(got.counters, st.counters)


def test_open_state_fresh_resume_and_mismatch(tmp_path):
    path = str(tmp_path / "run.npz")
    fresh = CK.open_state(path, "sig", (3, 4), 10)
    assert fresh.next_realization == 0 and fresh.counts.shape == (3, 4) and not fresh.counts.any()
    fresh.counts[1, 2] = 3
    fresh.next_realization = 4
    fresh.save(path)
    again = CK.open_state(path, "sig", (3, 4), 10)
    assert again.next_realization == 4 and again.counts[1, 2] == 3
    with pytest.raises(ValueError, match="different inputs"):
        CK.open_state(path, "other", (3, 4), 10)
    with pytest.raises(ValueError, match="grid"):
        CK.open_state(path, "sig", (4, 4), 10)
