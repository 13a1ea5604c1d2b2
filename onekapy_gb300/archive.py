"""Run archive of oneka/archive.py:46-89: a bz2-compressed pickle of a dict
with the reference's keys.  The ProbabilityField pickles as host arrays
(pgrid float64, rgrid bool), so an archive loads without a GPU."""
from __future__ import annotations

import bz2
import os
import pickle
from datetime import datetime

KEYS = ("projectname", "runtime", "target", "npaths", "duration", "nrealizations", "base", "c_dist",
        "p_dist", "t_dist", "stochastic_wells", "observations", "buffer", "spacing", "umbra", "smooth",
        "confined", "tol", "maxstep", "pfield")


def dump_oneka(projectname, runtime, target, npaths, duration, nrealizations, base, c_dist, p_dist,
               t_dist, stochastic_wells, observations, buffer, spacing, umbra, smooth, confined, tol,
               maxstep, pfield, directory="logs", filename=None):
    """Write the archive; returns its path (logs/Oneka<YYYYmmddTHHMMSS>.bz2 by default)."""
    if filename is None:
        os.makedirs(directory, exist_ok=True)
        filename = os.path.join(directory, "Oneka" + datetime.now().strftime("%Y%m%dT%H%M%S") + ".bz2")
    values = (projectname, runtime, target, npaths, duration, nrealizations, base, c_dist, p_dist,
              t_dist, stochastic_wells, observations, buffer, spacing, umbra, smooth, confined, tol,
              maxstep, pfield)
    with bz2.BZ2File(filename, "w") as fp:
        pickle.dump(dict(zip(KEYS, values)), fp)
    return filename


def load_oneka(filename):
    with bz2.BZ2File(filename, "r") as fp:
        return pickle.load(fp)
