"""Run archive of oneka/archive.py:46-89: a bz2-compressed pickle of a dict
with the reference's keys, interchangeable with the reference in both
directions.

* ``dump_oneka`` pickles ``pfield`` as an instance of the reference's class,
  ``oneka.probabilityfield.ProbabilityField``, whose state is the reference's
  attributes (deltax, deltay, nrows, ncols, xmin, xmax, ymin, ymax,
  total_weight, and pgrid / rgrid as NumPy float64 / bool arrays,
  oneka/probabilityfield.py:125-151).  The reference's ``load_oneka`` therefore
  opens it without this package.  When the reference is not installed, a
  stand-in class under that module path exists only while the pickle is
  written.
* ``load_oneka`` opens archives written by either side: the reference's
  class path, and this package's own, resolve to
  ``onekapy_gb300.probabilityfield.ProbabilityField``, which takes the
  reference's state (host arrays when no GPU is present).
"""
from __future__ import annotations

import bz2
import importlib
import os
import pickle
import sys
import types
from contextlib import contextmanager
from datetime import datetime

KEYS = ("projectname", "runtime", "target", "npaths", "duration", "nrealizations", "base", "c_dist",
        "p_dist", "t_dist", "stochastic_wells", "observations", "buffer", "spacing", "umbra", "smooth",
        "confined", "tol", "maxstep", "pfield")

REF_MODULE = "oneka.probabilityfield"
REF_CLASS = "ProbabilityField"


@contextmanager
def _reference_class():
    """The reference's ProbabilityField class, or, when the reference is not
    importable, a plain stand-in registered under its module path for the
    duration of the block (pickle writes classes by module and name)."""
    try:
        mod = importlib.import_module(REF_MODULE)
        cls = getattr(mod, REF_CLASS)
        if isinstance(cls, type):
            yield cls
            return
    except Exception:
        pass
    saved = {k: sys.modules.get(k) for k in ("oneka", REF_MODULE)}
    pkg = types.ModuleType("oneka")
    pkg.__path__ = []
    mod = types.ModuleType(REF_MODULE)
    cls = type(REF_CLASS, (), {"__module__": REF_MODULE, "__qualname__": REF_CLASS})
    setattr(mod, REF_CLASS, cls)
    pkg.probabilityfield = mod
    sys.modules["oneka"] = pkg
    sys.modules[REF_MODULE] = mod
    try:
        yield cls
    finally:
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v


def _as_reference(pfield, cls):
    """An instance of `cls` holding the reference attributes of this
    package's ProbabilityField `pfield`; anything else is returned as is."""
    from .probabilityfield import ProbabilityField
    if not isinstance(pfield, ProbabilityField):
        return pfield
    obj = cls.__new__(cls)
    obj.__dict__.update(pfield.__getstate__())
    return obj


def dump_oneka(projectname, runtime, target, npaths, duration, nrealizations, base, c_dist, p_dist,
               t_dist, stochastic_wells, observations, buffer, spacing, umbra, smooth, confined, tol,
               maxstep, pfield, directory="logs", filename=None):
    """Write the archive; returns its path (logs/Oneka<YYYYmmddTHHMMSS>.bz2 by default)."""
    if filename is None:
        os.makedirs(directory, exist_ok=True)
        filename = os.path.join(directory, "Oneka" + datetime.now().strftime("%Y%m%dT%H%M%S") + ".bz2")
    with _reference_class() as cls:
        pf = _as_reference(pfield, cls)
        values = (projectname, runtime, target, npaths, duration, nrealizations, base, c_dist, p_dist,
                  t_dist, stochastic_wells, observations, buffer, spacing, umbra, smooth, confined, tol,
                  maxstep, pf)
        with bz2.BZ2File(filename, "w") as fp:
            pickle.dump(dict(zip(KEYS, values)), fp)
    return filename


class _Unpickler(pickle.Unpickler):
    def find_class(self, module, name):
        if name == REF_CLASS and module in (REF_MODULE, "onekapy_gb300.probabilityfield"):
            from .probabilityfield import ProbabilityField
            return ProbabilityField
        return super().find_class(module, name)


def load_oneka(filename):
    """The archive's dict; its ``pfield`` is this package's ProbabilityField."""
    with bz2.BZ2File(filename, "r") as fp:
        return _Unpickler(fp).load()
