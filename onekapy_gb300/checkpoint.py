"""Checkpoint and resume of a stochastic capture-zone run.

The reference only archives a finished run (oneka/archive.py:46-89); a run
that stops early is lost.  Here a run on a fixed window can be saved after
every chunk of realizations and resumed later.  The state is small: the int32
count grid, the number of registered realizations, the index of the next
realization and the run's trace counters (attempts, accepted steps, chronicle
work, DRY / STEP_LIMIT traces, traces leaving the grid).  Resuming is exact -- the realization draws are Philox streams
keyed by (seed, realization index), so realization k is the same whichever
call draws it, and integer counts add exactly -- so an interrupted and
resumed run returns the same counts as an uninterrupted one.

A signature (SHA-256 over every input that determines the result) guards
against resuming with different inputs.
"""
from __future__ import annotations

import hashlib
import json
import os
from dataclasses import dataclass

import numpy as np

FORMAT = 2
NCOUNTERS = 8


def _canon(v):
    """JSON-able canonical form of the run inputs (floats by repr)."""
    if isinstance(v, (list, tuple)):
        return [_canon(x) for x in v]
    if isinstance(v, dict):
        return {str(k): _canon(x) for k, x in sorted(v.items())}
    if isinstance(v, (bool, np.bool_)):
        return bool(v)
    if isinstance(v, (int, np.integer)):
        return int(v)
    if isinstance(v, (float, np.floating)):
        return repr(float(v))
    if v is None or isinstance(v, str):
        return v
    if hasattr(v, "__dict__"):
        return {"type": type(v).__name__, **{k: _canon(x) for k, x in sorted(vars(v).items())}}
    return repr(v)


def signature(**inputs) -> str:
    return hashlib.sha256(json.dumps(_canon(inputs), sort_keys=True).encode()).hexdigest()


@dataclass
class RunState:
    signature: str
    counts: np.ndarray          # int32 [nrows][ncols]
    registered: int             # realizations registered so far
    next_realization: int       # first realization not yet tracked
    nrealizations: int
    counters: np.ndarray | None = None   # int64 [8] trace counters summed so far

    def __post_init__(self):
        if self.counters is None:
            self.counters = np.zeros(NCOUNTERS, dtype=np.int64)

    @property
    def complete(self) -> bool:
        return self.next_realization >= self.nrealizations

    def save(self, path: str) -> None:
        """Write atomically: a reader sees the old state or the new one."""
        tmp = f"{path}.tmp{os.getpid()}"
        with open(tmp, "wb") as f:
            np.savez(f, format=np.int64(FORMAT), signature=np.array(self.signature),
                     counts=np.ascontiguousarray(self.counts, dtype=np.int32),
                     registered=np.int64(self.registered), next_realization=np.int64(self.next_realization),
                     nrealizations=np.int64(self.nrealizations),
                     counters=np.ascontiguousarray(self.counters, dtype=np.int64))
            f.flush()
            os.fsync(f.fileno())
        os.replace(tmp, path)

    @staticmethod
    def load(path: str) -> "RunState":
        with np.load(path, allow_pickle=False) as z:
            if int(z["format"]) != FORMAT:
                raise ValueError(f"{path}: checkpoint format {int(z['format'])}, expected {FORMAT}")
            return RunState(str(z["signature"]), z["counts"].astype(np.int32), int(z["registered"]),
                            int(z["next_realization"]), int(z["nrealizations"]),
                            z["counters"].astype(np.int64))


def open_state(path: str | None, sig: str, shape, nrealizations: int) -> RunState:
    """The saved state at `path` if it belongs to this run, else a fresh one.
    A state saved by a run with other inputs raises ValueError."""
    if path and os.path.exists(path):
        st = RunState.load(path)
        if st.signature != sig:
            raise ValueError(f"{path} was written by a run with different inputs")
        if tuple(st.counts.shape) != tuple(shape):
            raise ValueError(f"{path}: grid {st.counts.shape} does not match {tuple(shape)}")
        return st
    return RunState(sig, np.zeros(shape, dtype=np.int32), 0, 0, nrealizations)
