"""Observation preprocessing of oneka/utilities.py:34-144, on the host.

It runs once per site, before the hot path.  The rules are the reference's:

- an observation within `buffer` (<=) of any well is dropped;
- each run of consecutive observations closer than 1 m to the run's first
  observation becomes one, with the minimum-variance weighted mean and
  sqrt(1/sum(1/sigma^2)) as its standard deviation.  The position is that of
  the run's first observation.
"""
from __future__ import annotations

import numpy as np

TOO_CLOSE = 1.0     # minimum distance for distinct observations [m]


def filter_obs(observations, wellfield, buffer):
    """Retained observations (same tuple layout as the input)."""
    obs = []
    for ob in observations:
        near = any(np.hypot(ob[0] - we[0], ob[1] - we[1]) <= buffer for we in wellfield)
        if not near:
            obs.append(ob)
    retained = []
    i = 0
    while i < len(obs):
        j = i + 1
        while j < len(obs) and np.hypot(obs[i][0] - obs[j][0], obs[i][1] - obs[j][1]) < TOO_CLOSE:
            j += 1
        if j - i > 1:
            num = 0
            den = 0
            for k in range(i, j):
                num += obs[k][2] / obs[k][3] ** 2
                den += 1 / obs[k][3] ** 2
            retained.append((obs[i][0], obs[i][1], num / den, np.sqrt(1 / den)))
        else:
            retained.append(obs[i])
        i = j
    return retained


def summary_statistics(values, names, formats, title):
    """Fixed-width table of count, min, median, max, mean and standard
    deviation per column, NaNs left out (oneka/utilities.py:148-256): the text
    the reference logs for the retained observations.  Returns an
    io.StringIO; use .getvalue() for the string."""
    import io
    ncol = len(values[0])
    widths = [len(format(1, f)) for f in formats]
    width = 5 + sum(widths)
    cols = []
    for j in range(ncol):
        x = np.array([v[j] for v in values], dtype=np.float64)
        cols.append(x[~np.isnan(x)])
    rows = [("min", np.min), ("med", np.median), ("max", np.max), ("avg", np.mean), ("std", np.std)]
    out = [f"{title:^{width}s}", "=" * width,
           "     " + "".join(f"{names[j]:>{widths[j]}s}" for j in range(ncol)), "-" * width,
           "cnt: " + "".join(f"{len(cols[j]):>{widths[j]}d}" for j in range(ncol))]
    for label, fn in rows:
        out.append(f"{label}: " + "".join(format(fn(cols[j]), formats[j]) for j in range(ncol)))
    out.append("=" * width)
    buf = io.StringIO()
    buf.write("\n".join(out) + "\n")
    return buf
