"""CPU oracle for the OnekaPy tracking and chronicle path -- TEST INFRASTRUCTURE.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, and only as the checker.  The product
(``onekapy_gb300``) never imports it.

Pieces and the reference code each one restates (paths within OnekaPy):

* ``track`` / ``evaluate``: ctypes front end of ``oneka_oracle.c``
  (oneka/model.py:207-427, oneka/capturezone.py:51-253,
  oneka/probabilityfield.py:264-427), FP64 with the reference's evaluation order.
* ``construct_fit`` / ``compute_fit``: NumPy restatement of
  oneka/model.py:497-606 (FOSM potentials, ``lstsq`` and ``inv``).
* ``release_points``: oneka/capturezone.py:110-115.
* ``replay_expand``: the expand loop of oneka/probabilityfield.py:175-261.
* ``philox4x32``, ``draw_*``: restatement of the counter-based random
  variates that the GPU realization kernel draws (Salmon et al., SC'11,
  "Parallel random numbers: as easy as 1, 2, 3"; Philox4x32-10).
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "liboneka_oracle.so")
_lib = None

ORC_OK, ORC_DRY, ORC_STEP_LIMIT = 0, 1, 2


def build(force: bool = False) -> str:
    """Compile the C oracle with the recipe in ``oracle/Makefile``."""
    src = os.path.join(_HERE, "oneka_oracle.c")
    if force or not os.path.exists(_SO) or os.path.getmtime(_SO) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _SO


class _Grid(ctypes.Structure):
    _fields_ = [("xmin", ctypes.c_double), ("ymin", ctypes.c_double),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double),
                ("nrows", ctypes.c_int32), ("ncols", ctypes.c_int32)]


class _Frame(ctypes.Structure):
    _fields_ = [("xmin", ctypes.c_double), ("ymin", ctypes.c_double),
                ("coff", ctypes.c_int32), ("roff", ctypes.c_int32),
                ("ncols", ctypes.c_int32), ("nrows", ctypes.c_int32)]


class _Opts(ctypes.Structure):
    _fields_ = [("duration", ctypes.c_double), ("tol", ctypes.c_double),
                ("maxstep", ctypes.c_double), ("umbra", ctypes.c_double),
                ("confined", ctypes.c_int32), ("pad", ctypes.c_int32),
                ("max_attempts", ctypes.c_int64)]


FRAME_DTYPE = np.dtype([("xmin", "<f8"), ("ymin", "<f8"), ("coff", "<i4"),
                        ("roff", "<i4"), ("ncols", "<i4"), ("nrows", "<i4")])


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_SO)
        P = ctypes.c_void_p
        L.orc_track.restype = ctypes.c_int64
        L.orc_track.argtypes = [P, ctypes.c_int32, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                P, P, P, P, ctypes.c_int32, P, ctypes.c_int32, P, P, P, P,
                                P, P, P, P, P, P, ctypes.c_int64, P, ctypes.c_int32]
        L.orc_evaluate.restype = None
        L.orc_evaluate.argtypes = [P, P, ctypes.c_int32, ctypes.c_double, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                   ctypes.c_double, P, P, ctypes.c_int64, P, P, P, P, P,
                                   ctypes.c_int32]
        L.orc_distancesquared.restype = ctypes.c_double
        L.orc_distancesquared.argtypes = [ctypes.c_double] * 6
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _f64(a, shape=None):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    if shape is not None:
        a = a.reshape(shape)
    return a


def track(wells_xy, coef, q, aquifer, release, grid, *, duration, tol, maxstep, umbra,
          confined, base=0.0, xo=0.0, yo=0.0, rskip=None, frames=None, max_attempts=0,
          want_counts=True, want_vertices=False, max_vertices=0, nthreads=0):
    """Track ``nreal`` realizations x ``npaths`` particles and chronicle them.

    ``grid`` is ``(xmin, ymin, dx, dy, nrows, ncols)``.  Returns a dict with
    ``counts`` (int32 [nrows, ncols]), ``registered`` and per-particle arrays.
    """
    wells_xy = _f64(wells_xy).reshape(-1, 2)
    nwells = wells_xy.shape[0]
    coef = _f64(coef).reshape(-1, 6)
    nreal = coef.shape[0]
    q = _f64(q).reshape(nreal, nwells)
    aquifer = _f64(aquifer).reshape(nreal, 3)
    release = _f64(release).reshape(-1, 2)
    npaths = release.shape[0]
    xmin, ymin, dx, dy, nrows, ncols = grid
    g = _Grid(float(xmin), float(ymin), float(dx), float(dy), int(nrows), int(ncols))
    o = _Opts(float(duration), float(tol), float(maxstep), float(umbra), int(bool(confined)), 0,
              int(max_attempts))
    if rskip is not None:
        rskip = np.ascontiguousarray(rskip, dtype=np.int32)
    if frames is not None:
        frames = np.ascontiguousarray(frames, dtype=FRAME_DTYPE).reshape(nreal, npaths)
    counts = np.zeros((int(nrows), int(ncols)), np.int32) if want_counts else None
    shp = (nreal, npaths)
    naccept = np.zeros(shp, np.int32)
    nattempt = np.zeros(shp, np.int32)
    status = np.zeros(shp, np.int32)
    endpoint = np.zeros(shp + (2,), np.float64)
    bbox = np.zeros(shp + (4,), np.float64)
    nvertices = np.zeros(shp, np.int64)
    vertices = None
    if want_vertices:
        vertices = np.full(shp + (max_vertices, 2), np.nan)
    reg = lib().orc_track(_ptr(wells_xy), nwells, float(base), float(xo), float(yo),
                          _ptr(coef), _ptr(q), _ptr(aquifer), _ptr(rskip), nreal,
                          _ptr(release), npaths, ctypes.byref(o), ctypes.byref(g),
                          _ptr(frames), _ptr(counts), _ptr(naccept), _ptr(nattempt),
                          _ptr(status), _ptr(endpoint), _ptr(bbox), _ptr(vertices),
                          int(max_vertices), _ptr(nvertices), int(nthreads))
    return dict(counts=counts, registered=int(reg), naccept=naccept, nattempt=nattempt,
                status=status, endpoint=endpoint, bbox=bbox, vertices=vertices,
                nvertices=nvertices)


def evaluate(wells_xy, q, base, K, n, H, xo, yo, coef, pts, confined=False):
    """Potential, discharge, head, velocity and status at points (oneka/model.py:207-427)."""
    wells_xy = _f64(wells_xy).reshape(-1, 2)
    q = _f64(q)
    pts = _f64(pts).reshape(-1, 2)
    coef = _f64(coef).reshape(6)
    N = pts.shape[0]
    pot = np.zeros(N)
    dis = np.zeros((N, 2))
    head = np.zeros(N)
    vel = np.zeros((N, 2))
    st = np.zeros(N, np.int32)
    lib().orc_evaluate(_ptr(wells_xy), _ptr(q), wells_xy.shape[0], float(base), float(K),
                       float(n), float(H), float(xo), float(yo), _ptr(coef), _ptr(pts), N,
                       _ptr(pot), _ptr(dis), _ptr(head), _ptr(vel), _ptr(st), int(bool(confined)))
    return dict(potential=pot, discharge=dis, head=head, velocity=vel, status=st)


def distancesquared(ax, ay, bx, by, cx, cy):
    return lib().orc_distancesquared(ax, ay, bx, by, cx, cy)


def rasterize(grid, xy, umbra, rgrid=None):
    """ProbabilityField.rasterize on a fixed grid; returns uint8 marks [nrows, ncols]."""
    xmin, ymin, dx, dy, nrows, ncols = grid
    g = _Grid(float(xmin), float(ymin), float(dx), float(dy), int(nrows), int(ncols))
    f = _Frame(float(xmin), float(ymin), 0, 0, int(ncols), int(nrows))
    if rgrid is None:
        rgrid = np.zeros((int(nrows), int(ncols)), np.uint8)
    xy = _f64(xy).reshape(-1, 2)
    L = lib()
    L.orc_rasterize.restype = None
    L.orc_rasterize.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                ctypes.c_int64, ctypes.c_double]
    L.orc_rasterize(ctypes.byref(g), ctypes.byref(f), _ptr(rgrid), _ptr(xy), xy.shape[0],
                    float(umbra))
    return rgrid


# ---------------------------------------------------------------------------
# Weighted least-squares fit: oneka/model.py:497-606, restated with NumPy.
# ---------------------------------------------------------------------------
class FitRangeError(Exception):
    pass


def construct_fit(obs, wells, base, conductivity, thickness, xo, yo):
    """``wells`` is a list of (xw, yw, rw, qw); ``obs`` of (x, y, z_ev, z_std)."""
    nobs = len(obs)
    WA = np.zeros([nobs, 6])
    Wb = np.zeros([nobs, 1])
    for i in range(nobs):
        x, y, z_ev, z_std = obs[i]
        head = z_ev - base
        if head >= thickness:
            pot_ev = (conductivity * thickness * (head - 0.5 * thickness))
            pot_std = conductivity * thickness * z_std
        elif head > 0:
            pot_ev = (0.5 * conductivity * (head**2 + z_std**2))
            pot_std = conductivity * head * z_std
        else:
            raise FitRangeError("elevation < base")
        dx = x - xo
        dy = y - yo
        WA[i, :] = np.array([dx**2, dy**2, dx * dy, dx, dy, 1]) / pot_std
        pw = 0.0
        for w in wells:
            ddx = x - w[0]
            ddy = y - w[1]
            r2 = ddx * ddx + ddy * ddy
            pw += w[3] * np.log(r2) * 0.07957747154594767
        Wb[i] = (pot_ev - pw) / pot_std
    return WA, Wb


def compute_fit(WA, Wb):
    coef_ev = np.linalg.lstsq(WA, Wb, rcond=-1)[0]
    coef_cov = np.linalg.inv(np.matmul(WA.T, WA))
    return coef_ev, coef_cov


def fit(obs, wells, base, conductivity, thickness, xo, yo):
    WA, Wb = construct_fit(obs, wells, base, conductivity, thickness, xo, yo)
    return compute_fit(WA, Wb)


# ---------------------------------------------------------------------------
# Release ring and grid geometry.
# ---------------------------------------------------------------------------
def release_points(xtarget, ytarget, rtarget, npaths):
    """oneka/capturezone.py:110-115, element by element."""
    STEPAWAY = 1.0
    pts = []
    for theta in np.linspace(0, 2 * np.pi, npaths + 1)[0:-1]:
        xs = (rtarget + STEPAWAY) * np.cos(theta) + xtarget
        ys = (rtarget + STEPAWAY) * np.sin(theta) + ytarget
        pts.append((float(xs), float(ys)))
    return np.array(pts, dtype=np.float64).reshape(-1, 2)


def replay_expand(xo, yo, dx, dy, bboxes):
    """Replay ProbabilityField(dx, dy, xo, yo) followed by expand(bbox) per trace.

    Returns the final (xmin, ymin, nrows, ncols, xmax, ymax) and, for each trace, the
    frame the reference held when it rasterized that trace (FRAME_DTYPE, with
    offsets into the final grid).  oneka/probabilityfield.py:140-151, 222-261.
    """
    xmin, xmax = xo - dx, xo + dx
    ymin, ymax = yo - dy, yo + dy
    ncols = nrows = 3
    cs = rs = 0                  # cumulative left/bottom growth
    recs = []
    for (bx0, bx1, by0, by1) in bboxes:
        if bx0 > bx1 or by0 > by1:
            raise ValueError("bad bbox")
        while bx0 <= xmin:
            xmin -= dx
            ncols += 1
            cs += 1
        while bx1 >= xmax:
            xmax += dx
            ncols += 1
        while by0 <= ymin:
            ymin -= dy
            nrows += 1
            rs += 1
        while by1 >= ymax:
            ymax += dy
            nrows += 1
        recs.append((xmin, ymin, cs, rs, ncols, nrows))
    frames = np.zeros(len(recs), FRAME_DTYPE)
    for k, (fx, fy, c, r, nc, nr) in enumerate(recs):
        frames[k] = (fx, fy, cs - c, rs - r, nc, nr)
    return (xmin, ymin, nrows, ncols, xmax, ymax), frames


def window(xo, yo, dx, dy, half_x, half_y):
    """Pre-expanded grid covering [xo-half_x, xo+half_x] x [yo-half_y, yo+half_y].

    It is the grid ProbabilityField(dx, dy, xo, yo).expand(...) produces for
    that request, so its node coordinates equal the reference's.
    """
    (xmin, ymin, nrows, ncols, _, _), _ = replay_expand(
        xo, yo, dx, dy, [(xo - half_x + 0.5 * dx, xo + half_x - 0.5 * dx,
                          yo - half_y + 0.5 * dy, yo + half_y - 0.5 * dy)])
    return (xmin, ymin, dx, dy, nrows, ncols)


# ---------------------------------------------------------------------------
# Philox4x32-10 and the realization variates (restated for checking K1).
# ---------------------------------------------------------------------------
PHILOX_M0, PHILOX_M1 = 0xD2511F53, 0xCD9E8D57
PHILOX_W0, PHILOX_W1 = 0x9E3779B9, 0xBB67AE85
STREAM_TAG = 0x4F4E454B            # b"ONEK": fourth counter word of every draw


def philox4x32(ctr, key, rounds=10):
    """ctr: 4 uint32, key: 2 uint32 -> 4 uint32 (Salmon et al. 2011)."""
    c0, c1, c2, c3 = (int(v) & 0xFFFFFFFF for v in ctr)
    k0, k1 = (int(v) & 0xFFFFFFFF for v in key)
    for _ in range(rounds):
        p0 = PHILOX_M0 * c0
        p1 = PHILOX_M1 * c2
        hi0, lo0 = p0 >> 32, p0 & 0xFFFFFFFF
        hi1, lo1 = p1 >> 32, p1 & 0xFFFFFFFF
        c0, c1, c2, c3 = (hi1 ^ c1 ^ k0), lo1, (hi0 ^ c3 ^ k1), lo0
        k0 = (k0 + PHILOX_W0) & 0xFFFFFFFF
        k1 = (k1 + PHILOX_W1) & 0xFFFFFFFF
    return c0, c1, c2, c3


def _u53(hi, lo):
    return ((((hi << 32) | lo) >> 11) * (1.0 / 9007199254740992.0))


def philox_uniforms(seed, realization, variate):
    """Two uniforms in [0, 1) for (seed, realization index, variate index)."""
    ctr = (variate, realization & 0xFFFFFFFF, (realization >> 32) & 0xFFFFFFFF, STREAM_TAG)
    key = (seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF)
    w = philox4x32(ctr, key)
    return _u53(w[0], w[1]), _u53(w[2], w[3])


DIST_CONST, DIST_UNIFORM, DIST_TRIANGULAR, DIST_LOGNORMAL = 0, 1, 2, 3


def variate(kind, p0, p1, p2, u0, u1):
    """Transform two uniforms into one variate of the given distribution."""
    if kind == DIST_CONST:
        return p0
    if kind == DIST_UNIFORM:
        return p0 + (p1 - p0) * u0
    if kind == DIST_TRIANGULAR:
        a, c, b = p0, p1, p2
        if b - a <= 0:
            return a
        fc = (c - a) / (b - a)
        if u0 < fc:
            return a + math.sqrt(u0 * (b - a) * (c - a))
        return b - math.sqrt((1.0 - u0) * (b - a) * (b - c))
    if kind == DIST_LOGNORMAL:
        z = math.sqrt(-2.0 * math.log(1.0 - u0)) * math.cos(2.0 * math.pi * u1)
        return math.exp(p0 + p1 * z)
    raise ValueError(kind)


def normal_pair(u0, u1):
    r = math.sqrt(-2.0 * math.log(1.0 - u0))
    return r * math.cos(2.0 * math.pi * u1), r * math.sin(2.0 * math.pi * u1)
