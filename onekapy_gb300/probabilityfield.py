"""Drop-in ``ProbabilityField`` of oneka/probabilityfield.py:53-427 with its
grids on the GPU.

``pgrid`` is a float64 device tensor [nrows, ncols]; the per-realization
registration grid is a device bitmask (``ceil(ncols/32)`` uint32 words per
row) that ``rgrid`` presents as a bool tensor.  ``insert`` / ``rasterize`` run
the FP64 ``oneka_rasterize`` kernel, ``register`` the ``oneka_register_weighted``
kernel; the geometry (expand) is host bookkeeping, as in the reference.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _capi as C
from .engine import Grid


class Error(Exception):
    """Base class for module errors (oneka/probabilityfield.py:41-43)."""


class RangeError(Error):
    """Passed argument out of valid range (oneka/probabilityfield.py:47-49)."""


def _unpack(mask: torch.Tensor, nrows: int, ncols: int, wpr: int) -> torch.Tensor:
    words = mask[: nrows * wpr].view(nrows, wpr).to(torch.int64) & 0xFFFFFFFF
    bits = torch.arange(32, device=mask.device, dtype=torch.int64)
    return (((words[:, :, None] >> bits) & 1).reshape(nrows, wpr * 32)[:, :ncols]).to(torch.bool)


def _pack(rgrid: torch.Tensor, wpr: int, total_words: int) -> torch.Tensor:
    nrows, ncols = rgrid.shape
    padded = torch.zeros((nrows, wpr * 32), dtype=torch.int64, device=rgrid.device)
    padded[:, :ncols] = rgrid.to(torch.int64)
    bits = torch.arange(32, device=rgrid.device, dtype=torch.int64)
    words = (padded.view(nrows, wpr, 32) << bits).sum(dim=2)
    out = torch.zeros(total_words, dtype=torch.int32, device=rgrid.device)
    out[: nrows * wpr] = torch.where(words >= 2**31, words - 2**32, words).view(-1).to(torch.int32)
    return out


class ProbabilityField:
    """An auto-expanding, axis-aligned-grid-based probability field."""

    def __init__(self, deltax, deltay, xo=np.nan, yo=np.nan):
        if deltax <= 0:
            raise RangeError("<deltax> must be > 0.")
        if deltay <= 0:
            raise RangeError("<deltay> must be > 0.")
        self.deltax = deltax
        self.deltay = deltay
        self._mask = None
        self.pgrid = None
        if np.isnan(xo) or np.isnan(yo):
            self.nrows = 0
            self.ncols = 0
        else:
            self.xmin = xo - deltax
            self.xmax = xo + deltax
            self.ymin = yo - deltay
            self.ymax = yo + deltay
            self.nrows = 3
            self.ncols = 3
            self._alloc()
            self.total_weight = 0.0

    # ---------------------------------------------------------------- storage
    def _grid(self) -> Grid:
        return Grid(self.xmin, self.ymin, float(self.deltax), float(self.deltay), self.nrows, self.ncols)

    def _mask_words(self) -> int:
        return self._grid().slot_bytes() // 4

    def _alloc(self):
        dev = C.device()
        self.pgrid = torch.zeros((self.nrows, self.ncols), dtype=torch.float64, device=dev)
        self._mask = torch.zeros(self._mask_words(), dtype=torch.int32, device=dev)

    @property
    def rgrid(self) -> torch.Tensor:
        """The registration grid of the current realization as bool [nrows, ncols]."""
        if self._mask is None and getattr(self, "_host_rgrid", None) is not None:
            return self._host_rgrid
        return _unpack(self._mask, self.nrows, self.ncols, (self.ncols + 31) // 32)

    @rgrid.setter
    def rgrid(self, value):
        v = torch.as_tensor(value, device=self._mask.device).to(torch.bool)
        self._mask = _pack(v, (self.ncols + 31) // 32, self._mask_words())

    @property
    def mask(self) -> torch.Tensor:
        """The registration bitmask (device int32 words, row-major)."""
        return self._mask

    def __repr__(self):
        if self.nrows == 0:
            return "ProbabilityField({0.deltax}, {0.deltay})".format(self)
        return ("ProbabilityField({0.deltax}, {0.deltay}, {0.nrows}, {0.ncols}, "
                "{0.xmin}, {0.xmax}, {0.ymin}, {0.ymax}, {0.total_weight})".format(self))

    def __str__(self):
        if self.nrows == 0:
            return "ProbabilityField({0.deltax}, {0.deltay}, {0.nrows}, {0.ncols})".format(self)
        return self.__repr__()

    # ---------------------------------------------------------------- geometry
    def expand(self, xmin, xmax, ymin, ymax):
        """Grow the grids to include the box; contents are kept
        (oneka/probabilityfield.py:175-261)."""
        if xmin > xmax:
            raise RangeError("<xmin> must be <= <xmax>.")
        if ymin > ymax:
            raise RangeError("<ymin> must be <= <ymax>.")
        if (self.ncols == 0) or (self.nrows == 0):
            self.xmin = xmin - self.deltax
            self.ymin = ymin - self.deltay
            self.ncols = max(3, math.ceil((xmax - self.xmin) / self.deltax) + 2)
            self.nrows = max(3, math.ceil((ymax - self.ymin) / self.deltay) + 2)
            self.xmax = self.xmin + (self.ncols - 1) * self.deltax
            self.ymax = self.ymin + (self.nrows - 1) * self.deltay
            self._alloc()
            self.total_weight = 0.0
            return
        nrows, ncols = self.nrows, self.ncols
        rshift = cshift = 0
        while xmin <= self.xmin:
            self.xmin -= self.deltax
            ncols += 1
            cshift += 1
        while xmax >= self.xmax:
            self.xmax += self.deltax
            ncols += 1
        while ymin <= self.ymin:
            self.ymin -= self.deltay
            nrows += 1
            rshift += 1
        while ymax >= self.ymax:
            self.ymax += self.deltay
            nrows += 1
        if (nrows != self.nrows) or (ncols != self.ncols):
            self._regrid(nrows, ncols, rshift, cshift)

    def _regrid(self, nrows, ncols, rshift, cshift):
        old_r = self.rgrid
        dev = self.pgrid.device
        pgrid = torch.zeros((nrows, ncols), dtype=torch.float64, device=dev)
        pgrid[rshift:rshift + self.nrows, cshift:cshift + self.ncols] = self.pgrid
        rgrid = torch.zeros((nrows, ncols), dtype=torch.bool, device=dev)
        rgrid[rshift:rshift + self.nrows, cshift:cshift + self.ncols] = old_r
        self.pgrid = pgrid
        self.nrows, self.ncols = nrows, ncols
        self._mask = _pack(rgrid, (ncols + 31) // 32, self._mask_words())

    # ---------------------------------------------------------------- chronicle
    def insert(self, ax, ay, bx, by, umbra):
        """Mark the nodes within umbra of one segment (probabilityfield.py:264-310)."""
        self._rasterize_device(np.array([[ax, ay], [bx, by]], dtype=np.float64), umbra)

    def rasterize(self, x, y, umbra):
        """Insert one track (probabilityfield.py:313-339)."""
        self.expand(min(x), max(x), min(y), max(y))
        xy = np.stack([np.asarray(x, dtype=np.float64), np.asarray(y, dtype=np.float64)], axis=1)
        self._rasterize_device(xy, umbra)

    def _rasterize_device(self, xy, umbra, frame=None):
        if self.nrows == 0:
            return
        dev = self._mask.device
        t = torch.as_tensor(np.ascontiguousarray(xy, dtype=np.float64), device=dev)
        g = self._grid().c()
        C.check(C.load().oneka_rasterize(ctypes.byref(g), ctypes.byref(frame) if frame else None,
                                         C.ptr(t), t.shape[0], float(umbra), C.ptr(self._mask),
                                         C.stream_ptr()))

    def register(self, weight):
        """pgrid[rgrid] += weight, then clear rgrid (probabilityfield.py:342-359)."""
        self.total_weight += weight
        g = self._grid().c()
        C.check(C.load().oneka_register_weighted(ctypes.byref(g), C.ptr(self._mask), float(weight),
                                                 C.ptr(self.pgrid), C.stream_ptr()))

    def reset(self):
        """Clear rgrid (probabilityfield.py:362-376)."""
        self._mask.zero_()

    @staticmethod
    def distancesquared(ax, ay, bx, by, cx, cy):
        """Squared distance from (cx, cy) to the segment (probabilityfield.py:380-427)."""
        dev = C.device()
        q = torch.tensor([[ax, ay, bx, by, cx, cy]], dtype=torch.float64, device=dev)
        out = torch.empty(1, dtype=torch.float64, device=dev)
        C.check(C.load().oneka_distancesquared(C.ptr(q), C.ptr(out), 1, C.stream_ptr()))
        return float(out.item())

    # ---------------------------------------------------------------- pickling
    def __getstate__(self):
        """Host arrays under the reference's attribute names (archive.py)."""
        st = {k: v for k, v in self.__dict__.items()
              if k not in ("_mask", "pgrid", "realizations", "counts", "_host_rgrid")}
        if self.nrows:
            st["pgrid"] = self.pgrid.detach().cpu().numpy()
            st["rgrid"] = self.rgrid.cpu().numpy()
        return st

    def __setstate__(self, st):
        st = dict(st)
        pgrid = st.pop("pgrid", None)
        rgrid = st.pop("rgrid", None)
        self.__dict__.update(st)
        self._mask = None
        self.pgrid = None
        self._host_rgrid = None
        if pgrid is not None:
            if torch.cuda.is_available():
                dev = C.device()
                self.pgrid = torch.as_tensor(pgrid, device=dev)
                self._mask = torch.zeros(self._mask_words(), dtype=torch.int32, device=dev)
                self.rgrid = torch.as_tensor(rgrid, device=dev)
            else:           # inspection without a GPU: host arrays
                self.pgrid = torch.as_tensor(pgrid)
                self._host_rgrid = torch.as_tensor(rgrid)

    # ---------------------------------------------------------------- helpers
    def probability(self) -> torch.Tensor:
        """pgrid / total_weight (the capture probability, oneka/visualize.py:230)."""
        return self.pgrid / self.total_weight
