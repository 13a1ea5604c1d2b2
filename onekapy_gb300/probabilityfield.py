"""Drop-in ``ProbabilityField`` of oneka/probabilityfield.py:53-427 with its
grids on the GPU.

The grids live on the device: ``pgrid_device`` is a float64 tensor
[nrows, ncols] and the per-realization registration grid is a device bitmask
(``ceil(ncols/32)`` uint32 words per row, ``mask``).  ``insert`` /
``rasterize`` run the FP64 ``oneka_rasterize`` kernel, ``register`` the
``oneka_register_weighted`` kernel; the geometry (expand) is host
bookkeeping, as in the reference.

``pgrid`` and ``rgrid`` are what the reference's callers read
(``pf.pgrid/pf.total_weight`` and ``np.sort(...)`` in oneka/visualize.py:230,
:318, :382): host NumPy arrays, float64 and bool, as in the reference.
``pgrid`` is copied back from the device once per change of the device grid
and cached; ``rgrid`` is unpacked from the bitmask on every read.  Writing an
element of the returned arrays does not reach the device: assign a whole
array (``pf.pgrid = a``, ``pf.rgrid = b``) instead.
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
        self._pdev = None        # device float64 [nrows, ncols]
        self._phost = None       # cached host copy of _pdev (None: not copied yet)
        self._rhost = None       # host rgrid of a field unpickled without a GPU
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
        self._pdev = torch.zeros((self.nrows, self.ncols), dtype=torch.float64, device=dev)
        self._phost = None
        self._mask = torch.zeros(self._mask_words(), dtype=torch.int32, device=dev)
        self._mask_clean = True     # no bit set since the last register / reset

    @property
    def pgrid(self) -> np.ndarray | None:
        """The weighted counts as a host float64 array [nrows, ncols] (the
        reference's type), copied from the device when it last changed."""
        if self._pdev is None:
            return self._phost
        if self._phost is None:
            # through page-locked memory (torch caches those blocks): a direct DMA copy
            host = torch.empty(self._pdev.shape, dtype=torch.float64, pin_memory=True)
            host.copy_(self._pdev)
            self._phost = host.numpy()
        return self._phost

    @pgrid.setter
    def pgrid(self, value):
        if isinstance(value, torch.Tensor):
            self._pdev = value.to(dtype=torch.float64, device=C.device())
        else:
            self._pdev = torch.as_tensor(np.asarray(value, dtype=np.float64), device=C.device())
        self._phost = None

    @property
    def pgrid_device(self) -> torch.Tensor | None:
        """The weighted counts on the device (float64 [nrows, ncols])."""
        return self._pdev

    @property
    def rgrid_device(self) -> torch.Tensor:
        """The registration grid of the current realization as a device bool tensor."""
        return _unpack(self._mask, self.nrows, self.ncols, (self.ncols + 31) // 32)

    @property
    def rgrid(self) -> np.ndarray:
        """The registration grid of the current realization as a host bool array [nrows, ncols]."""
        if self._mask is None:
            return self._rhost
        return self.rgrid_device.cpu().numpy()

    @rgrid.setter
    def rgrid(self, value):
        v = torch.as_tensor(np.asarray(value) if not isinstance(value, torch.Tensor) else value,
                            device=self._mask.device).to(torch.bool)
        self._mask = _pack(v, (self.ncols + 31) // 32, self._mask_words())
        self._mask_clean = False

    @property
    def mask(self) -> torch.Tensor:
        """The registration bitmask (device int32 words, row-major); a caller
        may mark nodes in it (oneka_track's mark-only mode)."""
        self._mask_clean = False
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
        dev = self._pdev.device
        pgrid = torch.zeros((nrows, ncols), dtype=torch.float64, device=dev)
        pgrid[rshift:rshift + self.nrows, cshift:cshift + self.ncols] = self._pdev
        if getattr(self, "_mask_clean", False):     # nothing to carry over: a fresh mask
            self._pdev = pgrid
            self._phost = None
            self.nrows, self.ncols = nrows, ncols
            self._mask = torch.zeros(self._mask_words(), dtype=torch.int32, device=dev)
            return
        old_r = self.rgrid_device
        rgrid = torch.zeros((nrows, ncols), dtype=torch.bool, device=dev)
        rgrid[rshift:rshift + self.nrows, cshift:cshift + self.ncols] = old_r
        self._pdev = pgrid
        self._phost = None
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
        self._mask_clean = False
        C.check(C.load().oneka_rasterize(ctypes.byref(g), ctypes.byref(frame) if frame else None,
                                         C.ptr(t), t.shape[0], float(umbra), C.ptr(self._mask),
                                         C.stream_ptr()))

    def register(self, weight):
        """pgrid[rgrid] += weight, then clear rgrid (probabilityfield.py:342-359)."""
        self.total_weight += weight
        g = self._grid().c()
        C.check(C.load().oneka_register_weighted(ctypes.byref(g), C.ptr(self._mask), float(weight),
                                                 C.ptr(self._pdev), C.stream_ptr()))
        self._phost = None
        self._mask_clean = True

    def reset(self):
        """Clear rgrid (probabilityfield.py:362-376)."""
        self._mask.zero_()
        self._mask_clean = True

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
        """The reference's attributes, with pgrid / rgrid as host NumPy arrays
        (oneka/probabilityfield.py:125-151), so that the state is the one a
        reference ProbabilityField pickles."""
        st = {k: v for k, v in self.__dict__.items()
              if not k.startswith("_") and k not in ("realizations", "counts")}
        if self.nrows:
            st["pgrid"] = np.array(self.pgrid, dtype=np.float64)
            st["rgrid"] = np.array(self.rgrid, dtype=bool)
        return st

    def __setstate__(self, st):
        st = dict(st)
        pgrid = st.pop("pgrid", None)
        rgrid = st.pop("rgrid", None)
        self.__dict__.update(st)
        self._mask = None
        self._pdev = None
        self._phost = None
        self._rhost = None
        if pgrid is None:
            return
        if torch.cuda.is_available():
            self.pgrid = pgrid
            self._mask = torch.zeros(self._mask_words(), dtype=torch.int32, device=C.device())
            self._mask_clean = True
            self.rgrid = rgrid
        else:           # inspection without a GPU: host arrays only
            self._phost = np.asarray(pgrid, dtype=np.float64)
            self._rhost = np.asarray(rgrid, dtype=bool)

    # ---------------------------------------------------------------- helpers
    def probability(self) -> torch.Tensor:
        """pgrid / total_weight on the device (the capture probability,
        oneka/visualize.py:230)."""
        from .outputs import probability
        return probability(self)
