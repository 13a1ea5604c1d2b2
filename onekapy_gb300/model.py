"""Drop-in ``Model`` of oneka/model.py:62-606, evaluated on the GPU.

Every method keeps the reference's name, arguments, return shape and
exceptions.  Point evaluations run the FP64 ``oneka_evaluate`` kernel and the
fit runs the FP64 ``oneka_realize`` kernel (ONEKA_MODE_GIVEN_EV).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _capi as C
from . import engine as E


class Error(Exception):
    """Base class for module errors (oneka/model.py:46-48)."""


class RangeError(Error):
    """Passed argument out of valid range (oneka/model.py:51-53)."""


class AquiferError(Error):
    """Dry aquifer (oneka/model.py:56-58)."""


class Model:
    """An Oneka-type analytic element model (oneka/model.py:62-128)."""

    def __init__(self, base, conductivity, porosity, thickness, wells, xo=0, yo=0,
                 coef=np.zeros((6, ))):
        self.base = base
        self.conductivity = conductivity
        self.porosity = porosity
        self.thickness = thickness
        self.wells = wells
        self.xo = xo
        self.yo = yo
        self.coef = coef

    @property
    def coef(self):
        return self._coef

    @coef.setter
    def coef(self, coef):
        self._coef = np.reshape(coef, [6, ])

    def __repr__(self):
        return 'Model({0.base}, {0.conductivity}, {0.porosity}, {0.thickness})'.format(self)

    __str__ = __repr__

    # ------------------------------------------------------------ device data
    def _site(self, dev):
        wells = torch.tensor([[float(w[0]), float(w[1]), float(w[2])] for w in self.wells],
                             dtype=torch.float64, device=dev).reshape(-1, 3).contiguous()
        q = torch.tensor([float(w[3]) for w in self.wells], dtype=torch.float64,
                         device=dev).contiguous()
        site = C.OnekaSite(len(self.wells), 0, 0, 0, float(self.base), float(self.xo),
                           float(self.yo), C.ptr(wells) if len(self.wells) else None, None)
        return site, wells, q

    def evaluate(self, points, confined=False):
        """Potential, discharge, head, velocity and status at ``points`` [n, 2]
        in one FP64 kernel launch (model.py:207-427)."""
        dev = C.device()
        pts = torch.as_tensor(np.asarray(points, dtype=np.float64).reshape(-1, 2), device=dev).contiguous()
        n = pts.shape[0]
        site, wells, q = self._site(dev)
        pot = torch.empty(n, dtype=torch.float64, device=dev)
        dis = torch.empty((n, 2), dtype=torch.float64, device=dev)
        head = torch.empty(n, dtype=torch.float64, device=dev)
        vel = torch.empty((n, 2), dtype=torch.float64, device=dev)
        st = torch.empty(n, dtype=torch.int32, device=dev)
        coef = (ctypes.c_double * 6)(*[float(c) for c in self.coef])
        C.check(C.load().oneka_evaluate(ctypes.byref(site), C.ptr(q) if len(self.wells) else None,
                                        float(self.conductivity), float(self.porosity),
                                        float(self.thickness), coef, C.ptr(pts), n,
                                        int(bool(confined)), C.ptr(pot), C.ptr(dis), C.ptr(head),
                                        C.ptr(vel), C.ptr(st), C.stream_ptr()))
        return dict(potential=pot.cpu().numpy(), discharge=dis.cpu().numpy(),
                    head=head.cpu().numpy(), velocity=vel.cpu().numpy(), status=st.cpu().numpy())

    def _one(self, x, y, confined=False):
        return self.evaluate([[float(x), float(y)]], confined=confined)

    # ------------------------------------------------------------ reference API
    def compute_potential(self, x, y):
        """Discharge potential [m^3/d] at (x, y) (model.py:207-237)."""
        return float(self._one(x, y)["potential"][0])

    def compute_potential_wells_only(self, x, y):
        """Potential of the wells alone (model.py:240-266)."""
        saved = self._coef
        try:
            self._coef = np.zeros(6)
            return float(self._one(x, y)["potential"][0])
        finally:
            self._coef = saved

    def compute_discharge(self, x, y):
        """Vertically integrated discharge [Qx, Qy] [m^2/d] (model.py:269-315)."""
        d = self._one(x, y)["discharge"][0]
        return [float(d[0]), float(d[1])]

    def compute_head(self, x, y):
        """Piezometric head [m] above the base (model.py:318-350)."""
        r = self._one(x, y)
        if r["status"][0] != C.TRACE_OK and not (r["potential"][0] > 0):
            raise AquiferError("potential_to_head: potential <= 0")
        return float(r["head"][0])

    def compute_velocity(self, x, y):
        """Seepage velocity (Vx, Vy) [m/d] (model.py:353-389)."""
        r = self._one(x, y, confined=False)
        if r["status"][0] != C.TRACE_OK:
            if not (r["potential"][0] > 0):
                raise AquiferError("potential_to_head: potential <= 0")
            raise AquiferError("discharge_to_velocity: head <= 0")
        v = r["velocity"][0]
        return (float(v[0]), float(v[1]))

    def compute_velocity_confined(self, x, y):
        """Seepage velocity assuming a confined aquifer (model.py:392-427)."""
        v = self._one(x, y, confined=True)["velocity"][0]
        return (float(v[0]), float(v[1]))

    def fit_regional_flow(self, obs, xo, yo):
        """Weighted least-squares fit of A..F (model.py:430-494).  Returns
        (coef_ev (6, 1), coef_cov (6, 6)) and sets xo, yo, coef."""
        coef_ev, coef_cov = fit(self, obs, xo, yo)
        self.xo = xo
        self.yo = yo
        self.coef = coef_ev
        return (coef_ev, coef_cov)

    def construct_fit(self, obs, xo, yo):
        """WA, Wb of the weighted least-squares problem (model.py:497-567),
        computed by the FP64 ``oneka_fit_rows`` kernel; host arrays
        (nobs, 6) and (nobs, 1) as in the reference."""
        nobs = len(obs)
        if nobs == 0:
            return (np.zeros([0, 6]), np.zeros([0, 1]))
        dev = C.device()
        site, wells, q = self._site(dev)
        o = torch.as_tensor(np.asarray(obs, dtype=np.float64).reshape(-1, 4), device=dev).contiguous()
        site.nobs, site.obs, site.xo, site.yo = nobs, C.ptr(o), float(xo), float(yo)
        WA = torch.empty((nobs, 6), dtype=torch.float64, device=dev)
        Wb = torch.empty((nobs, 1), dtype=torch.float64, device=dev)
        st = torch.empty(1, dtype=torch.int32, device=dev)
        C.check(C.load().oneka_fit_rows(ctypes.byref(site), C.ptr(q) if len(self.wells) else None,
                                        float(self.conductivity), float(self.thickness), C.ptr(WA), C.ptr(Wb),
                                        C.ptr(st), C.stream_ptr()))
        if int(st.item()) == C.REAL_RANGE:
            raise RangeError("model.fit_coeficient: elevation < base")
        return (WA.cpu().numpy(), Wb.cpu().numpy())

    @staticmethod
    def compute_fit(WA, Wb):
        """Least-squares coefficients (6, 1) and covariance inv(WA^T WA) (6, 6)
        (model.py:571-606), solved by the FP64 ``oneka_fit_solve`` kernel
        (normal equations with a Jacobi-scaled Cholesky factor)."""
        dev = C.device()
        A = torch.as_tensor(np.asarray(WA, dtype=np.float64).reshape(-1, 6), device=dev).contiguous()
        b = torch.as_tensor(np.asarray(Wb, dtype=np.float64).reshape(-1), device=dev).contiguous()
        if b.shape[0] != A.shape[0]:
            raise ValueError("WA and Wb must have the same number of rows")
        ev = torch.empty((1, 6), dtype=torch.float64, device=dev)
        cov = torch.empty((1, 36), dtype=torch.float64, device=dev)
        st = torch.empty(1, dtype=torch.int32, device=dev)
        C.check(C.load().oneka_fit_solve(C.ptr(A), C.ptr(b), A.shape[0], 1, C.ptr(ev), C.ptr(cov), C.ptr(st),
                                         C.stream_ptr()))
        s = int(st.item())
        if s == C.REAL_NOT_SPD:
            raise np.linalg.LinAlgError("normal equations are not positive definite")
        if s != C.REAL_OK:
            raise np.linalg.LinAlgError("WA or Wb is not finite")
        return (ev.cpu().numpy().reshape(6, 1), cov.cpu().numpy().reshape(6, 6))


def fit(model: Model, obs, xo, yo):
    """FOSM rows + FP64 normal equations on the GPU (oneka_realize with
    ONEKA_MODE_GIVEN_EV) for one model; raises like the reference."""
    dev = C.device()
    wells = [(w[0], w[1], w[2], 0.0) for w in model.wells]
    site = E.Site(wells, np.asarray(obs, dtype=np.float64).reshape(-1, 4), model.base, target=0,
                  xo=xo, yo=yo, device=dev)
    real = E.Realizations.empty(1, site.nwells, dev)
    real.q.copy_(torch.tensor([[float(w[3]) for w in model.wells]], dtype=torch.float64))
    real.aquifer.copy_(torch.tensor([[float(model.conductivity), float(model.porosity),
                                      float(model.thickness)]], dtype=torch.float64))
    E.realize(site, 1, mode=C.MODE_GIVEN_EV, out=real)
    st = int(real.status.item())
    if st == C.REAL_RANGE:
        raise RangeError("model.fit_coeficient: elevation < base")
    if st == C.REAL_NOT_SPD:
        raise np.linalg.LinAlgError("normal equations are not positive definite")
    ev = real.coef_ev.cpu().numpy().reshape(6, 1)
    cov = real.coef_cov.cpu().numpy().reshape(6, 6)
    return ev, cov


class ModelFeval:
    """The backtracing velocity function of oneka/stochastic.py:253-260:
    ``feval(xy) -> np.array([-Vx, -Vy])``.  compute_capturezone and
    compute_backtrace recognise it and run the whole trace on the GPU."""

    def __init__(self, model: Model, confined: bool):
        self.model = model
        self.confined = bool(confined)

    def __call__(self, xy):
        if self.confined:
            Vx, Vy = self.model.compute_velocity_confined(xy[0], xy[1])
        else:
            Vx, Vy = self.model.compute_velocity(xy[0], xy[1])
        return np.array([-Vx, -Vy])


def make_feval(model: Model, confined: bool) -> ModelFeval:
    return ModelFeval(model, confined)
