"""ETDRK integrators (exponax/etdrk/*).

The coefficient set-up (E = exp(dt L), the phi-function contour means with
``num_circle_points`` roots on a circle of ``circle_radius``, real part
kept) runs once per plan as an FP64 CUDA kernel; ``step_fourier`` runs the
fused stage kernels.  The tables are readable as ``_exp_term``,
``_half_exp_term`` and ``_coef_1`` .. ``_coef_6`` for inspection.
"""

from __future__ import annotations

import numpy as np

from . import _device
from ._lib import check, load
from ._plan import Plan
from .nonlin_fun import BaseNonlinearFun, ZeroNonlinearFun
from .spectral import wavenumber_shape


def roots_of_unity(M: int) -> np.ndarray:
    """etdrk/_utils.py:9-23: exp(2 pi i (j - 1/2) / M), j = 1..M."""
    return np.exp(2j * np.pi * (np.arange(1, M + 1) - 0.5) / M)


class BaseETDRK:
    """etdrk/_base_etdrk.py:15-80"""

    _order = 0

    def __init__(self, dt: float, linear_operator, nonlinear_fun: BaseNonlinearFun | None = None, *,
                 num_circle_points: int = 16, circle_radius: float = 1.0, num_points: int | None = None):
        self.dt = dt
        self.linear_operator = np.asarray(linear_operator, dtype=np.complex128)
        self._nonlinear_fun = nonlinear_fun
        self.num_circle_points = num_circle_points
        self.circle_radius = circle_radius
        D = self.linear_operator.ndim - 1
        if nonlinear_fun is not None:
            N = nonlinear_fun.num_points
            D = nonlinear_fun.num_spatial_dims
        elif num_points is not None:
            N = num_points
        elif D >= 2:
            N = self.linear_operator.shape[-2]
        else:
            N = 2 * (self.linear_operator.shape[-1] - 1)
        self.num_spatial_dims = D
        self.num_points = N
        if self.linear_operator.shape[1:] != wavenumber_shape(D, N):
            raise ValueError("linear operator does not match the spatial Fourier shape")
        self._plans = {}

    def _plan(self, num_channels: int) -> Plan:
        p = self._plans.get(num_channels)
        if p is None:
            nl = self._nonlinear_fun
            desc = nl._nl_desc() if nl is not None else {"nonlin_kind": 0}
            extent = getattr(nl, "_domain_extent", 1.0) if nl is not None else 1.0
            p = Plan(num_spatial_dims=self.num_spatial_dims, num_points=self.num_points, num_channels=num_channels,
                     order=self._order, domain_extent=extent, dt=self.dt, linear_operator=self.linear_operator,
                     num_circle_points=self.num_circle_points, circle_radius=self.circle_radius, nonlin=desc)
            self._plans[num_channels] = p
        return p

    def _any_plan(self) -> Plan:
        """A plan to read the coefficient tables from (they depend on the linear operator only): an
        existing one, else one at the first channel count the nonlinear function accepts among the
        linear operator's, the number of spatial dimensions, 2 and 3 (projected convection, for one,
        takes 3 channels with a single-channel operator)."""
        if self._plans:
            return next(iter(self._plans.values()))
        nl = self._nonlinear_fun
        for C in (self.linear_operator.shape[0], self.num_spatial_dims, 2, 3):
            if nl is not None:
                try:
                    nl._check_channels(C)
                except ValueError:
                    continue
            return self._plan(C)
        return self._plan(self.linear_operator.shape[0])

    @property
    def _exp_term(self):
        return self._any_plan().table(0)

    @property
    def _half_exp_term(self):
        return self._any_plan().table(1)

    def _coef(self, i):
        return self._any_plan().table(1 + i)

    _coef_1 = property(lambda self: self._coef(1))
    _coef_2 = property(lambda self: self._coef(2))
    _coef_3 = property(lambda self: self._coef(3))
    _coef_4 = property(lambda self: self._coef(4))
    _coef_5 = property(lambda self: self._coef(5))
    _coef_6 = property(lambda self: self._coef(6))

    def _run(self, u_hat, batched: bool, nsteps: int = 1):
        t, back = _device.to_device(u_hat, "complex64")
        D = self.num_spatial_dims
        C = t.shape[-D - 1]
        if self._nonlinear_fun is not None:
            self._nonlinear_fun._check_channels(C)
        B = t.shape[0] if batched else 1
        out = _device.empty(t.shape, "complex64")
        plan = self._plan(C)
        check(load().exgb_repeat_fourier(plan.handle, _device.stream(), _device.ptr(t), _device.ptr(out), B,
                                         nsteps), type(self).__name__)
        return back(out)

    def step_fourier(self, u_hat):
        """One ETDRK step in Fourier space (single sample (C, N..., N//2+1))."""
        return self._run(u_hat, batched=False)

    def _batched_step_fourier(self, u_hat):
        return self._run(u_hat, batched=True)


class ETDRK0(BaseETDRK):
    """etdrk/_etdrk_0.py:6-34: exact linear step u^ <- E u^."""

    _order = 0

    def __init__(self, dt, linear_operator, *, num_points=None):
        super().__init__(dt, linear_operator, None, num_points=num_points)


class ETDRK1(BaseETDRK):
    """etdrk/_etdrk_1.py:10-82"""

    _order = 1

    def __init__(self, dt, linear_operator, nonlinear_fun, *, num_circle_points=16, circle_radius=1.0):
        super().__init__(dt, linear_operator, nonlinear_fun, num_circle_points=num_circle_points,
                         circle_radius=circle_radius)


class ETDRK2(ETDRK1):
    """etdrk/_etdrk_2.py:10-102"""

    _order = 2


class ETDRK3(ETDRK1):
    """etdrk/_etdrk_3.py:10-212"""

    _order = 3


class ETDRK4(ETDRK1):
    """etdrk/_etdrk_4.py:10-224 (Cox-Matthews)"""

    _order = 4


def make_integrator(order, dt, linear_operator, nonlinear_fun, num_circle_points=16, circle_radius=1.0):
    """Order dispatch of BaseStepper.__init__ (_base_stepper.py:119-157)."""
    if order == 0:
        return ETDRK0(dt, linear_operator, num_points=nonlinear_fun.num_points)
    cls = {1: ETDRK1, 2: ETDRK2, 3: ETDRK3, 4: ETDRK4}.get(order)
    if cls is None:
        raise NotImplementedError(f"Order {order} not implemented.")
    if isinstance(nonlinear_fun, ZeroNonlinearFun):
        pass
    return cls(dt, linear_operator, nonlinear_fun, num_circle_points=num_circle_points, circle_radius=circle_radius)
