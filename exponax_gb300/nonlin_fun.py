"""Nonlinear functions of the ETDRK path (exponax/nonlin_fun/*).

Each class records its parameters, builds the same host-side arrays as the
reference (dealiasing mask, inverse Laplacian, forcing) and evaluates
N(u^) on the GPU through ``exgb_nonlinear``.  Single samples have shape
(C, N, ..., N//2+1); use :func:`exponax_gb300.vmap` for a leading batch axis.
"""

from __future__ import annotations

import numpy as np

from . import _device
from ._lib import (NL_CONVECTION, NL_GENERAL, NL_GRADIENT_NORM, NL_POLYNOMIAL, NL_PROJECTED_3D,
                   NL_PROJECTED_3D_KOLMOGOROV, NL_VORTICITY_2D, NL_VORTICITY_2D_KOLMOGOROV, NL_ZERO, check, load)
from ._plan import Plan
from .spectral import (build_laplace_operator, build_scaling_array, build_wavenumbers, dealias_kmax,
                       low_pass_filter_mask, spatial_shape, wavenumber_shape)
from .spectral import fft as _fft
from .spectral import ifft as _ifft


class BaseNonlinearFun:
    """nonlin_fun/_base.py:9-159"""

    _kind = NL_ZERO

    def __init__(self, num_spatial_dims: int, num_points: int, *, dealiasing_fraction: float | None = None):
        self.num_spatial_dims = num_spatial_dims
        self.num_points = num_points
        self.dealiasing_fraction = dealiasing_fraction
        if dealiasing_fraction is None:
            self.dealiasing_mask = None
        else:
            highest_resolved_mode = num_points // 2
            self.dealiasing_mask = low_pass_filter_mask(
                num_spatial_dims, num_points, cutoff=dealiasing_fraction * highest_resolved_mode - 1
            )
        self._plans = {}

    # ---------------------------------------------------------------- descriptors
    def _nl_desc(self) -> dict:
        return {"nonlin_kind": self._kind, "dealiasing_fraction": self.dealiasing_fraction}

    def _check_channels(self, num_channels: int) -> None:
        pass

    def kmax(self) -> int:
        return dealias_kmax(self.dealiasing_fraction, self.num_points)

    def _plan(self, num_channels: int) -> Plan:
        p = self._plans.get(num_channels)
        if p is None:
            shape = (1,) + wavenumber_shape(self.num_spatial_dims, self.num_points)
            p = Plan(num_spatial_dims=self.num_spatial_dims, num_points=self.num_points, num_channels=num_channels,
                     order=1, domain_extent=getattr(self, "_domain_extent", 1.0), dt=1.0,
                     linear_operator=np.zeros(shape, np.complex128), nonlin=self._nl_desc())
            self._plans[num_channels] = p
        return p

    # ---------------------------------------------------------------- reference methods
    def dealias(self, u_hat):
        """_base.py:73-97"""
        if self.dealiasing_mask is None:
            raise ValueError("Nonlinear function was set up without dealiasing")
        t, back = _device.to_device(u_hat, "complex64")
        m = _device.torch().from_numpy(self.dealiasing_mask.astype(np.float32)).to(t.device)
        return back(t * m)

    def fft(self, u):
        """_base.py:99-116 (post-dealiasing)"""
        u_hat = _fft(u, num_spatial_dims=self.num_spatial_dims)
        return self.dealias(u_hat) if self.dealiasing_mask is not None else u_hat

    def ifft(self, u_hat):
        """_base.py:118-137 (pre-dealiasing)"""
        if self.dealiasing_mask is not None:
            u_hat = self.dealias(u_hat)
        return _ifft(u_hat, num_spatial_dims=self.num_spatial_dims, num_points=self.num_points)

    def _eval(self, u_hat, batched: bool):
        t, back = _device.to_device(u_hat, "complex64")
        D = self.num_spatial_dims
        expect = wavenumber_shape(D, self.num_points)
        if tuple(t.shape[-D:]) != expect:
            raise ValueError(f"Expected spatial Fourier shape {expect}, got {tuple(t.shape[-D:])}.")
        C = t.shape[-D - 1]
        self._check_channels(C)
        B = t.shape[0] if batched else 1
        out = _device.empty(t.shape, "complex64")
        plan = self._plan(C)
        check(load().exgb_nonlinear(plan.handle, _device.stream(), _device.ptr(t), _device.ptr(out), B),
              type(self).__name__)
        return back(out)

    def __call__(self, u_hat):
        return self._eval(u_hat, batched=False)

    def _batched(self, u_hat):
        return self._eval(u_hat, batched=True)


class ZeroNonlinearFun(BaseNonlinearFun):
    """nonlin_fun/_zero.py:7-38"""

    _kind = NL_ZERO

    def __init__(self, num_spatial_dims: int, num_points: int):
        super().__init__(num_spatial_dims, num_points)

    def __call__(self, u_hat):
        t, back = _device.to_device(u_hat, "complex64")
        return back(_device.torch().zeros_like(t))

    _batched = __call__


class ConvectionNonlinearFun(BaseNonlinearFun):
    """nonlin_fun/_convection.py:7-245: -b/2 div(u u) or -b u.grad u (four
    variants; single-channel forms use the sum of the derivative operators)."""

    _kind = NL_CONVECTION

    def __init__(self, num_spatial_dims, num_points, *, derivative_operator, dealiasing_fraction=2 / 3, scale=1.0,
                 single_channel=False, conservative=False):
        self.derivative_operator = derivative_operator
        self.scale = scale
        self.single_channel = single_channel
        self.conservative = conservative
        super().__init__(num_spatial_dims, num_points, dealiasing_fraction=dealiasing_fraction)
        self._domain_extent = _extent_from_derivative(derivative_operator, num_points)

    def _nl_desc(self):
        d = super()._nl_desc()
        d.update(scale=self.scale, single_channel=self.single_channel, conservative=self.conservative)
        return d

    def _check_channels(self, C):
        if not self.single_channel and C != self.num_spatial_dims:
            raise ValueError("Number of channels in u_hat should match number of spatial dimensions")


class GradientNormNonlinearFun(BaseNonlinearFun):
    """nonlin_fun/_gradient_norm.py:8-101: -b/2 (|grad u|^2 - mean)."""

    _kind = NL_GRADIENT_NORM

    def __init__(self, num_spatial_dims, num_points, *, derivative_operator, dealiasing_fraction,
                 zero_mode_fix=True, scale=1.0):
        super().__init__(num_spatial_dims, num_points, dealiasing_fraction=dealiasing_fraction)
        self.derivative_operator = derivative_operator
        self.zero_mode_fix = zero_mode_fix
        self.scale = scale
        self._domain_extent = _extent_from_derivative(derivative_operator, num_points)

    def _nl_desc(self):
        d = super()._nl_desc()
        d.update(scale=self.scale, zero_mode_fix=self.zero_mode_fix)
        return d


class PolynomialNonlinearFun(BaseNonlinearFun):
    """nonlin_fun/_polynomial.py:6-76: sum_k c_k u^k."""

    _kind = NL_POLYNOMIAL

    def __init__(self, num_spatial_dims, num_points, *, dealiasing_fraction, coefficients):
        super().__init__(num_spatial_dims, num_points, dealiasing_fraction=dealiasing_fraction)
        self.coefficients = tuple(coefficients)

    def _nl_desc(self):
        d = super()._nl_desc()
        d.update(poly=self.coefficients)
        return d


class GeneralNonlinearFun(BaseNonlinearFun):
    """nonlin_fun/_general_nonlinear.py:9-119: b0 u^2 + b1/2 (1.grad)(u^2) +
    b2/2 |grad u|^2 (scale_list = (b0, b1, b2), with the reference's signs)."""

    _kind = NL_GENERAL

    def __init__(self, num_spatial_dims, num_points, *, derivative_operator, dealiasing_fraction,
                 scale_list=(0.0, -1.0, 0.0), zero_mode_fix=True):
        if len(scale_list) != 3:
            raise ValueError("The scale list must have exactly 3 elements")
        super().__init__(num_spatial_dims, num_points, dealiasing_fraction=dealiasing_fraction)
        self.derivative_operator = derivative_operator
        self.scale_list = tuple(scale_list)
        self.zero_mode_fix = zero_mode_fix
        self._domain_extent = _extent_from_derivative(derivative_operator, num_points)

    def _nl_desc(self):
        d = super()._nl_desc()
        d.update(scale_list=self.scale_list, zero_mode_fix=self.zero_mode_fix)
        return d


class VorticityConvection2d(BaseNonlinearFun):
    """nonlin_fun/_vorticity_convection.py:8-99: psi = w / Lap (1 at k=0),
    u = d_y psi, v = -d_x psi, -b (u w_x + v w_y)."""

    _kind = NL_VORTICITY_2D

    def __init__(self, num_spatial_dims, num_points, *, convection_scale=1.0, derivative_operator,
                 dealiasing_fraction):
        if num_spatial_dims != 2:
            raise ValueError(f"Expected num_spatial_dims = 2, got {num_spatial_dims}.")
        super().__init__(num_spatial_dims, num_points, dealiasing_fraction=dealiasing_fraction)
        self.convection_scale = convection_scale
        self.derivative_operator = derivative_operator
        lap = build_laplace_operator(derivative_operator, order=2)
        with np.errstate(divide="ignore", invalid="ignore"):
            self.inv_laplacian = np.where(lap == 0, 1.0, 1.0 / lap)
        self._domain_extent = _extent_from_derivative(derivative_operator, num_points)

    def _nl_desc(self):
        d = super()._nl_desc()
        d.update(scale=self.convection_scale)
        return d

    def _check_channels(self, C):
        if C != 1:
            raise ValueError("vorticity convection acts on a single channel")


class VorticityConvection2dKolmogorov(VorticityConvection2d):
    """nonlin_fun/_vorticity_convection.py:102-182: adds the forcing
    -k gamma * coef_extraction_scaling at (k_x=0, k_y=k)."""

    _kind = NL_VORTICITY_2D_KOLMOGOROV

    def __init__(self, num_spatial_dims, num_points, *, convection_scale=1.0, injection_mode=4,
                 injection_scale=1.0, derivative_operator, dealiasing_fraction):
        super().__init__(num_spatial_dims, num_points, convection_scale=convection_scale,
                         derivative_operator=derivative_operator, dealiasing_fraction=dealiasing_fraction)
        self.injection_mode = injection_mode
        self.injection_scale = injection_scale
        wn = build_wavenumbers(num_spatial_dims, num_points)
        m = (wn[0] == 0) & (wn[1] == injection_mode)
        self.injection = np.where(
            m, -injection_mode * injection_scale * build_scaling_array(2, num_points, mode="coef_extraction"), 0.0
        )

    def _nl_desc(self):
        d = super()._nl_desc()
        d.update(injection_mode=self.injection_mode, injection_scale=self.injection_scale)
        return d


class Leray(BaseNonlinearFun):
    """nonlin_fun/_leray.py:8-136: P(u^) = u^ + ik p^, p^ = -inv_lap (ik . u^),
    inv_lap = 0 at k = 0 (GPU kernel exgb_leray; Laplace order 2)."""

    def __init__(self, num_spatial_dims, num_points, *, derivative_operator, order=2):
        super().__init__(num_spatial_dims, num_points)
        self.order = order
        lap = build_laplace_operator(derivative_operator, order=order)
        with np.errstate(divide="ignore", invalid="ignore"):
            self.inv_laplacian = np.where(lap != 0, 1.0 / lap, 0.0)
        self.derivative_operator = derivative_operator
        self._domain_extent = _extent_from_derivative(derivative_operator, num_points)

    def _eval(self, u_hat, batched: bool):
        if self.order != 2:
            raise NotImplementedError("the GPU Leray projection uses the order-2 Laplacian")
        t, back = _device.to_device(u_hat, "complex64")
        D = self.num_spatial_dims
        if t.shape[-D - 1] != D:
            raise ValueError("Leray projection needs as many channels as spatial dimensions")
        count = t.shape[0] if batched else 1
        out = _device.empty(t.shape, "complex64")
        check(load().exgb_leray(_device.stream(), D, self.num_points, self._domain_extent, count, _device.ptr(t),
                                _device.ptr(out)), "Leray")
        return back(out)


class ProjectedConvection3d(BaseNonlinearFun):
    """nonlin_fun/_projected_convection.py:19-136: P F[u x (curl u)]."""

    _kind = NL_PROJECTED_3D

    def __init__(self, num_spatial_dims, num_points, *, derivative_operator, dealiasing_fraction=2 / 3):
        if num_spatial_dims != 3:
            raise ValueError("ProjectedConvection3d only supports 3 spatial dimensions.")
        super().__init__(num_spatial_dims, num_points, dealiasing_fraction=dealiasing_fraction)
        self.derivative_operator = derivative_operator
        self.leray_projection = Leray(num_spatial_dims, num_points, derivative_operator=derivative_operator)
        self._domain_extent = _extent_from_derivative(derivative_operator, num_points)

    def _check_channels(self, C):
        if C != 3:
            raise ValueError("Number of channels in u_hat should match number of spatial dimensions")


class ProjectedConvection3dKolmogorov(ProjectedConvection3d):
    """nonlin_fun/_projected_convection.py:139-226: forcing gamma * scaling
    at (0, k, 0) on the first velocity channel."""

    _kind = NL_PROJECTED_3D_KOLMOGOROV

    def __init__(self, num_spatial_dims, num_points, *, injection_mode=4, injection_scale=1.0,
                 derivative_operator, dealiasing_fraction):
        super().__init__(num_spatial_dims, num_points, derivative_operator=derivative_operator,
                         dealiasing_fraction=dealiasing_fraction)
        self.injection_mode = injection_mode
        self.injection_scale = injection_scale
        wn = build_wavenumbers(num_spatial_dims, num_points)
        m = (wn[0] == 0) & (wn[1] == injection_mode) & (wn[2] == 0)
        single = np.where(m, injection_scale * build_scaling_array(3, num_points, mode="coef_extraction"), 0.0)
        self.injection = np.concatenate([single, np.zeros_like(single), np.zeros_like(single)], axis=0)

    def _nl_desc(self):
        d = super()._nl_desc()
        d.update(injection_mode=self.injection_mode, injection_scale=self.injection_scale)
        return d


def _extent_from_derivative(derivative_operator, num_points) -> float:
    """Recover L from the derivative operator i 2 pi k / L (k = 1 mode of
    the last axis), so that plans rebuild the same scaled wavenumbers."""
    d = np.asarray(derivative_operator)
    last = d[-1]
    idx = (0,) * (last.ndim - 1) + (1,)
    k1 = float(np.imag(last[idx])) if last.shape[-1] > 1 else 0.0
    if k1 == 0.0:
        return 1.0
    return 2 * np.pi / k1
