"""Concrete PDE steppers (exponax/stepper/*) on the GB300 ETDRK path.

Each class assembles its linear operator and nonlinear function exactly as
the reference constructor does (host, once), then all stepping runs on the
GPU.  ``__call__`` checks the single-sample shape (C, N, ..., N) like the
reference; batches go through :func:`exponax_gb300.vmap`.
"""

from __future__ import annotations

import numpy as np

from . import _device
from ._lib import check, load
from .etdrk import make_integrator
from .nonlin_fun import (ConvectionNonlinearFun, GradientNormNonlinearFun, ProjectedConvection3d,
                         ProjectedConvection3dKolmogorov, VorticityConvection2d, VorticityConvection2dKolmogorov,
                         ZeroNonlinearFun)
from .spectral import (build_derivative_operator, build_gradient_inner_product_operator, build_laplace_operator,
                       spatial_shape, wavenumber_shape)


class BaseStepper:
    """_base_stepper.py:17-271"""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, num_channels, order,
                 num_circle_points=16, circle_radius=1.0):
        self.num_spatial_dims = num_spatial_dims
        self.domain_extent = domain_extent
        self.num_points = num_points
        self.dt = dt
        self.num_channels = num_channels
        self.dx = domain_extent / num_points
        self.order = order
        derivative_operator = build_derivative_operator(num_spatial_dims, domain_extent, num_points)
        lin = np.asarray(self._build_linear_operator(derivative_operator))
        ws = wavenumber_shape(num_spatial_dims, num_points)
        if lin.shape not in ((1,) + ws, (num_channels,) + ws):
            raise ValueError(
                f"Expected linear operator to have shape {(1,) + ws} or {(num_channels,) + ws}, got {lin.shape}."
            )
        self.linear_operator = lin
        nl = self._build_nonlinear_fun(derivative_operator)
        nl._domain_extent = domain_extent
        self.nonlinear_fun = nl
        self._integrator = make_integrator(order, dt, lin, nl, num_circle_points, circle_radius)

    def _build_linear_operator(self, derivative_operator):
        raise NotImplementedError

    def _build_nonlinear_fun(self, derivative_operator):
        raise NotImplementedError

    # ------------------------------------------------------------------ device plan
    @property
    def plan(self):
        return self._integrator._plan(self.num_channels)

    def set_dft_precision(self, mode: str = "fp32"):
        """Arithmetic of the transforms of the 2D vorticity steppers (no
        reference counterpart): "fp32" (default, FP32 FFTs) or "split_bf16"
        (dense DFT contractions on the tcgen05 tensor cores in split-BF16
        three-product form with FP32 accumulation; N = 128, dealiasing on).
        Returns the stepper."""
        self.plan.set_precision(mode)
        return self

    def _phys(self, u, batched: bool):
        t, back = _device.to_device(u, "float32")
        expected = (self.num_channels,) + spatial_shape(self.num_spatial_dims, self.num_points)
        got = tuple(t.shape[1:]) if batched else tuple(t.shape)
        if got != expected:
            raise ValueError(
                f"Expected shape {expected}, got {got}. For batched operation use exponax_gb300.vmap on the stepper."
            )
        return t, back, (t.shape[0] if batched else 1)

    # ------------------------------------------------------------------ reference API
    def step(self, u):
        """_base_stepper.py:201-220: fft -> step_fourier -> ifft."""
        return self._step(u, batched=False)

    def _step(self, u, batched):
        t, back, B = self._phys(u, batched)
        out = _device.empty(t.shape, "float32")
        check(load().exgb_step(self.plan.handle, _device.stream(), _device.ptr(t), _device.ptr(out), B),
              type(self).__name__)
        return back(out)

    def step_fourier(self, u_hat):
        """_base_stepper.py:222-239"""
        return self._integrator.step_fourier(u_hat)

    def __call__(self, u):
        """_base_stepper.py:241-271 (shape-checked single sample)."""
        return self.step(u)

    def _batched(self, u):
        return self._step(u, batched=True)

    def _batched_step_fourier(self, u_hat):
        return self._integrator._batched_step_fourier(u_hat)

    # fused multi-step paths used by rollout / repeat / RepeatedStepper
    def _repeat(self, u, n, batched):
        t, back, B = self._phys(u, batched)
        out = _device.empty(t.shape, "float32")
        check(load().exgb_repeat(self.plan.handle, _device.stream(), _device.ptr(t), _device.ptr(out), B, n),
              "repeat")
        return back(out)

    def _rollout(self, u, n, include_init, batched):
        t, back, B = self._phys(u, batched)
        T = n + (1 if include_init else 0)
        shape = ((B,) if batched else ()) + (T,) + tuple(t.shape[1:] if batched else t.shape)
        out = _device.empty(shape, "float32")
        check(load().exgb_rollout(self.plan.handle, _device.stream(), _device.ptr(t), _device.ptr(out), B, n,
                                  int(bool(include_init))), "rollout")
        return back(out)

    def _repeat_fourier(self, u_hat, n, batched):
        t, back = _device.to_device(u_hat, "complex64")
        B = t.shape[0] if batched else 1
        out = _device.empty(t.shape, "complex64")
        check(load().exgb_repeat_fourier(self.plan.handle, _device.stream(), _device.ptr(t), _device.ptr(out), B,
                                         n), "repeat_fourier")
        return back(out)


# ---------------------------------------------------------------------- concrete steppers

class KuramotoSivashinsky(BaseStepper):
    """stepper/_kuramoto_sivashinsky.py:8-168 (combustion / gradient-norm form)."""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, gradient_norm_scale=1.0,
                 second_order_scale=1.0, fourth_order_scale=1.0, dealiasing_fraction=2 / 3, order=2,
                 num_circle_points=16, circle_radius=1.0):
        self.gradient_norm_scale = gradient_norm_scale
        self.second_order_scale = second_order_scale
        self.fourth_order_scale = fourth_order_scale
        self.dealiasing_fraction = dealiasing_fraction
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=1, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius)

    def _build_linear_operator(self, d):
        return (-self.second_order_scale * build_laplace_operator(d, order=2)
                - self.fourth_order_scale * build_laplace_operator(d, order=4))

    def _build_nonlinear_fun(self, d):
        return GradientNormNonlinearFun(self.num_spatial_dims, self.num_points, derivative_operator=d,
                                        dealiasing_fraction=self.dealiasing_fraction, zero_mode_fix=True,
                                        scale=self.gradient_norm_scale)


class KuramotoSivashinskyConservative(BaseStepper):
    """stepper/_kuramoto_sivashinsky.py:171-315 (convection form)."""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, convection_scale=1.0,
                 second_order_scale=1.0, fourth_order_scale=1.0, single_channel=False, conservative=True,
                 dealiasing_fraction=2 / 3, order=2, num_circle_points=16, circle_radius=1.0):
        self.convection_scale = convection_scale
        self.second_order_scale = second_order_scale
        self.fourth_order_scale = fourth_order_scale
        self.single_channel = single_channel
        self.conservative = conservative
        self.dealiasing_fraction = dealiasing_fraction
        num_channels = 1 if single_channel else num_spatial_dims
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=num_channels, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius)

    def _build_linear_operator(self, d):
        return (-self.second_order_scale * build_laplace_operator(d, order=2)
                - self.fourth_order_scale * build_laplace_operator(d, order=4))

    def _build_nonlinear_fun(self, d):
        return ConvectionNonlinearFun(self.num_spatial_dims, self.num_points, derivative_operator=d,
                                      dealiasing_fraction=self.dealiasing_fraction, scale=self.convection_scale,
                                      single_channel=self.single_channel, conservative=self.conservative)


class Burgers(BaseStepper):
    """stepper/_burgers.py:8-155"""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, diffusivity=0.1, convection_scale=1.0,
                 single_channel=False, conservative=False, order=2, dealiasing_fraction=2 / 3,
                 num_circle_points=16, circle_radius=1.0):
        self.diffusivity = diffusivity
        self.convection_scale = convection_scale
        self.single_channel = single_channel
        self.conservative = conservative
        self.dealiasing_fraction = dealiasing_fraction
        num_channels = 1 if single_channel else num_spatial_dims
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=num_channels, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius)

    def _build_linear_operator(self, d):
        return self.diffusivity * build_laplace_operator(d)

    def _build_nonlinear_fun(self, d):
        return ConvectionNonlinearFun(self.num_spatial_dims, self.num_points, derivative_operator=d,
                                      dealiasing_fraction=self.dealiasing_fraction, scale=self.convection_scale,
                                      single_channel=self.single_channel, conservative=self.conservative)


class KortewegDeVries(BaseStepper):
    """stepper/_korteweg_de_vries.py:13-216"""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, convection_scale=-6.0, diffusivity=0.0,
                 dispersivity=1.0, hyper_diffusivity=0.01, advect_over_diffuse=False, diffuse_over_diffuse=False,
                 single_channel=False, conservative=False, order=2, dealiasing_fraction=2 / 3,
                 num_circle_points=16, circle_radius=1.0):
        self.convection_scale = convection_scale
        self.diffusivity = diffusivity
        self.dispersivity = dispersivity
        self.hyper_diffusivity = hyper_diffusivity
        self.advect_over_diffuse = advect_over_diffuse
        self.diffuse_over_diffuse = diffuse_over_diffuse
        self.single_channel = single_channel
        self.conservative = conservative
        self.dealiasing_fraction = dealiasing_fraction
        num_channels = 1 if single_channel else num_spatial_dims
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=num_channels, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius)

    def _build_linear_operator(self, d):
        velocity = self.dispersivity * np.ones(self.num_spatial_dims)
        lap = build_laplace_operator(d, order=2)
        diffusion = self.diffusivity * lap
        if self.advect_over_diffuse:
            dispersion = -build_gradient_inner_product_operator(d, velocity, order=1) * lap
        else:
            dispersion = -build_gradient_inner_product_operator(d, velocity, order=3)
        if self.diffuse_over_diffuse:
            hyper = -self.hyper_diffusivity * lap * lap
        else:
            hyper = -self.hyper_diffusivity * build_laplace_operator(d, order=4)
        return diffusion + dispersion + hyper

    def _build_nonlinear_fun(self, d):
        return ConvectionNonlinearFun(self.num_spatial_dims, self.num_points, derivative_operator=d,
                                      dealiasing_fraction=self.dealiasing_fraction, scale=self.convection_scale,
                                      single_channel=self.single_channel, conservative=self.conservative)


class NavierStokesVorticity(BaseStepper):
    """stepper/_navier_stokes.py:13-153: L = nu Lap + drag."""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, diffusivity=0.01,
                 vorticity_convection_scale=1.0, drag=0.0, order=2, dealiasing_fraction=2 / 3,
                 num_circle_points=16, circle_radius=1.0):
        if num_spatial_dims != 2:
            raise ValueError(f"Expected num_spatial_dims = 2, got {num_spatial_dims}. "
                             "For 3D, use NavierStokesVelocity instead.")
        self.diffusivity = diffusivity
        self.vorticity_convection_scale = vorticity_convection_scale
        self.drag = drag
        self.dealiasing_fraction = dealiasing_fraction
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=1, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius)

    def _build_linear_operator(self, d):
        return self.diffusivity * build_laplace_operator(d, order=2) + self.drag * build_laplace_operator(d, order=0)

    def _build_nonlinear_fun(self, d):
        return VorticityConvection2d(self.num_spatial_dims, self.num_points,
                                     convection_scale=self.vorticity_convection_scale, derivative_operator=d,
                                     dealiasing_fraction=self.dealiasing_fraction)


class KolmogorovFlowVorticity(BaseStepper):
    """stepper/_navier_stokes.py:156-327"""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, diffusivity=0.001, convection_scale=1.0,
                 drag=-0.1, injection_mode=4, injection_scale=1.0, order=2, dealiasing_fraction=2 / 3,
                 num_circle_points=16, circle_radius=1.0):
        if num_spatial_dims != 2:
            raise ValueError(f"Expected num_spatial_dims = 2, got {num_spatial_dims}. "
                             "For 3D, use KolmogorovFlowVelocity instead.")
        self.diffusivity = diffusivity
        self.convection_scale = convection_scale
        self.drag = drag
        self.injection_mode = injection_mode
        self.injection_scale = injection_scale
        self.dealiasing_fraction = dealiasing_fraction
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=1, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius)

    def _build_linear_operator(self, d):
        return self.diffusivity * build_laplace_operator(d, order=2) + self.drag * build_laplace_operator(d, order=0)

    def _build_nonlinear_fun(self, d):
        return VorticityConvection2dKolmogorov(self.num_spatial_dims, self.num_points,
                                               convection_scale=self.convection_scale,
                                               injection_mode=self.injection_mode,
                                               injection_scale=self.injection_scale, derivative_operator=d,
                                               dealiasing_fraction=self.dealiasing_fraction)


class NavierStokesVelocity(BaseStepper):
    """stepper/_navier_stokes.py:330-463: 3D velocity form with the projected
    convection (Leray) nonlinearity; L = nu Lap + drag."""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, diffusivity=0.01, drag=0.0, order=2,
                 dealiasing_fraction=2 / 3, num_circle_points=16, circle_radius=1.0):
        if num_spatial_dims != 3:
            raise ValueError(f"Expected num_spatial_dims = 3, got {num_spatial_dims}. "
                             "For 2D, use NavierStokesVorticity instead.")
        self.diffusivity = diffusivity
        self.drag = drag
        self.dealiasing_fraction = dealiasing_fraction
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=3, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius)

    def _build_linear_operator(self, d):
        return self.diffusivity * build_laplace_operator(d, order=2) + self.drag * build_laplace_operator(d, order=0)

    def _build_nonlinear_fun(self, d):
        return ProjectedConvection3d(self.num_spatial_dims, self.num_points, derivative_operator=d,
                                     dealiasing_fraction=self.dealiasing_fraction)


class KolmogorovFlowVelocity(BaseStepper):
    """stepper/_navier_stokes.py:466-598: 3D Kolmogorov flow (forcing on the
    first velocity channel at mode (0, k, 0))."""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, diffusivity=0.01, drag=0.0,
                 injection_mode=4, injection_scale=1.0, order=2, dealiasing_fraction=2 / 3, num_circle_points=16,
                 circle_radius=1.0):
        if num_spatial_dims != 3:
            raise ValueError(f"Expected num_spatial_dims = 3, got {num_spatial_dims}. "
                             "For 2D, use KolmogorovFlowVorticity instead.")
        self.diffusivity = diffusivity
        self.drag = drag
        self.injection_mode = injection_mode
        self.injection_scale = injection_scale
        self.dealiasing_fraction = dealiasing_fraction
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=3, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius)

    def _build_linear_operator(self, d):
        return self.diffusivity * build_laplace_operator(d, order=2) + self.drag * build_laplace_operator(d, order=0)

    def _build_nonlinear_fun(self, d):
        return ProjectedConvection3dKolmogorov(self.num_spatial_dims, self.num_points,
                                               injection_mode=self.injection_mode,
                                               injection_scale=self.injection_scale, derivative_operator=d,
                                               dealiasing_fraction=self.dealiasing_fraction)


class _LinearStepper(BaseStepper):
    def _build_nonlinear_fun(self, d):
        return ZeroNonlinearFun(self.num_spatial_dims, self.num_points)


def _diffusivity_matrix(num_spatial_dims, diffusivity):
    """stepper/_diffusion.py:84-89"""
    if np.isscalar(diffusivity):
        return np.eye(num_spatial_dims) * diffusivity
    diffusivity = np.asarray(diffusivity, dtype=np.float64)
    return np.diag(diffusivity) if diffusivity.ndim == 1 else diffusivity


class Advection(_LinearStepper):
    """stepper/_advection.py:13-104"""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, velocity=1.0):
        self.velocity = np.ones(num_spatial_dims) * velocity if np.isscalar(velocity) else np.asarray(velocity)
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=1, order=0)

    def _build_linear_operator(self, d):
        return -build_gradient_inner_product_operator(d, self.velocity, order=1)


class Diffusion(_LinearStepper):
    """stepper/_diffusion.py:12-122"""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, diffusivity=0.01):
        self.diffusivity = _diffusivity_matrix(num_spatial_dims, diffusivity)
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=1, order=0)

    def _build_linear_operator(self, d):
        return np.einsum("ij,ij...->...", self.diffusivity, d[:, None] * d[None, :])[None, ...]


class AdvectionDiffusion(_LinearStepper):
    """stepper/_advection_diffusion.py:107-128"""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, velocity=1.0, diffusivity=0.01):
        self.velocity = np.ones(num_spatial_dims) * velocity if np.isscalar(velocity) else np.asarray(velocity)
        self.diffusivity = _diffusivity_matrix(num_spatial_dims, diffusivity)
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=1, order=0)

    def _build_linear_operator(self, d):
        diff = np.einsum("ij,ij...->...", self.diffusivity, d[:, None] * d[None, :])[None, ...]
        return -build_gradient_inner_product_operator(d, self.velocity, order=1) + diff


class Dispersion(_LinearStepper):
    """stepper/_dispersion.py:102-117"""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, dispersivity=1.0,
                 advect_on_diffusion=False):
        self.dispersivity = (np.ones(num_spatial_dims) * dispersivity if np.isscalar(dispersivity)
                             else np.asarray(dispersivity))
        self.advect_on_diffusion = advect_on_diffusion
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=1, order=0)

    def _build_linear_operator(self, d):
        if self.advect_on_diffusion:
            return build_gradient_inner_product_operator(d, self.dispersivity, order=1) * build_laplace_operator(d)
        return build_gradient_inner_product_operator(d, self.dispersivity, order=3)


class HyperDiffusion(_LinearStepper):
    """stepper/_hyper_diffusion.py:95-110"""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, hyper_diffusivity=0.0001,
                 diffuse_on_diffuse=False):
        self.hyper_diffusivity = hyper_diffusivity
        self.diffuse_on_diffuse = diffuse_on_diffuse
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=1, order=0)

    def _build_linear_operator(self, d):
        if self.diffuse_on_diffuse:
            lap = build_laplace_operator(d)
            return -self.hyper_diffusivity * lap * lap
        return -self.hyper_diffusivity * build_laplace_operator(d, order=4)


class Wave(_LinearStepper):
    """stepper/_wave.py:8-197: the wave equation h_tt = c^2 Lap h as the system (h, v = h_t), advanced
    exactly.  The reference diagonalises per mode (w = i c |k| h, pos/neg = (w +- v)/sqrt(2), ETDRK0
    factors exp(+-i c |k| dt)) and adds dt v to the mean of h.  Composed, one step is the real map
      h' = cos(t) h + sin(t)/(c |k|) v,  v' = -c |k| sin(t) h + cos(t) v,  t = c |k| dt,
    and h' = h + dt v, v' = v at k = 0.  It is built once in FP64 (from the float32 |k| the reference
    uses) and applied on the device by exgb_mode_mix2, n steps per launch for repeat."""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, speed_of_sound=1.0):
        from .spectral import build_scaled_wavenumbers

        self.speed_of_sound = speed_of_sound
        k = build_scaled_wavenumbers(num_spatial_dims, domain_extent, num_points).astype(np.float32)
        self.wavenumber_norm = np.linalg.norm(k, axis=0, keepdims=True)
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=2, order=0)
        kn = self.wavenumber_norm.astype(np.float64).reshape(-1)
        c = float(speed_of_sound)
        th = c * kn * dt
        safe = np.where(kn == 0, 1.0, c * kn)
        m = np.stack([np.cos(th), np.where(kn == 0, dt, np.sin(th) / safe), -c * kn * np.sin(th), np.cos(th)])
        self._mix = m.astype(np.float32)
        self._mix_dev = None

    def _build_linear_operator(self, d):
        val = 1j * self.speed_of_sound * self.wavenumber_norm
        return np.concatenate((val, -val), axis=0)

    def _mix_table(self):
        if self._mix_dev is None:
            self._mix_dev = _device.torch().from_numpy(np.ascontiguousarray(self._mix)).cuda()
        return self._mix_dev

    def _apply(self, t_hat, B, n, out=None):
        per = self._mix.shape[1]
        out = _device.empty(t_hat.shape, "complex64") if out is None else out
        check(load().exgb_mode_mix2(_device.stream(), B, per, _device.ptr(self._mix_table()), _device.ptr(t_hat),
                                    _device.ptr(out), int(n)), "Wave")
        return out

    def _fourier(self, u_hat, n, batched):
        t, back = _device.to_device(u_hat, "complex64")
        ws = (2,) + wavenumber_shape(self.num_spatial_dims, self.num_points)
        got = tuple(t.shape[1:]) if batched else tuple(t.shape)
        if got != ws:
            raise ValueError(f"Expected Fourier shape {ws}, got {got}")
        return back(self._apply(t, t.shape[0] if batched else 1, n))

    def step_fourier(self, u_hat):
        return self._fourier(u_hat, 1, batched=False)

    def _batched_step_fourier(self, u_hat):
        return self._fourier(u_hat, 1, batched=True)

    def _repeat_fourier(self, u_hat, n, batched):
        return self._fourier(u_hat, n, batched)

    def _phys_steps(self, u, n, batched):
        from .spectral import fft, ifft

        t, back, B = self._phys(u, batched)
        D = self.num_spatial_dims
        hat = fft(t, num_spatial_dims=D)
        return ifft(self._apply(hat, B, n), num_spatial_dims=D, num_points=self.num_points), back

    def _step(self, u, batched):
        out, back = self._phys_steps(u, 1, batched)
        return back(out)

    def _repeat(self, u, n, batched):
        # the map is real and even in k, so it keeps rfftn spectra Hermitian: the reference's
        # per-step irfftn -> rfftn round trip changes nothing and the n steps run in one launch
        if n == 0:
            t, back, _ = self._phys(u, batched)
            return back(t.clone())
        out, back = self._phys_steps(u, n, batched)
        return back(out)

    def _rollout(self, u, n, include_init, batched):
        from .spectral import fft, ifft

        torch = _device.torch()
        t, back, B = self._phys(u, batched)
        D = self.num_spatial_dims
        hat = fft(t, num_spatial_dims=D)
        frames = [t] if include_init else []
        for _ in range(n):
            hat = self._apply(hat, B, 1)
            frames.append(ifft(hat, num_spatial_dims=D, num_points=self.num_points))
        if not frames:
            shape = ((B,) if batched else ()) + (0,) + tuple(t.shape[1:] if batched else t.shape)
            return back(_device.empty(shape, "float32"))
        return back(torch.stack(frames, dim=1 if batched else 0).contiguous())


# the reference's stepper sub-packages (stepper/generic, stepper/reaction)
from . import generic, reaction  # noqa: E402
