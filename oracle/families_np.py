"""NumPy restatement of exponax's reaction-diffusion and generic stepper families.

TEST INFRASTRUCTURE ONLY, like ``oracle/exponax_np.py`` on which it builds:
only ``tests/`` may import it; the product package never does.

Follows exponax 0.2.0:
  stepper/reaction/_fisher_kpp.py, _allen_cahn.py, _cahn_hilliard.py,
  _gray_scott.py, _swift_hohenberg.py, _belousov_zhabotinsky.py (each stepper
  and its nonlinear function);
  stepper/generic/_linear.py, _convection.py, _gradient_norm.py,
  _polynomial.py, _nonlinear.py, _vorticity_convection.py, _utils.py
  (General / Normalized / Difficulty steppers and the coefficient algebra).
"""

from __future__ import annotations

import numpy as np

from .exponax_np import (BaseNonlinearFun, BaseStepper, ConvectionNonlinearFun, GeneralNonlinearFun,
                         GradientNormNonlinearFun, PolynomialNonlinearFun, VorticityConvection2d,
                         VorticityConvection2dKolmogorov, ZeroNonlinearFun, build_laplace_operator)


# --------------------------------------------------------------------------
# reaction nonlinear functions
# --------------------------------------------------------------------------
class CahnHilliardNonlinearFun(BaseNonlinearFun):
    """stepper/reaction/_cahn_hilliard.py:12-45: scale * Lap F[u^3] (dealias applied before the ifft)."""

    def __init__(self, num_spatial_dims, num_points, *, derivative_operator, dealiasing_fraction, scale=1.0,
                 dtype="float32"):
        super().__init__(num_spatial_dims, num_points, dealiasing_fraction=dealiasing_fraction, dtype=dtype)
        self.laplace_operator = build_laplace_operator(derivative_operator)
        self.scale = scale

    def __call__(self, u_hat):
        u = self.ifft(self.dealias(u_hat))
        u_power_hat = self.fft(u[0] ** 3)
        return self.laplace_operator * u_power_hat * self.scale


class GrayScottNonlinearFun(BaseNonlinearFun):
    """stepper/reaction/_gray_scott.py:9-46"""

    def __init__(self, num_spatial_dims, num_points, *, dealiasing_fraction, feed_rate, kill_rate, dtype="float32"):
        super().__init__(num_spatial_dims, num_points, dealiasing_fraction=dealiasing_fraction, dtype=dtype)
        self.feed_rate = feed_rate
        self.kill_rate = kill_rate

    def __call__(self, u_hat):
        if u_hat.shape[0] != 2:
            raise ValueError("num_channels must be 2")
        u = self.ifft(self.dealias(u_hat))
        u_power = np.stack([
            self.feed_rate * (1 - u[0]) - u[0] * u[1] ** 2,
            -(self.feed_rate + self.kill_rate) * u[1] + u[0] * u[1] ** 2,
        ])
        return self.fft(u_power)


class BelousovZhabotinskyNonlinearFun(BaseNonlinearFun):
    """stepper/reaction/_belousov_zhabotinsky.py:14-51"""

    def __init__(self, num_spatial_dims, num_points, *, dealiasing_fraction, dtype="float32"):
        super().__init__(num_spatial_dims, num_points, dealiasing_fraction=dealiasing_fraction, dtype=dtype)

    def __call__(self, u_hat):
        if u_hat.shape[0] != 3:
            raise ValueError("num_channels must be 3")
        u = self.ifft(self.dealias(u_hat))
        u_power = np.stack([
            u[0] + u[1] - u[0] * u[1] - u[0] ** 2,
            u[2] - u[1] - u[0] * u[1],
            u[0] - u[2],
        ])
        return self.fft(u_power)


# --------------------------------------------------------------------------
# reaction steppers
# --------------------------------------------------------------------------
class FisherKPP(BaseStepper):
    """stepper/reaction/_fisher_kpp.py: L = nu Lap + r; N = F[-r u^2]."""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, diffusivity=0.01, reactivity=1.0, order=2,
                 dealiasing_fraction=2 / 3, num_circle_points=16, circle_radius=1.0, dtype="float32"):
        self.diffusivity = diffusivity
        self.reactivity = reactivity
        self.dealiasing_fraction = dealiasing_fraction
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=1, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius, dtype=dtype)

    def _build_linear_operator(self, d):
        return self.diffusivity * build_laplace_operator(d, order=2) + self.reactivity

    def _build_nonlinear_fun(self, d):
        return PolynomialNonlinearFun(self.num_spatial_dims, self.num_points,
                                      dealiasing_fraction=self.dealiasing_fraction,
                                      coefficients=[0.0, 0.0, -self.reactivity], dtype=self.dtype)


class AllenCahn(BaseStepper):
    """stepper/reaction/_allen_cahn.py: L = nu Lap + c1; N = F[c3 u^3]."""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, diffusivity=5e-3,
                 first_order_coefficient=1.0, third_order_coefficient=-1.0, order=2, dealiasing_fraction=1 / 2,
                 num_circle_points=16, circle_radius=1.0, dtype="float32"):
        self.diffusivity = diffusivity
        self.first_order_coefficient = first_order_coefficient
        self.third_order_coefficient = third_order_coefficient
        self.dealiasing_fraction = dealiasing_fraction
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=1, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius, dtype=dtype)

    def _build_linear_operator(self, d):
        return self.diffusivity * build_laplace_operator(d, order=2) + self.first_order_coefficient

    def _build_nonlinear_fun(self, d):
        return PolynomialNonlinearFun(self.num_spatial_dims, self.num_points,
                                      dealiasing_fraction=self.dealiasing_fraction,
                                      coefficients=[0.0, 0.0, 0.0, self.third_order_coefficient], dtype=self.dtype)


class CahnHilliard(BaseStepper):
    """stepper/reaction/_cahn_hilliard.py:48-158: L = nu Lap (c1 - gamma Lap); N = nu c3 Lap F[u^3]."""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, diffusivity=1e-2, gamma=1e-3,
                 first_order_coefficient=-1.0, third_order_coefficient=1.0, order=2, dealiasing_fraction=1 / 2,
                 num_circle_points=16, circle_radius=1.0, dtype="float32"):
        self.diffusivity = diffusivity
        self.gamma = gamma
        self.first_order_coefficient = first_order_coefficient
        self.third_order_coefficient = third_order_coefficient
        self.dealiasing_fraction = dealiasing_fraction
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=1, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius, dtype=dtype)

    def _build_linear_operator(self, d):
        lap = build_laplace_operator(d, order=2)
        return self.diffusivity * lap * (self.first_order_coefficient - self.gamma * lap)

    def _build_nonlinear_fun(self, d):
        return CahnHilliardNonlinearFun(self.num_spatial_dims, self.num_points, derivative_operator=d,
                                        dealiasing_fraction=self.dealiasing_fraction,
                                        scale=self.diffusivity * self.third_order_coefficient, dtype=self.dtype)


class GrayScott(BaseStepper):
    """stepper/reaction/_gray_scott.py:49-180: two species, L = (nu1 Lap, nu2 Lap)."""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, diffusivity_1=2e-5, diffusivity_2=1e-5,
                 feed_rate=0.04, kill_rate=0.06, order=2, dealiasing_fraction=1 / 2, num_circle_points=16,
                 circle_radius=1.0, dtype="float32"):
        self.diffusivity_1 = diffusivity_1
        self.diffusivity_2 = diffusivity_2
        self.feed_rate = feed_rate
        self.kill_rate = kill_rate
        self.dealiasing_fraction = dealiasing_fraction
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=2, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius, dtype=dtype)

    def _build_linear_operator(self, d):
        lap = build_laplace_operator(d, order=2)
        return np.concatenate([self.diffusivity_1 * lap, self.diffusivity_2 * lap])

    def _build_nonlinear_fun(self, d):
        return GrayScottNonlinearFun(self.num_spatial_dims, self.num_points,
                                     dealiasing_fraction=self.dealiasing_fraction, feed_rate=self.feed_rate,
                                     kill_rate=self.kill_rate, dtype=self.dtype)


class BelousovZhabotinsky(BaseStepper):
    """stepper/reaction/_belousov_zhabotinsky.py:54-118: three species, L = (nu_i Lap)."""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, diffusivities=(1e-5, 2e-5, 1e-5), order=2,
                 dealiasing_fraction=1 / 2, num_circle_points=16, circle_radius=1.0, dtype="float32"):
        self.diffusivities = diffusivities
        self.dealiasing_fraction = dealiasing_fraction
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=3, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius, dtype=dtype)

    def _build_linear_operator(self, d):
        lap = build_laplace_operator(d, order=2)
        return np.concatenate([nu * lap for nu in self.diffusivities])

    def _build_nonlinear_fun(self, d):
        return BelousovZhabotinskyNonlinearFun(self.num_spatial_dims, self.num_points,
                                               dealiasing_fraction=self.dealiasing_fraction, dtype=self.dtype)


class SwiftHohenberg(BaseStepper):
    """stepper/reaction/_swift_hohenberg.py: L = r - (k + Lap)^2; N = F[sum_i c_i u^i]."""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, reactivity=0.7, critical_number=1.0,
                 polynomial_coefficients=(0.0, 0.0, 1.0, -1.0), order=2, dealiasing_fraction=1 / 2,
                 num_circle_points=16, circle_radius=1.0, dtype="float32"):
        self.reactivity = reactivity
        self.critical_number = critical_number
        self.polynomial_coefficients = polynomial_coefficients
        self.dealiasing_fraction = dealiasing_fraction
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=1, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius, dtype=dtype)

    def _build_linear_operator(self, d):
        lap = build_laplace_operator(d, order=2)
        return self.reactivity - (self.critical_number + lap) ** 2

    def _build_nonlinear_fun(self, d):
        return PolynomialNonlinearFun(self.num_spatial_dims, self.num_points,
                                      dealiasing_fraction=self.dealiasing_fraction,
                                      coefficients=self.polynomial_coefficients, dtype=self.dtype)


# --------------------------------------------------------------------------
# generic steppers: coefficient algebra (stepper/generic/_utils.py)
# --------------------------------------------------------------------------
def normalize_coefficients(coefficients, *, domain_extent, dt):
    """_utils.py: alpha_i = a_i dt / L^i"""
    return tuple(c * dt / domain_extent**i for i, c in enumerate(coefficients))


def denormalize_coefficients(normalized_coefficients, *, domain_extent, dt):
    return tuple(c / dt * domain_extent**i for i, c in enumerate(normalized_coefficients))


def normalize_convection_scale(convection_scale, *, domain_extent, dt):
    return convection_scale * dt / domain_extent


def denormalize_convection_scale(normalized_convection_scale, *, domain_extent, dt):
    return normalized_convection_scale / dt * domain_extent


def normalize_gradient_norm_scale(gradient_norm_scale, *, domain_extent, dt):
    return gradient_norm_scale * dt / domain_extent**2


def denormalize_gradient_norm_scale(normalized_gradient_norm_scale, *, domain_extent, dt):
    return normalized_gradient_norm_scale / dt * domain_extent**2


def normalize_polynomial_scales(polynomial_scales, *, domain_extent=None, dt):
    return tuple(c * dt for c in polynomial_scales)


def denormalize_polynomial_scales(normalized_polynomial_scales, *, domain_extent=None, dt):
    return tuple(c / dt for c in normalized_polynomial_scales)


def reduce_normalized_coefficients_to_difficulty(normalized_coefficients, *, num_spatial_dims, num_points):
    """gamma_j = alpha_j N^j 2^(j-1) D, gamma_0 = alpha_0"""
    out = [a * num_points**j * 2 ** (j - 1) * num_spatial_dims for j, a in enumerate(normalized_coefficients)]
    out[0] = normalized_coefficients[0]
    return tuple(out)


def extract_normalized_coefficients_from_difficulty(difficulty_coefficients, *, num_spatial_dims, num_points):
    out = [g / (num_points**j * 2 ** (j - 1) * num_spatial_dims) for j, g in enumerate(difficulty_coefficients)]
    out[0] = difficulty_coefficients[0]
    return tuple(out)


def reduce_normalized_convection_scale_to_difficulty(normalized_convection_scale, *, num_spatial_dims, num_points,
                                                     maximum_absolute):
    return normalized_convection_scale * maximum_absolute * num_points * num_spatial_dims


def extract_normalized_convection_scale_from_difficulty(difficulty_convection_scale, *, num_spatial_dims, num_points,
                                                        maximum_absolute):
    return difficulty_convection_scale / (maximum_absolute * num_points * num_spatial_dims)


def reduce_normalized_gradient_norm_scale_to_difficulty(normalized_gradient_norm_scale, *, num_spatial_dims,
                                                        num_points, maximum_absolute):
    return normalized_gradient_norm_scale * maximum_absolute * num_points**2 * num_spatial_dims


def extract_normalized_gradient_norm_scale_from_difficulty(difficulty_gradient_norm_scale, *, num_spatial_dims,
                                                           num_points, maximum_absolute):
    return difficulty_gradient_norm_scale / (maximum_absolute * num_points**2 * num_spatial_dims)


def extract_normalized_nonlinear_scales_from_difficulty(nonlinear_difficulties, *, num_spatial_dims, num_points,
                                                        maximum_absolute):
    kw = dict(num_spatial_dims=num_spatial_dims, num_points=num_points, maximum_absolute=maximum_absolute)
    return (nonlinear_difficulties[0],
            extract_normalized_convection_scale_from_difficulty(nonlinear_difficulties[1], **kw),
            extract_normalized_gradient_norm_scale_from_difficulty(nonlinear_difficulties[2], **kw))


def _isotropic_linear(d, coefficients):
    """sum_i sum_axis a_i (ik_axis)^i (note a_0 is summed over the D axes)."""
    return sum(np.sum(c * d**i, axis=0, keepdims=True) for i, c in enumerate(coefficients))


# --------------------------------------------------------------------------
# generic steppers
# --------------------------------------------------------------------------
class GeneralLinearStepper(BaseStepper):
    """generic/_linear.py: ETDRK0 with L = sum_i a_i (1 . grad)^i."""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, linear_coefficients=(0.0, -0.1, 0.01),
                 dtype="float32"):
        self.linear_coefficients = linear_coefficients
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=1, order=0, dtype=dtype)

    def _build_linear_operator(self, d):
        return _isotropic_linear(d, self.linear_coefficients)

    def _build_nonlinear_fun(self, d):
        return ZeroNonlinearFun(self.num_spatial_dims, self.num_points, dtype=self.dtype)


class GeneralConvectionStepper(BaseStepper):
    """generic/_convection.py:12-152"""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, linear_coefficients=(0.0, 0.0, 0.01),
                 convection_scale=1.0, single_channel=False, conservative=False, order=2, dealiasing_fraction=2 / 3,
                 num_circle_points=16, circle_radius=1.0, dtype="float32"):
        self.linear_coefficients = linear_coefficients
        self.convection_scale = convection_scale
        self.single_channel = single_channel
        self.conservative = conservative
        self.dealiasing_fraction = dealiasing_fraction
        nc = 1 if single_channel else num_spatial_dims
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=nc, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius, dtype=dtype)

    def _build_linear_operator(self, d):
        return _isotropic_linear(d, self.linear_coefficients)

    def _build_nonlinear_fun(self, d):
        return ConvectionNonlinearFun(self.num_spatial_dims, self.num_points, derivative_operator=d,
                                      dealiasing_fraction=self.dealiasing_fraction, scale=self.convection_scale,
                                      single_channel=self.single_channel, conservative=self.conservative,
                                      dtype=self.dtype)


class GeneralGradientNormStepper(BaseStepper):
    """generic/_gradient_norm.py:12-130"""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *,
                 linear_coefficients=(0.0, 0.0, -1.0, 0.0, -1.0), gradient_norm_scale=1.0, order=2,
                 dealiasing_fraction=2 / 3, num_circle_points=16, circle_radius=1.0, dtype="float32"):
        self.linear_coefficients = linear_coefficients
        self.gradient_norm_scale = gradient_norm_scale
        self.dealiasing_fraction = dealiasing_fraction
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=1, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius, dtype=dtype)

    def _build_linear_operator(self, d):
        return _isotropic_linear(d, self.linear_coefficients)

    def _build_nonlinear_fun(self, d):
        return GradientNormNonlinearFun(self.num_spatial_dims, self.num_points, derivative_operator=d,
                                        dealiasing_fraction=self.dealiasing_fraction, scale=self.gradient_norm_scale,
                                        zero_mode_fix=True, dtype=self.dtype)


class GeneralPolynomialStepper(BaseStepper):
    """generic/_polynomial.py:10-120"""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, linear_coefficients=(10.0, 0.0, 1.0),
                 polynomial_coefficients=(0.0, 0.0, -10.0), order=2, dealiasing_fraction=2 / 3, num_circle_points=16,
                 circle_radius=1.0, dtype="float32"):
        self.linear_coefficients = linear_coefficients
        self.polynomial_coefficients = polynomial_coefficients
        self.dealiasing_fraction = dealiasing_fraction
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=1, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius, dtype=dtype)

    def _build_linear_operator(self, d):
        return _isotropic_linear(d, self.linear_coefficients)

    def _build_nonlinear_fun(self, d):
        return PolynomialNonlinearFun(self.num_spatial_dims, self.num_points,
                                      dealiasing_fraction=self.dealiasing_fraction,
                                      coefficients=self.polynomial_coefficients, dtype=self.dtype)


class GeneralNonlinearStepper(BaseStepper):
    """generic/_nonlinear.py:12-140"""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, linear_coefficients=(0.0, 0.0, 0.01),
                 nonlinear_coefficients=(0.0, -1.0, 0.0), order=2, dealiasing_fraction=2 / 3, num_circle_points=16,
                 circle_radius=1.0, dtype="float32"):
        if len(nonlinear_coefficients) != 3:
            raise ValueError("The nonlinear coefficients list must have exactly 3 elements")
        self.linear_coefficients = linear_coefficients
        self.nonlinear_coefficients = nonlinear_coefficients
        self.dealiasing_fraction = dealiasing_fraction
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=1, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius, dtype=dtype)

    def _build_linear_operator(self, d):
        return _isotropic_linear(d, self.linear_coefficients)

    def _build_nonlinear_fun(self, d):
        return GeneralNonlinearFun(self.num_spatial_dims, self.num_points, derivative_operator=d,
                                   dealiasing_fraction=self.dealiasing_fraction,
                                   scale_list=self.nonlinear_coefficients, zero_mode_fix=True, dtype=self.dtype)


class GeneralVorticityConvectionStepper(BaseStepper):
    """generic/_vorticity_convection.py:7-142"""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, vorticity_convection_scale=1.0,
                 linear_coefficients=(0.0, 0.0, 0.001), injection_mode=4, injection_scale=0.0, order=2,
                 dealiasing_fraction=2 / 3, num_circle_points=16, circle_radius=1.0, dtype="float32"):
        if num_spatial_dims != 2:
            raise ValueError(f"Expected num_spatial_dims = 2, got {num_spatial_dims}.")
        self.vorticity_convection_scale = vorticity_convection_scale
        self.linear_coefficients = linear_coefficients
        self.injection_mode = injection_mode
        self.injection_scale = injection_scale
        self.dealiasing_fraction = dealiasing_fraction
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=1, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius, dtype=dtype)

    def _build_linear_operator(self, d):
        return _isotropic_linear(d, self.linear_coefficients)

    def _build_nonlinear_fun(self, d):
        if self.injection_scale == 0.0:
            return VorticityConvection2d(self.num_spatial_dims, self.num_points,
                                         convection_scale=self.vorticity_convection_scale, derivative_operator=d,
                                         dealiasing_fraction=self.dealiasing_fraction, dtype=self.dtype)
        return VorticityConvection2dKolmogorov(self.num_spatial_dims, self.num_points,
                                               convection_scale=self.vorticity_convection_scale,
                                               derivative_operator=d, dealiasing_fraction=self.dealiasing_fraction,
                                               injection_mode=self.injection_mode,
                                               injection_scale=self.injection_scale, dtype=self.dtype)


class NormalizedLinearStepper(GeneralLinearStepper):
    """generic/_linear.py: L = 1, dt = 1."""

    def __init__(self, num_spatial_dims, num_points, *, normalized_linear_coefficients=(0.0, -0.5, 0.01),
                 dtype="float32"):
        self.normalized_linear_coefficients = normalized_linear_coefficients
        super().__init__(num_spatial_dims, 1.0, num_points, 1.0, linear_coefficients=normalized_linear_coefficients,
                         dtype=dtype)


class DifficultyLinearStepper(NormalizedLinearStepper):
    def __init__(self, num_spatial_dims=1, num_points=48, *, linear_difficulties=(0.0, -2.0), dtype="float32"):
        self.linear_difficulties = linear_difficulties
        super().__init__(num_spatial_dims, num_points, normalized_linear_coefficients=(
            extract_normalized_coefficients_from_difficulty(linear_difficulties, num_spatial_dims=num_spatial_dims,
                                                            num_points=num_points)), dtype=dtype)


class NormalizedConvectionStepper(GeneralConvectionStepper):
    def __init__(self, num_spatial_dims, num_points, *, normalized_linear_coefficients=(0.0, 0.0, 0.01 * 0.1),
                 normalized_convection_scale=1.0 * 0.1, **kw):
        self.normalized_linear_coefficients = normalized_linear_coefficients
        self.normalized_convection_scale = normalized_convection_scale
        super().__init__(num_spatial_dims, 1.0, num_points, 1.0, linear_coefficients=normalized_linear_coefficients,
                         convection_scale=normalized_convection_scale, **kw)


class DifficultyConvectionStepper(NormalizedConvectionStepper):
    def __init__(self, num_spatial_dims=1, num_points=48, *, linear_difficulties=(0.0, 0.0, 4.5),
                 convection_difficulty=5.0, maximum_absolute=1.0, **kw):
        g = dict(num_spatial_dims=num_spatial_dims, num_points=num_points)
        super().__init__(num_spatial_dims, num_points,
                         normalized_linear_coefficients=extract_normalized_coefficients_from_difficulty(
                             linear_difficulties, **g),
                         normalized_convection_scale=extract_normalized_convection_scale_from_difficulty(
                             convection_difficulty, maximum_absolute=maximum_absolute, **g), **kw)


class NormalizedGradientNormStepper(GeneralGradientNormStepper):
    def __init__(self, num_spatial_dims, num_points, *,
                 normalized_linear_coefficients=(0.0, 0.0, -1.0 * 0.1 / 60.0**2, 0.0, -1.0 * 0.1 / 60.0**4),
                 normalized_gradient_norm_scale=1.0 * 0.1 / 60.0**2, **kw):
        super().__init__(num_spatial_dims, 1.0, num_points, 1.0, linear_coefficients=normalized_linear_coefficients,
                         gradient_norm_scale=normalized_gradient_norm_scale, **kw)


class DifficultyGradientNormStepper(NormalizedGradientNormStepper):
    def __init__(self, num_spatial_dims=1, num_points=48, *, linear_difficulties=(0.0, 0.0, -0.128, 0.0, -0.32768),
                 gradient_norm_difficulty=0.064, maximum_absolute=1.0, **kw):
        g = dict(num_spatial_dims=num_spatial_dims, num_points=num_points)
        super().__init__(num_spatial_dims, num_points,
                         normalized_linear_coefficients=extract_normalized_coefficients_from_difficulty(
                             linear_difficulties, **g),
                         normalized_gradient_norm_scale=extract_normalized_gradient_norm_scale_from_difficulty(
                             gradient_norm_difficulty, maximum_absolute=maximum_absolute, **g), **kw)


class NormalizedPolynomialStepper(GeneralPolynomialStepper):
    def __init__(self, num_spatial_dims, num_points, *,
                 normalized_linear_coefficients=(10.0 * 0.001 / 10.0**0, 0.0, 1.0 * 0.001 / 10.0**2),
                 normalized_polynomial_coefficients=(0.0, 0.0, -10.0 * 0.001), **kw):
        super().__init__(num_spatial_dims, 1.0, num_points, 1.0, linear_coefficients=normalized_linear_coefficients,
                         polynomial_coefficients=normalized_polynomial_coefficients, **kw)


class DifficultyPolynomialStepper(NormalizedPolynomialStepper):
    def __init__(self, num_spatial_dims=1, num_points=48, *,
                 linear_difficulties=(10.0 * 0.001 / 10.0**0 * 48**0, 0.0, 1.0 * 0.001 / 10.0**2 * 48**2 * 2**1),
                 polynomial_difficulties=(0.0, 0.0, -10.0 * 0.001), **kw):
        super().__init__(num_spatial_dims, num_points,
                         normalized_linear_coefficients=extract_normalized_coefficients_from_difficulty(
                             linear_difficulties, num_spatial_dims=num_spatial_dims, num_points=num_points),
                         normalized_polynomial_coefficients=polynomial_difficulties, **kw)


class NormalizedNonlinearStepper(GeneralNonlinearStepper):
    def __init__(self, num_spatial_dims, num_points, *, normalized_linear_coefficients=(0.0, 0.0, 0.1 * 0.1),
                 normalized_nonlinear_coefficients=(0.0, -1.0 * 0.1, 0.0), **kw):
        super().__init__(num_spatial_dims, 1.0, num_points, 1.0, linear_coefficients=normalized_linear_coefficients,
                         nonlinear_coefficients=normalized_nonlinear_coefficients, **kw)


class DifficultyNonlinearStepper(NormalizedNonlinearStepper):
    def __init__(self, num_spatial_dims=1, num_points=48, *,
                 linear_difficulties=(0.0, 0.0, 0.1 * 0.1 / 1.0 * 48**2 * 2),
                 nonlinear_difficulties=(0.0, -1.0 * 0.1 / 1.0 * 48, 0.0), maximum_absolute=1.0, **kw):
        g = dict(num_spatial_dims=num_spatial_dims, num_points=num_points)
        super().__init__(num_spatial_dims, num_points,
                         normalized_linear_coefficients=extract_normalized_coefficients_from_difficulty(
                             linear_difficulties, **g),
                         normalized_nonlinear_coefficients=extract_normalized_nonlinear_scales_from_difficulty(
                             nonlinear_difficulties, maximum_absolute=maximum_absolute, **g), **kw)


class DifficultyLinearStepperSimple(DifficultyLinearStepper):
    """generic/_linear.py"""

    def __init__(self, num_spatial_dims=1, num_points=48, *, difficulty=-2.0, order=1, dtype="float32"):
        super().__init__(num_spatial_dims, num_points, linear_difficulties=(0.0,) * order + (difficulty,),
                         dtype=dtype)
