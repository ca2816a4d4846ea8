"""Reaction-diffusion steppers (exponax/stepper/reaction/*) on the GB300 ETDRK path.

FisherKPP, AllenCahn and SwiftHohenberg use the polynomial nonlinearity;
CahnHilliard, GrayScott and BelousovZhabotinsky bring their own nonlinear
functions.  In 2D and 3D (and the multi-species steppers in 1D) they run on
the staged N-D path of libexgb.so; the 1D single-species polynomial steppers
on the fused 1D kernel.  BelousovZhabotinsky is defined but not exported by the
reference (its module calls it experimental); it is importable from here as it
is from the reference's module.
"""

from __future__ import annotations

import numpy as np

from ._lib import NL_BELOUSOV_ZHABOTINSKY, NL_CAHN_HILLIARD, NL_GRAY_SCOTT
from .nonlin_fun import BaseNonlinearFun, PolynomialNonlinearFun, _extent_from_derivative
from .spectral import build_laplace_operator
from .stepper import BaseStepper


class CahnHilliardNonlinearFun(BaseNonlinearFun):
    """stepper/reaction/_cahn_hilliard.py:12-45: scale * Lap F[u^3] of the
    dealiased first channel."""

    _kind = NL_CAHN_HILLIARD

    def __init__(self, num_spatial_dims, num_points, *, derivative_operator, dealiasing_fraction, scale=1.0):
        super().__init__(num_spatial_dims, num_points, dealiasing_fraction=dealiasing_fraction)
        self.laplace_operator = build_laplace_operator(derivative_operator)
        self.scale = scale
        self._domain_extent = _extent_from_derivative(derivative_operator, num_points)

    def _nl_desc(self):
        d = super()._nl_desc()
        d.update(scale=self.scale)
        return d

    def _check_channels(self, C):
        if self.dealiasing_mask is None:
            raise ValueError("Nonlinear function was set up without dealiasing")


class GrayScottNonlinearFun(BaseNonlinearFun):
    """stepper/reaction/_gray_scott.py:9-46: F[f (1 - u0) - u0 u1^2], F[-(f + k) u1 + u0 u1^2]."""

    _kind = NL_GRAY_SCOTT

    def __init__(self, num_spatial_dims, num_points, *, dealiasing_fraction, feed_rate, kill_rate):
        super().__init__(num_spatial_dims, num_points, dealiasing_fraction=dealiasing_fraction)
        self.feed_rate = feed_rate
        self.kill_rate = kill_rate

    def _nl_desc(self):
        d = super()._nl_desc()
        d.update(reaction=(self.feed_rate, self.kill_rate))
        return d

    def _check_channels(self, C):
        if C != 2:
            raise ValueError("num_channels must be 2")
        if self.dealiasing_mask is None:
            raise ValueError("Nonlinear function was set up without dealiasing")


class BelousovZhabotinskyNonlinearFun(BaseNonlinearFun):
    """stepper/reaction/_belousov_zhabotinsky.py:14-51: three species,
    F[u0 + u1 - u0 u1 - u0^2], F[u2 - u1 - u0 u1], F[u0 - u2] of the dealiased state."""

    _kind = NL_BELOUSOV_ZHABOTINSKY

    def __init__(self, num_spatial_dims, num_points, *, dealiasing_fraction):
        super().__init__(num_spatial_dims, num_points, dealiasing_fraction=dealiasing_fraction)

    def _check_channels(self, C):
        if C != 3:
            raise ValueError("num_channels must be 3")
        if self.dealiasing_mask is None:
            raise ValueError("Nonlinear function was set up without dealiasing")


class FisherKPP(BaseStepper):
    """stepper/reaction/_fisher_kpp.py: u_t = nu Lap u + r u (1 - u)."""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, diffusivity=0.01, reactivity=1.0, order=2,
                 dealiasing_fraction=2 / 3, num_circle_points=16, circle_radius=1.0):
        self.diffusivity = diffusivity
        self.reactivity = reactivity
        self.dealiasing_fraction = dealiasing_fraction
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=1, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius)

    def _build_linear_operator(self, d):
        return self.diffusivity * build_laplace_operator(d, order=2) + self.reactivity

    def _build_nonlinear_fun(self, d):
        return PolynomialNonlinearFun(self.num_spatial_dims, self.num_points,
                                      dealiasing_fraction=self.dealiasing_fraction,
                                      coefficients=[0.0, 0.0, -self.reactivity])


class AllenCahn(BaseStepper):
    """stepper/reaction/_allen_cahn.py: u_t = nu Lap u + c1 u + c3 u^3."""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, diffusivity=5e-3,
                 first_order_coefficient=1.0, third_order_coefficient=-1.0, order=2, dealiasing_fraction=1 / 2,
                 num_circle_points=16, circle_radius=1.0):
        self.diffusivity = diffusivity
        self.first_order_coefficient = first_order_coefficient
        self.third_order_coefficient = third_order_coefficient
        self.dealiasing_fraction = dealiasing_fraction
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=1, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius)

    def _build_linear_operator(self, d):
        return self.diffusivity * build_laplace_operator(d, order=2) + self.first_order_coefficient

    def _build_nonlinear_fun(self, d):
        return PolynomialNonlinearFun(self.num_spatial_dims, self.num_points,
                                      dealiasing_fraction=self.dealiasing_fraction,
                                      coefficients=[0.0, 0.0, 0.0, self.third_order_coefficient])


class CahnHilliard(BaseStepper):
    """stepper/reaction/_cahn_hilliard.py:48-158: u_t = nu Lap (c3 u^3 + c1 u - gamma Lap u)."""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, diffusivity=1e-2, gamma=1e-3,
                 first_order_coefficient=-1.0, third_order_coefficient=1.0, order=2, dealiasing_fraction=1 / 2,
                 num_circle_points=16, circle_radius=1.0):
        self.diffusivity = diffusivity
        self.gamma = gamma
        self.first_order_coefficient = first_order_coefficient
        self.third_order_coefficient = third_order_coefficient
        self.dealiasing_fraction = dealiasing_fraction
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=1, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius)

    def _build_linear_operator(self, d):
        lap = build_laplace_operator(d, order=2)
        return self.diffusivity * lap * (self.first_order_coefficient - self.gamma * lap)

    def _build_nonlinear_fun(self, d):
        return CahnHilliardNonlinearFun(self.num_spatial_dims, self.num_points, derivative_operator=d,
                                        dealiasing_fraction=self.dealiasing_fraction,
                                        scale=self.diffusivity * self.third_order_coefficient)


class GrayScott(BaseStepper):
    """stepper/reaction/_gray_scott.py:49-180: two species with diffusivities nu1, nu2."""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, diffusivity_1=2e-5, diffusivity_2=1e-5,
                 feed_rate=0.04, kill_rate=0.06, order=2, dealiasing_fraction=1 / 2, num_circle_points=16,
                 circle_radius=1.0):
        self.diffusivity_1 = diffusivity_1
        self.diffusivity_2 = diffusivity_2
        self.feed_rate = feed_rate
        self.kill_rate = kill_rate
        self.dealiasing_fraction = dealiasing_fraction
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=2, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius)

    def _build_linear_operator(self, d):
        lap = build_laplace_operator(d, order=2)
        return np.concatenate([self.diffusivity_1 * lap, self.diffusivity_2 * lap])

    def _build_nonlinear_fun(self, d):
        return GrayScottNonlinearFun(self.num_spatial_dims, self.num_points,
                                     dealiasing_fraction=self.dealiasing_fraction, feed_rate=self.feed_rate,
                                     kill_rate=self.kill_rate)


class BelousovZhabotinsky(BaseStepper):
    """stepper/reaction/_belousov_zhabotinsky.py:54-118: three species with diffusivities
    (nu0, nu1, nu2) times the Laplacian, the nonlinearity above, dealiasing 1/2 by default."""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, diffusivities=(1e-5, 2e-5, 1e-5),
                 order=2, dealiasing_fraction=1 / 2, num_circle_points=16, circle_radius=1.0):
        self.diffusivities = diffusivities
        self.dealiasing_fraction = dealiasing_fraction
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=3, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius)

    def _build_linear_operator(self, d):
        lap = build_laplace_operator(d, order=2)
        return np.concatenate([nu * lap for nu in self.diffusivities])

    def _build_nonlinear_fun(self, d):
        return BelousovZhabotinskyNonlinearFun(self.num_spatial_dims, self.num_points,
                                               dealiasing_fraction=self.dealiasing_fraction)


class SwiftHohenberg(BaseStepper):
    """stepper/reaction/_swift_hohenberg.py: u_t = r u - (k + Lap)^2 u + sum_i c_i u^i."""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, reactivity=0.7, critical_number=1.0,
                 polynomial_coefficients=(0.0, 0.0, 1.0, -1.0), order=2, dealiasing_fraction=1 / 2,
                 num_circle_points=16, circle_radius=1.0):
        self.reactivity = reactivity
        self.critical_number = critical_number
        self.polynomial_coefficients = polynomial_coefficients
        self.dealiasing_fraction = dealiasing_fraction
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=1, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius)

    def _build_linear_operator(self, d):
        lap = build_laplace_operator(d, order=2)
        return self.reactivity - (self.critical_number + lap) ** 2

    def _build_nonlinear_fun(self, d):
        return PolynomialNonlinearFun(self.num_spatial_dims, self.num_points,
                                      dealiasing_fraction=self.dealiasing_fraction,
                                      coefficients=self.polynomial_coefficients)


__all__ = ["AllenCahn", "CahnHilliard", "FisherKPP", "GrayScott", "SwiftHohenberg", "CahnHilliardNonlinearFun",
           "GrayScottNonlinearFun"]
