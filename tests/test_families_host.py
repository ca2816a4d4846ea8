"""Host-side assembly of the reaction-diffusion and generic stepper families
(no GPU): linear operators, nonlinear-function descriptors and the generic
coefficient algebra against the oracle, and the error paths that the Python
layer raises before any device work."""

import warnings

import numpy as np
import pytest

import exponax_gb300 as ex
from exponax_gb300 import generic as gm
from oracle import families_np as f

REACTION = [
    ("FisherKPP", (2, 1.0, 32, 0.001), dict(diffusivity=0.02, reactivity=5.0)),
    ("AllenCahn", (1, 6.0, 64, 0.01), dict(first_order_coefficient=2.0)),
    ("CahnHilliard", (3, 2.0, 16, 0.001), dict(gamma=2e-3)),
    ("GrayScott", (2, 1.0, 32, 1.0), dict(feed_rate=0.03, kill_rate=0.05)),
    ("SwiftHohenberg", (2, 20.0, 32, 0.1), dict(critical_number=0.8)),
    ("BelousovZhabotinsky", (2, 1.0, 32, 0.01), dict(diffusivities=(1e-3, 3e-3, 2e-3))),
]


@pytest.mark.parametrize("name,args,kw", REACTION)
def test_reaction_linear_operators(name, args, kw):
    sm = getattr(ex.stepper.reaction, name)(*args, **kw)
    so = getattr(f, name)(*args, **kw)
    assert sm.num_channels == so.num_channels
    np.testing.assert_allclose(sm.linear_operator, so.linear_operator, rtol=2e-6, atol=1e-6 * np.abs(
        so.linear_operator).max())


def test_reaction_descriptors():
    gs = ex.stepper.reaction.GrayScott(2, 1.0, 32, 1.0, feed_rate=0.03, kill_rate=0.05)
    d = gs.nonlinear_fun._nl_desc()
    assert d["nonlin_kind"] == 10 and d["reaction"] == (0.03, 0.05) and d["dealiasing_fraction"] == 0.5
    ch = ex.stepper.reaction.CahnHilliard(2, 1.0, 32, 0.001, diffusivity=0.02, third_order_coefficient=3.0)
    d = ch.nonlinear_fun._nl_desc()
    assert d["nonlin_kind"] == 9 and d["scale"] == pytest.approx(0.06)
    fk = ex.stepper.reaction.FisherKPP(1, 1.0, 64, 0.001, reactivity=4.0)
    assert fk.nonlinear_fun._nl_desc()["poly"] == (0.0, 0.0, -4.0)
    plan = gs.plan.desc()
    assert plan.nonlin_kind == 10 and tuple(plan.reaction) == (0.03, 0.05) and plan.num_channels == 2
    bz = ex.stepper.reaction.BelousovZhabotinsky(1, 1.0, 64, 0.01)
    d = bz.nonlinear_fun._nl_desc()
    assert d["nonlin_kind"] == 11 and d["dealiasing_fraction"] == 0.5 and bz.num_channels == 3
    with pytest.raises(ValueError, match="3"):
        bz.nonlinear_fun._check_channels(2)


GENERIC = [
    ("GeneralLinearStepper", dict(num_spatial_dims=2, domain_extent=1.0, num_points=32, dt=0.01)),
    ("GeneralConvectionStepper", dict(num_spatial_dims=3, domain_extent=2.0, num_points=16, dt=0.01)),
    ("GeneralGradientNormStepper", dict(num_spatial_dims=2, domain_extent=30.0, num_points=32, dt=0.05)),
    ("GeneralPolynomialStepper", dict(num_spatial_dims=1, domain_extent=10.0, num_points=64, dt=0.001)),
    ("GeneralNonlinearStepper", dict(num_spatial_dims=2, domain_extent=1.0, num_points=32, dt=0.001)),
    ("GeneralVorticityConvectionStepper", dict(num_spatial_dims=2, domain_extent=6.0, num_points=32, dt=0.01,
                                               injection_scale=1.0)),
    ("NormalizedLinearStepper", dict(num_spatial_dims=2, num_points=32)),
    ("NormalizedConvectionStepper", dict(num_spatial_dims=2, num_points=32)),
    ("NormalizedGradientNormStepper", dict(num_spatial_dims=1, num_points=64)),
    ("NormalizedPolynomialStepper", dict(num_spatial_dims=2, num_points=32)),
    ("NormalizedNonlinearStepper", dict(num_spatial_dims=3, num_points=16)),
    ("DifficultyLinearStepper", dict(num_spatial_dims=2, num_points=40)),
    ("DifficultyLinearStepperSimple", dict(num_spatial_dims=1, difficulty=-3.0, order=3)),
    ("DifficultyConvectionStepper", dict(num_spatial_dims=2, num_points=32, maximum_absolute=2.0)),
    ("DifficultyGradientNormStepper", dict()),
    ("DifficultyPolynomialStepper", dict(num_spatial_dims=3, num_points=16)),
    ("DifficultyNonlinearStepper", dict(num_spatial_dims=2, num_points=48)),
]


@pytest.mark.parametrize("name,kw", GENERIC)
def test_generic_linear_operators(name, kw):
    sm = getattr(gm, name)(**kw)
    so = getattr(f, name)(**kw)
    assert (sm.num_spatial_dims, sm.num_points, sm.num_channels, sm.dt) == (
        so.num_spatial_dims, so.num_points, so.num_channels, so.dt)
    scale = max(np.abs(so.linear_operator).max(), 1e-30)
    np.testing.assert_allclose(sm.linear_operator, so.linear_operator, rtol=2e-6, atol=1e-6 * scale)


def test_generic_coefficient_algebra_roundtrips():
    c = (0.3, -1.2, 0.05, 0.0, -2e-4)
    for D, N, L, dt in [(1, 48, 3.0, 0.1), (2, 64, 1.0, 0.01), (3, 32, 20.0, 0.5)]:
        n = gm.normalize_coefficients(c, domain_extent=L, dt=dt)
        assert n == f.normalize_coefficients(c, domain_extent=L, dt=dt)
        np.testing.assert_allclose(gm.denormalize_coefficients(n, domain_extent=L, dt=dt), c, rtol=1e-12)
        g = gm.reduce_normalized_coefficients_to_difficulty(n, num_spatial_dims=D, num_points=N)
        assert g == f.reduce_normalized_coefficients_to_difficulty(n, num_spatial_dims=D, num_points=N)
        np.testing.assert_allclose(gm.extract_normalized_coefficients_from_difficulty(g, num_spatial_dims=D,
                                                                                      num_points=N), n, rtol=1e-12)
        kw = dict(num_spatial_dims=D, num_points=N, maximum_absolute=1.5)
        s = (0.2, -0.7, 0.4)
        r = gm.reduce_normalized_nonlinear_scales_to_difficulty(s, **kw)
        np.testing.assert_allclose(gm.extract_normalized_nonlinear_scales_from_difficulty(r, **kw), s, rtol=1e-12)
        assert gm.normalize_gradient_norm_scale(0.5, domain_extent=L, dt=dt) == pytest.approx(0.5 * dt / L**2)
        assert gm.denormalize_convection_scale(gm.normalize_convection_scale(0.5, domain_extent=L, dt=dt),
                                               domain_extent=L, dt=dt) == pytest.approx(0.5)
        assert gm.denormalize_polynomial_scales(gm.normalize_polynomial_scales((1.0, 2.0), dt=dt),
                                                dt=dt) == pytest.approx((1.0, 2.0))


def test_generic_errors_and_deprecation():
    with pytest.raises(ValueError):
        gm.GeneralVorticityConvectionStepper(3, 1.0, 16, 0.1)
    with pytest.raises(ValueError):
        gm.GeneralNonlinearStepper(1, 1.0, 32, 0.1, nonlinear_coefficients=(1.0, 2.0))
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        s = gm.DiffultyLinearStepperSimple(num_spatial_dims=1, difficulty=-1.0)
    assert any(issubclass(x.category, DeprecationWarning) for x in w)
    assert isinstance(s, gm.DifficultyLinearStepperSimple)


def test_stepper_subpackages_are_exposed():
    assert ex.stepper.generic is gm
    assert ex.stepper.reaction.FisherKPP.__name__ == "FisherKPP"
