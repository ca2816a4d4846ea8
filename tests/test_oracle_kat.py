"""Pin the NumPy oracle against the reference's own golden vectors and
known-answer tests (exponax 0.2.0 ``tests/`` and ``validation/``).

These run on CPU only.  Each test names the reference test it restates."""

import json
import os

import numpy as np
import pytest

from oracle import exponax_np as o

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


# ---------------------------------------------------------------- golden data

def _mask_cases():
    with open(os.path.join(GOLDEN, "filter_masks.json")) as f:
        return json.load(f)["cases"]


@pytest.mark.parametrize("case", _mask_cases(), ids=lambda c: f"{c['fn']}{tuple(c['args'])}{c['kwargs']}")
def test_filter_masks_golden(case):
    """tests/test_filter_masks.py (all 14 literal arrays)."""
    fn = getattr(o, case["fn"])
    got = fn(*case["args"], **case["kwargs"])
    exp = case["expected"]
    if isinstance(exp, dict):
        exp = np.ones(exp["ones_shape"], dtype=bool)
    np.testing.assert_array_equal(got, np.array(exp))


def _slice_cases():
    with open(os.path.join(GOLDEN, "mode_slices.json")) as f:
        return json.load(f)["cases"]


@pytest.mark.parametrize("case", _slice_cases(), ids=lambda c: str(tuple(c["args"])))
def test_mode_slices_golden(case):
    """tests/test_mode_slices_generation.py"""
    got = o.get_modes_slices(*case["args"])
    exp = tuple(tuple(slice(*s) for s in block) for block in case["expected"])
    assert got == exp


# ---------------------------------------------------------------- spectral

@pytest.mark.parametrize("D", [1, 2, 3])
def test_fft_ifft_roundtrip(D):
    """tests/test_spectral.py:19-31 (abs 1e-5)."""
    N = 16 if D == 3 else 32
    u = np.random.default_rng(0).standard_normal((1,) + (N,) * D).astype(np.float32)
    back = o.ifft(o.fft(u), num_spatial_dims=D, num_points=N)
    np.testing.assert_allclose(back, u, atol=1e-5)


@pytest.mark.parametrize("D,N", [(D, N) for D in (1, 2, 3) for N in (10, 11)])
def test_scaling_array_norm_compensation(D, N):
    """tests/test_spectral_scaling_arrays.py:8-37: backward-norm rfft divided
    by the norm_compensation array equals the forward-norm rfft."""
    u = np.random.default_rng(0).standard_normal((1,) + (N,) * D)
    axes = tuple(range(-D, 0))
    a = np.fft.rfftn(u, axes=axes) / o.build_scaling_array(D, N, mode="norm_compensation", dtype="float64")
    b = np.fft.rfftn(u, axes=axes, norm="forward")
    np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-14)


def test_derivative_of_sine_1d():
    """tests/test_spectral.py:34-84 (1D instance)."""
    L, N = 3.0, 48
    x = o.make_grid(1, L, N, dtype="float64")
    u = np.sin(2 * np.pi * x / L)
    d = o.build_derivative_operator(1, L, N, dtype="float64")
    du = o.ifft(d * o.fft(u), num_spatial_dims=1, num_points=N)
    np.testing.assert_allclose(du, 2 * np.pi / L * np.cos(2 * np.pi * x / L), atol=1e-10)


def test_laplace_eigenvalues():
    """tests/test_spectral.py:87-99, :148-156"""
    d = o.build_derivative_operator(2, 2 * np.pi, 16, dtype="float64")
    lap = o.build_laplace_operator(d, order=2)
    wn = o.build_wavenumbers(2, 16, dtype="float64")
    np.testing.assert_allclose(lap[0].real, -(wn[0] ** 2 + wn[1] ** 2))
    bih = o.build_laplace_operator(d, order=4)
    np.testing.assert_allclose(bih[0].real, wn[0] ** 4 + wn[1] ** 4)
    with pytest.raises(ValueError):
        o.build_laplace_operator(d, order=3)


def test_dealias_cutoffs_of_the_configs():
    """Kept |k| per axis for the N used on the hot path:
    floor(2/3 * (N//2) - 1), inclusive (nonlin_fun/_base.py:59-71)."""
    expect = {200: 65, 256: 84, 128: 41, 512: 169, 64: 20, 60: 19, 4096: 1364}
    for N, kmax in expect.items():
        nf = o.BaseNonlinearFun(1, N, dealiasing_fraction=2 / 3)
        kept = np.nonzero(nf.dealiasing_mask[0])[0]
        assert kept.max() == kmax, N


def test_spectrum_parseval_1d():
    """tests/test_spectrum.py (Parseval): sum(spectrum) = 0.5 mean(u^2)."""
    u = np.random.default_rng(1).standard_normal((1, 64))
    s = o.get_spectrum(u)
    np.testing.assert_allclose(s.sum(), 0.5 * np.mean(u**2), rtol=1e-10)


# ---------------------------------------------------------------- nonlinear functions

def test_convection_single_channel_kat():
    """tests/test_nonlinear_funs.py:17-52: -u u_x of sin -> -(pi/L) sin(2x')."""
    N, L = 64, 3.0
    d = o.build_derivative_operator(1, L, N)
    f = o.ConvectionNonlinearFun(1, N, derivative_operator=d, dealiasing_fraction=2 / 3, scale=1.0,
                                 single_channel=True, conservative=False)
    x = o.make_grid(1, L, N)
    u = np.sin(2 * np.pi * x / L).astype(np.float32)
    r = o.ifft(f(o.fft(u)), num_spatial_dims=1, num_points=N)
    np.testing.assert_allclose(r, -(np.pi / L) * np.sin(4 * np.pi * x / L), atol=1e-4)


def test_convection_conservative_equals_nonconservative():
    """tests/test_nonlinear_funs.py:55-93 (abs 1e-5)."""
    N, L = 64, 4.0
    d = o.build_derivative_operator(1, L, N)
    kw = dict(derivative_operator=d, dealiasing_fraction=2 / 3, scale=1.0, single_channel=True)
    fc = o.ConvectionNonlinearFun(1, N, conservative=True, **kw)
    fn = o.ConvectionNonlinearFun(1, N, conservative=False, **kw)
    x = o.make_grid(1, L, N)
    u = (0.5 * np.sin(2 * np.pi * x / L)).astype(np.float32)
    uh = o.fft(u)
    np.testing.assert_allclose(o.ifft(fc(uh), num_points=N), o.ifft(fn(uh), num_points=N), atol=1e-5)


def test_gradient_norm_zero_mode():
    """tests/test_nonlinear_funs.py:96-123"""
    N, L = 64, 3.0
    d = o.build_derivative_operator(1, L, N)
    f = o.GradientNormNonlinearFun(1, N, derivative_operator=d, dealiasing_fraction=2 / 3, zero_mode_fix=True)
    x = o.make_grid(1, L, N)
    u = (np.sin(2 * np.pi * x / L) + 0.5).astype(np.float32)
    assert abs(f(o.fft(u))[0, 0]) < 1e-5


def test_polynomial_constant_input():
    """tests/test_nonlinear_funs.py:126-152: constant c -> c0 + c1 c + c2 c^2."""
    N = 32
    f = o.PolynomialNonlinearFun(1, N, dealiasing_fraction=2 / 3, coefficients=(0.5, 2.0, -1.0))
    u = np.full((1, N), 1.5, dtype=np.float32)
    r = o.ifft(f(o.fft(u)), num_points=N)
    np.testing.assert_allclose(r, 0.5 + 2.0 * 1.5 - 1.5**2, atol=1e-5)


def test_leray_properties():
    """tests/test_nonlinear_funs.py:416-517: divergence-free, idempotent."""
    N = 16
    d = o.build_derivative_operator(3, 1.0, N, dtype="float64")
    P = o.Leray(3, N, derivative_operator=d, dtype="float64")
    u = np.random.default_rng(2).standard_normal((3, N, N, N))
    uh = o.fft(u)
    pu = P(uh)
    div = np.sum(d * pu, axis=0)
    assert np.max(np.abs(div)) < 1e-9 * np.max(np.abs(uh))
    np.testing.assert_allclose(P(pu), pu, atol=1e-9 * np.max(np.abs(uh)))


def test_projected_convection_divergence_free():
    """tests/test_nonlinear_funs.py:537-558"""
    N = 16
    d = o.build_derivative_operator(3, 2 * np.pi, N, dtype="float64")
    f = o.ProjectedConvection3d(3, N, derivative_operator=d, dtype="float64")
    rng = np.random.default_rng(3)
    u = rng.standard_normal((3, N, N, N))
    r = f(o.fft(u))
    div = np.sum(d * r, axis=0)
    assert np.max(np.abs(div)) < 1e-8 * np.max(np.abs(r))


def test_kolmogorov_injection_amplitude():
    """nonlin_fun/_vorticity_convection.py:166-176: -k*gamma*N^2/2 at (0,k), no 2pi/L."""
    N = 32
    d = o.build_derivative_operator(2, 2 * np.pi, N)
    f = o.VorticityConvection2dKolmogorov(2, N, injection_mode=4, injection_scale=1.0, derivative_operator=d,
                                          dealiasing_fraction=2 / 3)
    inj = f.injection[0]
    assert inj[0, 4] == pytest.approx(-4 * N * N / 2)
    assert np.count_nonzero(inj) == 1


def test_vorticity_inverse_laplacian_dc_is_one():
    """nonlin_fun/_vorticity_convection.py:76 vs _leray.py:108-110."""
    d = o.build_derivative_operator(2, 2 * np.pi, 8)
    assert o.VorticityConvection2d(2, 8, derivative_operator=d, dealiasing_fraction=2 / 3).inv_laplacian[0, 0, 0] == 1
    assert o.Leray(2, 8, derivative_operator=d).inv_laplacian[0, 0, 0] == 0


# ---------------------------------------------------------------- linear steppers (exact)

def test_advection_1d_exact():
    """tests/test_validation.py:13-37"""
    L, N, dt, c = 1.0, 32, 0.1, 0.1
    x = o.make_grid(1, L, N)
    st = o.Advection(1, L, N, dt, velocity=c)
    u0 = np.sin(2 * np.pi * x / L).astype(np.float32)
    np.testing.assert_allclose(st(u0), np.sin(2 * np.pi * (x - c * dt) / L), rtol=1e-4, atol=1e-5)


def test_diffusion_2d_exact():
    """tests/test_validation.py:131-168"""
    L, N, dt, nu = 2 * np.pi, 32, 0.1, 0.1
    g = o.make_grid(2, L, N)
    st = o.Diffusion(2, L, N, dt, diffusivity=nu)
    u0 = (np.sin(g[0:1]) * np.sin(2 * g[1:2])).astype(np.float32)
    np.testing.assert_allclose(st(u0), u0 * np.exp(-5 * nu * dt), atol=1e-5)


def test_poisson_1d_exact():
    """tests/test_validation.py:214-233: -u'' = f."""
    L, N = 2 * np.pi, 32
    x = o.make_grid(1, L, N, dtype="float64")
    p = o.Poisson(1, L, N, dtype="float64")
    f = 9 * np.sin(3 * x)
    np.testing.assert_allclose(p(f), np.sin(3 * x), atol=1e-6)


def test_etdrk0_exact_diffusion():
    """tests/test_etdrk.py:20-45"""
    L, N, dt, nu = 10.0, 100, 0.1, 0.1
    x = o.make_grid(1, L, N)

    def sol(t):
        return np.exp(-((4 * 2 * np.pi / L) ** 2) * nu * t) * np.sin(4 * 2 * np.pi * x / L)

    st = o.Diffusion(1, L, N, dt, diffusivity=nu)
    np.testing.assert_allclose(st(sol(0.0).astype(np.float32)), sol(dt), atol=1e-5)


def test_roots_of_unity():
    """tests/test_etdrk.py:8-17"""
    r = o.roots_of_unity(16)
    np.testing.assert_allclose(np.abs(r), 1, atol=1e-6)
    assert abs(r.sum()) < 1e-6


# ---------------------------------------------------------------- ETDRK convergence

@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_etdrk_convergence_order(order):
    """tests/test_etdrk.py:48-106: rate > order - 0.25 on Burgers."""
    L, N, nu, dt_base = 3.0, 64, 0.02, 0.2
    x = o.make_grid(1, L, N)
    u0 = np.sin(2 * np.pi * x / L).astype(np.float32)
    ref = o.repeat(o.Burgers(1, L, N, dt_base / 256, diffusivity=nu, order=4), 256)(u0)
    errs = []
    for r in (1, 2):
        st = o.Burgers(1, L, N, dt_base / r, diffusivity=nu, order=order)
        errs.append(float(np.sqrt(np.mean((o.repeat(st, r)(u0) - ref) ** 2))))
    assert np.log2(errs[0] / errs[1]) > order - 0.25


def test_higher_orders_agree_with_order_2():
    """tests/test_builtin_solvers.py:932-953 (within 5e-4 on Burgers)."""
    L, N = 1.0, 64
    x = o.make_grid(1, L, N)
    u0 = np.sin(2 * np.pi * x / L).astype(np.float32)
    base = o.Burgers(1, L, N, 0.01, diffusivity=0.01, order=2)(u0)
    for order in (3, 4):
        np.testing.assert_allclose(o.Burgers(1, L, N, 0.01, diffusivity=0.01, order=order)(u0), base, atol=5e-4)


# ---------------------------------------------------------------- validation notebooks

def test_taylor_green_published_errors():
    """validation/validate_taylor_green.ipynb cells 3-12: FP32 rel-L2 vs the
    analytic decay after 1/10/100 steps; published 1.85e-7 / 1.07e-6 / 1.00e-5.
    FFT rounding differs between backends, so allow 3x either way."""
    N, nu, dt = 60, 0.1, 0.01
    g = o.make_grid(2, 2 * np.pi, N)
    st = o.NavierStokesVorticity(2, 2 * np.pi, N, dt, diffusivity=nu)

    def tg(t):
        return (2 * np.sin(g[0:1]) * np.sin(g[1:2]) * np.exp(-2 * nu * t)).astype(np.float32)

    def rel(a, b):
        return np.linalg.norm(a - b) / np.linalg.norm(b)

    ic = tg(0.0)
    for n, pub in ((1, 1.85e-7), (10, 1.07e-6), (100, 1.00e-5)):
        e = rel(o.repeat(st, n)(ic), tg(n * dt))
        assert pub / 3 < e < pub * 3, (n, e)


def test_taylor_green_float64_is_exact():
    """The FP64 statement of the same case is exact to ~1e-13."""
    N, nu, dt = 60, 0.1, 0.01
    g = o.make_grid(2, 2 * np.pi, N, dtype="float64")
    st = o.NavierStokesVorticity(2, 2 * np.pi, N, dt, diffusivity=nu, dtype="float64")
    ic = 2 * np.sin(g[0:1]) * np.sin(g[1:2])
    u = o.repeat(st, 10)(ic)
    np.testing.assert_allclose(u, ic * np.exp(-2 * nu * 10 * dt), atol=1e-12)


def test_kdv_soliton():
    """validation/validate_kdv_against_analytical_soliton.ipynb: the soliton
    -c/2 sech^2(sqrt(c)/2 (x - c t - a)) travels with speed c (b=-6 form)."""
    L, N, dt, c, a = 20.0, 256, 1e-3, 5.0, 10.0
    x = o.make_grid(1, L, N, dtype="float64")

    def sol(t):
        return -c / 2 / np.cosh(np.sqrt(c) / 2 * (x - c * t - a)) ** 2

    def err(dt_, order):
        st = o.KortewegDeVries(1, L, N, dt_, hyper_diffusivity=0.0, order=order, dtype="float64")
        u = o.repeat(st, int(round(0.1 / dt_)))(sol(0.0))
        return np.linalg.norm(u - sol(0.1)) / np.linalg.norm(sol(0.1))

    # The notebook's comparison is qualitative; the soliton stays within 1 %.
    assert err(dt, 2) < 1e-2
    # The reference keeps only the real part of the phi-coefficients
    # (etdrk/_etdrk_2.py:80-81) although the dispersive L is imaginary, which
    # makes the scheme first order in dt whatever the ETDRK order.  The oracle
    # reproduces that quirk: the error drops 10x for a 10x smaller dt for
    # both orders 2 and 4.
    for order in (2, 4):
        ratio = err(dt, order) / err(dt / 10, order)
        assert 8 < ratio < 12, (order, ratio)


def test_repeated_stepper_matches_repeat():
    """tests/test_repeated_stepper.py:8-29 (rel 1e-3)."""
    st = o.KuramotoSivashinskyConservative(1, 60.0, 64, 0.05)
    u0 = np.sin(2 * np.pi * o.make_grid(1, 60.0, 64) / 60.0).astype(np.float32)
    a = o.RepeatedStepper(st, 5)(u0)
    b = o.repeat(st, 5)(u0)
    np.testing.assert_allclose(a, b, rtol=1e-3, atol=1e-5)


def test_map_between_resolutions_roundtrip():
    """tests/test_interpolation.py: band-limited fields map exactly."""
    N0, N1 = 64, 32
    g = o.make_grid(2, 2 * np.pi, N0, dtype="float64")
    u = np.sin(3 * g[0:1]) * np.cos(2 * g[1:2])
    d = o.map_between_resolutions(u, N1)
    g1 = o.make_grid(2, 2 * np.pi, N1, dtype="float64")
    np.testing.assert_allclose(d, np.sin(3 * g1[0:1]) * np.cos(2 * g1[1:2]), atol=1e-12)
    up = o.map_between_resolutions(d, N0)
    np.testing.assert_allclose(up, u, atol=1e-12)


def test_nrmse_and_correlation():
    """metrics/_spatial.py:537-586, metrics/_correlation.py:33-60"""
    u = np.random.default_rng(4).standard_normal((1, 32))
    assert o.nRMSE(u, u) == 0.0
    assert o.nRMSE(2 * u, u) == pytest.approx(1.0)
    assert o.correlation(3 * u, u) == pytest.approx(1.0)


def test_forced_stepper_oracle_splitting():
    """_forced_stepper.py: zero forcing reproduces the stepper; for a linear stepper the forced step
    is linear in f: step(u, f) = step(u) + step(dt f) (ETDRK0 diffusion)."""
    st = o.Diffusion(1, 1.0, 32, 0.01, diffusivity=0.05)
    fs = o.ForcedStepper(st)
    rng = np.random.default_rng(0)
    u = rng.standard_normal((1, 32)).astype(np.float64)
    f = rng.standard_normal((1, 32)).astype(np.float64)
    np.testing.assert_allclose(fs(u, 0 * f), st(u), rtol=0, atol=1e-6)
    np.testing.assert_allclose(fs(u, f), st(u) + st(0.01 * f), rtol=0, atol=1e-5)
    traj = o.rollout(fs, 3, takes_aux=True)(u, f)
    assert traj.shape == (3, 1, 32)
    np.testing.assert_allclose(traj[-1], o.repeat(fs, 3, takes_aux=True)(u, f), rtol=0, atol=0)
    fs_t = np.stack([f, 2 * f, 3 * f])
    traj2 = o.rollout(fs, 3, takes_aux=True, constant_aux=False)(u, fs_t)
    np.testing.assert_allclose(traj2[0], fs(u, f), rtol=0, atol=0)
