"""Staged N-D path on the GPU against the oracle: the convection (four
variants), gradient-norm, polynomial and general nonlinearities in 2D and 3D,
the Cahn-Hilliard, Gray-Scott and Belousov-Zhabotinsky reaction terms in 1D/2D/3D, and the steppers
built on them (Burgers / KS / KdV in 2D and 3D, the reaction-diffusion
family, the generic General / Normalized / Difficulty steppers).

Tolerances (relative L2, FP32 against the FP32 oracle): 2e-5 for one
nonlinear evaluation, 1e-5 per step, 1e-4 after 20-50 steps of the
non-chaotic cases."""

import numpy as np
import pytest

import exponax_gb300 as ex
from oracle import exponax_np as o
from oracle import families_np as f

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def rel(a, b):
    a = np.asarray(a).astype(np.complex128 if np.iscomplexobj(a) else np.float64)
    b = np.asarray(b).astype(np.complex128 if np.iscomplexobj(b) else np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def cu(x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def host(t):
    return t.cpu().numpy()


def field(D, N, C, key, cutoff=4):
    g = ex.ic.RandomAmplitudePhaseSeries(D, cutoff=cutoff, max_one=True)
    return np.concatenate([g(N, key=7 * key + c) for c in range(C)], axis=0).astype(np.float32)


def spectrum(D, N, C, key):
    return o.fft(field(D, N, C, key), num_spatial_dims=D).astype(np.complex64)


# ---------------------------------------------------------------------------- nonlinear functions
def _nl_pair(kind, D, N, L=2 * np.pi):
    dm = ex.spectral.build_derivative_operator(D, L, N)
    do = o.build_derivative_operator(D, L, N)
    if kind.startswith("conv"):
        sc = kind in ("conv_sc_cons", "conv_sc_noncons")
        cons = kind in ("conv_mc_cons", "conv_sc_cons")
        kw = dict(dealiasing_fraction=2 / 3, scale=0.7, single_channel=sc, conservative=cons)
        return (ex.nonlin_fun.ConvectionNonlinearFun(D, N, derivative_operator=dm, **kw),
                o.ConvectionNonlinearFun(D, N, derivative_operator=do, **kw), 1 if sc else D)
    if kind == "gradnorm":
        kw = dict(dealiasing_fraction=2 / 3, scale=0.9, zero_mode_fix=True)
        return (ex.nonlin_fun.GradientNormNonlinearFun(D, N, derivative_operator=dm, **kw),
                o.GradientNormNonlinearFun(D, N, derivative_operator=do, **kw), 1)
    if kind == "gradnorm_nofix":
        kw = dict(dealiasing_fraction=2 / 3, scale=0.9, zero_mode_fix=False)
        return (ex.nonlin_fun.GradientNormNonlinearFun(D, N, derivative_operator=dm, **kw),
                o.GradientNormNonlinearFun(D, N, derivative_operator=do, **kw), 1)
    if kind == "poly":
        kw = dict(dealiasing_fraction=1 / 2, coefficients=(0.3, -0.5, 1.0, -1.0))
        return ex.nonlin_fun.PolynomialNonlinearFun(D, N, **kw), o.PolynomialNonlinearFun(D, N, **kw), 1
    if kind == "general":
        kw = dict(dealiasing_fraction=2 / 3, scale_list=(0.4, -1.1, 0.6), zero_mode_fix=True)
        return (ex.nonlin_fun.GeneralNonlinearFun(D, N, derivative_operator=dm, **kw),
                o.GeneralNonlinearFun(D, N, derivative_operator=do, **kw), 1)
    if kind == "cahn_hilliard":
        kw = dict(dealiasing_fraction=1 / 2, scale=0.01)
        return (ex.stepper.reaction.CahnHilliardNonlinearFun(D, N, derivative_operator=dm, **kw),
                f.CahnHilliardNonlinearFun(D, N, derivative_operator=do, **kw), 1)
    if kind == "gray_scott":
        kw = dict(dealiasing_fraction=1 / 2, feed_rate=0.04, kill_rate=0.06)
        return ex.stepper.reaction.GrayScottNonlinearFun(D, N, **kw), f.GrayScottNonlinearFun(D, N, **kw), 2
    raise KeyError(kind)


ND_KINDS = ["conv_mc_cons", "conv_mc_noncons", "conv_sc_cons", "conv_sc_noncons", "gradnorm", "gradnorm_nofix",
            "poly", "general", "cahn_hilliard", "gray_scott"]


@pytest.mark.parametrize("kind", ND_KINDS)
@pytest.mark.parametrize("D,N", [(2, 32), (2, 48), (3, 16)])
def test_nonlinear_fun_matches_oracle(kind, D, N):
    fm, fo, C = _nl_pair(kind, D, N)
    uh = spectrum(D, N, C, key=N + D)
    got = host(fm(cu(uh)))
    want = fo(uh)
    assert got.shape == want.shape
    assert rel(got, want) < 2e-5, (kind, D, N)


@pytest.mark.parametrize("kind", ND_KINDS)
@pytest.mark.parametrize("D,N", [(2, 64), (3, 32)])
def test_nonlinear_fun_three_pass_register_sizes(kind, D, N):
    """Every staged nonlinearity at the sizes the register-FFT three-pass kernels take (2D 64^2, 3D 32^3):
    their derive (channel values loaded ahead), products (register inputs per channel / dimension count)
    and combine against the oracle, two samples at once."""
    fm, fo, C = _nl_pair(kind, D, N)
    uh = np.stack([spectrum(D, N, C, key=N + D + b) for b in range(2)])
    got = host(ex.vmap(fm)(cu(uh)))
    for b in range(2):
        assert rel(got[b], fo(uh[b])) < 2e-5, (kind, D, N, b)


@pytest.mark.parametrize("kind", ["cahn_hilliard", "gray_scott"])
@pytest.mark.parametrize("N", [64, 100])
def test_reaction_nonlinear_fun_1d(kind, N):
    fm, fo, C = _nl_pair(kind, 1, N, L=10.0)
    uh = spectrum(1, N, C, key=N)
    assert rel(host(fm(cu(uh))), fo(uh)) < 2e-5


def test_batched_nonlinear_fun():
    fm, fo, C = _nl_pair("conv_mc_noncons", 2, 32)
    uh = np.stack([spectrum(2, 32, C, key=k) for k in range(5)])
    got = host(ex.vmap(fm)(cu(uh)))
    for b in range(5):
        assert rel(got[b], fo(uh[b])) < 2e-5


# ---------------------------------------------------------------------------- steppers
def _ic_for(name, D, N, C, key):
    u = field(D, N, C, key)
    if name in ("FisherKPP",):
        return (0.5 + 0.4 * u).astype(np.float32)
    if name == "GrayScott":
        blob = 0.5 * (1 + field(D, N, 1, key, cutoff=2)[0])
        return np.stack([1.0 - 0.5 * blob, 0.25 * blob]).astype(np.float32)
    if name == "BelousovZhabotinsky":
        return (0.5 + 0.4 * u).astype(np.float32)
    return u


STEPPERS = [
    # (name, D, N, product ctor, oracle ctor, steps)
    ("Burgers", 2, 48, lambda m, D, N: m.Burgers(D, 2 * np.pi, N, 0.01, diffusivity=0.05), 30),
    ("Burgers_cons", 2, 32, lambda m, D, N: m.Burgers(D, 2 * np.pi, N, 0.01, diffusivity=0.05, conservative=True), 30),
    ("Burgers_sc", 2, 32, lambda m, D, N: m.Burgers(D, 2 * np.pi, N, 0.01, diffusivity=0.05, single_channel=True), 30),
    ("Burgers", 3, 16, lambda m, D, N: m.Burgers(D, 2 * np.pi, N, 0.01, diffusivity=0.05), 20),
    ("KortewegDeVries", 2, 32, lambda m, D, N: m.KortewegDeVries(D, 20.0, N, 0.005), 20),
    ("KuramotoSivashinsky", 2, 32, lambda m, D, N: m.KuramotoSivashinsky(D, 30.0, N, 0.05), 20),
    ("KuramotoSivashinskyConservative", 2, 32,
     lambda m, D, N: m.KuramotoSivashinskyConservative(D, 30.0, N, 0.05), 20),
]


@pytest.mark.parametrize("name,D,N,make,steps", STEPPERS)
def test_nd_stepper_matches_oracle(name, D, N, make, steps):
    sm, so = make(ex.stepper, D, N), make(o, D, N)
    u = np.stack([_ic_for(name, D, N, sm.num_channels, k) for k in range(3)])
    one = host(ex.vmap(sm)(cu(u)))
    for b in range(3):
        assert rel(one[b], so(u[b])) < 1e-5, (name, b)
    many = host(ex.vmap(ex.repeat(sm, steps))(cu(u)))
    for b in range(3):
        assert rel(many[b], o.repeat(so, steps)(u[b])) < 1e-4, (name, b)


REACTION = [
    ("FisherKPP", 2, 48, dict(domain_extent=1.0, dt=0.001, diffusivity=0.01, reactivity=10.0), 50),
    ("FisherKPP", 3, 16, dict(domain_extent=1.0, dt=0.001, diffusivity=0.01, reactivity=10.0), 20),
    ("AllenCahn", 2, 48, dict(domain_extent=2 * np.pi, dt=0.01), 50),
    ("SwiftHohenberg", 2, 48, dict(domain_extent=20 * np.pi, dt=0.05), 50),
    ("CahnHilliard", 1, 128, dict(domain_extent=2 * np.pi, dt=0.001, gamma=1e-3), 50),
    ("CahnHilliard", 2, 48, dict(domain_extent=2 * np.pi, dt=0.001, gamma=1e-3), 50),
    ("CahnHilliard", 3, 16, dict(domain_extent=2 * np.pi, dt=0.001, gamma=1e-3), 20),
    ("GrayScott", 1, 128, dict(domain_extent=1.0, dt=0.5, diffusivity_1=2e-5, diffusivity_2=1e-5), 50),
    ("GrayScott", 2, 48, dict(domain_extent=1.0, dt=0.5, diffusivity_1=2e-5, diffusivity_2=1e-5), 50),
    ("BelousovZhabotinsky", 1, 128, dict(domain_extent=1.0, dt=0.01), 50),
    ("BelousovZhabotinsky", 2, 48, dict(domain_extent=1.0, dt=0.01, diffusivities=(1e-3, 2e-3, 1e-3)), 50),
    ("BelousovZhabotinsky", 3, 16, dict(domain_extent=1.0, dt=0.01), 20),
    # N = 32: the three-pass 3D path (exgb_pass3d.cu); N = 16 above runs on the five-kernel path
    ("FisherKPP", 3, 32, dict(domain_extent=1.0, dt=0.001, diffusivity=0.01, reactivity=10.0), 10),
    ("CahnHilliard", 3, 32, dict(domain_extent=2 * np.pi, dt=0.001, gamma=1e-3), 10),
    ("GrayScott", 3, 32, dict(domain_extent=1.0, dt=0.5, diffusivity_1=2e-5, diffusivity_2=1e-5), 10),
    ("BelousovZhabotinsky", 3, 32, dict(domain_extent=1.0, dt=0.01), 10),
]


@pytest.mark.parametrize("name,D,N,kw,steps", REACTION)
def test_reaction_stepper_matches_oracle(name, D, N, kw, steps):
    kw = dict(kw)
    L, dt = kw.pop("domain_extent"), kw.pop("dt")
    sm = getattr(ex.stepper.reaction, name)(D, L, N, dt, **kw)
    so = getattr(f, name)(D, L, N, dt, **kw)
    u = np.stack([_ic_for(name, D, N, sm.num_channels, k) for k in range(2)])
    one = host(ex.vmap(sm)(cu(u)))
    for b in range(2):
        assert rel(one[b], so(u[b])) < 1e-5, (name, b)
    traj = host(ex.vmap(ex.rollout(sm, steps, include_init=True))(cu(u)))
    for b in range(2):
        want = o.rollout(so, steps, include_init=True)(u[b])
        assert rel(traj[b], want) < 1e-4, (name, b)


@pytest.mark.parametrize("order", [0, 1, 2, 3, 4])
def test_staged_all_orders(order):
    sm = ex.stepper.Burgers(2, 2 * np.pi, 32, 0.01, diffusivity=0.05, order=order)
    so = o.Burgers(2, 2 * np.pi, 32, 0.01, diffusivity=0.05, order=order)
    u = np.stack([field(2, 32, 2, k) for k in range(2)])
    got = host(ex.vmap(ex.repeat(sm, 10))(cu(u)))
    for b in range(2):
        assert rel(got[b], o.repeat(so, 10)(u[b])) < 1e-4, b


def test_staged_step_fourier_and_repeated_stepper():
    sm = ex.stepper.KuramotoSivashinsky(2, 30.0, 32, 0.05)
    so = o.KuramotoSivashinsky(2, 30.0, 32, 0.05)
    uh = spectrum(2, 32, 1, key=3)
    assert rel(host(sm.step_fourier(cu(uh))), so.step_fourier(uh)) < 1e-5
    u = field(2, 32, 1, key=4)
    rs = ex.RepeatedStepper(sm, 5)
    ro = o.RepeatedStepper(so, 5)
    assert rel(host(rs(cu(u))), ro(u)) < 1e-4


def test_staged_chunks_are_independent():
    """A 3D batch larger than one workspace chunk gives every sample the result it has alone."""
    N = 64
    sm = ex.stepper.Burgers(3, 2 * np.pi, N, 0.01, diffusivity=0.05)
    u0 = field(3, N, 3, key=1)
    alone = host(ex.vmap(sm)(cu(u0[None])))[0]
    batch = np.stack([u0 if b in (0, 27, 28, 33) else field(3, N, 3, key=10 + b) for b in range(34)])
    got = host(ex.vmap(sm)(cu(batch)))
    for b in (0, 27, 28, 33):
        np.testing.assert_array_equal(got[b], alone)
    assert rel(alone, o.Burgers(3, 2 * np.pi, N, 0.01, diffusivity=0.05)(u0)) < 1e-5


# ---------------------------------------------------------------------------- generic steppers
GENERIC = [
    ("GeneralConvectionStepper", dict(num_spatial_dims=2, domain_extent=1.0, num_points=32, dt=0.001)),
    ("GeneralGradientNormStepper", dict(num_spatial_dims=2, domain_extent=30.0, num_points=32, dt=0.05)),
    ("GeneralPolynomialStepper", dict(num_spatial_dims=2, domain_extent=10.0, num_points=32, dt=0.001)),
    ("GeneralNonlinearStepper", dict(num_spatial_dims=2, domain_extent=1.0, num_points=32, dt=0.001)),
    ("GeneralVorticityConvectionStepper", dict(num_spatial_dims=2, domain_extent=2 * np.pi, num_points=32,
                                               dt=0.01)),
    ("GeneralLinearStepper", dict(num_spatial_dims=3, domain_extent=1.0, num_points=16, dt=0.01)),
    ("DifficultyConvectionStepper", dict(num_spatial_dims=1)),
    ("DifficultyConvectionStepper", dict(num_spatial_dims=2, num_points=32)),
    ("DifficultyGradientNormStepper", dict(num_spatial_dims=1)),
    ("DifficultyGradientNormStepper", dict(num_spatial_dims=2, num_points=32)),
    ("DifficultyPolynomialStepper", dict(num_spatial_dims=2, num_points=32)),
    ("DifficultyNonlinearStepper", dict(num_spatial_dims=1)),
    ("DifficultyNonlinearStepper", dict(num_spatial_dims=2, num_points=32)),
    ("DifficultyLinearStepper", dict(num_spatial_dims=2, num_points=32)),
    ("DifficultyLinearStepperSimple", dict(num_spatial_dims=1, difficulty=2.0, order=2)),
]


@pytest.mark.parametrize("name,kw", GENERIC)
def test_generic_stepper_matches_oracle(name, kw):
    sm = getattr(ex.stepper.generic, name)(**kw)
    so = getattr(f, name)(**kw)
    D, N = sm.num_spatial_dims, sm.num_points
    u = np.stack([field(D, N, sm.num_channels, k, cutoff=3) for k in range(2)])
    got = host(ex.vmap(ex.repeat(sm, 10))(cu(u)))
    for b in range(2):
        assert rel(got[b], o.repeat(so, 10)(u[b])) < 1e-4, (name, b)


# ---------------------------------------------------------------------------- errors
def test_channel_errors():
    with pytest.raises(ValueError):
        ex.vmap(ex.stepper.reaction.GrayScott(2, 1.0, 32, 1.0).nonlinear_fun)(cu(np.zeros((1, 3, 32, 17),
                                                                                           np.complex64)))
    fm, _, _ = _nl_pair("conv_mc_cons", 2, 32)
    with pytest.raises(ValueError):
        fm(cu(np.zeros((3, 32, 17), np.complex64)))
    ch = ex.stepper.reaction.CahnHilliardNonlinearFun(2, 32, derivative_operator=ex.spectral.build_derivative_operator(
        2, 1.0, 32), dealiasing_fraction=None)
    with pytest.raises(ValueError):
        ch(cu(np.zeros((1, 32, 17), np.complex64)))
