"""The three-pass 3D path (exgb_pass3d.cu: N = 32, 64 and 128) against the oracle and
against the five-kernel 3D path (EXGB_3D_PATH=generic) on the same inputs.

Covers projected convection (NavierStokesVelocity, KolmogorovFlowVelocity with
its forcing at (0, k, 0)) at every ETDRK order, the staged nonlinearities in 3D
(Burgers' non-conservative convection: 12 derived fields; conservative
convection: 6 products; gradient norm; Cahn-Hilliard), batches that split into
workspace chunks, rollout / repeat semantics (the c2r projection of the kz = 0
plane after every step) and the nonlinear term alone.  Tolerances: 1e-5
relative L2 after one step, 1e-4 after 10 steps, 2e-5 for the nonlinear term
(the same bars as the other 3D tests)."""

import os

import numpy as np
import pytest

import exponax_gb300 as ex
from oracle import exponax_np as o

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


def velocity_ic(N, key, L=2 * np.pi, cutoff=5):
    g = ex.ic.RandomAmplitudePhaseSeries(3, cutoff=cutoff, max_one=True)
    u = np.concatenate([g(N, key=3 * key + c) for c in range(3)], axis=0).astype(np.float64)
    d = o.build_derivative_operator(3, L, N, dtype="float64")
    P = o.Leray(3, N, derivative_operator=d, dtype="float64")
    return o.ifft(P(o.fft(u)), num_spatial_dims=3, num_points=N).astype(np.float32)


def _generic(make):
    """The same stepper built on the five-kernel 3D path (the plan is created while the variable is set)."""
    os.environ["EXGB_3D_PATH"] = "generic"
    try:
        sm = make()
        sm.plan.handle
    finally:
        del os.environ["EXGB_3D_PATH"]
    return sm


@pytest.mark.parametrize("order", [1, 2, 3, 4])
@pytest.mark.parametrize("N", [32, 64])
def test_ns_velocity_step(N, order):
    mk = lambda: ex.stepper.NavierStokesVelocity(3, 2 * np.pi, N, 0.01, diffusivity=0.01, order=order)
    sm = mk()
    so = o.NavierStokesVelocity(3, 2 * np.pi, N, 0.01, diffusivity=0.01, order=order)
    u = np.stack([velocity_ic(N, k) for k in range(2)])
    got = host(ex.vmap(sm)(cu(u)))
    for b in range(2):
        assert rel(got[b], so(u[b])) < 1e-5, (N, order, b)
    gen = host(ex.vmap(_generic(mk))(cu(u)))
    assert rel(got, gen) < 2e-6


@pytest.mark.parametrize("order", [2, 4])
def test_ns_velocity_step_128(order):
    """N = 128: one 172 KB plane per CTA in passes 1 and 3."""
    N = 128
    mk = lambda: ex.stepper.NavierStokesVelocity(3, 2 * np.pi, N, 0.01, diffusivity=0.01, order=order)
    sm = mk()
    so = o.NavierStokesVelocity(3, 2 * np.pi, N, 0.01, diffusivity=0.01, order=order)
    u = velocity_ic(N, 2)
    got = host(sm(cu(u)))
    assert rel(got, so(u)) < 1e-5
    rep = host(ex.repeat(sm, 3)(cu(u)))
    assert rel(rep, host(ex.repeat(_generic(mk), 3)(cu(u)))) < 1e-5


@pytest.mark.parametrize("N", [32, 64])
def test_kolmogorov_velocity_repeat_and_rollout(N):
    mk = lambda: ex.stepper.KolmogorovFlowVelocity(3, 2 * np.pi, N, 0.01)
    sm = mk()
    so = o.KolmogorovFlowVelocity(3, 2 * np.pi, N, 0.01)
    u = velocity_ic(N, 4)
    assert rel(host(ex.repeat(sm, 10)(cu(u))), o.repeat(so, 10)(u)) < 1e-4
    tr = host(ex.rollout(sm, 3, include_init=True)(cu(u)))
    ref = o.rollout(so, 3, include_init=True)(u)
    assert tr.shape == (4, 3, N, N, N)
    for t in range(1, 4):
        assert rel(tr[t], ref[t]) < 1e-5 * t, t
    gen = host(ex.repeat(_generic(mk), 10)(cu(u)))
    assert rel(host(ex.repeat(sm, 10)(cu(u))), gen) < 1e-5


def test_ns_velocity_no_dealiasing_and_one_half():
    """No mask (every plane enters the nonlinear term, the Nyquist plane kz = N/2 included, with its
    c2r projection on the plane-major state), the 1.0 mask and the 1/2 mask."""
    N = 32
    u = velocity_ic(N, 7)
    for frac in (None, 1.0, 0.5):
        sm = ex.stepper.NavierStokesVelocity(3, 2 * np.pi, N, 0.005, diffusivity=0.02, dealiasing_fraction=frac)
        so = o.NavierStokesVelocity(3, 2 * np.pi, N, 0.005, diffusivity=0.02, dealiasing_fraction=frac)
        assert rel(host(ex.repeat(sm, 3)(cu(u))), o.repeat(so, 3)(u)) < 1e-5, frac


def test_batch_over_workspace_chunks():
    """A 64^3 batch larger than one workspace chunk: each sample as it is alone."""
    N = 64
    sm = ex.stepper.NavierStokesVelocity(3, 2 * np.pi, N, 0.01, diffusivity=0.01, order=2)
    u0 = velocity_ic(N, 1)
    B, same = 64, (0, 54, 55, 63)  # 55 samples per 1 GiB chunk at 64^3, ETDRK2
    batch = np.stack([u0 if b in same else np.roll(u0, b, axis=-1) * (1 + 0.01 * b) for b in range(B)])
    got = host(ex.vmap(sm)(cu(batch)))
    alone = host(sm(cu(u0)))
    for b in same:
        assert rel(got[b], alone) < 1e-6, b
    assert rel(alone, o.NavierStokesVelocity(3, 2 * np.pi, N, 0.01, diffusivity=0.01, order=2)(u0)) < 1e-5


def _field(N, C, key):
    g = ex.ic.RandomAmplitudePhaseSeries(3, cutoff=4, max_one=True)
    return np.concatenate([g(N, key=7 * key + c) for c in range(C)], axis=0).astype(np.float32)


@pytest.mark.parametrize("N", [32, 64])
def test_burgers_3d(N):
    """Non-conservative multi-channel convection: 12 derived fields per mode."""
    mk = lambda: ex.stepper.Burgers(3, 2 * np.pi, N, 0.01, diffusivity=0.05)
    sm = mk()
    so = o.Burgers(3, 2 * np.pi, N, 0.01, diffusivity=0.05)
    u = np.stack([_field(N, 3, k) for k in range(2)])
    got = host(ex.vmap(sm)(cu(u)))
    for b in range(2):
        assert rel(got[b], so(u[b])) < 1e-5
    got10 = host(ex.repeat(sm, 10)(cu(u[0])))
    assert rel(got10, o.repeat(so, 10)(u[0])) < 1e-4
    assert rel(got10, host(ex.repeat(_generic(mk), 10)(cu(u[0])))) < 1e-5


@pytest.mark.parametrize("name", ["conv_mc_cons", "conv_sc_noncons", "gradnorm", "cahn_hilliard"])
def test_staged_nonlinear_terms_3d(name):
    N, L = 32, 2 * np.pi
    dm = ex.spectral.build_derivative_operator(3, L, N)
    do = o.build_derivative_operator(3, L, N)
    if name == "conv_mc_cons":
        kw = dict(dealiasing_fraction=2 / 3, scale=0.7, conservative=True)
        fm = ex.nonlin_fun.ConvectionNonlinearFun(3, N, derivative_operator=dm, **kw)
        fo = o.ConvectionNonlinearFun(3, N, derivative_operator=do, **kw)
        C = 3
    elif name == "conv_sc_noncons":
        kw = dict(dealiasing_fraction=2 / 3, scale=0.7, single_channel=True)
        fm = ex.nonlin_fun.ConvectionNonlinearFun(3, N, derivative_operator=dm, **kw)
        fo = o.ConvectionNonlinearFun(3, N, derivative_operator=do, **kw)
        C = 1
    elif name == "gradnorm":
        kw = dict(dealiasing_fraction=2 / 3, scale=0.9, zero_mode_fix=True)
        fm = ex.nonlin_fun.GradientNormNonlinearFun(3, N, derivative_operator=dm, **kw)
        fo = o.GradientNormNonlinearFun(3, N, derivative_operator=do, **kw)
        C = 1
    else:
        from oracle import families_np as f

        kw = dict(dealiasing_fraction=1 / 2, scale=0.01)
        fm = ex.stepper.reaction.CahnHilliardNonlinearFun(3, N, derivative_operator=dm, **kw)
        fo = f.CahnHilliardNonlinearFun(3, N, derivative_operator=do, **kw)
        C = 1
    uh = np.stack([o.fft(_field(N, C, k), num_spatial_dims=3).astype(np.complex64) for k in range(3)])
    got = host(ex.vmap(fm)(cu(uh)))
    for b in range(3):
        assert rel(got[b], fo(uh[b])) < 2e-5, (name, b)


@pytest.mark.parametrize("kolmogorov", [False, True])
def test_projected_convection_term(kolmogorov):
    N, L = 64, 2 * np.pi
    dm = ex.spectral.build_derivative_operator(3, L, N)
    do = o.build_derivative_operator(3, L, N)
    if kolmogorov:
        fm = ex.nonlin_fun.ProjectedConvection3dKolmogorov(3, N, derivative_operator=dm, dealiasing_fraction=2 / 3)
        fo = o.ProjectedConvection3dKolmogorov(3, N, derivative_operator=do, dealiasing_fraction=2 / 3)
    else:
        fm = ex.nonlin_fun.ProjectedConvection3d(3, N, derivative_operator=dm)
        fo = o.ProjectedConvection3d(3, N, derivative_operator=do)
    uh = o.fft(velocity_ic(N, 3))
    got = host(fm(cu(uh)))
    assert rel(got, fo(uh)) < 2e-5


def test_128_batch_over_workspace_chunks_and_nonlinear_term():
    """128^3: 10 samples per 1 GiB workspace chunk (ETDRK2), so a batch of 12 splits in two; the
    projected-convection term alone at 128^3 against the oracle."""
    N = 128
    sm = ex.stepper.NavierStokesVelocity(3, 2 * np.pi, N, 0.01, diffusivity=0.01, order=2)
    u0 = velocity_ic(N, 5)
    B, same = 12, (0, 9, 10, 11)
    batch = np.stack([u0 if b in same else np.roll(u0, 3 * b, axis=-2) * (1 + 0.01 * b) for b in range(B)])
    got = host(ex.vmap(sm)(cu(batch)))
    alone = host(sm(cu(u0)))
    for b in same:
        assert rel(got[b], alone) < 1e-6, b
    dm = ex.spectral.build_derivative_operator(3, 2 * np.pi, N)
    do = o.build_derivative_operator(3, 2 * np.pi, N)
    fm = ex.nonlin_fun.ProjectedConvection3dKolmogorov(3, N, derivative_operator=dm, dealiasing_fraction=2 / 3)
    fo = o.ProjectedConvection3dKolmogorov(3, N, derivative_operator=do, dealiasing_fraction=2 / 3)
    uh = o.fft(u0)
    assert rel(host(fm(cu(uh))), fo(uh)) < 2e-5


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_burgers_3d_orders_64(order):
    N = 64
    sm = ex.stepper.Burgers(3, 2 * np.pi, N, 0.01, diffusivity=0.05, order=order)
    so = o.Burgers(3, 2 * np.pi, N, 0.01, diffusivity=0.05, order=order)
    u = _field(N, 3, 11)
    assert rel(host(sm(cu(u))), so(u)) < 1e-5


def test_kuramoto_sivashinsky_3d_32():
    """Gradient-norm nonlinearity (KuramotoSivashinsky, combustion form) on the three-pass 3D path."""
    N = 32
    sm = ex.stepper.KuramotoSivashinsky(3, 20.0, N, 0.05)
    so = o.KuramotoSivashinsky(3, 20.0, N, 0.05)
    u = _field(N, 1, 12)
    assert rel(host(sm(cu(u))), so(u)) < 1e-5
    assert rel(host(ex.repeat(sm, 10)(cu(u))), o.repeat(so, 10)(u)) < 1e-4
