"""3D path on the GPU against the oracle: transforms, Leray projection,
projected convection (+ Kolmogorov forcing), NavierStokesVelocity /
KolmogorovFlowVelocity steps, 3D linear ETDRK0.  Tolerances: 2e-6 for
transforms, 1e-5 relative L2 per step, 1e-4 after 10 steps."""

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


def velocity_ic(N, key, L=2 * np.pi):
    """Smooth random divergence-free velocity (3, N, N, N), float32."""
    g = ex.ic.RandomAmplitudePhaseSeries(3, cutoff=3, max_one=True)
    u = np.concatenate([g(N, key=3 * key + c) for c in range(3)], axis=0).astype(np.float64)
    d = o.build_derivative_operator(3, L, N, dtype="float64")
    P = o.Leray(3, N, derivative_operator=d, dtype="float64")
    return o.ifft(P(o.fft(u)), num_spatial_dims=3, num_points=N).astype(np.float32)


@pytest.mark.parametrize("N", [16, 32, 48])
def test_rfftn_irfftn_3d(N):
    rng = np.random.default_rng(N)
    u = rng.standard_normal((2, 3, N, N, N)).astype(np.float32)
    uh = host(ex.fft(cu(u), num_spatial_dims=3))
    ref = np.fft.rfftn(u.astype(np.float64), axes=(-3, -2, -1))
    assert rel(uh, ref) < 2e-6
    z = (rng.standard_normal(ref.shape) + 1j * rng.standard_normal(ref.shape)).astype(np.complex64)
    back = host(ex.ifft(cu(z), num_spatial_dims=3, num_points=N))
    assert rel(back, np.fft.irfftn(z.astype(np.complex128), s=(N,) * 3, axes=(-3, -2, -1))) < 2e-6


def test_leray_projection():
    """tests/test_nonlinear_funs.py:416-517 on the GPU: divergence-free,
    identity on divergence-free fields, idempotent; equal to the oracle."""
    N, L = 16, 2.0
    dm = ex.spectral.build_derivative_operator(3, L, N)
    do = o.build_derivative_operator(3, L, N)
    P = ex.nonlin_fun.Leray(3, N, derivative_operator=dm)
    Po = o.Leray(3, N, derivative_operator=do)
    u = np.random.default_rng(0).standard_normal((3, N, N, N)).astype(np.float32)
    uh = o.fft(u)
    pu = host(P(cu(uh)))
    assert rel(pu, Po(uh)) < 1e-6
    div = np.sum(do * pu, axis=0)
    assert np.max(np.abs(div)) < 1e-5 * np.max(np.abs(uh))
    assert rel(host(P(cu(pu))), pu) < 1e-6
    P2 = ex.nonlin_fun.Leray(2, 32, derivative_operator=ex.spectral.build_derivative_operator(2, L, 32))
    v = np.random.default_rng(1).standard_normal((2, 32, 32)).astype(np.float32)
    vh = o.fft(v)
    assert rel(host(P2(cu(vh))), o.Leray(2, 32, derivative_operator=o.build_derivative_operator(2, L, 32))(vh)) < 1e-6


@pytest.mark.parametrize("kolmogorov", [False, True])
@pytest.mark.parametrize("N", [16, 32])
def test_projected_convection_matches_oracle(N, kolmogorov):
    L = 2 * np.pi
    dm = ex.spectral.build_derivative_operator(3, L, N)
    do = o.build_derivative_operator(3, L, N)
    if kolmogorov:
        fm = ex.nonlin_fun.ProjectedConvection3dKolmogorov(3, N, derivative_operator=dm, dealiasing_fraction=2 / 3)
        fo = o.ProjectedConvection3dKolmogorov(3, N, derivative_operator=do, dealiasing_fraction=2 / 3)
    else:
        fm = ex.nonlin_fun.ProjectedConvection3d(3, N, derivative_operator=dm)
        fo = o.ProjectedConvection3d(3, N, derivative_operator=do)
    uh = o.fft(velocity_ic(N, 1))
    got = host(fm(cu(uh)))
    assert rel(got, fo(uh)) < 1e-5
    div = np.sum(do * got, axis=0)
    if not kolmogorov:
        assert np.max(np.abs(div)) < 1e-4 * np.max(np.abs(got))


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_navier_stokes_velocity_step(order):
    N = 32
    sm = ex.stepper.NavierStokesVelocity(3, 2 * np.pi, N, 0.01, diffusivity=0.01, order=order)
    so = o.NavierStokesVelocity(3, 2 * np.pi, N, 0.01, diffusivity=0.01, order=order)
    u = np.stack([velocity_ic(N, k) for k in range(2)])
    got = host(ex.vmap(sm)(cu(u)))
    for b in range(2):
        assert rel(got[b], so(u[b])) < 1e-5


def test_kolmogorov_velocity_repeat_10_steps():
    N = 32
    sm = ex.stepper.KolmogorovFlowVelocity(3, 2 * np.pi, N, 0.01)
    so = o.KolmogorovFlowVelocity(3, 2 * np.pi, N, 0.01)
    u = velocity_ic(N, 4)
    assert rel(host(ex.repeat(sm, 10)(cu(u))), o.repeat(so, 10)(u)) < 1e-4
    tr = host(ex.rollout(sm, 3, include_init=True)(cu(u)))
    ref = o.rollout(so, 3, include_init=True)(u)
    assert tr.shape == (4, 3, N, N, N)
    assert rel(tr[1:], ref[1:]) < 1e-5 * 3


def test_diffusion_3d_etdrk0():
    """tests/test_validation.py:171-211 on the GPU."""
    L, N, dt, nu = 2 * np.pi, 24, 0.1, 0.05
    g = ex.make_grid(3, L, N)
    st = ex.stepper.Diffusion(3, L, N, dt, diffusivity=nu)
    u0 = (np.sin(g[0:1]) * np.sin(2 * g[1:2]) * np.cos(g[2:3])).astype(np.float32)
    np.testing.assert_allclose(host(st(cu(u0))), u0 * np.exp(-6 * nu * dt), atol=1e-5)
