"""Edge cases of the stepping and transform entry points on the GPU: empty batches (torch hands
NULL data pointers for them), zero steps, zero states, in-place Fourier stepping, odd and
non-power-of-two grids, and sizes the library refuses with an error instead of a launch."""

import numpy as np
import pytest

import exponax_gb300 as ex
from oracle import exponax_np as o

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _steppers():
    return [
        ex.stepper.KuramotoSivashinskyConservative(1, 100.0, 200, 0.1),   # fused 1D kernel
        ex.stepper.NavierStokesVorticity(2, 2 * np.pi, 64, 0.01, diffusivity=1e-3),  # cluster kernel
        ex.stepper.NavierStokesVorticity(2, 2 * np.pi, 45, 0.01, diffusivity=1e-3),  # generic 2D kernel
        ex.stepper.Burgers(2, 2 * np.pi, 32, 0.01, diffusivity=0.05),     # staged N-D path
        ex.stepper.NavierStokesVelocity(3, 2 * np.pi, 16, 0.01),          # 3D path
        ex.stepper.Diffusion(2, 1.0, 32, 0.1),                            # ETDRK0
        ex.stepper.Wave(2, 1.0, 32, 0.01),                                # per-mode 2x2 map
    ]


@pytest.mark.parametrize("idx", range(7))
def test_empty_batches_and_zero_steps(idx):
    sm = _steppers()[idx]
    D, N, C = sm.num_spatial_dims, sm.num_points, sm.num_channels
    shape = (C,) + (N,) * D
    e = torch.empty((0,) + shape, dtype=torch.float32, device="cuda")
    assert tuple(ex.vmap(sm)(e).shape) == (0,) + shape
    assert tuple(ex.vmap(ex.repeat(sm, 4))(e).shape) == (0,) + shape
    assert tuple(ex.vmap(ex.rollout(sm, 3, include_init=True))(e).shape) == (0, 4) + shape
    eh = torch.empty((0, C) + (N,) * (D - 1) + (N // 2 + 1,), dtype=torch.complex64, device="cuda")
    assert tuple(ex.vmap(sm.step_fourier)(eh).shape) == tuple(eh.shape)
    assert tuple(ex.fft(e, num_spatial_dims=D).shape) == tuple(eh.shape)
    assert tuple(ex.ifft(eh, num_spatial_dims=D, num_points=N).shape) == tuple(e.shape)
    # zero steps return the state; rollout(0, include_init) is the initial state alone
    u = torch.from_numpy(np.random.default_rng(idx).standard_normal((2,) + shape).astype(np.float32)).cuda()
    np.testing.assert_array_equal(ex.vmap(ex.repeat(sm, 0))(u).cpu().numpy(), u.cpu().numpy())
    r = ex.vmap(ex.rollout(sm, 0, include_init=True))(u)
    assert tuple(r.shape) == (2, 1) + shape
    np.testing.assert_array_equal(r[:, 0].cpu().numpy(), u.cpu().numpy())
    # the zero state stays zero
    z = torch.zeros((1,) + shape, dtype=torch.float32, device="cuda")
    if not isinstance(sm, ex.stepper.Diffusion):
        assert float(ex.vmap(ex.repeat(sm, 3))(z).abs().max()) == 0.0


def test_empty_transforms_and_resampling():
    e = torch.empty((0, 1, 32, 32), dtype=torch.float32, device="cuda")
    assert tuple(ex.interpolation.map_between_resolutions_batched(e, 16).shape) == (0, 1, 16, 16)
    assert tuple(ex.spectral.derivative(torch.zeros((1, 8, 8), device="cuda"), 1.0).shape) == (2, 8, 8)


@pytest.mark.parametrize("kind", ["ks1d", "ns64"])
def test_in_place_fourier_stepping(kind):
    """exgb_repeat_fourier with the output buffer equal to the input buffer (the header allows aliasing)."""
    from exponax_gb300 import _device, _lib

    if kind == "ks1d":
        sm = ex.stepper.KuramotoSivashinskyConservative(1, 100.0, 200, 0.1)
        so = o.KuramotoSivashinskyConservative(1, 100.0, 200, 0.1)
        u = np.stack([ex.ic.RandomSineWaves1d(1)(200, key=k) for k in range(3)])
    else:
        sm = ex.stepper.NavierStokesVorticity(2, 2 * np.pi, 64, 0.01, diffusivity=1e-3)
        so = o.NavierStokesVorticity(2, 2 * np.pi, 64, 0.01, diffusivity=1e-3)
        u = np.stack([ex.ic.RandomAmplitudePhaseSeries(2, cutoff=5, max_one=True)(64, key=k) for k in range(3)])
    D = sm.num_spatial_dims
    uh = ex.fft(torch.from_numpy(u).cuda(), num_spatial_dims=D).contiguous()
    _lib.check(_lib.load().exgb_repeat_fourier(sm.plan.handle, _device.stream(), uh.data_ptr(), uh.data_ptr(), 3, 5))
    got = ex.ifft(uh, num_spatial_dims=D, num_points=sm.num_points).cpu().numpy()
    for b in range(3):
        assert rel(got[b], o.repeat(so, 5)(u[b])) < 1e-5, b


@pytest.mark.parametrize("name,order", [("KuramotoSivashinskyConservative", 2), ("Burgers", 1), ("Burgers", 3),
                                        ("KuramotoSivashinsky", 2), ("KortewegDeVries", 4), ("FisherKPP", 2)])
def test_1d_batches_larger_than_the_gpu(name, order):
    """A 1D batch with more work items than SMs runs the 1D kernel with the elementwise steps fused into
    the first and last radix passes (pack, products, trajectory stores); every sample of a 600-instance
    batch agrees with the oracle's single step (1e-5) and 10-step trajectory (1e-4), checked on a
    spread of samples, and with the same samples stepped in a small (unfused) batch."""
    N = 64
    if name == "FisherKPP":
        sm = ex.stepper.reaction.FisherKPP(1, 1.0, N, 0.001, reactivity=5.0, order=order)
        from oracle import families_np as f
        so = f.FisherKPP(1, 1.0, N, 0.001, reactivity=5.0, order=order)
        mk = lambda k: (0.5 + 0.4 * ex.ic.RandomSineWaves1d(1)(N, key=k)).astype(np.float32)  # noqa: E731
    else:
        args = {"KuramotoSivashinskyConservative": (1, 60.0, N, 0.05), "Burgers": (1, 1.0, N, 1e-3),
                "KuramotoSivashinsky": (1, 30.0, N, 0.05), "KortewegDeVries": (1, 20.0, N, 0.005)}[name]
        sm = getattr(ex.stepper, name)(*args, order=order)
        so = getattr(o, name)(*args, order=order)
        mk = lambda k: ex.ic.RandomSineWaves1d(1)(N, key=k)  # noqa: E731
    B = 600
    u = np.stack([mk(k) for k in range(B)])
    one = ex.vmap(sm)(torch.from_numpy(u).cuda()).cpu().numpy()
    traj = ex.vmap(ex.rollout(sm, 10, include_init=True))(torch.from_numpy(u).cuda()).cpu().numpy()
    small = ex.vmap(ex.rollout(sm, 10, include_init=True))(torch.from_numpy(u[:3]).cuda()).cpu().numpy()
    for b in (0, 1, 2, 151, 299, 300, 451, 598, 599):
        assert rel(one[b], so(u[b])) < 1e-5, b
        assert rel(traj[b], o.rollout(so, 10, include_init=True)(u[b])) < 1e-4, b
    assert rel(traj[:3], small) < 1e-6


@pytest.mark.parametrize("kind", ["ks1d", "ch1d", "ns2d", "burgers2d", "wave2d"])
@pytest.mark.parametrize("trajectory", [True, False])
def test_graph_rollout_replays_the_eager_result(kind, trajectory):
    """GraphRollout (rollouts captured as CUDA graphs): two replays with different initial states equal
    the eager vmap(rollout) / vmap(repeat) results within 1e-6 (the same kernels; in 1D the work queue
    may pair other instances in the packed output transform, which changes the last bit)."""
    if kind == "ks1d":
        sm = ex.stepper.KuramotoSivashinskyConservative(1, 100.0, 200, 0.1)
        mk = lambda k: ex.ic.RandomSineWaves1d(1)(200, key=k)  # noqa: E731
    elif kind == "ch1d":
        sm = ex.stepper.reaction.CahnHilliard(1, 2 * np.pi, 64, 0.001, gamma=1e-3)
        mk = lambda k: ex.ic.RandomSineWaves1d(1)(64, key=k)  # noqa: E731
    elif kind == "ns2d":
        sm = ex.stepper.NavierStokesVorticity(2, 2 * np.pi, 64, 0.01, diffusivity=1e-3)
        mk = lambda k: ex.ic.RandomAmplitudePhaseSeries(2, cutoff=5, max_one=True)(64, key=k)  # noqa: E731
    elif kind == "burgers2d":
        sm = ex.stepper.Burgers(2, 2 * np.pi, 32, 0.01, diffusivity=0.05)
        g = ex.ic.RandomAmplitudePhaseSeries(2, cutoff=3, max_one=True)
        mk = lambda k: np.concatenate([g(32, key=2 * k), g(32, key=2 * k + 1)])  # noqa: E731
    else:
        sm = ex.stepper.Wave(2, 1.0, 32, 0.01)
        g = ex.ic.RandomAmplitudePhaseSeries(2, cutoff=3, max_one=True)
        mk = lambda k: np.concatenate([g(32, key=2 * k), 0.3 * g(32, key=2 * k + 1)])  # noqa: E731
    B, n = 3, 7
    gr = ex.graphs.GraphRollout(sm, n, B, include_init=True, trajectory=trajectory)
    eager = ex.vmap(ex.rollout(sm, n, include_init=True)) if trajectory else ex.vmap(ex.repeat(sm, n))
    for base in (0, 10):
        u = torch.from_numpy(np.stack([mk(base + b) for b in range(B)]).astype(np.float32)).cuda()
        got = gr(u).clone()
        want = eager(u)
        assert tuple(got.shape) == tuple(want.shape)
        np.testing.assert_allclose(got.cpu().numpy(), want.cpu().numpy(), rtol=0, atol=1e-6)
    with pytest.raises(ValueError):
        gr(torch.zeros((B + 1,) + gr.shape[1:], device="cuda"))
