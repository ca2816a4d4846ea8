"""Grid sizes outside 2^a 3^b 5^c and 1D grids longer than one CTA's shared
memory, on the GPU against numpy.fft and the oracle.

The reference's spectral.fft / ifft (_spectral.py:614-721) accept any N;
its own 2D Kolmogorov validation runs at N = 513 = 3^3 19
(validation/validate_kolmogorov_2d_spectrum.ipynb) and it names 1D grids of
10k-100k points as practical (docs/examples/performance_hints.ipynb).  Here N
with a prime factor above 5 goes through Bluestein's chirp-z transform, and
long 1D 2^a 3^b 5^c grids through a four-step transform; the steppers of
those sizes run on the staged path.  Tolerances: transforms 2e-6 relative L2
against numpy.fft (FP32 Bluestein measures ~1.5e-7 in a float32 NumPy
model of the same arithmetic); steps 1e-5 relative L2 against the float32
oracle.
"""

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


@pytest.mark.parametrize("D,N", [(1, 7), (1, 77), (1, 154), (1, 1031), (1, 6007), (1, 65536), (1, 2 ** 18 * 3),
                                 (2, 21), (2, 110), (2, 513), (2, 2048), (3, 14), (3, 21)])
def test_rfftn_irfftn_any_n_match_numpy(D, N):
    rng = np.random.default_rng(N * 10 + D)
    B = 3 if N < 10000 else 2
    u = rng.standard_normal((B, 1) + (N,) * D).astype(np.float32)
    axes = tuple(range(-D, 0))
    uh = host(ex.fft(cu(u), num_spatial_dims=D))
    ref = np.fft.rfftn(u.astype(np.float64), axes=axes)
    assert rel(uh, ref) < 2e-6
    # irfftn of non-Hermitian input: the imaginary parts of the c2r DC (and even-N Nyquist) bins are dropped
    z = (rng.standard_normal(ref.shape) + 1j * rng.standard_normal(ref.shape)).astype(np.complex64)
    back = host(ex.ifft(cu(z), num_spatial_dims=D, num_points=N))
    assert rel(back, np.fft.irfftn(z.astype(np.complex128), s=(N,) * D, axes=axes)) < 2e-6


def _ic(D, N, key):
    if D == 1:
        return ex.ic.RandomSineWaves1d(1, cutoff=5)(N, key=key)
    return ex.ic.RandomAmplitudePhaseSeries(D, cutoff=5, max_one=True)(N, key=key)


@pytest.mark.parametrize("name,N,dt,steps", [
    ("Burgers", 77, 1e-3, 5),
    ("KuramotoSivashinskyConservative", 154, 0.1, 5),
    ("KortewegDeVries", 1031, 1e-3, 3),
    ("KuramotoSivashinskyConservative", 65536, 0.1, 3),
    ("Burgers", 65536, 1e-4, 3),
])
def test_1d_steppers_any_n(name, N, dt, steps):
    L = {"Burgers": 1.0, "KuramotoSivashinskyConservative": 100.0, "KortewegDeVries": 20.0}[name]
    sm = getattr(ex.stepper, name)(1, L, N, dt)
    so = getattr(o, name)(1, L, N, dt)
    u0 = np.stack([_ic(1, N, s) for s in range(3)])
    got = host(ex.vmap(ex.repeat(sm, steps))(cu(u0)))
    traj = host(ex.vmap(ex.rollout(sm, 2, include_init=True))(cu(u0[:1])))
    for b in range(3):
        assert rel(got[b], o.repeat(so, steps)(u0[b])) < 1e-5, b
    ref = o.rollout(so, 2, include_init=True)(u0[0])
    assert rel(traj[0, 1:], ref[1:]) < 1e-5


@pytest.mark.parametrize("N", [77, 65536])
def test_1d_linear_stepper_any_n(N):
    """ETDRK0 (Diffusion) on the general transforms and the 1D linear kernel."""
    sm = ex.stepper.Diffusion(1, 1.0, N, 1e-4, diffusivity=0.01)
    so = o.Diffusion(1, 1.0, N, 1e-4, diffusivity=0.01)
    u0 = np.stack([_ic(1, N, s) for s in range(2)])
    got = host(ex.vmap(ex.repeat(sm, 4))(cu(u0)))
    for b in range(2):
        assert rel(got[b], o.repeat(so, 4)(u0[b])) < 1e-5


@pytest.mark.parametrize("cls,kw", [("ConvectionNonlinearFun", {}), ("GradientNormNonlinearFun", {}),
                                    ("ConvectionNonlinearFun", {"conservative": True})])
def test_1d_nonlinear_term_any_n(cls, kw):
    N, L = 154, 30.0
    fm = getattr(ex.nonlin_fun, cls)(1, N, dealiasing_fraction=2 / 3,
                                     derivative_operator=ex.spectral.build_derivative_operator(1, L, N), **kw)
    fo = getattr(o, cls)(1, N, dealiasing_fraction=2 / 3, derivative_operator=o.build_derivative_operator(1, L, N),
                         **kw)
    uh = o.fft(_ic(1, N, 4))
    got = host(fm(cu(uh)))
    want = fo(uh)
    assert rel(got, want) < 1e-5


def test_kolmogorov_513_the_reference_validation_size():
    """KolmogorovFlowVorticity at N = 513 (the reference's own 2D Kolmogorov validation grid), on the
    staged path: 3 ETDRK2 steps within 1e-5 of the oracle, and the Fourier-space step of the first
    sample within 1e-5."""
    N = 513
    sm = ex.stepper.KolmogorovFlowVorticity(2, 2 * np.pi, N, 0.005)
    so = o.KolmogorovFlowVorticity(2, 2 * np.pi, N, 0.005)
    u0 = np.stack([_ic(2, N, s) for s in range(2)])
    got = host(ex.vmap(ex.repeat(sm, 3))(cu(u0)))
    for b in range(2):
        assert rel(got[b], o.repeat(so, 3)(u0[b])) < 1e-5, b
    uh = ex.fft(cu(u0[:1]), num_spatial_dims=2)
    step = host(ex.vmap(sm.step_fourier)(uh))
    assert rel(step[0], so.step_fourier(o.fft(u0[0]))) < 1e-5


@pytest.mark.parametrize("N,order", [(110, 2), (21, 4), (77, 1)])
def test_ns_vorticity_any_n(N, order):
    sm = ex.stepper.NavierStokesVorticity(2, 2 * np.pi, N, 0.01, diffusivity=1e-3, order=order)
    so = o.NavierStokesVorticity(2, 2 * np.pi, N, 0.01, diffusivity=1e-3, order=order)
    u0 = np.stack([_ic(2, N, s) for s in range(3)])
    got = host(ex.vmap(ex.repeat(sm, 5))(cu(u0)))
    for b in range(3):
        assert rel(got[b], o.repeat(so, 5)(u0[b])) < 1e-5, b


def test_burgers_2d_any_n():
    N = 110
    sm = ex.stepper.Burgers(2, 2 * np.pi, N, 0.01, diffusivity=0.05)
    so = o.Burgers(2, 2 * np.pi, N, 0.01, diffusivity=0.05)
    g = ex.ic.RandomAmplitudePhaseSeries(2, cutoff=4, max_one=True)
    u0 = np.stack([np.concatenate([g(N, key=2 * s + c) for c in range(2)]) for s in range(2)])
    got = host(ex.vmap(ex.repeat(sm, 3))(cu(u0)))
    for b in range(2):
        assert rel(got[b], o.repeat(so, 3)(u0[b])) < 1e-5, b


def test_ns_velocity_3d_n21():
    """3D NavierStokesVelocity (projected convection + Leray) at N = 21 = 3 x 7."""
    N, L = 21, 2 * np.pi
    g = ex.ic.RandomAmplitudePhaseSeries(3, cutoff=3, max_one=True)
    u = np.concatenate([g(N, key=c) for c in range(3)], axis=0).astype(np.float64)
    d = o.build_derivative_operator(3, L, N, dtype="float64")
    u0 = o.ifft(o.Leray(3, N, derivative_operator=d, dtype="float64")(o.fft(u)), num_spatial_dims=3,
                num_points=N).astype(np.float32)
    sm = ex.stepper.NavierStokesVelocity(3, L, N, 0.01)
    so = o.NavierStokesVelocity(3, L, N, 0.01)
    got = host(ex.vmap(ex.repeat(sm, 3))(cu(u0[None])))
    assert rel(got[0], o.repeat(so, 3)(u0)) < 1e-5


@pytest.mark.parametrize("n_old,n_new", [(513, 64), (64, 110), (77, 154)])
def test_map_between_resolutions_any_n(n_old, n_new):
    D = 2 if n_old != 77 else 1
    rng = np.random.default_rng(n_old + n_new)
    u = rng.standard_normal((1,) + (n_old,) * D).astype(np.float32)
    got = host(ex.map_between_resolutions(cu(u), n_new))
    assert rel(got, o.map_between_resolutions(u, n_new)) < 1e-5


def test_sizes_still_refused():
    """A prime N whose Bluestein length does not fit one CTA raises instead of launching; the library
    stays usable afterwards."""
    with pytest.raises((ValueError, ex.ExgbError)):
        ex.vmap(ex.stepper.Burgers(1, 1.0, 7919, 0.01))(torch.zeros((1, 1, 7919), device="cuda"))
    with pytest.raises((ValueError, ex.ExgbError)):
        ex.fft(torch.zeros((1, 1, 7919), device="cuda"), num_spatial_dims=1)
    sm = ex.stepper.Burgers(1, 1.0, 77, 0.01)
    u = _ic(1, 77, 1)
    assert rel(sm(cu(u)).cpu().numpy(), o.Burgers(1, 1.0, 77, 0.01)(u)) < 1e-5


@pytest.mark.parametrize("name,N,order", [("KolmogorovFlowVorticity", 512, 2), ("NavierStokesVorticity", 384, 3),
                                          ("NavierStokesVorticity", 2048, 2), ("Burgers", 256, 4),
                                          ("KuramotoSivashinsky", 160, 2)])
def test_three_pass_2d_path(name, N, order):
    """The three-pass 2D path (derive + inverse along kx / c2r, products, r2c / forward along x + ETDRK
    update): 2D vorticity from N = 320 on (and any N above the fused kernels' 1024), and every other 2D
    nonlinearity: 3 steps within 1e-5 of the oracle, the Fourier-space nonlinear term within 1e-5."""
    kw = {"diffusivity": 1e-3} if name == "NavierStokesVorticity" else {}
    if name == "Burgers":
        kw = {"diffusivity": 0.05}
    L = 2 * np.pi if name != "KuramotoSivashinsky" else 60.0
    dt = 0.001 if name != "KuramotoSivashinsky" else 0.05
    sm = getattr(ex.stepper, name)(2, L, N, dt, order=order, **kw)
    so = getattr(o, name)(2, L, N, dt, order=order, **kw)
    C = sm.num_channels
    g = ex.ic.RandomAmplitudePhaseSeries(2, cutoff=4, max_one=True)
    B = 2 if N < 1024 else 1
    u0 = np.stack([np.concatenate([g(N, key=C * s + c) for c in range(C)]) for s in range(B)]).astype(np.float32)
    got = host(ex.vmap(ex.repeat(sm, 3))(cu(u0)))
    for b in range(B):
        assert rel(got[b], o.repeat(so, 3)(u0[b])) < 1e-5, b
    nh = host(sm.nonlinear_fun(ex.fft(cu(u0[:1]), num_spatial_dims=2)[0]))
    ref32 = so.nonlinear_fun(o.fft(u0[0]))
    e32 = rel(nh, ref32)
    if N < 1024:
        assert e32 < 1e-5
    else:
        # At 2048^2 the term (derivative products of a band-limited field: exact zeros above |k| = 8,
        # FP32 rounding noise there) is 2.3e-5 from the float64 oracle, the float32 oracle 3.9e-6:
        # the FP32 Stockham transforms' rounding grows with N (the per-step state bar above holds).
        so64 = getattr(o, name)(2, L, N, dt, order=order, dtype="float64", **kw)
        ref64 = so64.nonlinear_fun(o.fft(u0[0].astype(np.float64)))
        assert rel(nh, ref64) < 5e-5, (e32, rel(nh, ref64), rel(ref32, ref64))
