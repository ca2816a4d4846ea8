"""ForcedStepper and auxiliary-input loops (_forced_stepper.py, _utils.py:137-163, :212-229) and the
device-built initial conditions, against the oracle / the host generators.

ForcedStepper: one step within 1e-5 relative L2 (1D Burgers, 2D NS vorticity), Fourier-space step,
batched calls, and 20-step rollouts with constant and time-varying forcing within 1e-4 (non-chaotic).
Device ICs: the same seeded draws as the host generators, built by scatter + inverse FFT + normalisation
on the GPU, within 2e-6 relative L2 of the host arrays (FP32 inverse FFT vs float64 synthesis)."""

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


def _case(name):
    if name == "burgers":
        args, kw = (1, 1.0, 128, 1e-3), {"diffusivity": 0.01}
        sm, so = ex.stepper.Burgers(*args, **kw), o.Burgers(*args, **kw)
        u = np.stack([ex.ic.RandomSineWaves1d(1, cutoff=5)(128, key=s) for s in range(3)])
    else:
        args, kw = (2, 2 * np.pi, 64, 0.01), {"diffusivity": 1e-3}
        sm, so = ex.stepper.NavierStokesVorticity(*args, **kw), o.NavierStokesVorticity(*args, **kw)
        u = np.stack([ex.ic.RandomAmplitudePhaseSeries(2, cutoff=5, max_one=True)(64, key=s) for s in range(3)])
    f = (0.5 * np.random.default_rng(7).standard_normal(u.shape)).astype(np.float32)
    return sm, so, u, f


@pytest.mark.parametrize("name", ["burgers", "ns"])
def test_forced_step_matches_oracle(name):
    sm, so, u, f = _case(name)
    fm, fo = ex.ForcedStepper(sm), o.ForcedStepper(so)
    got = ex.vmap(fm)(torch.from_numpy(u).cuda(), torch.from_numpy(f).cuda()).cpu().numpy()
    for b in range(3):
        want = fo(u[b], f[b])
        assert rel(got[b], want) < 1e-5, b
        assert rel(fm(u[b], f[b]), want) < 1e-5, b  # NumPy in, NumPy out
    D = sm.num_spatial_dims
    uh, fh = o.fft(u[0], num_spatial_dims=D), o.fft(f[0], num_spatial_dims=D)
    gh = fm.step_fourier(torch.from_numpy(uh.astype(np.complex64)).cuda(),
                         torch.from_numpy(fh.astype(np.complex64)).cuda()).cpu().numpy()
    wh = fo.step_fourier(uh.astype(np.complex64), fh.astype(np.complex64))
    assert rel(gh.view(np.float32), wh.astype(np.complex64).view(np.float32)) < 1e-5
    with pytest.raises(ValueError):
        fm(u[0], f[0][..., :-1])


@pytest.mark.parametrize("name", ["burgers", "ns"])
@pytest.mark.parametrize("constant", [True, False])
def test_forced_rollout_matches_oracle(name, constant):
    sm, so, u, f = _case(name)
    n = 20
    fm, fo = ex.ForcedStepper(sm), o.ForcedStepper(so)
    if constant:
        aux = f
    else:
        aux = np.stack([f * (1.0 + 0.1 * t) for t in range(n)], axis=1).astype(np.float32)  # (B, n, C, N...)
    roll = ex.vmap(ex.rollout(fm, n, include_init=True, takes_aux=True, constant_aux=constant))
    got = roll(torch.from_numpy(u).cuda(), torch.from_numpy(aux).cuda()).cpu().numpy()
    assert got.shape == (3, n + 1) + u.shape[1:]
    for b in range(3):
        want = o.rollout(fo, n, include_init=True, takes_aux=True, constant_aux=constant)(u[b], aux[b])
        assert rel(got[b], want) < 1e-4, b
    last = ex.repeat(fm, n, takes_aux=True, constant_aux=constant)(torch.from_numpy(u[0]).cuda(),
                                                                   torch.from_numpy(aux[0]).cuda())
    assert rel(last.cpu().numpy(), got[0, -1]) < 1e-6


@pytest.mark.parametrize("gen,N", [
    (ex.ic.RandomSineWaves1d(1, cutoff=5), 200),
    (ex.ic.RandomAmplitudePhaseSeries(1, cutoff=5), 128),
    (ex.ic.RandomAmplitudePhaseSeries(2, cutoff=5, max_one=True), 256),
    (ex.ic.RandomAmplitudePhaseSeries(2, cutoff=3), 60),
    (ex.ic.RandomAmplitudePhaseSeries(3, cutoff=2, max_one=True), 32),
])
def test_device_ics_match_host_generators(gen, N):
    keys = [0, 1, 17, 123456]
    got = gen.device_batch(N, keys).cpu().numpy()
    for i, k in enumerate(keys):
        want = gen(N, key=k)
        assert got[i].shape == want.shape
        assert rel(got[i], want) < 2e-6, k
    s = ex.ic.build_ic_set(gen, num_points=N, num_samples=3, key=5, device=True)
    assert isinstance(s, torch.Tensor) and s.is_cuda and s.shape[0] == 3
    assert rel(s[2].cpu().numpy(), gen(N, key=7)) < 2e-6


NOISE_GENS = [
    ("grf", 1, 128, dict(powerlaw_exponent=2.0, max_one=True)),
    ("grf", 2, 64, dict(domain_extent=2 * np.pi, powerlaw_exponent=3.0, std_one=True)),
    ("grf", 3, 32, dict(powerlaw_exponent=4.0)),
    ("diffused", 1, 200, dict(intensity=0.001, max_one=True)),
    ("diffused", 2, 60, dict(intensity=0.0005, std_one=True)),
    ("diffused", 3, 16, dict(domain_extent=3.0, intensity=0.01, zero_mean=False)),
]


@pytest.mark.parametrize("kind,D,N,kw", NOISE_GENS, ids=[f"{g[0]}{g[1]}d" for g in NOISE_GENS])
def test_noise_filter_ics_on_the_gpu_match_oracle(kind, D, N, kw):
    """GaussianRandomField / DiffusedNoise built on the GPU (rfftn, an ETDRK0 filter step, irfftn,
    device normalisation) from the same white noise as the oracle: within 1e-5 relative L2; and
    device_batch equals the host generator's fields for the same keys (same draws)."""
    cls = ex.ic.GaussianRandomField if kind == "grf" else ex.ic.DiffusedNoise
    gen = cls(D, **kw)
    ofun = o.gaussian_random_field_from_noise if kind == "grf" else o.diffused_noise_from_noise
    keys = [0, 3, 42]
    noise = np.stack([ex.ic.WhiteNoise(D)(N, key=k) for k in keys])
    got = gen.from_noise(torch.from_numpy(noise).cuda()).cpu().numpy()
    for i in range(len(keys)):
        want = ofun(noise[i], num_spatial_dims=D, **kw)
        assert got[i].shape == want.shape
        assert rel(got[i], want) < 1e-5, keys[i]
    dev = gen.device_batch(N, keys).cpu().numpy()
    np.testing.assert_allclose(dev, got, rtol=0, atol=1e-6)
    for i, k in enumerate(keys):
        assert rel(dev[i], gen(N, key=k)) < 1e-5


def test_normalize_ic_on_the_device():
    """normalize_ic of a CUDA tensor (one field over all entries) against the oracle: 1e-6."""
    u = (3.0 + 2.0 * np.random.default_rng(1).standard_normal((1, 48, 48))).astype(np.float32)
    for kw in (dict(), dict(std_one=True), dict(max_one=True), dict(zero_mean=False, max_one=True)):
        got = ex.ic.normalize_ic(torch.from_numpy(u).cuda(), **kw).cpu().numpy()
        assert rel(got, o.normalize_ic(u, **kw)) < 1e-6, kw
    with pytest.raises(ValueError):
        ex.ic.normalize_ic(torch.from_numpy(u).cuda(), zero_mean=False, std_one=True)


@pytest.mark.parametrize("gen,N", [
    (ex.ic.RandomTruncatedFourierSeries(1, cutoff=5), 128),
    (ex.ic.RandomTruncatedFourierSeries(2, cutoff=4, max_one=True), 64),
    (ex.ic.RandomTruncatedFourierSeries(2, cutoff=3, std_one=True), 48),
    (ex.ic.RandomTruncatedFourierSeries(3, cutoff=2, offset_range=(-1.0, 1.0)), 16),
    (ex.ic.RandomSineWaves1d(1, cutoff=4, offset_range=(0.5, 1.0), max_one=True), 100),
    (ex.ic.RandomSineWaves1d(1, cutoff=6, std_one=True), 64),
])
def test_device_ics_reference_recipes(gen, N):
    """The reference's RandomTruncatedFourierSeries (low-pass-filtered white noise with an offset) and
    RandomSineWaves1d with offset / std_one / max_one, built on the GPU from the host generator's draws:
    within 1e-5 relative L2 of the host fields (both FP32 transforms)."""
    keys = [0, 5, 77]
    got = gen.device_batch(N, keys).cpu().numpy()
    for i, k in enumerate(keys):
        want = gen(N, key=k)
        assert got[i].shape == want.shape
        assert rel(got[i], want) < 1e-5, k
