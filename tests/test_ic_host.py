"""Host side of the noise-based initial-condition generators (ic/_white_noise.py,
ic/_gaussian_random_field.py, ic/_diffused_noise.py, ic/_base_ic.py) against the oracle on the
same white noise: relative L2 within 1e-5 (both FP32), the reference's ValueErrors for invalid
normalisation options, and seeded determinism."""

import numpy as np
import pytest

import exponax_gb300 as ex
from oracle import exponax_np as o


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("D,N", [(1, 100), (2, 48), (3, 16)])
@pytest.mark.parametrize("norm", [dict(), dict(std_one=True), dict(max_one=True), dict(zero_mean=False)])
def test_gaussian_random_field_host(D, N, norm):
    gen = ex.ic.GaussianRandomField(D, domain_extent=2.0, powerlaw_exponent=3.0, **norm)
    u = gen(N, key=11)
    noise = ex.ic.WhiteNoise(D)(N, key=11)
    want = o.gaussian_random_field_from_noise(noise, num_spatial_dims=D, domain_extent=2.0, powerlaw_exponent=3.0,
                                              **norm)
    assert u.shape == (1,) + (N,) * D and u.dtype == np.float32
    assert rel(u, want) < 1e-5


@pytest.mark.parametrize("D,N", [(1, 128), (2, 40), (3, 12)])
def test_diffused_noise_host(D, N):
    gen = ex.ic.DiffusedNoise(D, intensity=0.002, max_one=True)
    want = o.diffused_noise_from_noise(ex.ic.WhiteNoise(D)(N, key=4), num_spatial_dims=D, intensity=0.002,
                                       max_one=True)
    assert rel(gen(N, key=4), want) < 1e-5


def test_white_noise_and_normalisation_options():
    w = ex.ic.WhiteNoise(2, std=0.5)
    a, b = w(32, key=9), w(32, key=9)
    np.testing.assert_array_equal(a, b)
    assert a.shape == (1, 32, 32) and abs(float(a.std()) - 0.5) < 0.05
    assert not np.array_equal(a, w(32, key=10))
    for cls in (ex.ic.GaussianRandomField, ex.ic.DiffusedNoise):
        with pytest.raises(ValueError):
            cls(1, zero_mean=False, std_one=True)
        with pytest.raises(ValueError):
            cls(1, std_one=True, max_one=True)
    u = np.random.default_rng(0).standard_normal((1, 20)).astype(np.float32) + 4
    for kw in (dict(), dict(std_one=True), dict(max_one=True)):
        np.testing.assert_allclose(ex.ic.normalize_ic(u, **kw), o.normalize_ic(u, **kw), rtol=1e-6, atol=1e-7)


def test_grf_power_spectrum_follows_the_power_law():
    """The radially binned power of a 2D field decays like |k|^-p (fit over the resolved range)."""
    p = 3.0
    gen = ex.ic.GaussianRandomField(2, powerlaw_exponent=p, zero_mean=True)
    spec = np.zeros(33)
    for key in range(16):
        uh = np.fft.rfft2(gen(64, key=key)[0])
        kx = np.fft.fftfreq(64, 1 / 64)[:, None]
        ky = np.fft.rfftfreq(64, 1 / 64)[None, :]
        kr = np.rint(np.sqrt(kx ** 2 + ky ** 2)).astype(int)
        np.add.at(spec, np.minimum(kr, 32).ravel(), (np.abs(uh) ** 2).ravel())
    k = np.arange(4, 24)
    # the half-plane shell of radius k holds ~pi k modes: power per mode ~ k^-p
    slope = np.polyfit(np.log(k), np.log(spec[k] / k), 1)[0]
    assert abs(slope + p) < 0.3, slope
