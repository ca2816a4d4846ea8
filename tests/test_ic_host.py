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


@pytest.mark.parametrize("D,N", [(1, 64), (2, 32), (3, 12)])
@pytest.mark.parametrize("kw", [dict(), dict(std_one=True), dict(max_one=True), dict(offset_range=(-1.0, 1.0))])
def test_random_truncated_fourier_series_follows_the_reference_recipe(D, N, kw):
    """ic/_truncated_fourier_series.py:65-100 (white noise -> low-pass -> offset -> irfftn -> normalise)
    against the oracle on the same noise and offset draws: 1e-5."""
    gen = ex.ic.RandomTruncatedFourierSeries(D, cutoff=3, **kw)
    noise, offset = gen._draws(N, 9)
    np.testing.assert_array_equal(noise, ex.ic.WhiteNoise(D)(N, key=9))
    zero_mean = kw.get("offset_range", (0.0, 0.0)) == (0.0, 0.0)
    want = o.truncated_fourier_series_from_noise(noise, num_spatial_dims=D, cutoff=3, offset=offset,
                                                 zero_mean=zero_mean, std_one=kw.get("std_one", False),
                                                 max_one=kw.get("max_one", False))
    got = gen(N, key=9)
    assert got.shape == (1,) + (N,) * D
    assert rel(got, want) < 1e-5
    # only the modes |k_d| <= cutoff carry energy
    hat = np.fft.rfftn(got[0].astype(np.float64))
    outside = ~o.low_pass_filter_mask(D, N, cutoff=3)[0]
    assert np.abs(hat[outside]).max() < 1e-4 * np.abs(hat).max()


def test_random_truncated_fourier_series_arguments():
    with pytest.raises(ValueError):
        ex.ic.RandomTruncatedFourierSeries(2, offset_range=(0.0, 1.0), std_one=True)
    with pytest.raises(ValueError):
        ex.ic.RandomTruncatedFourierSeries(2, std_one=True, max_one=True)


def test_sine_waves_1d_and_generator():
    """ic/_sine_waves_1d.py: the closed form on a grid, the generator's ranges and normalisations,
    gen_ic_fun evaluated on make_grid equal to the generator's own field."""
    L = 3.0
    x = ex.make_grid(1, L, 50)
    sw = ex.ic.SineWaves1d(L, (0.5, -2.0), (1, 3), (0.1, 1.0), offset=0.25)
    xd = x.astype(np.float64)
    want = 0.5 * np.sin(2 * np.pi / L * xd + 0.1) - 2.0 * np.sin(3 * 2 * np.pi / L * xd + 1.0) + 0.25
    np.testing.assert_allclose(sw(x), want, atol=1e-6)
    with pytest.raises(ValueError):
        ex.ic.SineWaves1d(L, (1.0,), (1, 2), (0.0,))
    with pytest.raises(ValueError):
        ex.ic.SineWaves1d(L, (1.0,), (1,), (0.0,), offset=1.0, std_one=True)
    g = ex.ic.RandomSineWaves1d(1, domain_extent=L, cutoff=4, amplitude_range=(0.5, 1.0), phase_range=(0.0, 0.1),
                                offset_range=(2.0, 3.0))
    u = g(64, key=5)
    assert 2.0 <= u.mean() <= 3.0
    np.testing.assert_allclose(g.gen_ic_fun(key=5)(ex.make_grid(1, L, 64)), u, atol=1e-5)
    assert abs(float(ex.ic.RandomSineWaves1d(1, std_one=True)(64, key=1).std()) - 1.0) < 1e-5
    assert abs(float(np.abs(ex.ic.RandomSineWaves1d(1, max_one=True)(64, key=1)).max()) - 1.0) < 1e-6
    with pytest.raises(ValueError):
        ex.ic.RandomSineWaves1d(2)


def test_blobs_discontinuities_and_wrappers():
    """The closed-form generators (ic/_gaussian_blob.py, _discontinuities.py) and the wrappers
    (_multi_channel.py, _scaled.py, _clamping.py)."""
    blob = ex.ic.GaussianBlob(np.array([0.5, 0.25]), np.diag([0.01, 0.02]))
    g = ex.make_grid(2, 1.0, 40)
    v = blob(g)
    assert v.shape == (1, 40, 40) and abs(v[0, 20, 10] - 1.0) < 1e-12
    np.testing.assert_allclose(ex.ic.GaussianBlob(np.array([0.5, 0.25]), np.diag([0.01, 0.02]),
                                                  one_complement=True)(g), 1 - v)
    rb = ex.ic.RandomGaussianBlobs(2, num_blobs=3)
    u = rb(32, key=1)
    assert u.shape == (1, 32, 32) and 0 < u.max() <= 1.0
    np.testing.assert_array_equal(u, rb(32, key=1))
    d = ex.ic.Discontinuity((0.2,), (0.6,), 2.0)(ex.make_grid(1, 1.0, 10))
    np.testing.assert_array_equal(d[0], [0, 0, 0, 2, 2, 2, 0, 0, 0, 0])
    rd = ex.ic.RandomDiscontinuities(2, num_discontinuities=4, zero_mean=True, max_one=True)
    w = rd(24, key=2)
    assert abs(w.mean()) < 1e-6 and abs(np.abs(w).max() - 1.0) < 1e-6
    mc = ex.ic.RandomMultiChannelICGenerator([ex.ic.RandomAmplitudePhaseSeries(2, cutoff=3),
                                              ex.ic.RandomGaussianBlobs(2)])
    m = mc(16, key=3)
    assert m.shape == (2, 16, 16)
    np.testing.assert_array_equal(m, mc(16, key=3))
    sc = ex.ic.ScaledICGenerator(ex.ic.RandomGaussianBlobs(1), 3.0)
    np.testing.assert_allclose(sc(32, key=4), 3.0 * ex.ic.RandomGaussianBlobs(1)(32, key=4))
    np.testing.assert_allclose(sc.gen_ic_fun(key=4)(ex.make_grid(1, 1.0, 32)), sc(32, key=4), atol=1e-6)
    cl = ex.ic.ClampingICGenerator(ex.ic.RandomAmplitudePhaseSeries(2, cutoff=3), limits=(-2.0, 5.0))
    c = cl(32, key=6)
    assert abs(c.min() + 2.0) < 1e-6 and abs(c.max() - 5.0) < 1e-5
    s = ex.ic.build_ic_set(ex.ic.RandomTruncatedFourierSeries(1), num_points=32, num_samples=4, key=7)
    assert s.shape == (4, 1, 32)
