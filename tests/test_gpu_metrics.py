"""Evaluation kernels against the oracle: get_spectrum (_spectral.py:866-1030) in 1D/2D/3D, power and
amplitude, sum and average binning (FP32, relative 1e-5 per bin where the bin is not tiny; binning and
NaN placement exact); nRMSE and correlation (metrics/_spatial.py:537-586, _correlation.py:33-60)
within 1e-6 relative."""

import numpy as np
import pytest

import exponax_gb300 as ex
from exponax_gb300 import metrics
from oracle import exponax_np as o

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.mark.parametrize("D,N", [(1, 64), (1, 200), (2, 64), (2, 128), (2, 45), (3, 32)])
@pytest.mark.parametrize("power", [True, False])
@pytest.mark.parametrize("binning", ["sum", "average"])
def test_get_spectrum_matches_oracle(D, N, power, binning):
    rng = np.random.default_rng(D * 1000 + N)
    u = rng.standard_normal((2,) + (N,) * D).astype(np.float32)
    got = metrics.get_spectrum(torch.from_numpy(u).cuda(), power=power, radial_binning=binning).cpu().numpy()
    if D == 1:
        want = o.get_spectrum(u, power=power)
    else:
        want = o.get_spectrum(u, power=power, radial_binning=binning)
    assert got.shape == want.shape == (2, N // 2 + 1)
    np.testing.assert_array_equal(np.isnan(got), np.isnan(want))
    ok = ~np.isnan(want)
    scale = np.nanmax(np.abs(want))
    assert np.max(np.abs(got[ok] - want[ok])) <= 1e-5 * scale


def test_get_spectrum_numpy_in_numpy_out_and_parseval():
    u = np.random.default_rng(3).standard_normal((1, 64, 64)).astype(np.float32)
    s = metrics.get_spectrum(u)
    assert isinstance(s, np.ndarray)
    # Parseval for a band-limited field (energy inside the Nyquist sphere)
    g = ex.ic.RandomAmplitudePhaseSeries(2, cutoff=5)
    v = g(64, key=1)
    sv = metrics.get_spectrum(v)
    assert abs(float(sv.sum()) - 0.5 * float(np.mean(v.astype(np.float64) ** 2))) < 1e-5 * float(np.mean(v ** 2))


def test_batched_spectrum():
    rng = np.random.default_rng(5)
    u = rng.standard_normal((3, 2, 32, 32)).astype(np.float32)
    got = metrics.get_spectrum(torch.from_numpy(u).cuda(), num_spatial_dims=2).cpu().numpy()
    for b in range(3):
        want = o.get_spectrum(u[b])
        assert np.max(np.abs(got[b] - want)) <= 1e-5 * np.max(np.abs(want))


def test_nrmse_and_correlation():
    rng = np.random.default_rng(11)
    ref = rng.standard_normal((2, 48, 48)).astype(np.float32)
    pred = (ref + 0.1 * rng.standard_normal(ref.shape)).astype(np.float32)
    want_n = sum(np.linalg.norm(pred[c].astype(np.float64) - ref[c]) / np.linalg.norm(ref[c]) for c in range(2))
    want_c = np.mean([np.sum(pred[c].astype(np.float64) * ref[c]) / (np.linalg.norm(pred[c]) * np.linalg.norm(ref[c]))
                      for c in range(2)])
    gn = float(metrics.nRMSE(torch.from_numpy(pred).cuda(), torch.from_numpy(ref).cuda()))
    gc = float(metrics.correlation(torch.from_numpy(pred).cuda(), torch.from_numpy(ref).cuda()))
    assert abs(gn - want_n) <= 1e-6 * want_n
    assert abs(gc - want_c) <= 1e-6
    assert isinstance(metrics.nRMSE(pred, ref), float)
    mm = metrics.mean_metric(metrics.nRMSE, torch.from_numpy(pred[None]).cuda(), torch.from_numpy(ref[None]).cuda())
    assert abs(float(mm) - want_n) <= 1e-6 * want_n


SPATIAL = ["MAE", "nMAE", "sMAE", "MSE", "nMSE", "sMSE", "RMSE", "nRMSE", "sRMSE"]
FOURIER = ["fourier_MAE", "fourier_nMAE", "fourier_MSE", "fourier_nMSE", "fourier_RMSE", "fourier_nRMSE"]
H1 = ["H1_MAE", "H1_nMAE", "H1_MSE", "H1_nMSE", "H1_RMSE", "H1_nRMSE"]


def _pair(D, N, C, key):
    rng = np.random.default_rng(key)
    a = rng.standard_normal((C,) + (N,) * D).astype(np.float32)
    b = (a + 0.3 * rng.standard_normal(a.shape)).astype(np.float32)
    return a, b


@pytest.mark.parametrize("D,N", [(1, 64), (2, 32), (3, 12)])
def test_metric_families_match_oracle(D, N):
    """Every spatial, Fourier and H1 metric (metrics/_spatial.py, _fourier.py, _derivative.py) on
    two-channel random fields against the oracle: 1e-5 relative; also without a reference where the
    metric allows it, with a band (low, high) and a derivative order, and on device tensors."""
    a, b = _pair(D, N, 2, 10 * D)
    for name in SPATIAL:
        got, want = getattr(ex.metrics, name)(a, b, domain_extent=2.0), getattr(o, name)(a, b, domain_extent=2.0)
        assert abs(got - want) <= 1e-5 * abs(want), (name, got, want)
    for name in FOURIER + H1:
        for kw in (dict(), dict(low=2, high=N // 4), dict(high=3)):
            got = getattr(ex.metrics, name)(a, b, domain_extent=2.0, **kw)
            want = getattr(o, name)(a, b, domain_extent=2.0, **kw)
            assert abs(got - want) <= 1e-5 * abs(want), (name, kw, got, want)
    for name in ("MAE", "MSE", "RMSE", "fourier_MAE", "fourier_MSE", "fourier_RMSE", "H1_MSE"):
        got, want = getattr(ex.metrics, name)(a), getattr(o, name)(a)
        assert abs(got - want) <= 1e-5 * abs(want), (name, got, want)
    for order in (0, 1, 2, 1.5):
        got = ex.metrics.fourier_nRMSE(a, b, derivative_order=order)
        want = o.fourier_nRMSE(a, b, derivative_order=order)
        assert abs(got - want) <= 1e-5 * abs(want), (order, got, want)
    t = ex.metrics.sMSE(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda())
    assert isinstance(t, torch.Tensor) and abs(float(t) - o.sMSE(a, b)) <= 1e-5 * o.sMSE(a, b)
    for p in (1.0, 3.0):
        got = ex.metrics.spatial_norm(a, b, mode="normalized", inner_exponent=p, outer_exponent=1 / p)
        want = o.spatial_norm(a, b, mode="normalized", inner_exponent=p, outer_exponent=1 / p)
        assert abs(got - want) <= 1e-5 * abs(want), (p, got, want)
    with pytest.raises(ValueError):
        ex.metrics.nMSE(a)


def test_fourier_and_spatial_norms_agree_by_parseval():
    """Size-independent property: the Fourier (R)MSE equals the spatial one (Parseval) for 256^2 fields."""
    a, b = _pair(2, 256, 1, 3)
    for fs, ss in (("fourier_MSE", "MSE"), ("fourier_nRMSE", "nRMSE")):
        f, s = getattr(ex.metrics, fs)(a, b), getattr(ex.metrics, ss)(a, b)
        assert abs(f - s) <= 1e-5 * abs(s), (fs, f, s)


def test_mean_metric_over_a_batch():
    a = np.stack([_pair(2, 32, 1, k)[0] for k in range(3)])
    b = np.stack([_pair(2, 32, 1, k)[1] for k in range(3)])
    got = ex.metrics.mean_metric(ex.metrics.nRMSE, a, b)
    want = np.mean([o.nRMSE(a[i], b[i]) for i in range(3)])
    assert abs(got - want) <= 1e-5 * want
