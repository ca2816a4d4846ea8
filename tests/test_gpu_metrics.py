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
    g = ex.ic.RandomTruncatedFourierSeries(2, cutoff=5)
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
