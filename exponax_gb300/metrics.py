"""Evaluation metrics (exponax/metrics/*, _spectral.get_spectrum) on device fields.

Device tensors go through the CUDA kernels of libexgb.so (``exgb_spectrum``,
``exgb_field_sums``); NumPy inputs are moved to the device and the result is
returned as NumPy.  Single fields have the reference's shape ``(C, N, ...)``;
``mean_metric`` averages over a leading batch axis."""

from __future__ import annotations

import numpy as np

from . import _device
from ._lib import check, load
from .spectral import fft


def _field_sums(u_pred, u_ref):
    """(C, 4) FP64 sums per channel: sum (a-b)^2, sum b^2, sum a b, sum a^2."""
    torch = _device.torch()
    a, back = _device.to_device(u_pred, "float32")
    b, _ = _device.to_device(u_ref, "float32")
    if a.shape != b.shape:
        raise ValueError(f"Shapes of u_pred {tuple(a.shape)} and u_ref {tuple(b.shape)} differ")
    C = a.shape[0]
    n = a.numel() // max(C, 1)
    out = torch.empty((C, 4), dtype=torch.float64, device=a.device)
    check(load().exgb_field_sums(_device.stream(), C, n, a.data_ptr(), b.data_ptr(), out.data_ptr()), "field_sums")
    return out, back


def nRMSE(u_pred, u_ref, *, domain_extent: float = 1.0):
    """metrics/_spatial.py:537-586: sum over channels of
    ||u_pred - u_ref||_2 / ||u_ref||_2 (the (L/N)^D factors cancel)."""
    s, back = _field_sums(u_pred, u_ref)
    v = (s[:, 0].sqrt() / s[:, 1].sqrt()).sum().float()
    return float(v) if not isinstance(u_pred, _device.torch().Tensor) else v


def correlation(u_pred, u_ref):
    """metrics/_correlation.py:33-60: channel mean of the normalised inner product."""
    s, back = _field_sums(u_pred, u_ref)
    v = (s[:, 2] / (s[:, 3].sqrt() * s[:, 1].sqrt())).mean().float()
    return float(v) if not isinstance(u_pred, _device.torch().Tensor) else v


def mean_metric(metric_fn, u_pred, u_ref, **kwargs):
    """metrics/_utils.py:5-18: batch mean of a per-sample metric."""
    vals = [metric_fn(u_pred[i], u_ref[i], **kwargs) for i in range(u_pred.shape[0])]
    if isinstance(vals[0], float):
        return float(np.mean(vals))
    t = _device.torch()
    return t.stack(vals).mean()


def get_spectrum(state, *, power: bool = True, radial_binning: str = "sum", num_spatial_dims: int | None = None):
    """_spectral.py:866-1030: power (or amplitude) spectrum of a state (C, N, ...),
    radially binned over |k| in [i - 1/2, i + 1/2) for D >= 2 ("sum" or "average");
    returns (C, N//2 + 1).  D = state.ndim - 1 as in the reference; pass
    num_spatial_dims for leading batch axes: (B, C, N, ...) -> (B, C, N//2 + 1)."""
    if radial_binning not in ("sum", "average"):
        raise ValueError(f"radial_binning must be 'sum' or 'average', got {radial_binning!r}")
    torch = _device.torch()
    t, back = _device.to_device(state, "float32")
    N = t.shape[-1]
    D = int(num_spatial_dims) if num_spatial_dims is not None else t.ndim - 1
    if D < 1 or D > 3 or any(int(x) != N for x in t.shape[-D:]):
        raise ValueError(f"Expected 1 to 3 spatial axes of equal length, got shape {tuple(t.shape)}")
    lead = t.shape[:-D]
    count = int(np.prod(lead)) if lead else 1
    uh = fft(t.reshape((count,) + tuple(t.shape[-D:])), num_spatial_dims=D).contiguous()
    out = torch.empty((count, N // 2 + 1), dtype=torch.float32, device=t.device)
    check(load().exgb_spectrum(_device.stream(), D, N, count, uh.data_ptr(), out.data_ptr(), int(bool(power)),
                               int(radial_binning == "average")), "spectrum")
    return back(out.reshape(tuple(lead) + (N // 2 + 1,)))
