"""Evaluation metrics (exponax/metrics/*, _spectral.get_spectrum) on device fields.

Device tensors go through the CUDA kernels of libexgb.so (``exgb_spectrum``,
``exgb_field_sums``, ``exgb_field_pnorms``, ``exgb_fourier_pnorms``); NumPy
inputs are moved to the device and the result is returned as a Python float
(device tensors give a 0-d tensor).  Single fields have the reference's shape
``(C, N, ...)``; ``mean_metric`` averages over a leading batch axis.  The
kernels return FP64 per-field sums; the per-channel exponents and the
normalized / symmetric combinations are applied to those few numbers."""

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


def mean_metric(metric_fn, *args, **kwargs):
    """metrics/_utils.py:5-18: batch mean of a per-sample metric over the leading axis of every argument."""
    vals = [metric_fn(*(a[i] for a in args), **kwargs) for i in range(args[0].shape[0])]
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


# ---------------------------------------------------------------------------- spatial family
def _ret(v, like):
    """A 0-d FP32 tensor for tensor inputs, a Python float otherwise."""
    t = _device.torch()
    v = v.float() if isinstance(v, t.Tensor) else t.tensor(float(v))
    return v if isinstance(like, t.Tensor) else float(v)


def _pnorm_sums(state, state_ref, p):
    """(C, 3) FP64 per-channel sums |a - b|^p, |a|^p, |b|^p (exgb_field_pnorms); b may be None."""
    torch = _device.torch()
    a, _ = _device.to_device(state, "float32")
    b = None
    if state_ref is not None:
        b, _ = _device.to_device(state_ref, "float32")
        if a.shape != b.shape:
            raise ValueError(f"Shapes of the state {tuple(a.shape)} and the reference {tuple(b.shape)} differ")
    C = a.shape[0]
    n = a.numel() // max(C, 1)
    out = torch.empty((C, 3), dtype=torch.float64, device=a.device)
    check(load().exgb_field_pnorms(_device.stream(), C, n, a.data_ptr(), b.data_ptr() if b is not None else None,
                                   float(inner_exponent_checked(p)), out.data_ptr()), "field_pnorms")
    return out, a


def inner_exponent_checked(p):
    if not p > 0:
        raise ValueError(f"inner_exponent must be positive, got {p}")
    return p


def spatial_aggregator(state_no_channel, *, num_spatial_dims=None, domain_extent: float = 1.0, num_points=None,
                       inner_exponent: float = 2.0, outer_exponent=None):
    """metrics/_spatial.py:8-83: (scale * sum |u|^p)^q with scale = (L / N)^D of one channel-less field."""
    t, _ = _device.to_device(state_no_channel, "float32")
    D = t.ndim if num_spatial_dims is None else num_spatial_dims
    N = t.shape[-1] if num_points is None else num_points
    q = 1 / inner_exponent if outer_exponent is None else outer_exponent
    s, _ = _pnorm_sums(t.reshape(1, -1), None, inner_exponent)
    return _ret(((domain_extent / N) ** D * s[0, 0]) ** q, state_no_channel)


def spatial_norm(state, state_ref=None, *, mode: str = "absolute", domain_extent: float = 1.0,
                 inner_exponent: float = 2.0, outer_exponent=None):
    """metrics/_spatial.py:86-195: per channel (scale sum |u - u_ref|^p)^q, optionally divided by the
    reference's norm ("normalized") or by the mean of both norms ("symmetric"), summed over channels."""
    if mode not in ("absolute", "normalized", "symmetric"):
        raise ValueError(f"unknown mode {mode!r}")
    if state_ref is None and mode != "absolute":
        raise ValueError(f"mode '{mode}' requires state_ref")
    s, a = _pnorm_sums(state, state_ref, inner_exponent)
    D = a.ndim - 1
    N = a.shape[-1]
    q = 1 / inner_exponent if outer_exponent is None else outer_exponent
    norms = ((domain_extent / N) ** D * s) ** q  # (C, 3): diff, state, ref
    if mode == "normalized":
        v = (norms[:, 0] / norms[:, 2]).sum()
    elif mode == "symmetric":
        v = (2 * norms[:, 0] / (norms[:, 1] + norms[:, 2])).sum()
    else:
        v = norms[:, 0].sum()
    return _ret(v, state)


def _spatial_metric(name, mode, p, q, ref_required):
    def metric(u_pred, u_ref=None, *, domain_extent: float = 1.0):
        if ref_required and u_ref is None:
            raise ValueError(f"{name} requires u_ref")
        return spatial_norm(u_pred, u_ref, mode=mode, domain_extent=domain_extent, inner_exponent=p,
                            outer_exponent=q)

    metric.__name__ = name
    metric.__doc__ = f"metrics/_spatial.py: {mode} spatial norm, inner exponent {p}, outer exponent {q}."
    return metric


MAE = _spatial_metric("MAE", "absolute", 1.0, 1.0, False)
nMAE = _spatial_metric("nMAE", "normalized", 1.0, 1.0, True)
sMAE = _spatial_metric("sMAE", "symmetric", 1.0, 1.0, True)
MSE = _spatial_metric("MSE", "absolute", 2.0, 1.0, False)
nMSE = _spatial_metric("nMSE", "normalized", 2.0, 1.0, True)
sMSE = _spatial_metric("sMSE", "symmetric", 2.0, 1.0, True)
RMSE = _spatial_metric("RMSE", "absolute", 2.0, 0.5, False)
sRMSE = _spatial_metric("sRMSE", "symmetric", 2.0, 0.5, True)


# ---------------------------------------------------------------------------- Fourier and H1 families
def _fourier_sums(fields, D, p, low, high, derivative_order, domain_extent):
    """(F, Dd) FP64 sums of exgb_fourier_pnorms over F channel-less fields (F, N, ..., N)."""
    torch = _device.torch()
    N = fields.shape[-1]
    if low is not None or high is not None:
        lo = 0 if low is None else int(low)
        hi = (N // 2) + 1 if high is None else int(high)
    else:
        lo, hi = 0, 1 << 30
    uh = fft(fields, num_spatial_dims=D).contiguous()
    F = fields.shape[0]
    Dd = D if derivative_order is not None else 1
    out = torch.empty((F, Dd), dtype=torch.float64, device=fields.device)
    check(load().exgb_fourier_pnorms(_device.stream(), D, N, F, uh.data_ptr(), float(inner_exponent_checked(p)),
                                     float(derivative_order) if derivative_order is not None else -1.0, lo, hi,
                                     float(domain_extent), out.data_ptr()), "fourier_pnorms")
    return out


def _fourier_norms(fields, D, *, domain_extent, inner_exponent, outer_exponent, low, high, derivative_order):
    N = fields.shape[-1]
    q = 1 / inner_exponent if outer_exponent is None else outer_exponent
    s = _fourier_sums(fields, D, inner_exponent, low, high, derivative_order, domain_extent)
    return (((domain_extent / N) ** D) * s).pow(q).sum(dim=1)


def fourier_aggregator(state_no_channel, *, num_spatial_dims=None, domain_extent: float = 1.0, num_points=None,
                       inner_exponent: float = 2.0, outer_exponent=None, low=None, high=None, derivative_order=None):
    """metrics/_fourier.py:15-140: the norm of one channel-less field from its rfftn coefficients
    (|c| < 1e-5 dropped, optional band low <= |k| <= high, optional derivative, reconstruction
    scaling), summed over the derivative components."""
    t, _ = _device.to_device(state_no_channel, "float32")
    D = t.ndim if num_spatial_dims is None else num_spatial_dims
    if num_points is not None and num_points != t.shape[-1]:
        raise ValueError("num_points must match the field")
    v = _fourier_norms(t[None], D, domain_extent=domain_extent, inner_exponent=inner_exponent,
                       outer_exponent=outer_exponent, low=low, high=high, derivative_order=derivative_order)
    return _ret(v[0], state_no_channel)


def fourier_norm(state, state_ref=None, *, mode: str = "absolute", domain_extent: float = 1.0,
                 inner_exponent: float = 2.0, outer_exponent=None, low=None, high=None, derivative_order=None):
    """metrics/_fourier.py:143-235: per-channel Fourier aggregation of state - state_ref (absolute) or
    divided by that of state_ref (normalized), summed over channels."""
    if mode not in ("absolute", "normalized"):
        raise ValueError(f"unknown mode {mode!r}")
    if state_ref is None and mode == "normalized":
        raise ValueError("mode 'normalized' requires state_ref")
    torch = _device.torch()
    a, _ = _device.to_device(state, "float32")
    D = a.ndim - 1
    fields = a
    if state_ref is not None:
        b, _ = _device.to_device(state_ref, "float32")
        if a.shape != b.shape:
            raise ValueError(f"Shapes of the state {tuple(a.shape)} and the reference {tuple(b.shape)} differ")
        C = a.shape[0]
        fields = torch.empty((2 * C,) + tuple(a.shape[1:]), dtype=torch.float32, device=a.device)
        # fields[:C] = a - b (exgb_axpy), fields[C:] = b
        check(load().exgb_axpy(_device.stream(), a.numel(), -1.0, a.data_ptr(), b.data_ptr(), fields.data_ptr()),
              "fourier_norm")
        fields[C:].copy_(b)
    kw = dict(domain_extent=domain_extent, inner_exponent=inner_exponent, outer_exponent=outer_exponent, low=low,
              high=high, derivative_order=derivative_order)
    n = _fourier_norms(fields, D, **kw)
    C = a.shape[0]
    v = (n[:C] / n[C:]).sum() if mode == "normalized" else n[:C].sum()
    return _ret(v, state)


def _fourier_metric(name, mode, p, q, ref_required):
    def metric(u_pred, u_ref=None, *, domain_extent: float = 1.0, low=None, high=None, derivative_order=None):
        if ref_required and u_ref is None:
            raise ValueError(f"{name} requires u_ref")
        return fourier_norm(u_pred, u_ref, mode=mode, domain_extent=domain_extent, inner_exponent=p,
                            outer_exponent=q, low=low, high=high, derivative_order=derivative_order)

    metric.__name__ = name
    metric.__doc__ = f"metrics/_fourier.py: {mode} Fourier norm, inner exponent {p}, outer exponent {q}."
    return metric


fourier_MAE = _fourier_metric("fourier_MAE", "absolute", 1.0, 1.0, False)
fourier_nMAE = _fourier_metric("fourier_nMAE", "normalized", 1.0, 1.0, True)
fourier_MSE = _fourier_metric("fourier_MSE", "absolute", 2.0, 1.0, False)
fourier_nMSE = _fourier_metric("fourier_nMSE", "normalized", 2.0, 1.0, True)
fourier_RMSE = _fourier_metric("fourier_RMSE", "absolute", 2.0, 0.5, False)
fourier_nRMSE = _fourier_metric("fourier_nRMSE", "normalized", 2.0, 0.5, True)


def _h1_metric(name, fm):
    def metric(u_pred, u_ref=None, *, domain_extent: float = 1.0, low=None, high=None):
        kw = dict(domain_extent=domain_extent, low=low, high=high)
        a = fm(u_pred, u_ref, derivative_order=None, **kw)
        b = fm(u_pred, u_ref, derivative_order=1, **kw)
        return a + b

    metric.__name__ = name
    metric.__doc__ = f"metrics/_derivative.py: {fm.__name__} of the field plus that of its first derivative."
    return metric


H1_MAE = _h1_metric("H1_MAE", fourier_MAE)
H1_nMAE = _h1_metric("H1_nMAE", fourier_nMAE)
H1_MSE = _h1_metric("H1_MSE", fourier_MSE)
H1_nMSE = _h1_metric("H1_nMSE", fourier_nMSE)
H1_RMSE = _h1_metric("H1_RMSE", fourier_RMSE)
H1_nRMSE = _h1_metric("H1_nRMSE", fourier_nRMSE)

