"""Spectral helpers: operator assembly on the host and the device FFTs.

Operator builders (wavenumbers, derivative / Laplace / gradient-inner-product
operators, masks, scaling arrays, mode slices) run once per stepper
construction on the host in NumPy.  They follow exponax/_spectral.py of the
reference (file:line given per function) and return complex128 / float64
arrays (the plan rounds to float32 on the device, as the reference works in
float32).  ``fft`` / ``ifft`` run on the GPU through libexgb.so.
"""

from __future__ import annotations

from itertools import product

import numpy as np

from . import _device
from ._lib import check, load


def spatial_shape(num_spatial_dims: int, num_points: int) -> tuple:
    """_spectral.py:230-250"""
    return (num_points,) * num_spatial_dims


def wavenumber_shape(num_spatial_dims: int, num_points: int) -> tuple:
    """_spectral.py:253-275"""
    return (num_points,) * (num_spatial_dims - 1) + (num_points // 2 + 1,)


def space_indices(num_spatial_dims: int) -> tuple:
    """_spectral.py:212-227"""
    return tuple(range(-num_spatial_dims, 0))


def build_wavenumbers(num_spatial_dims: int, num_points: int) -> np.ndarray:
    """_spectral.py:13-49: integer wavenumbers, fftfreq on the leading axes
    and rfftfreq on the last, 'ij' indexing; shape (D, N, ..., N//2+1)."""
    last = np.arange(num_points // 2 + 1, dtype=np.float64)
    lead = np.fft.fftfreq(num_points, 1.0 / num_points)
    axes = [lead] * (num_spatial_dims - 1) + [last]
    return np.stack(np.meshgrid(*axes, indexing="ij"))


def build_scaled_wavenumbers(num_spatial_dims: int, domain_extent: float, num_points: int) -> np.ndarray:
    """_spectral.py:52-83: wavenumbers times 2 pi / L."""
    return (2 * np.pi / domain_extent) * build_wavenumbers(num_spatial_dims, num_points)


def build_derivative_operator(num_spatial_dims: int, domain_extent: float, num_points: int) -> np.ndarray:
    """_spectral.py:86-115: i k, shape (D, N, ..., N//2+1)."""
    return 1j * build_scaled_wavenumbers(num_spatial_dims, domain_extent, num_points)


def build_laplace_operator(derivative_operator: np.ndarray, *, order: int = 2) -> np.ndarray:
    """_spectral.py:118-155: sum_d (i k_d)^order (order even, 0 -> ones)."""
    if order % 2 != 0:
        raise ValueError("Order must be even.")
    if order == 0:
        return np.ones((1,) + derivative_operator.shape[1:], dtype=derivative_operator.dtype)
    return np.sum(derivative_operator**order, axis=0, keepdims=True)


def build_gradient_inner_product_operator(derivative_operator: np.ndarray, velocity, *, order: int = 1):
    """_spectral.py:158-209: sum_d c_d (i k_d)^order (order odd)."""
    if order % 2 != 1:
        raise ValueError("Order must be odd.")
    velocity = np.asarray(velocity, dtype=np.float64)
    if velocity.shape != (derivative_operator.shape[0],):
        raise ValueError(
            f"Expected velocity shape to be {derivative_operator.shape[0]}, got {velocity.shape}."
        )
    return np.tensordot(velocity, derivative_operator**order, axes=(0, 0))[None, ...]


def low_pass_filter_mask(num_spatial_dims: int, num_points: int, *, cutoff: float, axis_separate: bool = True):
    """_spectral.py:278-342: keep |k_d| <= cutoff (inclusive), compared in
    float32 as the reference does under its default precision."""
    wn = build_wavenumbers(num_spatial_dims, num_points).astype(np.float32)
    cut = np.float32(cutoff)
    if axis_separate:
        mask = np.all(np.abs(wn) <= cut, axis=0)
    else:
        mask = np.linalg.norm(wn, axis=0) <= cut
    return mask[None, ...]


def oddball_filter_mask(num_spatial_dims: int, num_points: int):
    """_spectral.py:345-400: all modes except the Nyquist planes (even N)."""
    if num_points % 2 == 1:
        return np.ones((1,) + wavenumber_shape(num_spatial_dims, num_points), dtype=bool)
    return low_pass_filter_mask(num_spatial_dims, num_points, cutoff=num_points // 2 - 1)


def build_scaling_array(num_spatial_dims: int, num_points: int, *, mode: str) -> np.ndarray:
    """_spectral.py:403-527: per-mode normalisers of the unnormalised rfftn."""
    dens = {"norm_compensation": (1, 1), "reconstruction": (2, 1), "coef_extraction": (2, 2)}
    if mode not in dens:
        raise ValueError("Invalid mode.")
    right_den, other_den = dens[mode]
    n = num_points
    right_k = np.arange(n // 2 + 1)
    other_k = np.fft.fftfreq(n, 1.0 / n)
    right = np.full(right_k.shape, n / right_den)
    other = np.full(other_k.shape, n / other_den)
    right[right_k == 0] = n
    other[other_k == 0] = n
    if n % 2 == 0:
        right[right_k == n // 2] = n
        other[other_k == -(n // 2)] = n
    axes = [other] * (num_spatial_dims - 1) + [right]
    return np.prod(np.stack(np.meshgrid(*axes, indexing="ij")), axis=0, keepdims=True)


def get_modes_slices(num_spatial_dims: int, num_points: int):
    """_spectral.py:530-611: index blocks of positive / negative wavenumbers."""
    nyq = num_points // 2
    if num_points % 2 == 0:
        left, right = slice(None, nyq), slice(-nyq, None)
    else:
        left, right = slice(None, nyq + 1), slice(-nyq, None)
    per_axis = [[slice(None, nyq + 1)]] + [[left, right]] * (num_spatial_dims - 1)
    return tuple(tuple([slice(None)] + list(reversed(p))) for p in product(*per_axis))


def dealias_kmax(dealiasing_fraction, num_points: int) -> int:
    """Largest |k| kept by BaseNonlinearFun's mask (nonlin_fun/_base.py:59-71)."""
    if dealiasing_fraction is None:
        return num_points
    cutoff = np.float32(dealiasing_fraction * (num_points // 2) - 1)
    k = -1
    while k + 1 <= num_points // 2 and np.float32(k + 1) <= cutoff:
        k += 1
    return k


# --------------------------------------------------------------------- device transforms

def fft(field, *, num_spatial_dims: int | None = None):
    """spectral.fft (_spectral.py:614-656) on the GPU: rfftn over the last D
    axes.  Accepts any leading axes (batch, channels)."""
    t, back = _device.to_device(field, "float32")
    D = t.ndim - 1 if num_spatial_dims is None else num_spatial_dims
    N = t.shape[-1]
    if any(s != N for s in t.shape[-D:]):
        raise ValueError("all spatial axes must have the same length")
    lead = t.shape[:-D]
    count = int(np.prod(lead)) if lead else 1
    out = _device.empty(tuple(lead) + wavenumber_shape(D, N), "complex64")
    check(load().exgb_rfftn(_device.stream(), D, N, count, _device.ptr(t), _device.ptr(out)), "fft")
    return back(out)


def ifft(field_hat, *, num_spatial_dims: int | None = None, num_points: int | None = None):
    """spectral.ifft (_spectral.py:659-721) on the GPU: irfftn with
    s=(N,)*D; the imaginary parts of the c2r axis' DC and Nyquist bins are
    ignored as in the reference's FFT backends."""
    t, back = _device.to_device(field_hat, "complex64")
    D = t.ndim - 1 if num_spatial_dims is None else num_spatial_dims
    if num_points is None:
        if D >= 2:
            num_points = t.shape[-2]
        else:
            raise ValueError("num_points must be provided if num_spatial_dims == 1.")
    N = num_points
    lead = t.shape[:-D]
    count = int(np.prod(lead)) if lead else 1
    out = _device.empty(tuple(lead) + spatial_shape(D, N), "float32")
    check(load().exgb_irfftn(_device.stream(), D, N, count, _device.ptr(t), _device.ptr(out)), "ifft")
    return back(out)


def derivative(field, domain_extent: float, *, order: int = 1, indexing: str = "ij"):
    """spectral.derivative (_spectral.py:724-791) on the GPU: every axis' order-th spectral derivative of a
    state (C, N, ..., N); (D, N, ...) for one channel, else (C, D, N, ...).  rfftn, the (i k_d)^order
    multipliers (exgb_spectral_derivative), irfftn."""
    if indexing != "ij":
        raise NotImplementedError("only indexing='ij' is supported")
    if int(order) != order or order < 0:
        raise ValueError("order must be a non-negative integer")
    t, back = _device.to_device(field, "float32")
    C, D, N = t.shape[0], t.ndim - 1, t.shape[-1]
    hat = fft(t, num_spatial_dims=D).contiguous()
    dh = _device.empty((C, D) + wavenumber_shape(D, N), "complex64")
    check(load().exgb_spectral_derivative(_device.stream(), D, N, C, int(order), float(domain_extent),
                                          _device.ptr(hat), _device.ptr(dh)), "derivative")
    out = ifft(dh, num_spatial_dims=D, num_points=N)
    return back(out[0] if C == 1 else out)


def make_incompressible(field, *, indexing: str = "ij"):
    """spectral.make_incompressible (_spectral.py:794-863) on the GPU: the divergence-free part of a
    velocity field (D, N, ..., N) (Leray projection; rfftn, exgb_make_incompressible, irfftn)."""
    if indexing != "ij":
        raise NotImplementedError("only indexing='ij' is supported")
    t, back = _device.to_device(field, "float32")
    D, N = t.ndim - 1, t.shape[-1]
    if t.shape[0] != D:
        raise ValueError(f"Expected the number of channels ({t.shape[0]}) to match the number of spatial "
                         f"dimensions ({D}).")
    hat = fft(t, num_spatial_dims=D).contiguous()
    check(load().exgb_make_incompressible(_device.stream(), D, N, 1, _device.ptr(hat), _device.ptr(hat)),
          "make_incompressible")
    return back(ifft(hat, num_spatial_dims=D, num_points=N))


def get_fourier_coefficients(state, *, scaling_compensation_mode: str | None = "coef_extraction", round=5,
                             indexing: str = "ij"):
    """spectral.get_fourier_coefficients (_spectral.py:1033-1172): rfftn of a state (C, N, ..., N) divided
    by a scaling array (exgb_mode_scale) and rounded to `round` decimals (None: no rounding)."""
    if indexing != "ij":
        raise NotImplementedError("only indexing='ij' is supported")
    t, back = _device.to_device(state, "float32")
    D, N = t.ndim - 1, t.shape[-1]
    hat = fft(t, num_spatial_dims=D).contiguous()
    if scaling_compensation_mode is not None:
        sc = build_scaling_array(D, N, mode=scaling_compensation_mode).reshape(-1)
        table = _device.torch().from_numpy(np.ascontiguousarray((1.0 / sc).astype(np.complex64))).cuda()
        check(load().exgb_mode_scale(_device.stream(), t.shape[0], table.numel(), _device.ptr(table),
                                     _device.ptr(hat), _device.ptr(hat)), "get_fourier_coefficients")
    if round is not None:
        # round half to even of re and im at `round` decimals, as jnp.round does on complex arrays
        torch = _device.torch()
        hat = torch.complex(torch.round(hat.real, decimals=int(round)), torch.round(hat.imag, decimals=int(round)))
    return back(hat)


def get_spectrum(state, **kwargs):
    """spectral.get_spectrum (_spectral.py:866-1030); see exponax_gb300.metrics.get_spectrum."""
    from .metrics import get_spectrum as _gs

    return _gs(state, **kwargs)
