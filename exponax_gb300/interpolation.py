"""map_between_resolutions and FourierInterpolator (exponax/_interpolation.py) on the GPU."""

from __future__ import annotations

import numpy as np

from . import _device
from ._lib import check, load


def _map(state, new_num_points: int, oddball_zero: bool, batched: bool):
    t, back = _device.to_device(state, "float32")
    D = t.ndim - (2 if batched else 1)
    old = t.shape[-1]
    if old == new_num_points:
        return back(t.clone())
    lead = t.shape[:-D]
    count = int(np.prod(lead))
    out = _device.empty(tuple(lead) + (new_num_points,) * D, "float32")
    check(load().exgb_map_between_resolutions(_device.stream(), D, old, new_num_points, count, _device.ptr(t),
                                              _device.ptr(out), int(bool(oddball_zero))), "map_between_resolutions")
    return back(out)


def map_between_resolutions(state, new_num_points: int, *, oddball_zero: bool = True):
    """Spectral re-sampling of a (C, N, ..., N) state to new_num_points."""
    return _map(state, new_num_points, oddball_zero, batched=False)


def map_between_resolutions_batched(states, new_num_points: int, *, oddball_zero: bool = True):
    """Same for a leading batch axis (B, C, N, ..., N)."""
    return _map(states, new_num_points, oddball_zero, batched=True)


class FourierInterpolator:
    """_interpolation.py:22-112: the trigonometric interpolant of a periodic state (C, N, ..., N),
    evaluated at arbitrary points of the domain.  At construction the state's rfftn is divided by the
    "reconstruction" scaling array on the device (exgb_rfftn + exgb_mode_scale); __call__(x) for one
    point x (D,) returns (C,), and vmap(interpolator)(points) evaluates (P, D) points in one
    exgb_fourier_interp launch (one warp per point).  indexing "ij" (the reference's default)."""

    def __init__(self, state, *, domain_extent: float = 1.0, indexing: str = "ij"):
        from .spectral import build_scaling_array, fft

        if indexing != "ij":
            raise NotImplementedError("only indexing='ij' is supported")
        t, back = _device.to_device(state, "float32")
        self._back = back
        self.num_spatial_dims = t.ndim - 1
        self.domain_extent = domain_extent
        self.num_points = t.shape[-1]
        self.num_channels = t.shape[0]
        D, N = self.num_spatial_dims, self.num_points
        hat = fft(t, num_spatial_dims=D).contiguous()
        recon = build_scaling_array(D, N, mode="reconstruction").reshape(-1)
        table = _device.torch().from_numpy(np.ascontiguousarray((1.0 / recon).astype(np.complex64))).cuda()
        check(load().exgb_mode_scale(_device.stream(), self.num_channels, table.numel(), _device.ptr(table),
                                     _device.ptr(hat), _device.ptr(hat)), "FourierInterpolator")
        self.state_hat_scaled = hat

    def _eval(self, x, batched):
        t, back = _device.to_device(x, "float32")
        D = self.num_spatial_dims
        pts = t.reshape(-1, D) if batched else t.reshape(1, D)
        if (batched and (t.ndim != 2 or t.shape[1] != D)) or (not batched and t.numel() != D):
            raise ValueError(f"Expected points of {D} coordinates, got shape {tuple(t.shape)}")
        P, C = pts.shape[0], self.num_channels
        out = _device.empty((P, C), "float32")
        check(load().exgb_fourier_interp(_device.stream(), D, self.num_points, C, _device.ptr(self.state_hat_scaled),
                                         float(self.domain_extent), P, _device.ptr(pts), _device.ptr(out)),
              "FourierInterpolator")
        return back(out if batched else out[0])

    def __call__(self, x):
        """The interpolant's channels at one point x of shape (D,)."""
        return self._eval(x, batched=False)

    def _batched(self, xs):
        return self._eval(xs, batched=True)
