"""Poisson (exponax/_poisson.py:14-128): exact periodic solve of Lap^(order/2) u = -f.

The inverse operator -1/Lap^(order/2) (0 where the operator vanishes, so the
solution has zero mean) is built once on the host in complex64, as the
reference builds it, and kept on the device; step_fourier is one
exgb_mode_scale launch, step / __call__ add the rfftn and irfftn launches.
"""

from __future__ import annotations

import numpy as np

from . import _device
from ._lib import check, load
from .spectral import build_derivative_operator, build_laplace_operator, fft, ifft, spatial_shape


class Poisson:
    def __init__(self, num_spatial_dims: int, domain_extent: float, num_points: int, *, order: int = 2):
        self.num_spatial_dims = num_spatial_dims
        self.domain_extent = domain_extent
        self.num_points = num_points
        self.dx = domain_extent / num_points
        d = build_derivative_operator(num_spatial_dims, domain_extent, num_points).astype(np.complex64)
        op = build_laplace_operator(d, order=order)
        with np.errstate(divide="ignore", invalid="ignore"):
            inv = np.where(op == 0, 0.0, 1 / op).astype(np.complex64)
        # what step_fourier multiplies by: -inv (_poisson.py:82)
        self._inv_operator = inv
        self._table = None

    def _device_table(self):
        if self._table is None:
            torch = _device.torch()
            self._table = torch.from_numpy(np.ascontiguousarray(-self._inv_operator.reshape(-1))).cuda()
        return self._table

    def step_fourier(self, f_hat):
        """-inv(Lap) f^ on (..., N, ..., N//2+1) complex64 fields (any leading axes)."""
        t, back = _device.to_device(f_hat, "complex64")
        table = self._device_table()
        per = table.numel()
        if t.numel() % per != 0 or tuple(t.shape[-self.num_spatial_dims:]) != self._inv_operator.shape[1:]:
            raise ValueError(f"Fourier shape {tuple(t.shape)} does not match {self._inv_operator.shape[1:]}")
        out = _device.empty(t.shape, "complex64")
        check(load().exgb_mode_scale(_device.stream(), t.numel() // per, per, _device.ptr(table), _device.ptr(t),
                                     _device.ptr(out)), "Poisson.step_fourier")
        return back(out)

    def step(self, f):
        """Solve in state space (any leading axes before the D spatial axes)."""
        D = self.num_spatial_dims
        f_hat = fft(f, num_spatial_dims=D)
        return ifft(self.step_fourier(f_hat), num_spatial_dims=D, num_points=self.num_points)

    def __call__(self, f):
        """Single right-hand side (C, N, ..., N) with the reference's shape check."""
        if tuple(f.shape[1:]) != spatial_shape(self.num_spatial_dims, self.num_points):
            raise ValueError(f"Shape of f[1:] is {tuple(f.shape[1:])} but should be "
                             f"{spatial_shape(self.num_spatial_dims, self.num_points)}")
        return self.step(f)
