"""Owning wrapper around an ``exgb_plan*`` (created lazily on first device
use, so that operator assembly can be inspected without a GPU)."""

from __future__ import annotations

import ctypes

import numpy as np

from . import _device
from ._lib import PlanDesc, check, load


class Plan:
    """Immutable stepping plan: dims, L, ETDRK order, nonlinearity."""

    def __init__(self, *, num_spatial_dims, num_points, num_channels, order, domain_extent, dt, linear_operator,
                 num_circle_points=16, circle_radius=1.0, nonlin=None):
        self.num_spatial_dims = int(num_spatial_dims)
        self.num_points = int(num_points)
        self.num_channels = int(num_channels)
        self.order = int(order)
        self.domain_extent = float(domain_extent)
        self.dt = float(dt)
        L = np.ascontiguousarray(np.asarray(linear_operator, dtype=np.complex128))
        self.linear_operator = L
        self.num_circle_points = int(num_circle_points)
        self.circle_radius = float(circle_radius)
        self.nonlin = dict(nonlin or {"nonlin_kind": 0})
        self._handle = None

    def desc(self) -> PlanDesc:
        d = PlanDesc()
        d.num_spatial_dims = self.num_spatial_dims
        d.num_points = self.num_points
        d.num_channels = self.num_channels
        d.order = self.order
        d.domain_extent = self.domain_extent
        d.dt = self.dt
        d.linear_operator = self.linear_operator.ctypes.data
        d.linear_operator_channels = self.linear_operator.shape[0]
        d.num_circle_points = self.num_circle_points
        d.circle_radius = self.circle_radius
        nl = self.nonlin
        d.nonlin_kind = int(nl.get("nonlin_kind", 0))
        frac = nl.get("dealiasing_fraction", None)
        d.dealiasing_fraction = -1.0 if frac is None else float(frac)
        d.scale = float(nl.get("scale", 1.0))
        d.single_channel = int(bool(nl.get("single_channel", False)))
        d.conservative = int(bool(nl.get("conservative", False)))
        d.zero_mode_fix = int(bool(nl.get("zero_mode_fix", True)))
        sl = list(nl.get("scale_list", (0.0, 0.0, 0.0)))
        for i in range(3):
            d.scale_list[i] = float(sl[i])
        poly = list(nl.get("poly", ()))
        if len(poly) > 8:
            raise ValueError("at most 8 polynomial coefficients are supported")
        d.num_poly = len(poly)
        for i, c in enumerate(poly):
            d.poly[i] = float(c)
        d.injection_mode = int(nl.get("injection_mode", -1))
        d.injection_scale = float(nl.get("injection_scale", 0.0))
        rx = list(nl.get("reaction", (0.0, 0.0)))
        for i in range(2):
            d.reaction[i] = float(rx[i])
        return d

    @property
    def handle(self):
        if self._handle is None:
            _device.require_cuda()
            _device.torch().cuda.init()
            lib = load()
            h = ctypes.c_void_p()
            d = self.desc()
            check(lib.exgb_plan_create(ctypes.byref(d), ctypes.byref(h)), "plan")
            self._handle = h
        return self._handle

    def table(self, which: int) -> np.ndarray:
        """Coefficient table from the device (0=E, 1=E_half, 2..7 = coef_1..6)."""
        shape = self.linear_operator.shape
        if which <= 1:
            out = np.empty(shape, dtype=np.complex64)
        else:
            out = np.empty(shape, dtype=np.float32)
        check(load().exgb_plan_get_table(self.handle, which, out.ctypes.data, out.nbytes), "table")
        return out

    def kmax(self) -> int:
        return load().exgb_plan_kmax(self.handle)

    PRECISIONS = {"fp32": 0, "split_bf16": 1}

    def set_precision(self, mode: str) -> None:
        """Arithmetic of the 2D vorticity transforms: "fp32" (FP32 FFTs) or
        "split_bf16" (tcgen05 DFT contractions, split-BF16, FP32 accumulation)."""
        if mode not in self.PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(self.PRECISIONS)}, got {mode!r}")
        arr = (ctypes.c_int * 1)(self.PRECISIONS[mode])
        check(load().exgb_plan_tune(self.handle, 3, arr, 1), "set_precision")

    def status(self) -> None:
        """Raise if a bounded device wait of this plan's kernels gave up (synchronises)."""
        check(load().exgb_plan_status(self.handle), "plan status")

    def __del__(self):
        try:
            if self._handle is not None:
                load().exgb_plan_destroy(self._handle)
        except Exception:
            pass
