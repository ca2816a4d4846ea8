"""ctypes binding of libexgb.so (the C ABI declared in include/exgb.h).

The library is the product: there is no CPU fallback.  Loading fails loudly
if ``libexgb.so`` has not been built (``python -m exponax_gb300.build``).
"""

from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libexgb.so")

EXGB_OK = 0
EXGB_EINVAL = -1
EXGB_ESHAPE = -2
EXGB_ENOTFACTORABLE = -3
EXGB_ECUDA = -4
EXGB_ETIMEOUT = -5
EXGB_EGUARD = -6
EXGB_ENOMEM = -7
EXGB_EUNSUPPORTED = -8
EXGB_ENOTIMPL = -9

# exgb_plan_tune knob of the tensor-core kernel's timeout path (tests only)
EXGB_TUNE_WAIT_BUDGET = 5

NL_ZERO = 0
NL_CONVECTION = 1
NL_GRADIENT_NORM = 2
NL_POLYNOMIAL = 3
NL_GENERAL = 4
NL_VORTICITY_2D = 5
NL_VORTICITY_2D_KOLMOGOROV = 6
NL_PROJECTED_3D = 7
NL_PROJECTED_3D_KOLMOGOROV = 8
NL_CAHN_HILLIARD = 9
NL_GRAY_SCOTT = 10
NL_BELOUSOV_ZHABOTINSKY = 11


class PlanDesc(ctypes.Structure):
    """Mirror of exgb_plan_desc."""

    _fields_ = [
        ("num_spatial_dims", ctypes.c_int32),
        ("num_points", ctypes.c_int32),
        ("num_channels", ctypes.c_int32),
        ("order", ctypes.c_int32),
        ("domain_extent", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("linear_operator", ctypes.c_void_p),
        ("linear_operator_channels", ctypes.c_int32),
        ("num_circle_points", ctypes.c_int32),
        ("circle_radius", ctypes.c_double),
        ("nonlin_kind", ctypes.c_int32),
        ("dealiasing_fraction", ctypes.c_double),
        ("scale", ctypes.c_double),
        ("single_channel", ctypes.c_int32),
        ("conservative", ctypes.c_int32),
        ("zero_mode_fix", ctypes.c_int32),
        ("scale_list", ctypes.c_double * 3),
        ("num_poly", ctypes.c_int32),
        ("poly", ctypes.c_double * 8),
        ("injection_mode", ctypes.c_int32),
        ("injection_scale", ctypes.c_double),
        ("reaction", ctypes.c_double * 2),
    ]


class WorkItem(ctypes.Structure):
    """Mirror of exgb_work_item."""

    _fields_ = [("plan", ctypes.c_void_p), ("u0", ctypes.c_void_p), ("traj", ctypes.c_void_p)]


# (name, restype, argtypes) of every symbol include/exgb.h declares
_VP = ctypes.c_void_p
_I = ctypes.c_int
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
SIGNATURES = [
    ("exgb_version", _I, []),
    ("exgb_last_error", ctypes.c_char_p, []),
    ("exgb_device_info", _I, [ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    ("exgb_plan_create", _I, [ctypes.POINTER(PlanDesc), ctypes.POINTER(_VP)]),
    ("exgb_plan_destroy", _I, [_VP]),
    ("exgb_plan_get_table", _I, [_VP, _I, _VP, ctypes.c_size_t]),
    ("exgb_plan_kmax", _I, [_VP]),
    ("exgb_rfftn", _I, [_VP, _I, _I, _I64, _VP, _VP]),
    ("exgb_irfftn", _I, [_VP, _I, _I, _I64, _VP, _VP]),
    ("exgb_step_fourier", _I, [_VP, _VP, _VP, _VP, _I64]),
    ("exgb_step", _I, [_VP, _VP, _VP, _VP, _I64]),
    ("exgb_nonlinear", _I, [_VP, _VP, _VP, _VP, _I64]),
    ("exgb_repeat", _I, [_VP, _VP, _VP, _VP, _I64, _I32]),
    ("exgb_repeat_fourier", _I, [_VP, _VP, _VP, _VP, _I64, _I32]),
    ("exgb_rollout", _I, [_VP, _VP, _VP, _VP, _I64, _I32, _I32]),
    ("exgb_repeat_fourier_noalloc", _I, [_VP, _VP, _VP, _VP, _I64, _I32]),
    ("exgb_queue_rollout", _I, [ctypes.POINTER(WorkItem), _I64, _I32, _I32, _VP]),
    ("exgb_map_between_resolutions", _I, [_VP, _I, _I, _I, _I64, _VP, _VP, _I]),
    ("exgb_fourier_interp", _I, [_VP, _I, _I, _I, _VP, ctypes.c_float, _I64, _VP, _VP]),
    ("exgb_leray", _I, [_VP, _I, _I, ctypes.c_double, _I64, _VP, _VP]),
    ("exgb_plan_tune", _I, [_VP, _I, ctypes.POINTER(_I), _I]),
    ("exgb_plan_get_tuning", _I, [_VP, ctypes.POINTER(_I), _I]),
    ("exgb_plan_fused_launches", _I, [_VP, ctypes.c_int64, ctypes.POINTER(_I)]),
    ("exgb_plan_status", _I, [_VP]),
    ("exgb_tc_gemm_check", _I, [_VP, _I, _I, _VP, _VP, _VP, _I]),
    ("exgb_spectrum", _I, [_VP, _I, _I, _I64, _VP, _VP, _I, _I]),
    ("exgb_field_sums", _I, [_VP, _I64, _I64, _VP, _VP, _VP]),
    ("exgb_field_pnorms", _I, [_VP, _I64, _I64, _VP, _VP, ctypes.c_float, _VP]),
    ("exgb_fourier_pnorms", _I, [_VP, _I, _I, _I64, _VP, ctypes.c_float, ctypes.c_float, _I, _I, ctypes.c_float, _VP]),
    ("exgb_axpy", _I, [_VP, _I64, ctypes.c_float, _VP, _VP, _VP]),
    ("exgb_scatter_modes", _I, [_VP, _I64, _I64, _I, _VP, _VP, _VP]),
    ("exgb_normalize_fields", _I, [_VP, _I64, _I64, _VP, _I, _I, _I]),
    ("exgb_mode_scale", _I, [_VP, _I64, _I64, _VP, _VP, _VP]),
    ("exgb_mode_mix2", _I, [_VP, _I64, _I64, _VP, _VP, _VP, _I]),
    ("exgb_spectral_derivative", _I, [_VP, _I, _I, _I64, _I, ctypes.c_float, _VP, _VP]),
    ("exgb_make_incompressible", _I, [_VP, _I, _I, _I64, _VP, _VP]),
    ("exgb_queue_prepare", _I, [ctypes.POINTER(WorkItem), _I64, _I32, _I32, ctypes.POINTER(_VP)]),
    ("exgb_queue_launch", _I, [_VP, _VP]),
    ("exgb_queue_destroy", _I, [_VP]),
]

_lib = None


class ExgbError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"exgb error {code}: {msg}")
        self.code = code


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load libexgb.so and declare the C signatures (no GPU needed)."""
    global _lib
    if _lib is not None and path == LIB_PATH:
        return _lib
    if not os.path.exists(path):
        raise ImportError(
            f"{path} is missing: build the CUDA library first (python -m exponax_gb300.build)"
        )
    lib = ctypes.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path == LIB_PATH:
        _lib = lib
    return lib


def check(rc: int, what: str = "") -> None:
    """Raise the reference's exception type for a failed call."""
    if rc == EXGB_OK:
        return
    msg = load().exgb_last_error().decode(errors="replace")
    if what:
        msg = f"{what}: {msg}"
    if rc == EXGB_ESHAPE or rc == EXGB_EINVAL or rc == EXGB_ENOTFACTORABLE:
        raise ValueError(msg)
    if rc == EXGB_ENOTIMPL:
        raise NotImplementedError(msg)
    raise ExgbError(rc, msg)
