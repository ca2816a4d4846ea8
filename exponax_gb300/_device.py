"""Device memory plumbing (PyTorch tensors hold the buffers; libexgb.so
does the work).

Inputs may be torch tensors (any device; moved to the current CUDA device)
or NumPy arrays (copied to the GPU; results come back as NumPy).  Everything
runs on torch's current CUDA stream.
"""

from __future__ import annotations

import numpy as np

_TORCH = None


def torch():
    global _TORCH
    if _TORCH is None:
        import torch as _t

        _TORCH = _t
    return _TORCH


_DT = {"float32": "float32", "complex64": "complex64"}


def _tdtype(name):
    t = torch()
    return {"float32": t.float32, "complex64": t.complex64}[name]


def require_cuda():
    t = torch()
    if not t.cuda.is_available():
        raise RuntimeError("exponax_gb300 needs a CUDA GPU (sm_103a); no CPU fallback exists")


def to_device(x, dtype: str):
    """Return (contiguous CUDA tensor of `dtype`, function mapping a result
    tensor back to the caller's array type)."""
    require_cuda()
    t = torch()
    if isinstance(x, t.Tensor):
        y = x
        if not y.is_cuda:
            y = y.cuda()
        if y.dtype != _tdtype(dtype):
            y = y.to(_tdtype(dtype))
        return y.contiguous(), (lambda r: r)
    a = np.asarray(x)
    np_dtype = np.float32 if dtype == "float32" else np.complex64
    y = t.from_numpy(np.ascontiguousarray(a.astype(np_dtype, copy=False))).cuda()
    return y, (lambda r: r.cpu().numpy())


def empty(shape, dtype: str):
    t = torch()
    return t.empty(tuple(int(s) for s in shape), dtype=_tdtype(dtype), device="cuda")


def ptr(t) -> int:
    return int(t.data_ptr())


def stream() -> int:
    """cudaStream_t of torch's current stream as an integer handle."""
    return int(torch().cuda.current_stream().cuda_stream)
