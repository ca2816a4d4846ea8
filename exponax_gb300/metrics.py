"""Evaluation metrics (exponax/metrics/*) on device tensors.

Not on the stepping path; computed with plain tensor reductions on the GPU
(or NumPy for NumPy inputs)."""

from __future__ import annotations

import numpy as np

from . import _device


def _lib(x):
    t = _device.torch()
    return t if isinstance(x, t.Tensor) else np


def nRMSE(u_pred, u_ref, *, domain_extent: float = 1.0):
    """metrics/_spatial.py:537-586: sum over channels of
    ||u_pred - u_ref||_2 / ||u_ref||_2 (the (L/N)^D factors cancel)."""
    xp = _lib(u_pred)
    C = u_pred.shape[0]
    d = (u_pred - u_ref).reshape(C, -1)
    r = u_ref.reshape(C, -1)
    if xp is np:
        return float(np.sum(np.linalg.norm(d, axis=1) / np.linalg.norm(r, axis=1)))
    return (d.norm(dim=1) / r.norm(dim=1)).sum()


def correlation(u_pred, u_ref):
    """metrics/_correlation.py:33-60: channel mean of the normalised inner product."""
    xp = _lib(u_pred)
    C = u_pred.shape[0]
    a = u_pred.reshape(C, -1)
    b = u_ref.reshape(C, -1)
    if xp is np:
        return float(np.mean(np.sum(a * b, axis=1) / (np.linalg.norm(a, axis=1) * np.linalg.norm(b, axis=1))))
    return ((a * b).sum(dim=1) / (a.norm(dim=1) * b.norm(dim=1))).mean()


def mean_metric(metric_fn, u_pred, u_ref, **kwargs):
    """metrics/_utils.py:5-18: batch mean of a per-sample metric."""
    vals = [metric_fn(u_pred[i], u_ref[i], **kwargs) for i in range(u_pred.shape[0])]
    if isinstance(vals[0], float):
        return float(np.mean(vals))
    t = _device.torch()
    return t.stack(vals).mean()
