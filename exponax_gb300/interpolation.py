"""map_between_resolutions (exponax/_interpolation.py:195-285) on the GPU."""

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
