"""Autotuner for radix plans and launch shapes.

For a stepper and a representative batch it times the candidate
configurations of its plan on the device (CUDA events, median of
`repeats` runs of `repeat_fourier`), applies the fastest and records it in
a JSON cache keyed by device, dimension, N, order, nonlinearity and batch
bucket, so later plans with the same key start tuned.

Knobs (exgb_plan_tune):
  * radix order of the length-N Stockham FFT (1D kernel, transforms,
    generic 2D kernel): every ordering of the factorisations of N into
    {8, 4, 2, 5, 3}, capped;
  * CTAs per cluster of the 2D cluster kernels: 1..8 (those that fit; for the
    generic kernel searched after its radix order);
  * instances per work item of the 1D kernel;
  * threads per CTA of the 1D kernel (searched after the two above).
"""

from __future__ import annotations

import ctypes
import itertools
import json
import os

import numpy as np

from . import _device
from ._lib import EXGB_OK, check, load

KMAX = 12


def cache_path() -> str:
    return os.environ.get("EXGB_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "exponax_gb300", "autotune.json"))


def _factorisations(n, radices=(8, 4, 2, 5, 3)):
    out = []

    def rec(m, cur):
        if m == 1:
            out.append(tuple(cur))
            return
        for r in radices:
            if m % r == 0 and (not cur or r <= cur[-1] or r in (5, 3)):
                rec(m // r, cur + [r])

    rec(n, [])
    return out


def radix_candidates(n, cap=12):
    seen = []
    for f in _factorisations(n):
        for p in itertools.permutations(f):
            if p not in seen:
                seen.append(p)
            if len(seen) >= 200:
                break
    # fewest passes first, then keep a spread of orderings
    seen.sort(key=lambda p: (len(p), p))
    return seen[:cap]


def get_tuning(plan):
    buf = (ctypes.c_int * (KMAX + 5))()
    check(load().exgb_plan_get_tuning(plan.handle, buf, KMAX + 5), "get_tuning")
    npass = buf[0]
    return {"radices": [buf[1 + i] for i in range(npass)], "cluster": buf[1 + KMAX], "items_per_cta": buf[2 + KMAX],
            "threads": buf[4 + KMAX]}


def _set(plan, kind, values):
    arr = (ctypes.c_int * max(1, len(values)))(*values)
    return load().exgb_plan_tune(plan.handle, kind, arr, len(values))


def _key(stepper, batch):
    torch = _device.torch()
    name = torch.cuda.get_device_name()
    nl = type(stepper.nonlinear_fun).__name__
    bucket = 1 << int(np.ceil(np.log2(max(1, batch))))
    return f"{name}|D{stepper.num_spatial_dims}|N{stepper.num_points}|o{stepper.order}|{nl}|B{bucket}"


def _time(plan, uh, out, batch, nsteps, repeats):
    torch = _device.torch()
    lib = load()
    ms = []
    for r in range(repeats + 1):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        rc = lib.exgb_repeat_fourier(plan.handle, _device.stream(), uh.data_ptr(), out.data_ptr(), batch, nsteps)
        e1.record()
        torch.cuda.synchronize()
        if rc != EXGB_OK:
            return float("inf")
        if r:
            ms.append(e0.elapsed_time(e1))
    return float(np.median(ms))


def tune(stepper, *, batch=64, nsteps=10, repeats=3, use_cache=True, write_cache=True, seed=0):
    """Tune the plan of `stepper` in place; returns the chosen configuration
    and the timings of every candidate."""
    torch = _device.torch()
    plan = stepper.plan
    key = _key(stepper, batch)
    path = cache_path()
    cache = {}
    if os.path.exists(path):
        try:
            cache = json.load(open(path))
        except Exception:
            cache = {}
    if use_cache and key in cache:
        apply(stepper, cache[key])
        return {"key": key, "best": cache[key], "cached": True}
    D, N, C = stepper.num_spatial_dims, stepper.num_points, stepper.num_channels
    shape = (batch, C) + (N,) * (D - 1) + (N // 2 + 1,)
    g = torch.Generator(device="cuda").manual_seed(seed)
    uh = torch.randn(shape, dtype=torch.complex64, device="cuda", generator=g) * 1e-3
    out = torch.empty_like(uh)
    results = []
    cfg = get_tuning(plan)
    is_reg2d = D == 2 and cfg["cluster"] > 0 and N in (64, 128, 256) and stepper.order > 0
    if is_reg2d:
        for G in range(1, 9):
            if _set(plan, 1, [G]) != EXGB_OK:
                continue
            results.append(({"cluster": G}, _time(plan, uh, out, batch, nsteps, repeats)))
    else:
        ms_options = [0, 1, 2, 4, 8, 16] if D == 1 else [0]
        for rad in radix_candidates(N):
            if _set(plan, 0, list(rad)) != EXGB_OK:
                continue
            for m in ms_options:
                if D == 1:
                    _set(plan, 2, [m])
                results.append(({"radices": list(rad), "items_per_cta": m},
                                _time(plan, uh, out, batch, nsteps, repeats)))
        if D == 1:
            # threads per CTA for the best radix order / items per CTA found so far
            fin = [r for r in results if np.isfinite(r[1])]
            if fin:
                base = min(fin, key=lambda r: r[1])[0]
                _set(plan, 0, list(base["radices"]))
                _set(plan, 2, [base["items_per_cta"]])
                for t in (64, 128, 256):
                    if _set(plan, 4, [t]) != EXGB_OK:
                        continue
                    results.append((dict(base, threads=t), _time(plan, uh, out, batch, nsteps, repeats)))
                _set(plan, 4, [0])
        if D == 2 and cfg["cluster"] > 0 and stepper.order > 0:
            # generic 2D cluster kernel: cluster size for the best radix order found so far
            fin = [r for r in results if np.isfinite(r[1])]
            if fin:
                base = min(fin, key=lambda r: r[1])[0]
                _set(plan, 0, list(base["radices"]))
                for G in range(1, 9):
                    if _set(plan, 1, [G]) != EXGB_OK:
                        continue
                    results.append((dict(base, cluster=G), _time(plan, uh, out, batch, nsteps, repeats)))
                _set(plan, 1, [0])
    results = [r for r in results if np.isfinite(r[1])]
    best = min(results, key=lambda r: r[1])[0] if results else {}
    apply(stepper, best)
    if write_cache and best:
        cache[key] = best
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as f:
            json.dump(cache, f, indent=1)
    return {"key": key, "best": best, "cached": False, "timings_ms": [(c, t) for c, t in results]}


def apply(stepper, best):
    plan = stepper.plan
    if "radices" in best:
        _set(plan, 0, list(best["radices"]))
    if "items_per_cta" in best:
        _set(plan, 2, [int(best["items_per_cta"])])
    if "threads" in best:
        _set(plan, 4, [int(best["threads"])])
    if "cluster" in best:
        _set(plan, 1, [int(best["cluster"])])
