"""Time loops and batching (exponax/_utils.py, exponax/_repeated_stepper.py).

``rollout`` and ``repeat`` return callables like the reference.  When the
stepped function is a stepper of this package, the whole loop runs as one
fused device call (1D: one kernel for all steps; 2D: one kernel per step for
trajectories, one kernel for ``repeat``).  Other callables are stepped in a
Python loop of device calls.  ``vmap`` maps a leading batch axis onto the
batched device entry points (the reference batches with ``jax.vmap``).
"""

from __future__ import annotations

import numpy as np

from . import _device
from .stepper import BaseStepper


def make_grid(num_spatial_dims: int, domain_extent: float, num_points: int, *, full: bool = False,
              zero_centered: bool = False) -> np.ndarray:
    """_utils.py:10-62 (float32 grid, 'ij' indexing, shape (D, N, ..., N))."""
    if full:
        g = np.linspace(0, domain_extent, num_points + 1, endpoint=True)
    else:
        g = np.linspace(0, domain_extent, num_points, endpoint=False)
    if zero_centered:
        g = g - domain_extent / 2
    return np.stack(np.meshgrid(*([g] * num_spatial_dims), indexing="ij")).astype(np.float32)


class _Rollout:
    def __init__(self, stepper_fn, n, include_init):
        self.stepper_fn = stepper_fn
        self.n = int(n)
        self.include_init = bool(include_init)

    def _loop(self, u0, batched):
        fn = vmap(self.stepper_fn) if batched else self.stepper_fn
        t = _device.torch()
        u = u0
        frames = [u0] if self.include_init else []
        for _ in range(self.n):
            u = fn(u)
            frames.append(u)
        ax = 1 if batched else 0
        if isinstance(u0, t.Tensor):
            return t.stack(frames, dim=ax)
        return np.stack([np.asarray(f) for f in frames], axis=ax)

    def __call__(self, u0):
        if isinstance(self.stepper_fn, BaseStepper):
            return self.stepper_fn._rollout(u0, self.n, self.include_init, batched=False)
        return self._loop(u0, batched=False)

    def _batched(self, u0):
        if isinstance(self.stepper_fn, BaseStepper):
            return self.stepper_fn._rollout(u0, self.n, self.include_init, batched=True)
        return self._loop(u0, batched=True)


def rollout(stepper_fn, n: int, *, include_init: bool = False, takes_aux: bool = False, constant_aux: bool = True):
    """_utils.py:92-186: callable returning the trajectory (n [+1], C, N...)."""
    if takes_aux:
        raise NotImplementedError("rollouts with auxiliary inputs (ForcedStepper) are not built in this version")
    return _Rollout(stepper_fn, n, include_init)


class _Repeat:
    def __init__(self, stepper_fn, n):
        self.stepper_fn = stepper_fn
        self.n = int(n)

    def __call__(self, u0):
        if isinstance(self.stepper_fn, BaseStepper):
            return self.stepper_fn._repeat(u0, self.n, batched=False)
        u = u0
        for _ in range(self.n):
            u = self.stepper_fn(u)
        return u

    def _batched(self, u0):
        if isinstance(self.stepper_fn, BaseStepper):
            return self.stepper_fn._repeat(u0, self.n, batched=True)
        fn = vmap(self.stepper_fn)
        u = u0
        for _ in range(self.n):
            u = fn(u)
        return u


def repeat(stepper_fn, n: int, *, takes_aux: bool = False, constant_aux: bool = True):
    """_utils.py:189-254: callable returning the state after n steps."""
    if takes_aux:
        raise NotImplementedError("repeat with auxiliary inputs (ForcedStepper) is not built in this version")
    return _Repeat(stepper_fn, n)


class RepeatedStepper:
    """_repeated_stepper.py:9-139: num_sub_steps steps kept in Fourier space."""

    def __init__(self, stepper: BaseStepper, num_sub_steps: int):
        self.stepper = stepper
        self.num_sub_steps = num_sub_steps
        self.dt = stepper.dt * num_sub_steps
        self.num_spatial_dims = stepper.num_spatial_dims
        self.domain_extent = stepper.domain_extent
        self.num_points = stepper.num_points
        self.num_channels = stepper.num_channels
        self.dx = stepper.dx

    def step_fourier(self, u_hat):
        return self.stepper._repeat_fourier(u_hat, self.num_sub_steps, batched=False)

    def _batched_step_fourier(self, u_hat):
        return self.stepper._repeat_fourier(u_hat, self.num_sub_steps, batched=True)

    def _do(self, u, batched):
        from .spectral import fft, ifft

        D = self.num_spatial_dims
        u_hat = fft(u, num_spatial_dims=D)
        u_hat = self.stepper._repeat_fourier(u_hat, self.num_sub_steps, batched=batched)
        return ifft(u_hat, num_spatial_dims=D, num_points=self.num_points)

    def step(self, u):
        return self._do(u, batched=False)

    def __call__(self, u):
        t, _ = _device.to_device(u, "float32")
        expected = (self.num_channels,) + (self.num_points,) * self.num_spatial_dims
        if tuple(t.shape) != expected:
            raise ValueError(f"Expected shape {expected}, got {tuple(t.shape)}.")
        return self._do(u, batched=False)

    def _batched(self, u):
        return self._do(u, batched=True)


def vmap(fn):
    """Batched version of a stepper / rollout / repeat / nonlinear function /
    step_fourier method of this package (the role jax.vmap plays for the
    reference)."""
    if hasattr(fn, "_batched"):
        return fn._batched
    owner = getattr(fn, "__self__", None)
    name = getattr(fn, "__name__", "")
    if owner is not None and name == "step_fourier" and hasattr(owner, "_batched_step_fourier"):
        return owner._batched_step_fourier
    if owner is not None and name in ("step", "__call__") and hasattr(owner, "_batched"):
        return owner._batched

    def looped(u):
        t = _device.torch()
        outs = [fn(u[i]) for i in range(u.shape[0])]
        if isinstance(outs[0], t.Tensor):
            return t.stack(outs)
        return np.stack(outs)

    return looped
