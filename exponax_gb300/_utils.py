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


def wrap_bc(u):
    """_utils.py:65-89: a state (C, N, ..., N) padded periodically to (C, N+1, ..., N+1) (the first point
    of every spatial axis repeated at its end), for plotting on closed grids."""
    t = _device.torch()
    if isinstance(u, t.Tensor):
        out = u
        for ax in range(1, u.ndim):
            out = t.cat([out, out.narrow(ax, 0, 1)], dim=ax)
        return out
    u = np.asarray(u)
    return np.pad(u, ((0, 0),) + ((0, 1),) * (u.ndim - 1), mode="wrap")


def stack_sub_trajectories(trj, sub_len: int):
    """_utils.py:257-313: all windows of sub_len consecutive time steps of a trajectory (n, ...) ->
    (n - sub_len + 1, sub_len, ...); a tuple / list / dict of trajectories is mapped leaf by leaf
    (all leaves must have the same number of time steps)."""
    t = _device.torch()
    leaves = []

    def collect(x):
        if isinstance(x, dict):
            for v in x.values():
                collect(v)
        elif isinstance(x, (list, tuple)):
            for v in x:
                collect(v)
        else:
            leaves.append(x)

    collect(trj)
    steps = {int(x.shape[0]) for x in leaves}
    if len(steps) != 1:
        raise ValueError("All arrays in trj must have the same number of time steps in the leading axis")
    n = steps.pop()
    if sub_len > n:
        raise ValueError("n must be smaller than or equal to the number of time steps in trj")

    def windows(x):
        if isinstance(x, t.Tensor):
            return t.stack([x[i:i + sub_len] for i in range(n - sub_len + 1)])
        x = np.asarray(x)
        return np.stack([x[i:i + sub_len] for i in range(n - sub_len + 1)])

    def rebuild(x):
        if isinstance(x, dict):
            return {k: rebuild(v) for k, v in x.items()}
        if isinstance(x, (list, tuple)):
            return type(x)(rebuild(v) for v in x)
        return windows(x)

    return rebuild(trj)


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
    """_utils.py:92-186: callable returning the trajectory (n [+1], C, N...).
    takes_aux: the callable is (u0, aux) -> trajectory with stepper_fn(u, aux);
    aux is the same every step (constant_aux) or has a leading time axis of n."""
    if takes_aux:
        return _AuxLoop(stepper_fn, n, include_init, constant_aux, trajectory=True)
    return _Rollout(stepper_fn, n, include_init)


def _aux_at(aux, t, constant, batched):
    if constant:
        return aux
    return aux[:, t] if batched else aux[t]


class _AuxLoop:
    """Time loop over stepper_fn(u, aux) (_utils.py:137-163 for rollout, :212-229 for repeat)."""

    def __init__(self, stepper_fn, n, include_init, constant_aux, trajectory):
        self.stepper_fn = stepper_fn
        self.n = int(n)
        self.include_init = bool(include_init)
        self.constant_aux = bool(constant_aux)
        self.trajectory = trajectory

    def _run(self, u0, aux, batched):
        fn = self.stepper_fn
        if batched:
            fn = fn._batched if hasattr(fn, "_batched") else _looped2(fn)
        u = u0
        frames = [u0] if self.include_init else []
        for t in range(self.n):
            u = fn(u, _aux_at(aux, t, self.constant_aux, batched))
            if self.trajectory:
                frames.append(u)
        if not self.trajectory:
            return u
        tt = _device.torch()
        ax = 1 if batched else 0
        if isinstance(u0, tt.Tensor):
            return tt.stack(frames, dim=ax)
        return np.stack([np.asarray(f) for f in frames], axis=ax)

    def __call__(self, u0, aux):
        return self._run(u0, aux, batched=False)

    def _batched(self, u0, aux):
        return self._run(u0, aux, batched=True)


def _looped2(fn):
    def looped(u, aux):
        t = _device.torch()
        outs = [fn(u[i], aux[i]) for i in range(u.shape[0])]
        return t.stack(outs) if isinstance(outs[0], t.Tensor) else np.stack(outs)

    return looped


class ForcedStepper:
    """_forced_stepper.py:7-108: turns a stepper u -> u_next of u_t = Lu + N(u)
    into (u, f) -> u_next of u_t = Lu + N(u) + f by operator splitting: one
    explicit Euler substep with the forcing (u + dt f, exgb_axpy on the device)
    followed by the wrapped stepper (first order in time, as in the reference)."""

    def __init__(self, stepper):
        self.stepper = stepper

    def __getattr__(self, name):
        if name in ("num_spatial_dims", "domain_extent", "num_points", "num_channels", "dt", "dx"):
            return getattr(self.stepper, name)
        raise AttributeError(name)

    def _add_forcing(self, u, f, dtype):
        from ._lib import check, load

        t, back = _device.to_device(u, dtype)
        tf, _ = _device.to_device(f, dtype)
        if tuple(t.shape) != tuple(tf.shape):
            raise ValueError(f"Forcing shape {tuple(tf.shape)} does not match the state shape {tuple(t.shape)}")
        out = _device.torch().empty_like(t)
        n = t.numel() * (2 if dtype == "complex64" else 1)
        check(load().exgb_axpy(_device.stream(), n, float(self.stepper.dt), t.data_ptr(), tf.data_ptr(),
                               out.data_ptr()), "forcing")
        return out, back

    def step(self, u, f):
        w, back = self._add_forcing(u, f, "float32")
        return back(self.stepper.step(w))

    def step_fourier(self, u_hat, f_hat):
        w, back = self._add_forcing(u_hat, f_hat, "complex64")
        return back(self.stepper.step_fourier(w))

    def __call__(self, u, f):
        return self.step(u, f)

    def _batched(self, u, f):
        w, back = self._add_forcing(u, f, "float32")
        return back(vmap(self.stepper)(w))

    def _batched_step_fourier(self, u_hat, f_hat):
        w, back = self._add_forcing(u_hat, f_hat, "complex64")
        return back(vmap(self.stepper.step_fourier)(w))


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
        return _AuxLoop(stepper_fn, n, False, constant_aux, trajectory=False)
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
