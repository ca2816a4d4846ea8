"""Rollouts captured as CUDA graphs.

``GraphRollout(stepper, n, batch)`` records ``vmap(rollout(stepper, n))`` (or ``vmap(repeat(stepper, n))``
with ``trajectory=False``) over a fixed batch once as a CUDA graph; each call copies the new initial
states into the graph's input buffer and replays it, so a rollout costs one graph launch whatever its
number of kernel launches.  1D single-channel steppers are recorded as one launch of the device work
queue (``exgb_queue_prepare`` / ``exgb_queue_launch``, the capturable 1D entry point); every other
stepper by capturing its batched rollout after a warm-up call (which sizes the library's workspaces,
so nothing is allocated during capture).  The output tensor is reused by every call.
"""

from __future__ import annotations

from . import _device
from ._utils import repeat, rollout, vmap


class GraphRollout:
    def __init__(self, stepper, n: int, batch: int, *, include_init: bool = False, trajectory: bool = True):
        torch = _device.torch()
        _device.require_cuda()
        self.stepper = stepper
        self.n = int(n)
        self.trajectory = bool(trajectory)
        D, N, C = stepper.num_spatial_dims, stepper.num_points, stepper.num_channels
        self.shape = (int(batch), C) + (N,) * D
        self._queue = None
        if D == 1 and C == 1 and self._capture_queue(stepper, int(batch), include_init):
            return
        fn = vmap(rollout(stepper, self.n, include_init=include_init)) if trajectory else vmap(repeat(stepper, self.n))
        self._input = torch.zeros(self.shape, dtype=torch.float32, device="cuda")
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            fn(self._input)  # warm-up: plans, kernel attributes and workspaces exist before capture
        torch.cuda.current_stream().wait_stream(side)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.output = fn(self._input)
        self._graph = g

    def _capture_queue(self, stepper, batch, include_init):
        """Record the rollout as one work-queue launch; False for 1D plans the queue does not run (those
        on the staged N-D path, e.g. Cahn-Hilliard), which are then captured like the rest."""
        from ._lib import ExgbError
        from .batching import QueueRollout

        torch = _device.torch()
        u0 = torch.zeros(self.shape, dtype=torch.float32, device="cuda")
        try:
            q = QueueRollout([(stepper, u0[b]) for b in range(batch)], self.n,
                             include_init=include_init or not self.trajectory)
        except (ExgbError, ValueError):
            return False
        q.capture()
        self._queue = q
        self._input = q._u0[0]
        traj = q._traj[0]  # (B, T, 1, N)
        self.output = traj if self.trajectory else traj[:, -1]
        self._graph = q._graph
        return True

    def __call__(self, u0):
        """Replay for the batch of initial states u0 (batch, C, N, ..., N); returns the graph's output
        tensor ((batch, T, C, N, ...) or (batch, C, N, ...)), overwritten by the next call."""
        t, _ = _device.to_device(u0, "float32")
        if tuple(t.shape) != self.shape:
            raise ValueError(f"Expected initial states of shape {self.shape}, got {tuple(t.shape)}")
        self._input.copy_(t.reshape(self._input.shape))
        self._graph.replay()
        return self.output
