"""Uneven batches: many 1D instances of different PDEs, resolutions and
time steps in one persistent launch fed by a device work queue.

The reference can only ``jax.vmap`` over identical shapes, so an uneven
batch there is one ``vmap(rollout)`` per (PDE, N) group run in sequence.
Here every instance is an item of one queue (longest items first) and the
whole rollout of every instance runs in a single kernel launch, which can
be captured in a CUDA graph and replayed.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _device
from ._lib import WorkItem, check, load
from .stepper import BaseStepper


class QueueRollout:
    """Rollout of `nsteps` steps for every (stepper, u0) instance.

    ``instances``: sequence of ``(stepper, u0)`` with 1D steppers of this
    package and ``u0`` of shape (1, N).  Instances of the same stepper that
    follow each other share a work item.  ``trajectories[i]`` has shape
    (nsteps + include_init, 1, N)."""

    def __init__(self, instances, nsteps: int, *, include_init: bool = True):
        torch = _device.torch()
        _device.require_cuda()
        self.nsteps = int(nsteps)
        self.include_init = bool(include_init)
        T = self.nsteps + (1 if include_init else 0)
        # group instances by stepper so each group is one contiguous buffer
        order = []
        groups = {}
        for i, (st, u0) in enumerate(instances):
            if not isinstance(st, BaseStepper) or st.num_spatial_dims != 1:
                raise ValueError("QueueRollout runs 1D steppers of exponax_gb300")
            groups.setdefault(id(st), (st, []))[1].append(i)
        self._u0 = []
        self._traj = []
        self.trajectories = [None] * len(instances)
        items = []
        for st, idx in groups.values():
            N = st.num_points
            u = torch.stack([_device.to_device(instances[i][1], "float32")[0].reshape(1, N) for i in idx])
            tr = torch.empty((len(idx), T, 1, N), dtype=torch.float32, device="cuda")
            self._u0.append(u)
            self._traj.append(tr)
            h = st.plan.handle.value
            for k, i in enumerate(idx):
                items.append(WorkItem(h, u.data_ptr() + k * N * 4, tr.data_ptr() + k * T * N * 4))
                self.trajectories[i] = tr[k]
            order.extend(idx)
        arr = (WorkItem * len(items))(*items)
        q = ctypes.c_void_p()
        check(load().exgb_queue_prepare(arr, len(items), self.nsteps, int(self.include_init), ctypes.byref(q)),
              "queue")
        self._q = q
        self._graph = None

    def launch(self):
        """One launch on torch's current stream (no allocation, capturable)."""
        check(load().exgb_queue_launch(self._q, _device.stream()), "queue launch")

    def capture(self):
        """Capture the launch in a CUDA graph; later `replay()` calls run it."""
        torch = _device.torch()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self.launch()  # warm-up outside the graph (sets kernel attributes)
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.launch()
        self._graph = g
        return g

    def replay(self):
        if self._graph is None:
            self.capture()
        self._graph.replay()

    def __del__(self):
        try:
            if getattr(self, "_q", None) is not None:
                load().exgb_queue_destroy(self._q)
        except Exception:
            pass


def uneven_config3(num_instances=3000, nsteps=100, seed=0):
    """The uneven 1D benchmark batch: a seeded
    multinomial over Burgers (L=1, nu=0.01, dt=1e-3), KdV (L=20, dispersion 1,
    hyper-diffusion 0.01, dt=0.01) and KS-conservative (L=100, dt=0.1), N
    uniform over {128, ..., 4096}, sine-series ICs (cutoff 5) per seed.
    Returns (instances, steppers)."""
    from . import ic, stepper

    rng = np.random.default_rng(seed)
    pde = rng.integers(0, 3, size=num_instances)
    Ns = rng.choice([128, 256, 512, 1024, 2048, 4096], size=num_instances)
    steppers = {}

    def get(p, N):
        key = (int(p), int(N))
        if key not in steppers:
            if p == 0:
                steppers[key] = stepper.Burgers(1, 1.0, int(N), 1e-3, diffusivity=0.01)
            elif p == 1:
                steppers[key] = stepper.KortewegDeVries(1, 20.0, int(N), 0.01, dispersivity=1.0,
                                                        hyper_diffusivity=0.01)
            else:
                steppers[key] = stepper.KuramotoSivashinskyConservative(1, 100.0, int(N), 0.1)
        return steppers[key]

    g = ic.RandomSineWaves1d(1, cutoff=5)
    instances = [(get(p, N), g(int(N), key=i)) for i, (p, N) in enumerate(zip(pde, Ns))]
    return instances, steppers
