"""Run one stepping workload for profiling (e.g. under ncu).

    python profile_case.py --dims 2 --n 256 --batch 32 --steps 10 --reps 3
    python profile_case.py --dims 2 --n 128 --kolmogorov --precision split_bf16
    python profile_case.py --uneven 600 --steps 100 --reps 3
    python profile_case.py --corrector 256 --reps 10

Builds the stepper (NavierStokesVorticity in 2D, KuramotoSivashinsky-
Conservative in 1D), creates device-resident Fourier states and launches
``repeat_fourier`` --reps times (one fused-kernel launch each), then
synchronises.  Prints the CUDA-event time per launch.  With --uneven K it
instead builds the first K instances of the uneven 1D batch (Burgers / KdV /
KS-conservative, N in {128 .. 4096}), captures their work-queue rollout in a
CUDA graph and replays it --reps times.  With --corrector B it runs the
learned corrector's forward pass (64 x 64 grids, batch B, inference) --reps
times after 5 warm-up passes.
"""

from __future__ import annotations

import argparse

import numpy as np


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--dims", type=int, default=2)
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--batch", type=int, default=32)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--order", type=int, default=2)
    ap.add_argument("--kolmogorov", action="store_true")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "split_bf16"])
    ap.add_argument("--uneven", type=int, default=0, help="instances of the uneven 1D work-queue batch")
    ap.add_argument("--corrector", type=int, default=0, help="batch of the learned corrector's forward pass")
    ap.add_argument("--pde", default="", choices=["", "burgers", "grayscott"],
                    help="2D/3D Burgers or Gray-Scott on the staged N-D path instead of the vorticity / KS steppers")
    a = ap.parse_args()

    import torch

    import exponax_gb300 as ex
    from exponax_gb300 import _device, _lib

    if a.corrector:
        from exponax_gb300.learned import PeriodicConvCorrector

        net = PeriodicConvCorrector(64, seed=0, max_batch=a.corrector)
        v = torch.randn(a.corrector, 64, 64, device="cuda")
        for _ in range(5):
            net(v)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(a.reps):
            net(v)
        e1.record()
        torch.cuda.synchronize()
        net.status()
        print(f"corrector forward (batch {a.corrector}): {e0.elapsed_time(e1) / a.reps:.3f} ms")
        return

    if a.uneven:
        from exponax_gb300.batching import QueueRollout, uneven_config3

        instances, _ = uneven_config3(a.uneven, a.steps, seed=0)
        q = QueueRollout(instances, a.steps, include_init=True)
        q.capture()
        for _ in range(a.reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            q.replay()
            e1.record()
            torch.cuda.synchronize()
            print(f"uneven queue ({a.uneven} instances, {a.steps} steps): {e0.elapsed_time(e1):.3f} ms")
        return

    if a.pde == "burgers":
        st = ex.stepper.Burgers(a.dims, 2 * np.pi, a.n, 0.01, diffusivity=0.05, order=a.order)
        g = ex.ic.RandomAmplitudePhaseSeries(a.dims, cutoff=4, max_one=True)
    elif a.pde == "grayscott":
        st = ex.stepper.reaction.GrayScott(a.dims, 1.0, a.n, 0.5, order=a.order)
        g = ex.ic.RandomAmplitudePhaseSeries(a.dims, cutoff=2, max_one=True)
    elif a.dims == 3:
        st = ex.stepper.NavierStokesVelocity(3, 2 * np.pi, a.n, 0.01, order=a.order)
        g = ex.ic.RandomAmplitudePhaseSeries(3, cutoff=3, max_one=True)
    elif a.dims == 2:
        cls = ex.stepper.KolmogorovFlowVorticity if a.kolmogorov else ex.stepper.NavierStokesVorticity
        kw = {} if a.kolmogorov else {"diffusivity": 1e-3}
        st = cls(2, 2 * np.pi, a.n, 0.01, order=a.order, **kw)
        if a.precision != "fp32":
            st.set_dft_precision(a.precision)
        g = ex.ic.RandomAmplitudePhaseSeries(2, cutoff=5, max_one=True)
    else:
        st = ex.stepper.KuramotoSivashinskyConservative(1, 100.0, a.n, 0.1, order=a.order)
        g = ex.ic.RandomSineWaves1d(1, cutoff=5)
    C = st.num_channels
    u0 = torch.from_numpy(np.stack([np.concatenate([g(a.n, key=C * s + c) for c in range(C)])
                                    for s in range(a.batch)])).cuda()
    if a.pde == "grayscott":
        u0 = torch.stack([1.0 - 0.25 * (1 + u0[:, 0]), 0.25 * (1 + u0[:, 1])], dim=1).contiguous()
    uh = ex.fft(u0, num_spatial_dims=a.dims)
    out = torch.empty_like(uh)
    lib = _lib.load()
    h = st.plan.handle
    for _ in range(a.reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        _lib.check(lib.exgb_repeat_fourier(h, _device.stream(), uh.data_ptr(), out.data_ptr(), a.batch, a.steps))
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        dofs = a.batch * st.num_channels * a.n**a.dims * a.steps  # channels x grid points
        print(f"repeat_fourier: {ms:.3f} ms, {dofs / ms * 1e3:.3e} DOF-steps/s")


if __name__ == "__main__":
    main()
