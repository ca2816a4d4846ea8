"""Throughput of the ETDRK2 stepping path on batched 2D vorticity.

Workload (one bench step): NavierStokesVorticity(2, 2*pi, 256, dt=0.01,
diffusivity=1e-3), ETDRK2, batch 128, 200 steps (``repeat``), float32,
seeded random truncated Fourier series ICs (cutoff 5, max|w| = 1).
Metric: DOF-steps/s = batch * 256^2 * 200 / time.

Arms:
  default            the GB300 path (libexgb.so), one JSON line on rank 0
  --impl reference   the reference algorithm's CPU path: the NumPy oracle
                     (restatement of exponax; JAX is not installed), run on
                     all host cores with one process per sample

Timing: W warm-up steps, then K steps each bracketed by CUDA events on the
launching stream; L2 is flushed (write of a 256 MiB buffer) between timed
steps outside the events; max over ranks; nvidia-smi clocks sampled during
the timed region.
"""

from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N = 256
BATCH = 128
NSTEPS = 200
DT = 0.01
NU = 1e-3
# algorithmic HBM bytes per DOF-step of ETDRK2 with the Fourier state
# resident between steps: 6 passes over a complex64 half-spectrum
BYTES_PER_DOF_STEP = 6 * 8 * (N // 2 + 1) / N
# algorithmic FP32 transform flops per DOF-step of the fused kernel (5 n log2 n per complex length-n FFT):
# per stage 4 inverse + 1 forward transforms of the K + 1 dealiased columns (K = 2/3 (N/2) - 1 = 84)
# and 2 inverse + 1/2 forward (two rows packed) transforms per row; two stages per ETDRK2 step
KEEP = int(2 / 3 * (N // 2)) - 1
FFT_FLOPS_PER_DOF_STEP = 2 * (5 * (KEEP + 1) + 2.5 * N) * 5 * N * np.log2(N) / (N * N)


def metric_name():
    return "ETDRK DOF-steps/s at 1 GB300"


def config(extra=None):
    c = {"workload": "NavierStokesVorticity 2D 256^2, nu=1e-3, dt=0.01, ETDRK2, batch 128, 200 steps (repeat)",
         "global_batch": BATCH, "num_points": N, "steps_per_bench_step": NSTEPS, "dt": DT,
         "parallelism": "replicas (batch shards, no collective)", "l2": "flushed between timed steps (256 MiB write)"}
    if extra:
        c.update(extra)
    return c


def make_ics(b0, count):
    from exponax_gb300.ic import RandomAmplitudePhaseSeries

    g = RandomAmplitudePhaseSeries(2, cutoff=5, max_one=True)
    return np.stack([g(N, key=s) for s in range(b0, b0 + count)])


# ------------------------------------------------------------------ clocks
class ClockSampler:
    def __init__(self, out_path):
        self.path = out_path
        self.proc = None

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self, gpu_index=0):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9 or not p[0].isdigit() or int(p[0]) != gpu_index:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() in ("active", "1"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------ CPU baseline (oracle)
def _oracle_worker(args):
    seed, nsteps = args
    from oracle import exponax_np as o

    st = o.NavierStokesVorticity(2, 2 * np.pi, N, DT, diffusivity=NU)
    u = make_ics(seed, 1)[0]
    t0 = time.perf_counter()
    for _ in range(nsteps):
        u = st(u)
    return time.perf_counter() - t0


def cpu_baseline(samples=None, nsteps=NSTEPS):
    """NumPy oracle of the same workload on the host cores, one process per
    sample (spawn), bounded sample of `samples` x `nsteps` sample-steps (by default one
    sample per core, each the full 200-step trajectory of one initial condition)."""
    import multiprocessing as mp

    cores = os.cpu_count() or 1
    try:
        cores = len(os.sched_getaffinity(0))
    except Exception:
        pass
    samples = samples or cores
    ctx = mp.get_context("spawn")
    with ctx.Pool(min(cores, samples)) as pool:
        worker_s = pool.map(_oracle_worker, [(s, nsteps) for s in range(samples)])
    # the workers run concurrently (one per core): the slowest one bounds the job
    wall = max(worker_s)
    dofs = samples * N * N * nsteps
    return {"value": dofs / wall, "unit": "DOF-steps/s", "cores": min(cores, samples), "kind": "port",
            "sample": f"NumPy oracle (exponax restatement), {samples} samples x {nsteps} steps of the same "
                      f"256^2 ETDRK2 problem, one spawn process per sample; slowest worker {wall:.2f} s"}


# ------------------------------------------------------------------ float64 check (oracle as the checker)
def _rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def fp64_check_ns256(st, ex, torch):
    """Relative L2 of the GPU path against the float64 oracle (stand-in for a JAX float64 run) on the
    first two initial conditions of the workload, after 1, 20 and 200 steps (outside any timed region)."""
    from oracle import exponax_np as o

    so = o.NavierStokesVorticity(2, 2 * np.pi, N, DT, diffusivity=NU, dtype="float64")
    u0 = make_ics(0, 2)
    got = ex.vmap(ex.rollout(st, NSTEPS))(torch.from_numpy(u0).cuda()).cpu().numpy()
    errs = {}
    refs = [o.rollout(so, NSTEPS)(u0[b].astype(np.float64)) for b in range(2)]
    for nn in (1, 20, NSTEPS):
        errs[f"rel_l2_vs_fp64_after_{nn}"] = max(_rel(got[b, nn - 1], refs[b][nn - 1]) for b in range(2))
    errs["sample"] = "2 initial conditions, NumPy float64 oracle"
    return errs


# ------------------------------------------------------------------ arms
def dist_init():
    """One process per GPU (torchrun); replicas over batch shards, no data-path collective."""
    from exponax_gb300 import replicas

    return replicas.init("nccl")


def run_reference(args, rank, ws):
    if rank != 0:
        return
    # warm-up (pool start, imports) then K timed bounded samples
    cores = os.cpu_count() or 1
    for _ in range(max(0, min(args.warmup, 1))):
        cpu_baseline(samples=min(cores, 4), nsteps=2)
    vals = []
    for _ in range(args.steps):
        vals.append(cpu_baseline())
    v = float(np.median([x["value"] for x in vals]))
    base = dict(vals[0])
    base["value"] = v
    line = {"metric": metric_name(), "value": v, "unit": "DOF-steps/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": BATCH * N * N * NSTEPS / v * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config({"note": "ms_per_step extrapolates the measured rate to the full bench step"}),
            "impl": "reference", "cpu_baseline": base,
            "e2e": {"value": v, "unit": "DOF-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gb300(args, rank, ws):
    import torch

    import exponax_gb300 as ex
    from exponax_gb300 import _device, _lib

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    lib = _lib.load()
    st = ex.stepper.NavierStokesVorticity(2, 2 * np.pi, N, DT, diffusivity=NU)
    plan = st.plan.handle
    stream = torch.cuda.current_stream()
    sptr = _device.stream()

    from exponax_gb300 import replicas

    seeds = replicas.shard(BATCH, rank)  # this rank's contiguous shard of seeds
    u0_host = make_ics(seeds.start, BATCH)
    u0 = torch.from_numpy(u0_host).cuda()
    uh0 = ex.fft(u0, num_spatial_dims=2)
    out_h = torch.empty_like(uh0)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def fourier_run():
        _lib.check(lib.exgb_repeat_fourier(plan, sptr, uh0.data_ptr(), out_h.data_ptr(), BATCH, NSTEPS))

    # ---- warm-up
    for _ in range(args.warmup):
        fourier_run()
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()

    # ---- value: device-resident inputs, the fused 2D kernel (1 launch per bench step, 2 when the
    #      samples of a partial last wave run on the tail configuration)
    import tempfile

    clocks = ClockSampler(os.path.join(os.environ.get("EXGB_CLOCKS_DIR", tempfile.gettempdir()),
                                       f"bench_clocks_r{rank}.csv"))
    clocks.start()
    times = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fourier_run()
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    total_ms = replicas.max_over_ranks(float(np.sum(times)))
    ms_step = total_ms / args.steps
    value = replicas.aggregate_throughput(BATCH * N * N * NSTEPS, ws, ms_step)

    # ---- e2e: public API, pinned host buffers, H2D + repeat + D2H inside the timed region
    pin_in = torch.from_numpy(u0_host).pin_memory()
    pin_out = torch.empty_like(pin_in).pin_memory()
    rep = ex.vmap(ex.repeat(st, NSTEPS))
    for _ in range(max(1, args.warmup)):
        dev = pin_in.cuda(non_blocking=True)
        pin_out.copy_(rep(dev), non_blocking=True)
    torch.cuda.synchronize()
    etimes = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        dev = pin_in.cuda(non_blocking=True)
        res = rep(dev)
        pin_out.copy_(res, non_blocking=True)
        e1.record(stream)
        torch.cuda.synchronize()
        etimes.append(e0.elapsed_time(e1))
    clk = clocks.stop(local)
    e_ms = replicas.max_over_ranks(float(np.sum(etimes)) / args.steps)
    e2e = replicas.aggregate_throughput(BATCH * N * N * NSTEPS, ws, e_ms)

    # ---- roofline of the dominant kernel (vort2d_kernel: every launch of fourier_run)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    alg_bytes = BATCH * N * N * NSTEPS * BYTES_PER_DOF_STEP
    achieved = alg_bytes / (ms_step * 1e-3) / 1e9
    traffic = None
    tf = os.path.join(ROOT, "profiles", "vort2d_kernel_ns256_b128_traffic.txt")
    if os.path.exists(tf):
        for line in open(tf):
            if line.startswith(("dram_bytes_per_launch=", "dram_bytes_per_bench_step=")):
                traffic = float(line.split("=")[1])

    # the kernel keeps its stage buffers in L2 and shared memory, so the FP32 pipes bound it: transform
    # flops against the nominal FP32 rate (152 SMs x 128 FMA lanes x 2) at the SM clock sampled under load
    sm_mhz = float((clk or {}).get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0))
    fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
    fp32_ach = FFT_FLOPS_PER_DOF_STEP * value / ws / 1e12  # per GPU
    fp32 = {"achieved": fp32_ach, "peak": fp32_peak, "unit": "TFLOP/s", "frac": fp32_ach / fp32_peak,
            "note": f"{FFT_FLOPS_PER_DOF_STEP:.0f} transform flop/DOF-step (5 n log2 n per complex FFT); "
                    f"peak nominal at {sm_mhz:.0f} MHz"}

    # launches per call of the fused kernel (2 when a partial last wave runs on larger clusters)
    nfl = ctypes.c_int(0)
    lib_rc = lib.exgb_plan_fused_launches(plan, BATCH, ctypes.byref(nfl))
    fused = nfl.value if lib_rc == 0 and nfl.value > 0 else 1

    if rank == 0:
        cpu = cpu_baseline() if ws == 1 and not args.no_cpu else None
        fp64 = fp64_check_ns256(st, ex, torch) if ws == 1 and not args.no_cpu else None
        line = {"metric": metric_name(), "value": value, "unit": "DOF-steps/s", "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded truncated Fourier series ICs)",
                "config": config({"value_path": "exgb_repeat_fourier on device-resident Fourier states",
                                  "e2e_path": "vmap(repeat(stepper, 200)) with pinned host in/out"}),
                "e2e": {"value": e2e, "unit": "DOF-steps/s", "ms_per_step": e_ms,
                        "h2d_bytes_per_step": int(pin_in.numel() * 4), "d2h_bytes_per_step": int(pin_out.numel() * 4)},
                "gpu_launches": args.steps * fused + args.steps * (4 + fused),
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "traffic": traffic,
                             "kernel": "vort2d_kernel<256,512>",
                             "note": f"algorithmic {BYTES_PER_DOF_STEP:.2f} B/DOF-step (ETDRK2, 6 complex64 "
                                     f"half-spectrum passes) x {BATCH}x{N}^2x{NSTEPS} per bench step "
                                     f"({fused} kernel launch{'es' if fused > 1 else ''}); peak {peak_src}",
                             "fp32": fp32},
                "clocks": clk, "cpu_baseline": cpu, "fp64_check": fp64}
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.barrier()


# ------------------------------------------------------------------ other benchmark configurations
# MMA work of tcdft2d_kernel per sample and ETDRK2 step (N = 128): per stage 4 x (128x96x96 + 128x128x96)
# + 128x128x128 + 128x96x128 multiply-adds, x 2 flop, x 3 split-BF16 products; 2 stages.
TC128_MMA_FLOPS_PER_SAMPLE_STEP = 2 * 3 * 2 * (4 * (128 * 96 * 96 + 128 * 128 * 96) + 128 * 128 * 128 + 128 * 96 * 128)


def _traffic(name):
    """DRAM bytes per launch from the committed ncu summary profiles/<name>_traffic.txt, or None."""
    tf = os.path.join(ROOT, "profiles", f"{name}_traffic.txt")
    if os.path.exists(tf):
        for ln in open(tf):
            if ln.startswith("dram_bytes_per_launch=") or ln.startswith("dram_bytes_per_call="):
                return float(ln.split("=")[1])
    return None


def _timed(fn, steps, warmup, flush=None):
    import torch

    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ts = []
    for _ in range(steps):
        if flush is not None:
            flush.fill_(1.0)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    return float(np.mean(ts))


def _oracle_ks_worker(args):
    seed, nsteps = args
    from exponax_gb300.ic import RandomSineWaves1d
    from oracle import exponax_np as o

    st = o.KuramotoSivashinskyConservative(1, 100.0, 200, 0.1)
    u = RandomSineWaves1d(1, cutoff=5)(200, key=seed)
    t0 = time.perf_counter()
    o.rollout(st, nsteps, include_init=True)(u)
    return time.perf_counter() - t0


def _ns3d_ic(N, key):
    """Smooth divergence-free velocity (3, N, N, N), float32: amplitude-phase series per channel, Leray-projected."""
    from exponax_gb300.ic import RandomAmplitudePhaseSeries
    from oracle import exponax_np as o

    g = RandomAmplitudePhaseSeries(3, cutoff=5, max_one=True)
    u = np.concatenate([g(N, key=3 * key + c) for c in range(3)], axis=0).astype(np.float64)
    d = o.build_derivative_operator(3, 2 * np.pi, N, dtype="float64")
    P = o.Leray(3, N, derivative_operator=d, dtype="float64")
    return o.ifft(P(o.fft(u)), num_spatial_dims=3, num_points=N).astype(np.float32)


def _oracle_ns3d_worker(args):
    seed, nsteps = args
    from oracle import exponax_np as o

    st = o.NavierStokesVelocity(3, 2 * np.pi, 64, 0.01, diffusivity=0.01)
    u = _ns3d_ic(64, seed)
    t0 = time.perf_counter()
    o.repeat(st, nsteps)(u)
    return time.perf_counter() - t0


def _oracle_uneven_worker(args):
    idx, nsteps = args
    from oracle import exponax_np as o

    rng = np.random.default_rng(0)
    pde = rng.integers(0, 3, size=3000)
    Ns = rng.choice([128, 256, 512, 1024, 2048, 4096], size=3000)
    from exponax_gb300.ic import RandomSineWaves1d

    t = 0.0
    dofs = 0
    for i in idx:
        p, N = int(pde[i]), int(Ns[i])
        if p == 0:
            st = o.Burgers(1, 1.0, N, 1e-3, diffusivity=0.01)
        elif p == 1:
            st = o.KortewegDeVries(1, 20.0, N, 0.01, dispersivity=1.0, hyper_diffusivity=0.01)
        else:
            st = o.KuramotoSivashinskyConservative(1, 100.0, N, 0.1)
        u = RandomSineWaves1d(1, cutoff=5)(N, key=i)
        t0 = time.perf_counter()
        o.rollout(st, nsteps, include_init=True)(u)
        t += time.perf_counter() - t0
        dofs += N * nsteps
    return t, dofs


def _pool_map(fn, jobs):
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    with ctx.Pool(len(jobs)) as pool:
        return pool.map(fn, jobs)


def _cores():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def run_other(args, rank, ws):
    import torch

    import exponax_gb300 as ex

    if rank != 0:
        return
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    cores = _cores()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    line = {"n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "metric": metric_name(), "unit": "DOF-steps/s"}
    if args.workload == "ks1d":
        B, Nk, n = 16, 200, 500
        st = ex.stepper.KuramotoSivashinskyConservative(1, 100.0, Nk, 0.1)
        u0h = np.stack([ex.ic.RandomSineWaves1d(1, cutoff=5)(Nk, key=s) for s in range(B)])
        u0 = torch.from_numpy(u0h).cuda()
        roll = ex.vmap(ex.rollout(st, n, include_init=True))
        ms = _timed(lambda: roll(u0), args.steps, args.warmup, flush)
        pin = torch.from_numpy(u0h).pin_memory()
        out = torch.empty((B, n + 1, 1, Nk), dtype=torch.float32).pin_memory()
        ems = _timed(lambda: out.copy_(roll(pin.cuda(non_blocking=True)), non_blocking=True), args.steps,
                     args.warmup)
        dof = B * Nk * n
        line.update(value=dof / (ms * 1e-3), ms_per_step=ms,
                    config={"workload": "KuramotoSivashinskyConservative 1D, L=100, N=200, dt=0.1, ETDRK2, batch 16, "
                                        "500-step rollout with include_init (one fused launch writing Fourier states, "
                                        "one batched inverse transform)"},
                    e2e={"value": dof / (ems * 1e-3), "unit": "DOF-steps/s", "ms_per_step": ems,
                         "h2d_bytes_per_step": int(pin.numel() * 4), "d2h_bytes_per_step": int(out.numel() * 4)},
                    gpu_launches=2 * args.steps)
        if not args.no_cpu:
            ts = _pool_map(_oracle_ks_worker, [(s, n) for s in range(min(cores, B))])
            line["cpu_baseline"] = {"value": min(cores, B) * Nk * n / max(ts), "unit": "DOF-steps/s",
                                    "cores": min(cores, B), "kind": "port",
                                    "sample": f"NumPy oracle, {min(cores, B)} samples x {n}-step rollout, one process each"}
            # float64 check: rel-L2 after 1 and 20 steps (chaotic case) and the time-averaged energy
            # spectra of the last 100 steps (sum_k |E_gpu - E_fp64| / sum_k E_fp64)
            from oracle import exponax_np as o

            so = o.KuramotoSivashinskyConservative(1, 100.0, Nk, 0.1, dtype="float64")
            got = roll(u0[:2]).cpu().numpy()
            errs = {}
            refs = [o.rollout(so, n, include_init=True)(u0h[b].astype(np.float64)) for b in range(2)]
            for nn in (1, 20):
                errs[f"rel_l2_vs_fp64_after_{nn}"] = max(_rel(got[b, nn], refs[b][nn]) for b in range(2))
            spec = lambda tr: np.mean(np.abs(np.fft.rfft(tr[-100:, 0].astype(np.float64), axis=-1)) ** 2, axis=0)  # noqa
            errs["energy_spectrum_rel_diff_last_100_steps"] = max(
                float(np.sum(np.abs(spec(got[b]) - spec(refs[b]))) / np.sum(spec(refs[b]))) for b in range(2))
            errs["sample"] = "2 initial conditions, NumPy float64 oracle"
            line["fp64_check"] = errs
    elif args.workload == "uneven1d":
        from exponax_gb300.batching import QueueRollout, uneven_config3

        n = 100
        instances, steppers = uneven_config3(3000, n, seed=0)
        q = QueueRollout(instances, n, include_init=True)
        q.capture()
        ms = _timed(q.replay, args.steps, args.warmup, flush)
        dof = sum(st.num_points for st, _ in instances) * n
        # e2e: host ICs -> device, one graph replay, whole trajectories back to pinned host memory
        pin_in = [uq.cpu().pin_memory() for uq in q._u0]  # one host buffer per (PDE, N) group
        tot_out = sum(t.numel() for t in q.trajectories)
        pin_out = torch.empty(tot_out, dtype=torch.float32).pin_memory()
        groups = [(uq, tr) for uq, tr in zip(q._u0, q._traj)]

        def e2e():
            for (uq, _), ph in zip(groups, pin_in):
                uq.copy_(ph, non_blocking=True)
            q.replay()
            off = 0
            for _, tr in groups:
                pin_out[off:off + tr.numel()].copy_(tr.reshape(-1), non_blocking=True)
                off += tr.numel()

        ems = _timed(e2e, args.steps, args.warmup)
        line.update(value=dof / (ms * 1e-3), ms_per_step=ms,
                    config={"workload": "3000 1D instances, seeded multinomial over Burgers / KdV / KS-conservative, "
                                        "N uniform in {128..4096}, ETDRK2, 100-step rollouts with include_init, one "
                                        "persistent work-queue launch captured as a CUDA graph",
                            "instances": 3000, "distinct_plans": len(steppers)},
                    e2e={"value": dof / (ems * 1e-3), "unit": "DOF-steps/s", "ms_per_step": ems,
                         "h2d_bytes_per_step": int(sum(p.numel() * 4 for p in pin_in)),
                         "d2h_bytes_per_step": int(tot_out * 4)},
                    gpu_launches=args.steps)
        if not args.no_cpu:
            nproc = min(cores, 16)
            jobs = [(list(range(p, 96, nproc)), n) for p in range(nproc)]
            res = _pool_map(_oracle_uneven_worker, jobs)
            line["cpu_baseline"] = {"value": sum(r[1] for r in res) / max(r[0] for r in res), "unit": "DOF-steps/s",
                                    "cores": nproc, "kind": "port",
                                    "sample": f"NumPy oracle rollouts of the first 96 instances, {nproc} processes"}
            # float64 check: the first instance of each PDE, 100-step trajectory after the graph replay
            from oracle import exponax_np as o

            q.replay()
            torch.cuda.synchronize()
            errs = {}
            for i, (stp, u) in enumerate(instances):
                name = type(stp).__name__
                if f"{name}_rel_l2_vs_fp64_after_{n}" in errs:
                    continue
                if name == "Burgers":
                    so = o.Burgers(1, 1.0, stp.num_points, 1e-3, diffusivity=0.01, dtype="float64")
                elif name == "KortewegDeVries":
                    so = o.KortewegDeVries(1, 20.0, stp.num_points, 0.01, dispersivity=1.0, hyper_diffusivity=0.01,
                                           dtype="float64")
                else:
                    so = o.KuramotoSivashinskyConservative(1, 100.0, stp.num_points, 0.1, dtype="float64")
                ref = o.rollout(so, n, include_init=True)(np.asarray(u, dtype=np.float64))
                got = q.trajectories[i].cpu().numpy()
                errs[f"{name}_rel_l2_vs_fp64_after_{n}"] = _rel(got[-1], ref[-1])
                errs[f"{name}_N"] = int(stp.num_points)
            errs["sample"] = "first instance of each PDE, NumPy float64 oracle"
            line["fp64_check"] = errs
    elif args.workload == "kolmo128":
        from exponax_gb300 import _device, _lib

        Nk, B, n = 128, 1024, 100
        st = ex.stepper.KolmogorovFlowVorticity(2, 2 * np.pi, Nk, 0.01)
        if args.precision != "fp32":
            st.set_dft_precision(args.precision)
        g = ex.ic.RandomAmplitudePhaseSeries(2, cutoff=5, max_one=True)
        u0h = np.stack([g(Nk, key=s) for s in range(B)])
        uh = ex.fft(torch.from_numpy(u0h).cuda(), num_spatial_dims=2)
        out = torch.empty_like(uh)
        lib = _lib.load()
        h = st.plan.handle

        def run():
            _lib.check(lib.exgb_repeat_fourier(h, _device.stream(), uh.data_ptr(), out.data_ptr(), B, n))

        ms = _timed(run, args.steps, args.warmup, flush)
        rep = ex.vmap(ex.repeat(st, n))
        pin = torch.from_numpy(u0h).pin_memory()
        pout = torch.empty_like(pin).pin_memory()
        ems = _timed(lambda: pout.copy_(rep(pin.cuda(non_blocking=True)), non_blocking=True), args.steps,
                     args.warmup)
        dof = B * Nk * Nk * n
        line.update(value=dof / (ms * 1e-3), ms_per_step=ms,
                    config={"workload": "KolmogorovFlowVorticity 2D 128^2, nu=1e-3, drag=-0.1, forcing k=4 amplitude "
                                        "1, dt=0.01, ETDRK2, batch 1024, 100 steps ("
                                        + ("FP32 transforms" if args.precision == "fp32" else
                                           "split-BF16 tcgen05 DFT contractions, FP32 accumulation") + ")"},
                    dtype="f32" if args.precision == "fp32" else "bf16x3 (split) / f32 accumulate",
                    e2e={"value": dof / (ems * 1e-3), "unit": "DOF-steps/s", "ms_per_step": ems,
                         "h2d_bytes_per_step": int(pin.numel() * 4), "d2h_bytes_per_step": int(pout.numel() * 4)},
                    gpu_launches=args.steps)
        peaks = {}
        try:
            peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        except Exception:
            pass
        if args.precision == "fp32":
            peak = float(peaks.get("hbm_gbs", 6800.0))
            bpd = 6 * 8 * (Nk // 2 + 1) / Nk  # 6 complex64 half-spectrum passes per ETDRK2 step
            achieved = dof * bpd / (ms * 1e-3) / 1e9
            line["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                                "frac": achieved / peak, "traffic": _traffic("vort2d_kernel_kolmo128_b1024"),
                                "kernel": "vort2d_kernel<128,512>",
                                "note": f"algorithmic {bpd:.3f} B/DOF-step x {B}x{Nk}^2x{n} per launch; peak "
                                        + ("measured" if "hbm_gbs" in peaks else "fallback")}
        else:
            peak = float(peaks.get("bf16_tflops", 1900.0))
            flops = TC128_MMA_FLOPS_PER_SAMPLE_STEP * B * n
            achieved = flops / (ms * 1e-3) / 1e12
            line["roofline"] = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                                "frac": achieved / peak, "traffic": _traffic("tcdft2d_kernel_kolmo128_b1024"),
                                "kernel": "tcdft2d_kernel",
                                "note": f"{TC128_MMA_FLOPS_PER_SAMPLE_STEP} MMA flop per sample-step (10 split-BF16 "
                                        "contraction chains, 3 products each, as issued) x "
                                        f"{B}x{n} per launch; peak bf16 burst "
                                        + ("measured" if "bf16_tflops" in peaks else "fallback")}
        if not args.no_cpu:
            from oracle import exponax_np as o

            so64 = o.KolmogorovFlowVorticity(2, 2 * np.pi, Nk, 0.01, dtype="float64")
            errs = {}
            for nn in (1, 100):
                got = ex.vmap(ex.repeat(st, nn))(torch.from_numpy(u0h[:2]).cuda()).cpu().numpy()
                e = []
                for b in range(2):
                    ref = o.repeat(so64, nn)(u0h[b].astype(np.float64))
                    e.append(float(np.linalg.norm(got[b] - ref) / np.linalg.norm(ref)))
                errs[f"rel_l2_vs_fp64_after_{nn}"] = float(np.max(e))
            line["precision"] = dict(errs, note=("FP32 register transforms" if args.precision == "fp32" else
                                                 "split-BF16 tensor-core DFT") + " vs the float64 oracle, 2 seeds")
    elif args.workload == "ns3d64":
        from exponax_gb300 import _device, _lib

        Nk, B, n = 64, 32, 20
        st = ex.stepper.NavierStokesVelocity(3, 2 * np.pi, Nk, 0.01, diffusivity=0.01)
        u0h = np.stack([_ns3d_ic(Nk, s) for s in range(B)])
        uh = ex.fft(torch.from_numpy(u0h).cuda(), num_spatial_dims=3)
        out = torch.empty_like(uh)
        lib = _lib.load()
        h = st.plan.handle

        def run():
            _lib.check(lib.exgb_repeat_fourier(h, _device.stream(), uh.data_ptr(), out.data_ptr(), B, n))

        ms = _timed(run, args.steps, args.warmup, flush)
        rep = ex.vmap(ex.repeat(st, n))
        pin = torch.from_numpy(u0h).pin_memory()
        pout = torch.empty_like(pin).pin_memory()
        ems = _timed(lambda: pout.copy_(rep(pin.cuda(non_blocking=True)), non_blocking=True), args.steps,
                     args.warmup)
        dof = B * 3 * Nk ** 3 * n
        # launches per repeat call: 2 transposes + 1 linear-planes kernel + 4 kernels x 2 stages x n steps
        # (no projection between steps in Fourier space; ncu counts 163 for n = 20)
        launches = 3 + n * 2 * 4
        line.update(value=dof / (ms * 1e-3), ms_per_step=ms,
                    config={"workload": "NavierStokesVelocity 3D 64^3 (projected convection + Leray), domain 2pi, "
                                        "nu=0.01, dt=0.01, ETDRK2, 2/3 dealiasing, batch 32, 20 steps (repeat), "
                                        "three-pass 3D path", "l2": "flushed (256 MB write) between timed steps"},
                    e2e={"value": dof / (ems * 1e-3), "unit": "DOF-steps/s", "ms_per_step": ems,
                         "h2d_bytes_per_step": int(pin.numel() * 4), "d2h_bytes_per_step": int(pout.numel() * 4)},
                    gpu_launches=args.steps * launches)
        peaks = {}
        try:
            peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        except Exception:
            pass
        peak = float(peaks.get("hbm_gbs", 6800.0))
        bpd = 6 * 8 * (Nk // 2 + 1) / Nk  # 6 complex64 half-spectrum passes per ETDRK2 step
        achieved = dof * bpd / (ms * 1e-3) / 1e9
        line["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                            "frac": achieved / peak, "traffic": _traffic("pass3d_ns3d64_b32"),
                            "kernel": "pass1/2/3_3d_kernel<64> + combine_planes_kernel (one ETDRK stage)",
                            "note": f"algorithmic {bpd:.3f} B/DOF-step (state read + write per stage) x "
                                    f"{B}x3x{Nk}^3x{n} per repeat call, against the call's event time; "
                                    "traffic = DRAM bytes of the whole call (ncu); peak "
                                    + ("measured" if "hbm_gbs" in peaks else "fallback")}
        if not args.no_cpu:
            nproc = min(cores, 16)
            ncs = 5
            ts = _pool_map(_oracle_ns3d_worker, [(s, ncs) for s in range(nproc)])
            line["cpu_baseline"] = {"value": nproc * 3 * Nk ** 3 * ncs / max(ts), "unit": "DOF-steps/s",
                                    "cores": nproc, "kind": "port",
                                    "sample": f"NumPy oracle, {nproc} samples x {ncs} steps, one process each"}
            from oracle import exponax_np as o

            so64 = o.NavierStokesVelocity(3, 2 * np.pi, Nk, 0.01, diffusivity=0.01, dtype="float64")
            errs = {}
            for nn in (1, 20):
                got = ex.vmap(ex.repeat(st, nn))(torch.from_numpy(u0h[:2]).cuda()).cpu().numpy()
                e = []
                for b in range(2):
                    ref = o.repeat(so64, nn)(u0h[b].astype(np.float64))
                    e.append(float(np.linalg.norm(got[b] - ref) / np.linalg.norm(ref)))
                errs[f"rel_l2_vs_fp64_after_{nn}"] = float(np.max(e))
            errs["sample"] = "2 initial conditions, NumPy float64 oracle"
            line["fp64_check"] = errs
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "split_bf16"],
                    help="transform arithmetic of the kolmo128 workload")
    ap.add_argument("--workload", default="ns256", choices=["ns256", "ks1d", "uneven1d", "kolmo128", "ns3d64"],
                    help="ns256 (default, the headline metric) or one of the other benchmark configurations")
    args = ap.parse_args()
    rank, ws = dist_init()
    if args.workload != "ns256":
        run_other(args, rank, ws)
    elif args.impl == "reference":
        run_reference(args, rank, ws)
    else:
        run_gb300(args, rank, ws)
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
