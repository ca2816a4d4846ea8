"""Parity of the benchmark workloads at their configured scale (through the
C ABI), against the float32 NumPy oracle on sampled members of the batch.

* The uneven 1D batch: 3000 Burgers / KdV / KS-conservative instances with N
  drawn from {128, ..., 4096}, 100 steps in one work-queue launch replayed
  from a CUDA graph (the reference runs one jax.vmap(rollout) per (PDE, N)
  group, _utils.py:92-186).  A seeded sample covering every (PDE, N) cell --
  including the N = 4096 items whose ETDRK state lives in a per-CTA global
  slot -- is compared instance by instance: within 1e-4 relative L2 after
  100 steps for Burgers and KdV (non-chaotic), within 1e-4 over the first 20
  steps for KS (chaotic).
* 2D Navier-Stokes vorticity 256^2 (nu 1e-3, dt 0.01, ETDRK2), batch 128 --
  which takes the partial-last-wave launch on larger clusters -- over 200
  steps: four sampled seeds within 1e-5 after one step and 1e-4 over the
  first 20 steps, and time-averaged energy spectra over steps 100..200 within
  5 %.  The final states after 200 steps are also held to 1e-4 (this flow at
  this horizon stays within a few 1e-6 of a float64 run).
"""

import numpy as np
import pytest

import exponax_gb300 as ex
from oracle import exponax_np as o

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _oracle_1d(sm):
    """The oracle stepper with the same class and parameters as a 1D stepper of uneven_config3."""
    name = type(sm).__name__
    N = sm.num_points
    if name == "Burgers":
        return o.Burgers(1, 1.0, N, 1e-3, diffusivity=0.01)
    if name == "KortewegDeVries":
        return o.KortewegDeVries(1, 20.0, N, 0.01, dispersivity=1.0, hyper_diffusivity=0.01)
    assert name == "KuramotoSivashinskyConservative", name
    return o.KuramotoSivashinskyConservative(1, 100.0, N, 0.1)


def test_uneven_batch_3000_instances_sampled_against_oracle():
    from exponax_gb300.batching import QueueRollout, uneven_config3

    nsteps = 100
    instances, _ = uneven_config3(3000, nsteps, seed=0)
    q = QueueRollout(instances, nsteps, include_init=True)
    q.capture()
    q.replay()
    q.replay()  # a second replay recomputes the same trajectories from the same u0
    torch.cuda.synchronize()

    cells = {}
    for i, (sm, _) in enumerate(instances):
        cells.setdefault((type(sm).__name__, sm.num_points), []).append(i)
    assert len(cells) == 18, sorted(cells)
    rng = np.random.default_rng(1234)
    sample = []
    for key in sorted(cells):
        idx = cells[key]
        sample.extend(int(i) for i in rng.choice(idx, size=min(3, len(idx)), replace=False))
    extra = rng.choice(len(instances), size=60 - len(sample), replace=False)
    sample.extend(int(i) for i in extra if int(i) not in sample)
    assert len(sample) >= 54

    worst = {}
    for i in sample:
        sm, u0 = instances[i]
        so = _oracle_1d(sm)
        got = q.trajectories[i].cpu().numpy()
        assert got.shape == (nsteps + 1, 1, sm.num_points)
        np.testing.assert_array_equal(got[0], np.asarray(u0, np.float32).reshape(1, -1))
        name = type(sm).__name__
        if name == "KuramotoSivashinskyConservative":
            ref = o.rollout(so, 20, include_init=True)(u0)
            e = max(rel(got[t], ref[t]) for t in range(1, 21))
        else:
            ref = o.repeat(so, nsteps)(u0)
            e = rel(got[nsteps], ref)
        key = (name, sm.num_points)
        worst[key] = max(worst.get(key, 0.0), e)
        assert e < 1e-4, (i, key, e)
    assert {k[1] for k in worst} == {128, 256, 512, 1024, 2048, 4096}


def _avg_power_spectrum(states):
    """Radially binned ("sum") power spectrum of _spectral.py:866-1030 averaged over
    the leading axis of `states` (T, N, N): the binning is linear, so the per-mode
    power is averaged first and binned once (float64)."""
    N = states.shape[-1]
    u = np.fft.rfft2(np.asarray(states, np.float64))
    rec = o.build_scaling_array(2, N, mode="reconstruction", dtype="float64")[0]
    nc = o.build_scaling_array(2, N, mode="norm_compensation", dtype="float64")[0]
    q = (0.5 * np.abs(u) ** 2 / (rec * nc)).mean(axis=0)
    wn = o.build_wavenumbers(2, N, dtype="float64")
    norm = np.linalg.norm(wn, axis=0)
    out = np.zeros(N // 2 + 1)
    for k in range(N // 2 + 1):
        m = (norm >= k - 0.5) & (norm < k + 0.5)
        out[k] = q[m].sum()
    return out


def test_ns256_batch128_200_steps_sampled_against_oracle():
    from exponax_gb300 import _lib

    import ctypes

    B, N, n = 128, 256, 200
    sm = ex.stepper.NavierStokesVorticity(2, 2 * np.pi, N, 0.01, diffusivity=1e-3)
    so = o.NavierStokesVorticity(2, 2 * np.pi, N, 0.01, diffusivity=1e-3)
    cnt = ctypes.c_int(0)
    assert _lib.load().exgb_plan_fused_launches(sm.plan.handle, B, ctypes.byref(cnt)) == 0
    assert cnt.value == 2, "batch 128 at 256^2 runs its partial last wave on the tail configuration"
    g = ex.ic.RandomAmplitudePhaseSeries(2, cutoff=5, max_one=True)
    u0 = np.stack([g(N, key=s) for s in range(B)])
    u0d = torch.from_numpy(u0).cuda()
    one = ex.vmap(sm)(u0d).cpu().numpy()
    traj = ex.vmap(ex.rollout(sm, n, include_init=True))(u0d)  # (B, n + 1, 1, N, N) on the device
    assert tuple(traj.shape) == (B, n + 1, 1, N, N)
    fin = ex.vmap(ex.repeat(sm, n))(u0d).cpu().numpy()
    seeds = [0, 41, 86, 127]  # both launches: the main waves and the tail samples
    spec_m, spec_o = 0.0, 0.0
    for s in seeds:
        ref = o.rollout(so, n, include_init=True)(u0[s])
        got = traj[s].cpu().numpy()
        assert rel(one[s], ref[1]) < 1e-5, (s, rel(one[s], ref[1]))
        for t in range(1, 21):
            assert rel(got[t], ref[t]) < 1e-4, (s, t)
        assert rel(got[n], ref[n]) < 1e-4, (s, rel(got[n], ref[n]))
        assert rel(fin[s], ref[n]) < 1e-4, (s, rel(fin[s], ref[n]))
        spec_m = spec_m + _avg_power_spectrum(got[100:, 0])
        spec_o = spec_o + _avg_power_spectrum(ref[100:, 0])
    k = slice(1, 85)  # the modes the 2/3 mask keeps
    assert rel(spec_m[k], spec_o[k]) < 0.05
    assert np.max(np.abs(np.log(spec_m[1:30] / spec_o[1:30]))) < np.log(1.05)
