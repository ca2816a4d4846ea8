"""Autotuner: candidates time on the device, the winner is applied and
cached, and the tuned plan still matches the oracle (1e-5 per step)."""

import json

import numpy as np
import pytest

import exponax_gb300 as ex
from exponax_gb300 import autotune
from oracle import exponax_np as o

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


def test_radix_candidates_multiply_to_n():
    for n in (60, 128, 200, 256, 4096):
        cands = autotune.radix_candidates(n)
        assert cands
        for c in cands:
            assert int(np.prod(c)) == n


@pytest.mark.parametrize("case", ["ks1d", "ns2d", "ns2d_generic"])
def test_tune_apply_cache_and_parity(case, tmp_path, monkeypatch):
    monkeypatch.setenv("EXGB_AUTOTUNE_CACHE", str(tmp_path / "cache.json"))
    if case == "ks1d":
        sm = ex.stepper.KuramotoSivashinskyConservative(1, 100.0, 200, 0.1)
        so = o.KuramotoSivashinskyConservative(1, 100.0, 200, 0.1)
        u = np.stack([ex.ic.RandomSineWaves1d(1, cutoff=5)(200, key=s) for s in range(3)])
    else:
        n = 128 if case == "ns2d" else 96
        sm = ex.stepper.NavierStokesVorticity(2, 2 * np.pi, n, 0.01, diffusivity=1e-3)
        so = o.NavierStokesVorticity(2, 2 * np.pi, n, 0.01, diffusivity=1e-3)
        g = ex.ic.RandomAmplitudePhaseSeries(2, cutoff=5, max_one=True)
        u = np.stack([g(n, key=s) for s in range(3)])
    res = autotune.tune(sm, batch=32, nsteps=4, repeats=2)
    assert not res["cached"] and res["best"] and len(res["timings_ms"]) >= 2
    if case == "ns2d_generic":
        # radix orders first, then every cluster size for the best of them
        assert "cluster" in res["best"] and "radices" in res["best"]
        assert autotune.get_tuning(sm.plan)["cluster"] == res["best"]["cluster"]
    cache = json.load(open(tmp_path / "cache.json"))
    assert res["key"] in cache
    got = ex.vmap(sm)(torch.from_numpy(u).cuda()).cpu().numpy()
    for b in range(3):
        assert rel(got[b], so(u[b])) < 1e-5
    again = autotune.tune(sm, batch=32, nsteps=4)
    assert again["cached"] and again["best"] == res["best"]


@pytest.mark.parametrize("n", [64, 128, 256, 96, 512])
def test_every_cluster_size_matches_oracle(n):
    """The 2D cluster kernels (register FFTs at N = 64 / 128 / 256, the generic kernel at 96 and
    512) with each cluster size 1..8 that fits (rows split unevenly when G does not divide N): one
    ETDRK2 step within 1e-5 of the oracle; sizes that do not fit are refused with
    EXGB_EUNSUPPORTED and leave the plan usable."""
    import os

    from exponax_gb300._lib import EXGB_OK
    os.environ["EXGB_2D_PATH"] = "fused"  # 512^2 runs on the three-pass path unless asked otherwise
    try:
        sm = ex.stepper.NavierStokesVorticity(2, 2 * np.pi, n, 0.01, diffusivity=1e-3)
        sm.plan.handle  # the plan (and its path) is made here, while the variable is set
    finally:
        del os.environ["EXGB_2D_PATH"]
    so = o.NavierStokesVorticity(2, 2 * np.pi, n, 0.01, diffusivity=1e-3)
    g = ex.ic.RandomAmplitudePhaseSeries(2, cutoff=5, max_one=True)
    u = np.stack([g(n, key=s) for s in range(3)])
    want = [so(u[b]) for b in range(3)]
    ran = []
    for G in range(1, 9):
        if autotune._set(sm.plan, 1, [G]) != EXGB_OK:
            continue
        assert autotune.get_tuning(sm.plan)["cluster"] == G
        got = ex.vmap(sm)(torch.from_numpy(u).cuda()).cpu().numpy()
        for b in range(3):
            assert rel(got[b], want[b]) < 1e-5, (G, b)
        ran.append(G)
    assert len(ran) >= 2, ran
    assert autotune._set(sm.plan, 1, [0]) == EXGB_OK


@pytest.mark.parametrize("n,batch", [(200, 3), (64, 40), (1024, 2)])
def test_1d_threads_per_cta_match_oracle(n, batch):
    """Every threads-per-CTA setting of the 1D kernel (64, 128, 256 and the automatic choice) gives
    the oracle's step within 1e-5 and the same 20-step rollout within 1e-4; other values are refused."""
    from exponax_gb300._lib import EXGB_OK
    sm = ex.stepper.KuramotoSivashinskyConservative(1, 100.0, n, 0.1)
    so = o.KuramotoSivashinskyConservative(1, 100.0, n, 0.1)
    u = np.stack([ex.ic.RandomSineWaves1d(1, cutoff=5)(n, key=s) for s in range(batch)])
    want1 = [so(u[b]) for b in range(batch)]
    want20 = [o.rollout(so, 20, include_init=True)(u[b]) for b in range(batch)]
    for t in (64, 128, 256, 0):
        assert autotune._set(sm.plan, 4, [t]) == EXGB_OK
        assert autotune.get_tuning(sm.plan)["threads"] == t
        got = ex.vmap(sm)(torch.from_numpy(u).cuda()).cpu().numpy()
        traj = ex.vmap(ex.rollout(sm, 20, include_init=True))(torch.from_numpy(u).cuda()).cpu().numpy()
        for b in range(batch):
            assert rel(got[b], want1[b]) < 1e-5, (t, b)
            assert rel(traj[b], want20[b]) < 1e-4, (t, b)
    assert autotune._set(sm.plan, 4, [96]) != EXGB_OK
