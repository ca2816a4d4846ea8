"""Split-BF16 tensor-core DFT path (tcgen05) of the 2D vorticity steppers.

1. The tcgen05 layer (exgb_tc_gemm_check) against float64 GEMMs: with
   bf16-rounded inputs the products are exact and only the FP32
   accumulation rounds (rel 2e-6); split-BF16 of FP32 inputs keeps about
   16 significant bits per product (rel 3e-5).
2. KolmogorovFlowVorticity 128^2 (the precision-study configuration) with
   precision "split_bf16" against the oracle: the nonlinear term within
   1e-4 relative L2 (a chain of four split-BF16 contractions), one step
   within 1e-5, 100 steps within 1e-4 of the FP32 oracle; the errors of the
   FP32 and split-BF16 paths against a float64 oracle run are printed.
"""

import ctypes

import numpy as np
import pytest

import exponax_gb300 as ex
from exponax_gb300 import _device
from exponax_gb300._lib import check, load
from oracle import exponax_np as o

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def cu(x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def bf16(x):
    return torch.from_numpy(np.asarray(x, np.float32)).to(torch.bfloat16).to(torch.float32).numpy()


@pytest.mark.parametrize("n,k", [(16, 16), (96, 96), (128, 128), (176, 64), (256, 128)])
@pytest.mark.parametrize("split", [0, 1])
def test_tcgen05_gemm_layer(n, k, split):
    rng = np.random.default_rng(n * 1000 + k)
    a = rng.standard_normal((128, k)).astype(np.float32)
    b = rng.standard_normal((n, k)).astype(np.float32)
    d = torch.empty((128, n), dtype=torch.float32, device="cuda")
    da, db = cu(a), cu(b)
    check(load().exgb_tc_gemm_check(_device.stream(), n, k, da.data_ptr(), db.data_ptr(), d.data_ptr(), split),
          "tc_gemm_check")
    got = d.cpu().numpy()
    if split:
        want = a.astype(np.float64) @ b.astype(np.float64).T
        assert rel(got, want) < 3e-5
    else:
        want = bf16(a).astype(np.float64) @ bf16(b).astype(np.float64).T
        assert rel(got, want) < 2e-6


def _kolmo(dtype="float32", n=128):
    return o.KolmogorovFlowVorticity(2, 2 * np.pi, n, 0.01, dtype=dtype)


def _ics(B, n=128, seed0=0):
    g = ex.ic.RandomAmplitudePhaseSeries(2, cutoff=5, max_one=True)
    return np.stack([g(n, key=seed0 + s) for s in range(B)])


def test_split_bf16_requires_supported_plan():
    sm = ex.stepper.KolmogorovFlowVorticity(2, 2 * np.pi, 64, 0.01)
    with pytest.raises(Exception):
        sm.set_dft_precision("split_bf16")
    with pytest.raises(ValueError):
        sm.set_dft_precision("tf16")


def test_split_bf16_nonlinear_term_matches_oracle():
    sm = ex.stepper.KolmogorovFlowVorticity(2, 2 * np.pi, 128, 0.01).set_dft_precision("split_bf16")
    so = _kolmo()
    B = 4
    u = _ics(B)
    uh = np.stack([o.fft(x) for x in u]).astype(np.complex64)
    t = cu(uh)
    out = torch.empty_like(t)
    check(load().exgb_nonlinear(sm.plan.handle, _device.stream(), t.data_ptr(), out.data_ptr(), B), "nonlinear")
    sm.plan.status()
    got = out.cpu().numpy()
    for b in range(B):
        want = so.nonlinear_fun(uh[b])
        assert rel(got[b].view(np.float32), want.astype(np.complex64).view(np.float32)) < 1e-4, b


def test_split_bf16_single_step_matches_oracle():
    sm = ex.stepper.KolmogorovFlowVorticity(2, 2 * np.pi, 128, 0.01).set_dft_precision("split_bf16")
    so = _kolmo()
    B = 6
    u = _ics(B)
    got = ex.vmap(sm)(cu(u)).cpu().numpy()
    sm.plan.status()
    for b in range(B):
        assert rel(got[b], so(u[b])) < 1e-5, b


@pytest.mark.parametrize("order", [1, 3, 4])
def test_split_bf16_other_orders(order):
    sm = ex.stepper.KolmogorovFlowVorticity(2, 2 * np.pi, 128, 0.01, order=order).set_dft_precision("split_bf16")
    so = o.KolmogorovFlowVorticity(2, 2 * np.pi, 128, 0.01, order=order)
    u = _ics(2, seed0=7)
    got = ex.vmap(sm)(cu(u)).cpu().numpy()
    for b in range(2):
        assert rel(got[b], so(u[b])) < 1e-5, b


def test_split_bf16_100_steps_against_fp32_and_fp64():
    """Precision study: errors after 1 and 100 steps of both transform
    arithmetics against a float64 oracle run (printed), and the split-BF16
    path within 1e-4 of the FP32 oracle after 100 steps."""
    B, n = 4, 100
    u = _ics(B, seed0=100)
    s32 = _kolmo("float32")
    s64 = _kolmo("float64")
    fp32 = ex.stepper.KolmogorovFlowVorticity(2, 2 * np.pi, 128, 0.01)
    tc = ex.stepper.KolmogorovFlowVorticity(2, 2 * np.pi, 128, 0.01).set_dft_precision("split_bf16")
    res = {}
    for steps in (1, n):
        g32 = ex.vmap(ex.repeat(fp32, steps))(cu(u)).cpu().numpy()
        gtc = ex.vmap(ex.repeat(tc, steps))(cu(u)).cpu().numpy()
        w64 = np.stack([o.repeat(s64, steps)(u[b].astype(np.float64)) for b in range(B)])
        w32 = np.stack([o.repeat(s32, steps)(u[b]) for b in range(B)])
        res[steps] = (rel(g32, w64), rel(gtc, w64), rel(w32, w64), rel(gtc, w32))
    tc.plan.status()
    for steps, (e32, etc, eo32, d) in res.items():
        print(f"steps={steps}: rel-L2 vs float64 oracle: fp32 CUDA {e32:.2e}, split-bf16 CUDA {etc:.2e}, "
              f"fp32 oracle {eo32:.2e}; split-bf16 vs fp32 oracle {d:.2e}")
    assert res[1][3] < 1e-5
    assert res[n][3] < 1e-4


def test_split_bf16_navier_stokes_rollout_and_switch_back():
    """Plain NavierStokesVorticity (no forcing) on the tensor-core path: a 10-step physical rollout
    (c2r projection between steps) within 1e-4 of the oracle, and switching the plan back to FP32
    transforms reproduces the FP32 path."""
    sm = ex.stepper.NavierStokesVorticity(2, 2 * np.pi, 128, 0.01, diffusivity=1e-3)
    so = o.NavierStokesVorticity(2, 2 * np.pi, 128, 0.01, diffusivity=1e-3)
    u = _ics(3, seed0=40)
    fp32 = ex.vmap(ex.rollout(sm, 10, include_init=True))(cu(u)).cpu().numpy()
    sm.set_dft_precision("split_bf16")
    tc = ex.vmap(ex.rollout(sm, 10, include_init=True))(cu(u)).cpu().numpy()
    sm.plan.status()
    for b in range(3):
        want = o.rollout(so, 10, include_init=True)(u[b])
        assert rel(tc[b], want) < 1e-4, b
    sm.set_dft_precision("fp32")
    again = ex.vmap(ex.rollout(sm, 10, include_init=True))(cu(u)).cpu().numpy()
    np.testing.assert_array_equal(again, fp32)


def test_split_bf16_batch_not_multiple_of_ctas():
    """Batches smaller and larger than the persistent grid (152 CTAs) give the same per-sample result."""
    sm = ex.stepper.KolmogorovFlowVorticity(2, 2 * np.pi, 128, 0.01).set_dft_precision("split_bf16")
    u = _ics(2, seed0=60)
    small = ex.vmap(ex.repeat(sm, 3))(cu(u)).cpu().numpy()
    big = np.concatenate([u] * 101)  # 202 samples
    out = ex.vmap(ex.repeat(sm, 3))(cu(big)).cpu().numpy()
    for rep in (0, 77, 100):
        np.testing.assert_array_equal(out[2 * rep:2 * rep + 2], small)


def test_bounded_wait_runs_out_and_reports_timeout():
    """The timeout path of the tensor-core kernel's bounded device waits, with no fault: a test-only
    knob gives the first MMA-completion wait of each launch a budget of 2 clock cycles, so it gives up
    while its MMAs are in flight.  The kernel then drains them with the normal budget, releases its
    tensor memory and sets the status word: exgb_plan_status returns EXGB_ETIMEOUT (and clears it),
    the context stays usable, and with the normal budget restored the next call matches the oracle
    within 1e-5 after one step."""
    from exponax_gb300 import _lib, autotune

    lib = load()
    N = 128
    sm = ex.stepper.KolmogorovFlowVorticity(2, 2 * np.pi, N, 0.01).set_dft_precision("split_bf16")
    so = o.KolmogorovFlowVorticity(2, 2 * np.pi, N, 0.01)
    u0 = np.stack([ex.ic.RandomAmplitudePhaseSeries(2, cutoff=5, max_one=True)(N, key=s) for s in range(4)])
    assert autotune._set(sm.plan, _lib.EXGB_TUNE_WAIT_BUDGET, [2]) == 0
    ex.vmap(sm)(cu(u0))
    torch.cuda.synchronize()
    assert lib.exgb_plan_status(sm.plan.handle) == _lib.EXGB_ETIMEOUT
    assert b"gave up" in lib.exgb_last_error()
    assert lib.exgb_plan_status(sm.plan.handle) == 0  # cleared on read
    assert autotune._set(sm.plan, _lib.EXGB_TUNE_WAIT_BUDGET, [0]) == 0
    got = ex.vmap(sm)(cu(u0)).cpu().numpy()
    sm.plan.status()
    for b in range(4):
        assert rel(got[b], so(u0[b])) < 1e-5
