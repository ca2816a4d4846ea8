"""Learned corrector kernels against the NumPy oracle (oracle/corrector_np.py):
forward, loss and every parameter gradient (BF16 weights / activations /
gradients on the GPU against an FP64 oracle: 3e-2 relative L2), one Adam
step (1e-5 on the FP32 master weights), the training signal on a synthetic
task, and the spectral-energy guard."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def rel(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def _net(B=3, H=8, seed=1, in_scale=0.7, out_scale=0.5):
    from exponax_gb300.learned import PeriodicConvCorrector

    net = PeriodicConvCorrector(H, seed=seed, max_batch=B, in_scale=in_scale, out_scale=out_scale)
    # a larger last layer and non-zero biases so every gradient is exercised
    rng = np.random.default_rng(seed + 10)
    w = net.w.cpu().numpy()
    o, n = net.layout["W6"]
    w[o:o + n] = rng.standard_normal(n) / np.sqrt(9 * 48)
    for k in ("b1", "b2", "b3", "b4", "b5", "b6"):
        o, n = net.layout[k]
        w[o:o + n] = 0.1 * rng.standard_normal(n)
    net.set_params(w)
    return net


def _data(B, H, seed=0):
    rng = np.random.default_rng(seed)
    v = rng.standard_normal((B, H, 64)).astype(np.float32)
    tgt = (v + 0.3 * rng.standard_normal((B, H, 64))).astype(np.float32)
    return v, tgt


@pytest.mark.parametrize("B,H", [(3, 8), (2, 64)])
def test_forward_and_gradients_match_oracle(B, H):
    from oracle import corrector_np as co

    net = _net(B, H)
    v, tgt = _data(B, H)
    loss, pred = net.loss_and_grads(torch.from_numpy(v).cuda(), torch.from_numpy(tgt).cuda())
    params = net.params_numpy()
    loss_o, pred_o, grads_o = co.loss_and_grads(params, v.astype(np.float64), tgt.astype(np.float64),
                                                in_scale=net.in_scale, out_scale=net.out_scale)
    assert rel(pred.cpu().numpy() - v, pred_o - v) < 3e-2
    assert abs(float(loss) - loss_o) / loss_o < 1e-2
    g = net.g.cpu().numpy()
    for i, (gw, gb) in enumerate(grads_o):
        wo, wl = net.layout[f"W{i + 1}"]
        bo, bl = net.layout[f"b{i + 1}"]
        assert rel(g[wo:wo + wl], gw) < 3e-2, f"W{i + 1}"
        assert rel(g[bo:bo + bl], gb) < 3e-2, f"b{i + 1}"


def test_adam_step_matches_oracle():
    from oracle import corrector_np as co

    B, H = 2, 8
    net = _net(B, H)
    v, tgt = _data(B, H, 3)
    params = net.params_numpy()
    net.loss_and_grads(torch.from_numpy(v).cuda(), torch.from_numpy(tgt).cuda())
    g = net.g.cpu().numpy().astype(np.float64)
    grads = []
    for i in range(len(params)):
        wo, wl = net.layout[f"W{i + 1}"]
        bo, bl = net.layout[f"b{i + 1}"]
        grads.append((g[wo:wo + wl].reshape(params[i][0].shape), g[bo:bo + bl]))
    state = {"t": 0, "m": [[np.zeros_like(w), np.zeros_like(b)] for w, b in params],
             "v": [[np.zeros_like(w), np.zeros_like(b)] for w, b in params]}
    new = co.adam(params, grads, state, lr=1e-3)
    net.adam_step(lr=1e-3)
    got = net.params_numpy()
    for (wa, ba), (wb, bb) in zip(got, new):
        np.testing.assert_allclose(wa, wb, rtol=1e-5, atol=1e-7)
        np.testing.assert_allclose(ba, bb, rtol=1e-5, atol=1e-7)


def test_training_reduces_loss():
    """A fixed periodic smoothing is learnable: 200 Adam steps must cut the
    loss by 5x."""
    from exponax_gb300.learned import PeriodicConvCorrector

    B, H = 16, 16
    rng = np.random.default_rng(5)
    v = rng.standard_normal((B, H, 64)).astype(np.float32)
    tgt = v + 0.5 * (np.roll(v, 1, axis=2) + np.roll(v, -1, axis=1) - 2 * v)
    net = PeriodicConvCorrector(H, seed=2, max_batch=B)
    vt, tt = torch.from_numpy(v).cuda(), torch.from_numpy(tgt.astype(np.float32)).cuda()
    first = float(net.train_step(vt, tt, lr=3e-3))
    for _ in range(200):
        last = float(net.train_step(vt, tt, lr=3e-3))
    assert last < first / 5, (first, last)


def test_guard_trips_on_energetic_corrections():
    import exponax_gb300 as ex
    from exponax_gb300.learned import GuardedCorrectedStepper, PeriodicConvCorrector

    st = ex.stepper.KolmogorovFlowVorticity(2, 2 * np.pi, 64, 0.04)
    g = ex.ic.RandomAmplitudePhaseSeries(2, cutoff=5, max_one=True)
    u = torch.from_numpy(np.stack([g(64, key=s) for s in range(4)])).cuda()
    plain = ex.vmap(st)(u)
    quiet = PeriodicConvCorrector(64, seed=0, max_batch=4, out_scale=1e-6)
    gs = GuardedCorrectedStepper(st, quiet, kg=8, thresh=0.05)
    out = gs(u)
    assert int(gs.last_tripped.sum()) == 0
    assert torch.allclose(out, plain, atol=1e-3)
    loud = PeriodicConvCorrector(64, seed=0, max_batch=4, out_scale=1e3)
    gs = GuardedCorrectedStepper(st, loud, kg=8, thresh=0.05)
    out = gs(u)
    assert int(gs.last_tripped.sum()) == 4
    assert torch.equal(out, plain)


def test_trained_corrector_beats_the_plain_coarse_stepper():
    """The learned part's gain, end to end on the GPU at small scale: Kolmogorov flow (nu 1e-3, drag
    0.1, forcing k = 4) solved at 128^2 (dt 0.002, 3000-step spin-up) and downsampled to 64^2 every 8
    fine steps; 64 trajectories x 30 pairs train the corrector (20 epochs, the project's BF16 kernels
    and Adam); on 16 held-out seeds the guarded corrected 64^2 stepper (dt 0.016) has at most 0.85x
    the relative L2 error of the plain 64^2 stepper after 1, 10 and 30 coarse steps (measured about
    0.72x, 0.78x, 0.76x)."""
    import exponax_gb300 as ex
    from exponax_gb300 import learned as ke
    from exponax_gb300.learned import PeriodicConvCorrector

    kw = dict(n_fine=128, n_coarse_grid=64, dt=0.002, ratio=8, spinup=3000, n_coarse=30)
    train_data, _ = ke.fine_coarse_trajectories(list(range(1000, 1064)), **kw)
    eval_data, _ = ke.fine_coarse_trajectories(list(range(5000, 5016)), **kw)
    coarse = ex.stepper.KolmogorovFlowVorticity(2, 2 * np.pi, 64, 0.016, **ke.KW)
    net = PeriodicConvCorrector(H=64, seed=0, max_batch=128)
    hist = ke.train(net, coarse, train_data, epochs=20, batch=128)
    assert hist[-1] < 0.7 * hist[0]
    res = ke.evaluate(eval_data, coarse, net)
    plain, learned = res["plain"][0], res["learned"][0]
    for t in (1, 10, 30):
        assert learned[t] < 0.85 * plain[t], (t, learned[t], plain[t])


def _conv_ref(x, w, dy_dx_taps=True):
    """Periodic 3x3 conv in float64: out[b, y, x, co] = sum_tap sum_ci w[tap, co, ci] x[b, y + dy, x + dx, ci],
    tap = (dy + 1) * 3 + (dx + 1)."""
    out = 0.0
    for tap in range(9):
        dy, dx = tap // 3 - 1, tap % 3 - 1
        xs = np.roll(x, shift=(-dy, -dx), axis=(1, 2))
        out = out + np.einsum("byxc,oc->byxo", xs, w[tap])
    return out


def _bf16(a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(torch.bfloat16)


@pytest.mark.parametrize("B,H", [(1, 64), (16, 64), (3, 6)])
@pytest.mark.parametrize("mode", [0, 1])
def test_conv48_tensor_core_layer(B, H, mode):
    """The 48 -> 48 tcgen05 implicit-GEMM layer alone against a float64 periodic convolution of the same
    bf16 inputs and weights: forward (bias, tanh-form GELU) and backward-data (times its derivative at the
    layer below) within
    the bf16 rounding of the outputs (relative L2 <= 4e-3, measured against the float64 result); B = 16
    at 64 rows is 512 tiles, more than one per SM, so the two-stage pipeline runs."""
    from exponax_gb300 import _device
    from oracle import corrector_np as co
    from exponax_gb300.learned import PeriodicConvCorrector, _lib

    rng = np.random.default_rng(B * 100 + H + mode)
    x = _bf16(rng.standard_normal((B, H, 64, 48))).float().numpy().astype(np.float64)
    w = _bf16(rng.standard_normal((9, 48, 48)) / np.sqrt(9 * 48)).float().numpy().astype(np.float64)
    bias = (0.1 * rng.standard_normal(48)).astype(np.float32)
    aux = _bf16(rng.standard_normal((B, H, 64, 48))).float().numpy().astype(np.float64)
    xd = _bf16(x).cuda()
    wd = _bf16(w).cuda()
    bd = torch.from_numpy(bias).cuda()
    auxd = _bf16(aux).cuda()
    pre = torch.full((B, H, 64, 48), float("nan"), dtype=torch.bfloat16, device="cuda")
    post = torch.full_like(pre, float("nan"))
    lib = _lib()
    from exponax_gb300.learned import _p

    rc = lib.exgb_conv48(_device.stream(), _p(xd), B, H, _p(wd), _p(bd) if mode == 0 else None, mode,
                         _p(auxd) if mode == 1 else None, _p(pre), _p(post) if mode == 0 else None)
    assert rc == 0
    PeriodicConvCorrector.status()
    ref = _conv_ref(x, w)
    if mode == 0:
        ref = ref + bias.astype(np.float64)
        assert rel(pre.float().cpu().numpy(), ref) < 4e-3
        assert rel(post.float().cpu().numpy(), co.gelu(ref)) < 4e-3
    else:
        assert rel(pre.float().cpu().numpy(), ref * co.gelu_d(aux)) < 4e-3


@pytest.mark.parametrize("B,H", [(1, 64), (16, 64), (3, 13), (2, 2), (2, 1)])
def test_thin_layers(B, H):
    """The 1 -> 48 and 48 -> 1 layers alone against float64 periodic convolutions of the same inputs:
    1 -> 48 (FP32 input, bias, tanh-form GELU, bf16 outputs) within the bf16 rounding (relative L2 <=
    4e-3), 48 -> 1 (bf16 input, FP32 tap sums, out = base + scale (conv + b)) within 1e-5.  H = 13 leaves
    a partial block of output rows, H = 1 and 2 make the periodic halo rows repeat."""
    from exponax_gb300 import _device
    from oracle import corrector_np as co
    from exponax_gb300.learned import PeriodicConvCorrector, _lib, _p

    rng = np.random.default_rng(7 * B + H)
    lib = _lib()
    # 1 -> 48
    x = rng.standard_normal((B, H, 64)).astype(np.float32)
    w1 = (rng.standard_normal((9, 48)) / 3.0).astype(np.float32)
    b1 = (0.1 * rng.standard_normal(48)).astype(np.float32)
    pre = torch.full((B, H, 64, 48), float("nan"), dtype=torch.bfloat16, device="cuda")
    post = torch.full_like(pre, float("nan"))
    xd, w1d, b1d = (torch.from_numpy(a).cuda() for a in (x, w1, b1))
    assert lib.exgb_conv_in1(_device.stream(), _p(xd), B, H, _p(w1d), _p(b1d), _p(pre), _p(post)) == 0
    PeriodicConvCorrector.status()
    ref = _conv_ref(x.astype(np.float64)[..., None], w1.astype(np.float64)[:, :, None]) + b1
    assert rel(pre.float().cpu().numpy(), ref) < 4e-3
    assert rel(post.float().cpu().numpy(), co.gelu(ref)) < 4e-3
    # 48 -> 1
    h = _bf16(rng.standard_normal((B, H, 64, 48))).float().numpy().astype(np.float64)
    w6 = (rng.standard_normal((9, 48)) / np.sqrt(9 * 48)).astype(np.float32)
    b6 = np.array([0.3], np.float32)
    base = rng.standard_normal((B, H, 64)).astype(np.float32)
    out = torch.full((B, H, 64), float("nan"), dtype=torch.float32, device="cuda")
    hd = _bf16(h).cuda()
    w6d, b6d, based = (torch.from_numpy(a).cuda() for a in (w6, b6, base))
    for with_base in (True, False):
        assert lib.exgb_conv_out1(_device.stream(), _p(hd), B, H, _p(w6d), _p(b6d), _p(based) if with_base else None,
                                  0.7, _p(out)) == 0
        PeriodicConvCorrector.status()
        ref = 0.7 * (_conv_ref(h, w6.astype(np.float64)[:, None, :])[..., 0] + b6[0])
        if with_base:
            ref = ref + base
        assert rel(out.cpu().numpy(), ref) < 1e-5


@pytest.mark.parametrize("B,H", [(2, 64), (3, 13)])
def test_backward_kernels_per_layer(B, H):
    """The backward kernels alone against float64 on the same bf16 / FP32 inputs, at the bar of their
    FP32 accumulation: the weight and bias gradients of all three layer kinds (per-chunk FP32 partial
    sums over 512 pixels, then an FP32 reduction) within 2e-6 relative L2, and the 48 -> 1 layer's
    backward-data (FP32 sums, bf16 output) within the bf16 rounding (4e-3)."""
    from exponax_gb300 import _device
    from oracle import corrector_np as co
    from exponax_gb300.learned import PeriodicConvCorrector, _lib, _p

    rng = np.random.default_rng(11 * B + H)
    lib = _lib()
    s = _device.stream()
    n = B * H * 64
    nchunk = (n + 511) // 512
    part = torch.empty(nchunk * 9 * 48 * 48, dtype=torch.float32, device="cuda")
    part_b = torch.empty(nchunk * 48, dtype=torch.float32, device="cuda")
    dpre = _bf16(rng.standard_normal((B, H, 64, 48))).float().numpy().astype(np.float64)
    x48 = _bf16(rng.standard_normal((B, H, 64, 48))).float().numpy().astype(np.float64)
    x1 = rng.standard_normal((B, H, 64)).astype(np.float32)
    dout = rng.standard_normal((B, H, 64)).astype(np.float32)
    dw = torch.full((9 * 48 * 48,), float("nan"), device="cuda")
    db = torch.full((48,), float("nan"), device="cuda")
    dpre_d, x48_d = _bf16(dpre).cuda(), _bf16(x48).cuda()
    x1_d, dout_d = torch.from_numpy(x1).cuda(), torch.from_numpy(dout).cuda()
    # 48 -> 48
    assert lib.exgb_wgrad(s, 0, _p(dpre_d), _p(x48_d), B, H, _p(part), _p(part_b), _p(dw), _p(db)) == 0
    assert rel(dw.cpu().numpy(), co.conv_wgrad(dpre, x48)) < 2e-6
    assert rel(db.cpu().numpy(), dpre.sum(axis=(0, 1, 2))) < 2e-6
    # 1 -> 48: the input field is the single channel
    assert lib.exgb_wgrad(s, 1, _p(dpre_d), _p(x1_d), B, H, _p(part), _p(part_b), _p(dw), _p(db)) == 0
    ref = co.conv_wgrad(dpre, x1.astype(np.float64)[..., None])[:, :, 0]  # (9, 48) = W[tap][co]
    assert rel(dw[:9 * 48].cpu().numpy(), ref) < 2e-6
    assert rel(db.cpu().numpy(), dpre.sum(axis=(0, 1, 2))) < 2e-6
    # 48 -> 1: the output gradient is the single channel
    assert lib.exgb_wgrad(s, 2, _p(dout_d), _p(x48_d), B, H, _p(part), _p(part_b), _p(dw), _p(db)) == 0
    ref = co.conv_wgrad(dout.astype(np.float64)[..., None], x48)[:, 0, :]  # (9, 48) = W[tap][ci]
    assert rel(dw[:9 * 48].cpu().numpy(), ref) < 2e-6
    assert abs(float(db[0]) - float(dout.astype(np.float64).sum())) <= 2e-6 * float(np.abs(dout).sum())
    # 48 -> 1 backward-data, times gelu' of the pre-activations
    w6 = (rng.standard_normal((9, 48)) / np.sqrt(9 * 48)).astype(np.float32)
    pre = _bf16(rng.standard_normal((B, H, 64, 48))).float().numpy().astype(np.float64)
    out = torch.full((B, H, 64, 48), float("nan"), dtype=torch.bfloat16, device="cuda")
    assert lib.exgb_conv_out1_bwd_data(s, _p(dout_d), B, H, _p(torch.from_numpy(w6).cuda()), _p(_bf16(pre).cuda()),
                                       _p(out)) == 0
    ref = co.conv_T(dout.astype(np.float64)[..., None], w6.astype(np.float64)[:, None, :]) * co.gelu_d(pre)
    assert rel(out.float().cpu().numpy(), ref) < 4e-3
    PeriodicConvCorrector.status()
