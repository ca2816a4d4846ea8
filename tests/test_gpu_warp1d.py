"""The 1D latency kernel's one-warp transforms (N = 64, 128, 200, 256; one CTA per work item when the
items do not outnumber the SMs) against the NumPy oracle: every ETDRK order, a rollout, a uniform-N
work queue whose items hold several instances (one warp per instance), and a mixed queue that keeps
the block transforms.  Tolerances: 1e-5 relative L2 for one step, 1e-4 over 20 steps."""

import numpy as np
import pytest

import exponax_gb300 as ex
from oracle import exponax_np as o

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

WARP_SIZES = [64, 128, 200, 256]


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def cu(x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def host(t):
    return t.cpu().numpy()


def _ic(N, key):
    return ex.ic.RandomSineWaves1d(1, cutoff=5)(N, key=key)


@pytest.mark.parametrize("N", WARP_SIZES)
@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_single_step_every_order(N, order):
    """KS-conservative (convection) and KS (gradient norm) steps, batch 3: one item per SM."""
    for name in ("KuramotoSivashinskyConservative", "KuramotoSivashinsky"):
        sm = getattr(ex.stepper, name)(1, 60.0, N, 0.05, order=order)
        so = getattr(o, name)(1, 60.0, N, 0.05, order=order)
        u = np.stack([_ic(N, k) for k in range(3)])
        got = host(ex.vmap(sm)(cu(u)))
        for b in range(3):
            assert rel(got[b], so(u[b])) < 1e-5, (name, b)


@pytest.mark.parametrize("N", WARP_SIZES)
def test_rollout_20_steps(N):
    """Burgers (non-chaotic) and KdV, 20-step rollouts of 4 samples: within 1e-4."""
    cases = [
        (ex.stepper.Burgers(1, 1.0, N, 1e-3, diffusivity=0.01), o.Burgers(1, 1.0, N, 1e-3, diffusivity=0.01)),
        (ex.stepper.KortewegDeVries(1, 20.0, N, 0.005), o.KortewegDeVries(1, 20.0, N, 0.005)),
    ]
    for sm, so in cases:
        u = np.stack([_ic(N, 10 + k) for k in range(4)])
        got = host(ex.vmap(ex.rollout(sm, 20, include_init=True))(cu(u)))
        for b in range(4):
            ref = o.rollout(so, 20, include_init=True)(u[b])
            assert rel(got[b, 1:], ref[1:]) < 1e-4, (type(sm).__name__, b)


def _queue(specs, order, n):
    from exponax_gb300 import _device, _lib

    u0s, trajs, items = [], [], []
    for i, s in enumerate(order):
        sm, _ = specs[s]
        u0 = cu(_ic(sm.num_points, i))
        tr = torch.empty((n + 1, 1, sm.num_points), dtype=torch.float32, device="cuda")
        u0s.append(u0)
        trajs.append(tr)
        items.append(_lib.WorkItem(sm.plan.handle.value, u0.data_ptr(), tr.data_ptr()))
    arr = (_lib.WorkItem * len(items))(*items)
    _lib.check(_lib.load().exgb_queue_rollout(arr, len(items), n, 1, _device.stream()))
    torch.cuda.synchronize()
    for i, s in enumerate(order):
        ref = o.rollout(specs[s][1], n, include_init=True)(host(u0s[i]))
        assert rel(host(trajs[i])[1:], ref[1:]) < 1e-4, (i, s)


def test_uniform_queue_items_with_several_instances():
    """40 consecutive N = 128 instances of one plan: work items of up to 16 instances, fewer items
    than SMs, so the latency kernel's warps each take one instance of an item."""
    from exponax_gb300 import _device, _lib

    sm = ex.stepper.Burgers(1, 1.0, 128, 1e-3, diffusivity=0.01)
    so = o.Burgers(1, 1.0, 128, 1e-3, diffusivity=0.01)
    B, n, N = 40, 20, 128
    u0 = np.stack([_ic(N, k) for k in range(B)])  # (B, 1, N), contiguous per instance
    u0d = cu(u0)
    tr = torch.empty((B, n + 1, 1, N), dtype=torch.float32, device="cuda")
    items = [_lib.WorkItem(sm.plan.handle.value, u0d[b].data_ptr(), tr[b].data_ptr()) for b in range(B)]
    arr = (_lib.WorkItem * B)(*items)
    _lib.check(_lib.load().exgb_queue_rollout(arr, B, n, 1, _device.stream()))
    torch.cuda.synchronize()
    got = host(tr)
    for b in range(B):
        ref = o.rollout(so, n, include_init=True)(u0[b])
        assert rel(got[b, 1:], ref[1:]) < 1e-4, b


def test_mixed_queue_keeps_block_transforms():
    """Items of N = 200 and N = 256 in one queue (block transforms) next to the same PDEs alone."""
    specs = [
        (ex.stepper.KuramotoSivashinskyConservative(1, 100.0, 200, 0.1),
         o.KuramotoSivashinskyConservative(1, 100.0, 200, 0.1)),
        (ex.stepper.Burgers(1, 1.0, 256, 1e-3, diffusivity=0.01), o.Burgers(1, 1.0, 256, 1e-3, diffusivity=0.01)),
    ]
    _queue(specs, [0, 1, 0, 1, 1], 20)
    _queue(specs, [0, 0, 0], 20)
