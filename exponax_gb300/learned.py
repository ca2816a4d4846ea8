"""Learned coarse-step correction for 2D Kolmogorov flow.

A small periodic convolutional residual network corrects every coarse
(64^2, dt = 0.04) ETDRK2 step:  u_{n+1} = v + out_scale * NN(in_scale * v),
v = coarse_step(u_n).  Network: 3x3 periodic convolutions 1 -> 48 -> 48 x 4
-> 1 with GELU in its tanh form (six layers, ~84 k parameters), BF16 weights and
activations, FP32 accumulation; the 48 -> 48 layers (forward and
backward-data) run on the tcgen05 tensor cores (exgb_conv48).  Training
(Adam, lr 1e-3, mean squared error against the downsampled fine solution)
and inference use only the kernels of libexgb.so.  A spectral-energy guard replaces a corrected state by the plain
coarse state when the correction puts too much energy above |k| > kg or is
not finite.

No counterpart in the reference (its closest precedent is the 1D CNN
emulator notebook); the plain method (exponax_gb300.stepper) generates the
training data and measures the error.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _device, ic, stepper
from ._lib import check, load
from ._utils import rollout, vmap
from .interpolation import map_between_resolutions_batched
from .spectral import fft, ifft

C = 48
NMID = 4
TAPS = 9


_V, _I, _I64, _F = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_float
# argument types of the corrector entry points (include/exgb_corrector.h)
CORRECTOR_SIGNATURES = {
    "exgb_conv48": [_V, _V, _I, _I, _V, _V, _I, _V, _V, _V],
    "exgb_conv_in1": [_V, _V, _I, _I, _V, _V, _V, _V],
    "exgb_conv_out1": [_V, _V, _I, _I, _V, _V, _V, _F, _V],
    "exgb_conv_out1_bwd_data": [_V, _V, _I, _I, _V, _V, _V],
    "exgb_wgrad": [_V, _I, _V, _V, _I, _I, _V, _V, _V, _V],
    "exgb_adam": [_V, _V, _V, _V, _V, _I64, _F, _F, _F, _F, _I64, _V, _V, _I],
    "exgb_cast_weights": [_V, _V, _I64, _V, _V, _I],
    "exgb_mse": [_V, _V, _V, _I64, _F, _V, _V, _I],
    "exgb_guard": [_V, _V, _V, _I, _I, _I, _F, _V, _V, _V],
    "exgb_conv_status": [],
}


def _lib():
    lib = load()
    if not hasattr(lib, "_conv_sigs"):
        for name, args in CORRECTOR_SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        lib._conv_sigs = True
    return lib


def _p(t):
    return ctypes.c_void_p(int(t.data_ptr()))


class PeriodicConvCorrector:
    """Parameters live in one FP32 device buffer (plus Adam moments and bf16
    working copies); activations for up to `max_batch` samples are kept for
    the backward pass."""

    def __init__(self, H: int = 64, *, seed: int = 0, max_batch: int = 256, in_scale: float = 1.0,
                 out_scale: float = 1.0):
        torch = _device.torch()
        _device.require_cuda()
        if H % 2:
            raise ValueError("grid height must be even")
        self.H, self.Wd = H, 64
        self.in_scale, self.out_scale = float(in_scale), float(out_scale)
        self.max_batch = int(max_batch)
        # parameter layout: W1 (9,48), b1 (48), [Wm (9,48,48), bm (48)] x 4, W6 (9,48), b6 (1)
        sizes = [("W1", TAPS * C), ("b1", C)]
        for i in range(NMID):
            sizes += [(f"W{i + 2}", TAPS * C * C), (f"b{i + 2}", C)]
        sizes += [("W6", TAPS * C), ("b6", 1)]
        self.layout = {}
        off = 0
        for name, n in sizes:
            self.layout[name] = (off, n)
            off += n
        self.num_params = off
        rng = np.random.default_rng(seed)
        init = np.zeros(off, np.float32)
        for name, (o, n) in self.layout.items():
            if name.startswith("W"):
                fan_in = TAPS * (1 if name == "W1" else C)
                gain = np.sqrt(2.0) if name != "W6" else 0.1  # small last layer: start near the plain method
                init[o:o + n] = rng.standard_normal(n) * gain / np.sqrt(fan_in)
        dev = "cuda"
        self.w = torch.from_numpy(init).to(dev)
        self.g = torch.zeros_like(self.w)
        self.m = torch.zeros_like(self.w)
        self.v = torch.zeros_like(self.w)
        self.t = 0
        self.w16 = [torch.empty(TAPS * C * C, dtype=torch.bfloat16, device=dev) for _ in range(NMID)]
        self.wflip = [torch.empty(TAPS * C * C, dtype=torch.bfloat16, device=dev) for _ in range(NMID)]
        self._alloc(self.max_batch)
        self._cast()

    # ------------------------------------------------------------------ buffers
    def _alloc(self, B):
        torch = _device.torch()
        px = B * self.H * self.Wd
        bf = dict(dtype=torch.bfloat16, device="cuda")
        self.pre = [torch.empty(px * C, **bf) for _ in range(NMID + 1)]
        self.h = [torch.empty(px * C, **bf) for _ in range(NMID + 1)]
        self.dpre = [torch.empty(px * C, **bf) for _ in range(2)]
        self.x0 = torch.empty(px, dtype=torch.float32, device="cuda")
        self.out = torch.empty(px, dtype=torch.float32, device="cuda")
        self.dout = torch.empty(px, dtype=torch.float32, device="cuda")
        nchunk = (px + 511) // 512
        self.part = torch.empty(nchunk * TAPS * C * C, dtype=torch.float32, device="cuda")
        self.part_b = torch.empty(nchunk * C, dtype=torch.float32, device="cuda")
        self.loss_part = torch.empty(1024, dtype=torch.float32, device="cuda")

    def _view(self, t, name):
        o, n = self.layout[name]
        return t[o:o + n]

    def _cast(self):
        lib = _lib()
        s = _device.stream()
        for i in range(NMID):
            wv = self._view(self.w, f"W{i + 2}")
            check(lib.exgb_cast_weights(s, _p(wv), wv.numel(), _p(self.w16[i]), _p(self.wflip[i]), 1), "cast")

    def set_params(self, flat: np.ndarray):
        torch = _device.torch()
        self.w.copy_(torch.from_numpy(np.asarray(flat, np.float32)))
        self._cast()

    def params_numpy(self):
        """Parameters in the oracle's layout: list of (w, b) arrays."""
        w = self.w.cpu().numpy().astype(np.float64)
        out = []
        for i in range(NMID + 2):
            wn, bn = f"W{i + 1}", f"b{i + 1}"
            wo, wl = self.layout[wn]
            bo, bl = self.layout[bn]
            if i == 0:
                ww = w[wo:wo + wl].reshape(TAPS, C, 1)
            elif i == NMID + 1:
                ww = w[wo:wo + wl].reshape(TAPS, 1, C)
            else:
                ww = w[wo:wo + wl].reshape(TAPS, C, C)
            out.append((ww, w[bo:bo + bl]))
        return out

    # ------------------------------------------------------------------ forward / backward
    def forward(self, v, out=None, keep=False):
        """v: (B, H, 64) float32 CUDA tensor -> corrected state (B, H, 64).  keep: also store the
        pre-activations that a following backward pass needs (inference skips those writes)."""
        torch = _device.torch()
        lib = _lib()
        s = _device.stream()
        v = v.contiguous()
        B = v.shape[0]
        if B > self.max_batch:
            self.max_batch = B
            self._alloc(B)
        H = self.H
        torch.mul(v.reshape(-1), self.in_scale, out=self.x0[:B * H * 64])
        check(lib.exgb_conv_in1(s, _p(self.x0), B, H, _p(self._view(self.w, "W1")), _p(self._view(self.w, "b1")),
                                _p(self.pre[0]) if keep else None, _p(self.h[0])), "conv_in1")
        for i in range(NMID):
            check(lib.exgb_conv48(s, _p(self.h[i]), B, H, _p(self.w16[i]), _p(self._view(self.w, f"b{i + 2}")), 0,
                                  None, _p(self.pre[i + 1]) if keep else None, _p(self.h[i + 1])), "conv48")
        if out is None:
            out = torch.empty_like(v)
        check(lib.exgb_conv_out1(s, _p(self.h[NMID]), B, H, _p(self._view(self.w, "W6")),
                                 _p(self._view(self.w, "b6")), _p(v), self.out_scale, _p(out)), "conv_out1")
        self._B = B
        return out

    __call__ = forward

    def loss_and_grads(self, v, target):
        """Forward, MSE loss against `target` and all parameter gradients (in self.g)."""
        torch = _device.torch()
        lib = _lib()
        s = _device.stream()
        pred = self.forward(v, keep=True)
        B, H = self._B, self.H
        n = B * H * 64
        nb = 256
        check(lib.exgb_mse(s, _p(pred), _p(target.contiguous()), n, self.out_scale, _p(self.dout),
                           _p(self.loss_part), nb), "mse")
        # last layer (48 -> 1)
        check(lib.exgb_wgrad(s, 2, _p(self.dout), _p(self.h[NMID]), B, H, _p(self.part), _p(self.part_b),
                             _p(self._view(self.g, "W6")), _p(self._view(self.g, "b6"))), "wgrad6")
        check(lib.exgb_conv_out1_bwd_data(s, _p(self.dout), B, H, _p(self._view(self.w, "W6")),
                                          _p(self.pre[NMID]), _p(self.dpre[0])), "bwd6")
        cur = 0
        for i in range(NMID - 1, -1, -1):
            # layer i+2: input h[i], output pre[i+1]; dpre[cur] = dL/dpre[i+1]
            check(lib.exgb_wgrad(s, 0, _p(self.dpre[cur]), _p(self.h[i]), B, H, _p(self.part), _p(self.part_b),
                                 _p(self._view(self.g, f"W{i + 2}")), _p(self._view(self.g, f"b{i + 2}"))),
                  "wgrad48")
            check(lib.exgb_conv48(s, _p(self.dpre[cur]), B, H, _p(self.wflip[i]), None, 1, _p(self.pre[i]),
                                  _p(self.dpre[1 - cur]), None), "conv48 bwd")
            cur = 1 - cur
        check(lib.exgb_wgrad(s, 1, _p(self.dpre[cur]), _p(self.x0), B, H, _p(self.part), _p(self.part_b),
                             _p(self._view(self.g, "W1")), _p(self._view(self.g, "b1"))), "wgrad1")
        loss = self.loss_part[:nb].sum() / n
        return loss, pred

    @staticmethod
    def status():
        """Synchronise and raise if a bounded device wait of the tensor-core conv kernel gave up
        since the last check (the results of that launch are then invalid)."""
        check(_lib().exgb_conv_status(), "conv status")

    def adam_step(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        lib = _lib()
        s = _device.stream()
        self.t += 1
        check(lib.exgb_adam(s, _p(self.w), _p(self.m), _p(self.v), _p(self.g), self.num_params, lr, b1, b2, eps,
                            self.t, None, None, 0), "adam")
        self._cast()

    def train_step(self, v, target, lr=1e-3):
        loss, _ = self.loss_and_grads(v, target)
        self.adam_step(lr)
        return loss

    def save(self, path):
        np.savez(path, w=self.w.cpu().numpy(), m=self.m.cpu().numpy(), v=self.v.cpu().numpy(), t=self.t,
                 in_scale=self.in_scale, out_scale=self.out_scale)

    def load(self, path):
        torch = _device.torch()
        d = np.load(path)
        self.w.copy_(torch.from_numpy(d["w"]))
        self.m.copy_(torch.from_numpy(d["m"]))
        self.v.copy_(torch.from_numpy(d["v"]))
        self.t = int(d["t"])
        self.in_scale, self.out_scale = float(d["in_scale"]), float(d["out_scale"])
        self._cast()


class GuardedCorrectedStepper:
    """Coarse ETDRK2 step followed by the corrector, with the spectral-energy
    guard: a sample whose correction carries more than `thresh` of the plain
    state's energy above |k| > kg (or is not finite) keeps the plain step."""

    def __init__(self, coarse_stepper, corrector: PeriodicConvCorrector, *, kg: int = 16, thresh: float = 0.05):
        self.coarse = coarse_stepper
        self.net = corrector
        self.kg, self.thresh = int(kg), float(thresh)
        self.trips = 0

    def step(self, u):
        """u: (B, 1, H, 64) -> (B, 1, H, 64)."""
        torch = _device.torch()
        lib = _lib()
        plain = vmap(self.coarse)(u)
        B, _, H, Wd = plain.shape
        corrected = self.net(plain.reshape(B, H, Wd)).reshape(B, 1, H, Wd)
        corr_hat = fft((corrected - plain).reshape(B, H, Wd), num_spatial_dims=2)
        plain_hat = fft(plain.reshape(B, H, Wd), num_spatial_dims=2)
        tripped = torch.empty(B, dtype=torch.int32, device="cuda")
        check(lib.exgb_guard(_device.stream(), _p(corr_hat), _p(plain_hat), B, H, self.kg, self.thresh, _p(plain),
                             _p(corrected), _p(tripped)), "guard")
        self.last_tripped = tripped
        return corrected

    __call__ = step


# ---- training data, training and evaluation of the corrector (2D Kolmogorov flow) ----

KW = dict(diffusivity=1e-3, drag=-0.1, injection_mode=4, injection_scale=1.0)


def _events():
    torch = _device.torch()
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def fine_coarse_trajectories(seeds, *, n_fine=512, n_coarse_grid=64, dt=0.001, ratio=8, spinup=1000, n_coarse=200,
                             batch=256):
    """Downsampled fine trajectories (len(seeds), n_coarse + 1, n_coarse_grid, n_coarse_grid) on the GPU, and
    the GPU milliseconds of the post-spin-up fine steps."""
    torch = _device.torch()
    fine = stepper.KolmogorovFlowVorticity(2, 2 * np.pi, n_fine, dt, **KW)
    h = fine.plan.handle
    lib = load()
    g = ic.RandomAmplitudePhaseSeries(2, cutoff=5, max_one=True)
    out = torch.empty((len(seeds), n_coarse + 1, n_coarse_grid, n_coarse_grid), dtype=torch.float32, device="cuda")
    fine_ms = 0.0
    for b0 in range(0, len(seeds), batch):
        sb = seeds[b0:b0 + batch]
        B = len(sb)
        u0 = torch.from_numpy(np.stack([g(n_fine, key=int(s)) for s in sb])).cuda()
        uh = fft(u0, num_spatial_dims=2)
        tmp = torch.empty_like(uh)
        check(lib.exgb_repeat_fourier(h, _device.stream(), uh.data_ptr(), tmp.data_ptr(), B, spinup), "spin-up")
        uh, tmp = tmp, uh
        for t in range(n_coarse + 1):
            if t > 0:
                e0, e1 = _events()
                e0.record()
                check(lib.exgb_repeat_fourier(h, _device.stream(), uh.data_ptr(), tmp.data_ptr(), B, ratio), "fine")
                e1.record()
                uh, tmp = tmp, uh
                torch.cuda.synchronize()
                fine_ms += e0.elapsed_time(e1)
            phys = ifft(uh, num_spatial_dims=2, num_points=n_fine)  # (B, 1, N, N)
            out[b0:b0 + B, t] = map_between_resolutions_batched(phys, n_coarse_grid)[:, 0]
    return out, fine_ms


def train(net, coarse, data, *, epochs=4, batch=256, lr=1e-3, seed=0, log=None):
    """data: (T, n_coarse + 1, H, W) coarse snapshots."""
    torch = _device.torch()
    T, S, H, W = data.shape
    x = data[:, :-1].reshape(-1, 1, H, W)
    y = data[:, 1:].reshape(-1, H, W)
    v = torch.empty_like(x)
    for i in range(0, x.shape[0], 4096):
        v[i:i + 4096] = vmap(coarse)(x[i:i + 4096])
    v = v.reshape(-1, H, W)
    net.in_scale = float(1.0 / v.std())
    net.out_scale = float((y - v).std())
    rng = np.random.default_rng(seed)
    n = v.shape[0]
    hist = []
    for ep in range(epochs):
        perm = torch.from_numpy(rng.permutation(n)).cuda()
        tot, cnt = 0.0, 0
        for i in range(0, n - batch + 1, batch):
            idx = perm[i:i + batch]
            loss = net.train_step(v[idx], y[idx], lr=lr)
            if (i // batch) % 50 == 0:
                tot += float(loss)
                cnt += 1
        hist.append(tot / max(cnt, 1))
        if log:
            log(f"epoch {ep}: mean loss {hist[-1]:.3e} (normalised by out_scale^2: {hist[-1] / net.out_scale ** 2:.3e})")
    return hist


def evaluate(ref, coarse, net, *, kg=16, thresh=0.05):
    """ref: (B, S, H, W) downsampled fine trajectories.  Returns metrics and GPU ms."""
    torch = _device.torch()
    B, S, H, W = ref.shape
    u0 = ref[:, 0:1].contiguous()  # (B, 1, H, W)
    roll = vmap(rollout(coarse, S - 1, include_init=True))
    e0, e1 = _events()
    e0.record()
    plain = roll(u0)[:, :, 0]  # (B, S, H, W)
    e1.record()
    torch.cuda.synchronize()
    plain_ms = e0.elapsed_time(e1)
    gs = GuardedCorrectedStepper(coarse, net, kg=kg, thresh=thresh)
    learned = torch.empty_like(ref)
    learned[:, 0] = ref[:, 0]
    u = u0
    trips = 0
    e0, e1 = _events()
    e0.record()
    for t in range(1, S):
        u = gs(u)
        learned[:, t] = u[:, 0]
        trips += gs.last_tripped.sum()
    e1.record()
    torch.cuda.synchronize()
    learned_ms = e0.elapsed_time(e1)

    def metrics(pred):
        d = (pred - ref).reshape(B, S, -1)
        r = ref.reshape(B, S, -1)
        rel = (d.norm(dim=2) / r.norm(dim=2)).mean(dim=0)  # per step, mean over seeds
        p = pred.reshape(B, S, -1)
        corr = ((p * r).sum(dim=2) / (p.norm(dim=2) * r.norm(dim=2))).mean(dim=0)
        below = (corr < 0.8).nonzero()
        ct = int(below[0, 0]) if below.numel() else S - 1
        return rel.cpu().numpy(), corr.cpu().numpy(), ct

    rp, cp, ctp = metrics(plain)
    rl, cl, ctl = metrics(learned)
    return {"plain": (rp, cp, ctp), "learned": (rl, cl, ctl), "plain_ms": plain_ms, "learned_ms": learned_ms,
            "guard_trips": int(trips), "guard_checks": int(B * (S - 1))}
