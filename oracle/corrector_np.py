"""NumPy statement of the learned coarse-step corrector (test infrastructure).

The corrector has no counterpart in the reference; this module is the CPU
oracle its CUDA forward / backward kernels are checked against.  Network:
x0 = in_scale * v; h1 = gelu(conv(x0; W1, b1)) (1 -> C); h_i = gelu(conv(h_{i-1};
W_i, b_i)) (C -> C, i = 2..L-1); out = conv(h_{L-1}; W_L, b_L) (C -> 1);
pred = v + out_scale * out.  3x3 periodic convolutions, GELU in its tanh
form (Hendrycks & Gimpel 2016: x / 2 (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3)))),
weights laid out [tap][co][ci] with tap = (dy + 1) * 3 + (dx + 1) and
input pixel (y + dy, x + dx) (wrapped).  Loss = mean (pred - target)^2.
"""

import numpy as np

_A = np.sqrt(2.0 / np.pi)
_B = 0.044715


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(_A * (x + _B * x ** 3)))


def gelu_d(x):
    t = np.tanh(_A * (x + _B * x ** 3))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * _A * (1.0 + 3.0 * _B * x * x)


def _shift(x, dy, dx):
    """x[..., y + dy, x + dx, :] for NHWC x (periodic)."""
    return np.roll(x, shift=(-dy, -dx), axis=(1, 2))


def conv(x, w, b):
    """x (B, H, W, Cin), w (9, Cout, Cin), b (Cout,) -> (B, H, W, Cout)."""
    out = np.zeros(x.shape[:3] + (w.shape[1],), dtype=np.float64)
    for tap in range(9):
        dy, dx = tap // 3 - 1, tap % 3 - 1
        out += _shift(x, dy, dx) @ w[tap].T
    return out + b


def conv_T(g, w):
    """Adjoint of conv w.r.t. its input: g (B, H, W, Cout) -> (B, H, W, Cin)."""
    out = np.zeros(g.shape[:3] + (w.shape[2],), dtype=np.float64)
    for tap in range(9):
        dy, dx = tap // 3 - 1, tap % 3 - 1
        out += _shift(g @ w[tap], -dy, -dx)
    return out


def conv_wgrad(g, x):
    """dL/dw for out = conv(x, w): g (B,H,W,Cout), x (B,H,W,Cin) -> (9, Cout, Cin)."""
    gw = np.zeros((9, g.shape[-1], x.shape[-1]))
    gf = g.reshape(-1, g.shape[-1])
    for tap in range(9):
        dy, dx = tap // 3 - 1, tap % 3 - 1
        gw[tap] = gf.T @ _shift(x, dy, dx).reshape(-1, x.shape[-1])
    return gw


def forward(params, v, in_scale=1.0, out_scale=1.0):
    """params: list of (w, b); w of the first layer (9, C, 1), last (9, 1, C).
    Returns pred and the cache for backward."""
    x = (in_scale * v)[..., None].astype(np.float64)
    cache = {"x0": x, "pre": [], "h": [x]}
    h = x
    for i, (w, b) in enumerate(params[:-1]):
        pre = conv(h, w, b)
        cache["pre"].append(pre)
        h = gelu(pre)
        cache["h"].append(h)
    w, b = params[-1]
    out = conv(h, w, b)[..., 0]
    pred = v + out_scale * out
    return pred, cache


def loss_and_grads(params, v, target, in_scale=1.0, out_scale=1.0):
    pred, cache = forward(params, v, in_scale, out_scale)
    n = pred.size
    loss = float(np.mean((pred - target) ** 2))
    dout = (2.0 * (pred - target) / n * out_scale)[..., None]
    grads = [None] * len(params)
    w, b = params[-1]
    h = cache["h"][-1]
    grads[-1] = (conv_wgrad(dout, h), dout.sum(axis=(0, 1, 2)))
    dh = conv_T(dout, w)
    for i in range(len(params) - 2, -1, -1):
        dpre = dh * gelu_d(cache["pre"][i])
        wi, bi = params[i]
        grads[i] = (conv_wgrad(dpre, cache["h"][i]), dpre.sum(axis=(0, 1, 2)))
        if i > 0:
            dh = conv_T(dpre, wi)
    return loss, pred, grads


def adam(params, grads, state, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (bias-corrected), state = dict(t, m, v) lists."""
    state["t"] += 1
    t = state["t"]
    out = []
    for k, ((w, b), (gw, gb)) in enumerate(zip(params, grads)):
        new = []
        for j, (p, g) in enumerate(((w, gw), (b, gb))):
            m = state["m"][k][j] = b1 * state["m"][k][j] + (1 - b1) * g
            v = state["v"][k][j] = b2 * state["v"][k][j] + (1 - b2) * g * g
            new.append(p - lr * (m / (1 - b1**t)) / (np.sqrt(v / (1 - b2**t)) + eps))
        out.append(tuple(new))
    return out
