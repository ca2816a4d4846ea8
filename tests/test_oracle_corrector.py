"""The corrector oracle's gradients agree with central finite differences
(CPU only; pins oracle/corrector_np.py before the GPU kernels are checked
against it)."""

import numpy as np

from oracle import corrector_np as co


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    C = 4
    params = [(rng.standard_normal((9, C, 1)) * 0.3, rng.standard_normal(C) * 0.1),
              (rng.standard_normal((9, C, C)) * 0.3, rng.standard_normal(C) * 0.1),
              (rng.standard_normal((9, 1, C)) * 0.3, rng.standard_normal(1) * 0.1)]
    v = rng.standard_normal((2, 5, 6))
    t = rng.standard_normal((2, 5, 6))
    _, _, grads = co.loss_and_grads(params, v, t, 0.7, 0.5)
    eps = 1e-6
    for li in range(3):
        for j in range(2):
            p, g = params[li][j], grads[li][j]
            for _ in range(3):
                idx = tuple(rng.integers(0, s) for s in p.shape)
                old = p[idx]
                p[idx] = old + eps
                lp = co.loss_and_grads(params, v, t, 0.7, 0.5)[0]
                p[idx] = old - eps
                lm = co.loss_and_grads(params, v, t, 0.7, 0.5)[0]
                p[idx] = old
                assert abs((lp - lm) / (2 * eps) - g[idx]) < 1e-6 * max(1.0, abs(g[idx]))


def test_conv_adjoint_identity():
    """<conv(x), g> = <x, conv_T(g)> (zero bias)."""
    rng = np.random.default_rng(1)
    x = rng.standard_normal((2, 6, 7, 3))
    g = rng.standard_normal((2, 6, 7, 5))
    w = rng.standard_normal((9, 5, 3))
    lhs = np.sum(co.conv(x, w, np.zeros(5)) * g)
    rhs = np.sum(x * co.conv_T(g, w))
    assert abs(lhs - rhs) < 1e-9 * abs(lhs)
