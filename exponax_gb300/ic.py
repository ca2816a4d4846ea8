"""Initial-condition generators for the benchmark configurations.

The reference draws its random fields with jax.random (threefry); those
streams are not reproduced.  These generators follow the configuration
wording with NumPy's seeded PCG64: per seed s, ``np.random.default_rng(s)``.
Parity tests feed identical arrays to the GPU path and the oracle, so the
generator choice does not affect parity.
"""

from __future__ import annotations

import numpy as np


def _device_series(num_spatial_dims, num_points, keys, draw, zero_mean, max_one):
    """Batch of random Fourier-series fields built on the device: the per-key
    coefficients (`draw(key) -> (flat mode indices, complex64 values)`, same
    positions for every key) are scattered into zeroed rfftn spectra
    (exgb_scatter_modes), inverse-transformed (exgb_irfftn) and normalised
    (exgb_normalize_fields).  Returns a (B, 1, N, ...) float32 CUDA tensor."""
    from . import _device
    from ._lib import check, load

    torch = _device.torch()
    _device.require_cuda()
    D, N = num_spatial_dims, num_points
    idx, vals = None, []
    for k in keys:
        i, v = draw(int(k))
        if idx is None:
            idx = i
        vals.append(v)
    B = len(vals)
    field_elems = (N // 2 + 1) * N ** (D - 1)
    d_idx = torch.from_numpy(np.ascontiguousarray(idx, dtype=np.int64)).cuda()
    d_vals = torch.from_numpy(np.ascontiguousarray(np.stack(vals).astype(np.complex64))).cuda()
    hat = torch.empty((B, field_elems), dtype=torch.complex64, device="cuda")
    lib = load()
    st = _device.stream()
    check(lib.exgb_scatter_modes(st, B, field_elems, len(idx), d_idx.data_ptr(), d_vals.data_ptr(), hat.data_ptr()),
          "scatter_modes")
    out = torch.empty((B, 1) + (N,) * D, dtype=torch.float32, device="cuda")
    check(lib.exgb_irfftn(st, D, N, B, hat.data_ptr(), out.data_ptr()), "irfftn")
    if zero_mean or max_one:
        check(lib.exgb_normalize_fields(st, B, N ** D, out.data_ptr(), int(zero_mean), int(max_one)), "normalize")
    return out


class RandomSineWaves1d:
    """u(x) = sum_{k=1..cutoff} a_k sin(2 pi k x / L + phi_k), a_k ~ U(-1, 1),
    phi_k ~ U(0, 2 pi), zero mean (the 1D sine-series reading of
    ic/_sine_waves_1d.py:82-179)."""

    def __init__(self, num_spatial_dims: int = 1, *, cutoff: int = 5):
        if num_spatial_dims != 1:
            raise ValueError("RandomSineWaves1d is one-dimensional")
        self.cutoff = cutoff

    def __call__(self, num_points: int, *, key: int) -> np.ndarray:
        rng = np.random.default_rng(key)
        a = rng.uniform(-1.0, 1.0, self.cutoff)
        phi = rng.uniform(0.0, 2 * np.pi, self.cutoff)
        x = np.arange(num_points) / num_points
        k = np.arange(1, self.cutoff + 1)
        u = np.sum(a[:, None] * np.sin(2 * np.pi * k[:, None] * x[None, :] + phi[:, None]), axis=0)
        return u[None, :].astype(np.float32)

    def _draw(self, num_points):
        N = num_points

        def draw(key):
            rng = np.random.default_rng(key)
            a = rng.uniform(-1.0, 1.0, self.cutoff)
            phi = rng.uniform(0.0, 2 * np.pi, self.cutoff)
            # a sin(theta + phi) -> rfft coefficient N a e^{i phi} / (2 i) at k
            return np.arange(1, self.cutoff + 1), 0.5 * N * a * (np.sin(phi) - 1j * np.cos(phi))

        return draw

    def device_batch(self, num_points: int, keys) -> "torch.Tensor":
        """The fields of `keys` (same draws as __call__), built on the GPU: (B, 1, N)."""
        return _device_series(1, num_points, keys, self._draw(num_points), False, False)


class RandomTruncatedFourierSeries:
    """Random-phase, random-amplitude Fourier series with |k_d| <= cutoff on
    every axis (the hypercube low-pass of
    ic/_truncated_fourier_series.py:17-100), zero mean; optional rescaling
    to max |u| = 1 (normalize_ic, ic/_base_ic.py:18-32)."""

    def __init__(self, num_spatial_dims: int, *, cutoff: int = 5, max_one: bool = False):
        self.num_spatial_dims = num_spatial_dims
        self.cutoff = cutoff
        self.max_one = max_one

    def __call__(self, num_points: int, *, key: int) -> np.ndarray:
        if self.num_spatial_dims == 1:
            u = RandomSineWaves1d(1, cutoff=self.cutoff)(num_points, key=key)[0]
        else:
            # one random cosine per +-k pair (the last nonzero component of k positive), drawn in
            # mode order; summed by an inverse real FFT of the half-spectrum _draw lays out
            idx, z = self._draw(num_points)(key)
            D, N = self.num_spatial_dims, num_points
            H = np.zeros(N ** (D - 1) * (N // 2 + 1), dtype=np.complex128)
            np.add.at(H, idx, z)
            u = np.fft.irfftn(H.reshape((N,) * (D - 1) + (N // 2 + 1,)), s=(N,) * D)
        u = u - u.mean()
        if self.max_one:
            u = u / np.max(np.abs(u))
        return u[None, ...].astype(np.float32)

    def _draw(self, num_points):
        """Per key: flat rfftn positions and coefficients of the series drawn by __call__ (2D / 3D):
        a cos(k.x + phi) contributes z = N^D a e^{i phi} / 2 at k (last axis >= 0) and conj(z) at -k
        when k's last component is 0."""
        D, N, c = self.num_spatial_dims, num_points, self.cutoff
        M = N // 2 + 1
        pos, neg = [], []
        for m in np.ndindex(*([2 * c + 1] * D)):
            k = np.array(m) - c
            nz = np.nonzero(k)[0]
            if nz.size == 0 or k[nz[-1]] < 0:
                continue
            if D == 2 and (k[1] < 0 or (k[1] == 0 and k[0] < 0)):
                continue

            def flat(kk):
                f = 0
                for d in range(D - 1):
                    f = f * N + int(kk[d]) % N
                return f * M + int(kk[-1])

            pos.append(flat(k))
            neg.append(flat(-k) if k[-1] == 0 else -1)
        pos, neg = np.array(pos), np.array(neg)
        has = neg >= 0
        idx = np.concatenate([pos, neg[has]])
        scale = 0.5 * float(N) ** D

        def draw(key):
            rng = np.random.default_rng(key)
            z = np.empty(len(pos), dtype=np.complex128)
            for i in range(len(pos)):
                a = rng.uniform(-1.0, 1.0)
                phi = rng.uniform(0.0, 2 * np.pi)
                z[i] = scale * a * np.exp(1j * phi)
            return idx, np.concatenate([z, np.conj(z[has])])

        return draw

    def device_batch(self, num_points: int, keys) -> "torch.Tensor":
        """The fields of `keys` (same draws as __call__), built on the GPU: (B, 1, N, ...)."""
        if self.num_spatial_dims == 1:
            return _device_series(1, num_points, keys, RandomSineWaves1d(1, cutoff=self.cutoff)._draw(num_points),
                                  True, self.max_one)
        return _device_series(self.num_spatial_dims, num_points, keys, self._draw(num_points), True, self.max_one)


def build_ic_set(ic_generator, *, num_points: int, num_samples: int, key: int = 0, device: bool = False):
    """_utils.py:316-348: stack of num_samples ICs; sample i uses seed key + i.
    device=True builds them on the GPU (generators with `device_batch`) and returns a CUDA tensor."""
    if device and hasattr(ic_generator, "device_batch"):
        return ic_generator.device_batch(num_points, range(key, key + num_samples))
    return np.stack([ic_generator(num_points, key=key + i) for i in range(num_samples)])
