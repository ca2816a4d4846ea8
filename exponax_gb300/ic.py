"""Initial-condition generators for the benchmark configurations.

The reference draws its random fields with jax.random (threefry); those
streams are not reproduced.  These generators follow the configuration
wording with NumPy's seeded PCG64: per seed s, ``np.random.default_rng(s)``.
Parity tests feed identical arrays to the GPU path and the oracle, so the
generator choice does not affect parity.
"""

from __future__ import annotations

import numpy as np


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
        elif self.num_spatial_dims == 2:
            # same draws and modes as the general branch, summed by an inverse
            # real FFT instead of mode by mode
            rng = np.random.default_rng(key)
            c, N = self.cutoff, num_points
            H = np.zeros((N, N // 2 + 1), dtype=np.complex128)
            for m in np.ndindex(2 * c + 1, 2 * c + 1):
                kx, ky = m[0] - c, m[1] - c
                if (kx, ky) == (0, 0) or ky < 0 or (ky == 0 and kx < 0):
                    continue
                a = rng.uniform(-1.0, 1.0)
                phi = rng.uniform(0.0, 2 * np.pi)
                z = 0.5 * a * np.exp(1j * phi) * N * N
                H[kx % N, ky] += z
                if ky == 0:
                    H[(-kx) % N, 0] += np.conj(z)
            u = np.fft.irfft2(H, s=(N, N))
        else:
            rng = np.random.default_rng(key)
            c = self.cutoff
            x = np.arange(num_points) / num_points
            grids = np.meshgrid(*([x] * self.num_spatial_dims), indexing="ij")
            u = np.zeros((num_points,) * self.num_spatial_dims)
            modes = [m for m in np.ndindex(*([2 * c + 1] * self.num_spatial_dims))]
            for m in modes:
                k = np.array(m) - c
                # one representative of each +-k pair (last axis >= 0 half space)
                nz = np.nonzero(k)[0]
                if nz.size == 0 or k[nz[-1]] < 0:
                    continue
                a = rng.uniform(-1.0, 1.0)
                phi = rng.uniform(0.0, 2 * np.pi)
                arg = sum(2 * np.pi * k[d] * grids[d] for d in range(self.num_spatial_dims))
                u += a * np.cos(arg + phi)
        u = u - u.mean()
        if self.max_one:
            u = u / np.max(np.abs(u))
        return u[None, ...].astype(np.float32)


def build_ic_set(ic_generator, *, num_points: int, num_samples: int, key: int = 0) -> np.ndarray:
    """_utils.py:316-348: stack of num_samples ICs; sample i uses seed key + i."""
    return np.stack([ic_generator(num_points, key=key + i) for i in range(num_samples)])
