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
        check(lib.exgb_normalize_fields(st, B, N ** D, out.data_ptr(), int(zero_mean), 0, int(max_one)), "normalize")
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


def validate_normalization_options(*, zero_mean: bool, std_one: bool, max_one: bool):
    """ic/_base_ic.py:8-13: ValueError for the invalid combinations."""
    if not zero_mean and std_one:
        raise ValueError("Cannot have `zero_mean=False` and `std_one=True`.")
    if std_one and max_one:
        raise ValueError("Cannot have `std_one=True` and `max_one=True`.")


def normalize_ic(ic, *, zero_mean: bool = True, std_one: bool = False, max_one: bool = False):
    """normalize_ic (ic/_base_ic.py:18-32) of one field over all its entries: subtract the mean, then
    divide by the population standard deviation or by max |u|.  A CUDA tensor is normalised on the
    device (exgb_normalize_fields); a NumPy array on the host."""
    validate_normalization_options(zero_mean=zero_mean, std_one=std_one, max_one=max_one)
    if isinstance(ic, np.ndarray):
        if zero_mean:
            ic = ic - ic.mean()
        if std_one:
            ic = ic / ic.std()
        if max_one:
            ic = ic / np.max(np.abs(ic))
        return ic
    return _normalize_device(ic.clone().reshape(1, -1), zero_mean, std_one, max_one).reshape(ic.shape)


def _normalize_device(fields, zero_mean, std_one, max_one):
    """In place over a contiguous float32 CUDA tensor whose leading axis counts the fields."""
    from . import _device
    from ._lib import check, load

    if not (zero_mean or std_one or max_one):
        return fields
    B = fields.shape[0]
    n = fields.numel() // max(B, 1)
    check(load().exgb_normalize_fields(_device.stream(), B, n, fields.data_ptr(), int(zero_mean), int(std_one),
                                       int(max_one)), "normalize_ic")
    return fields


class WhiteNoise:
    """i.i.d. normal samples in physical space, no normalisation (ic/_white_noise.py:8-32); NumPy's
    seeded PCG64 in place of jax.random."""

    def __init__(self, num_spatial_dims: int, std: float = 1.0):
        self.num_spatial_dims = num_spatial_dims
        self.std = std

    def __call__(self, num_points: int, *, key: int) -> np.ndarray:
        rng = np.random.default_rng(key)
        shape = (1,) + (num_points,) * self.num_spatial_dims
        return (self.std * rng.standard_normal(shape)).astype(np.float32)

    def device_batch(self, num_points: int, keys) -> "torch.Tensor":
        """The noise fields of `keys` (same draws as __call__) as a (B, 1, N, ...) CUDA tensor."""
        from . import _device

        torch = _device.torch()
        _device.require_cuda()
        host = np.stack([self(num_points, key=int(k)) for k in keys])
        return torch.from_numpy(host).pin_memory().cuda(non_blocking=True)


class _NoiseFilterIC:
    """Shared part of the generators that filter white noise (GaussianRandomField, DiffusedNoise):
    __call__ runs the filter on the host (NumPy, float32 like the reference's default precision);
    from_noise / device_batch run it on the GPU through the library."""

    def __init__(self, num_spatial_dims, domain_extent, zero_mean, std_one, max_one):
        validate_normalization_options(zero_mean=zero_mean, std_one=std_one, max_one=max_one)
        self.num_spatial_dims = num_spatial_dims
        self.domain_extent = domain_extent
        self.zero_mean = zero_mean
        self.std_one = std_one
        self.max_one = max_one
        self.white_noise = WhiteNoise(num_spatial_dims)
        self._filters = {}

    def __call__(self, num_points: int, *, key: int) -> np.ndarray:
        u = self._host_filter(self.white_noise(num_points, key=key))
        return normalize_ic(u, zero_mean=self.zero_mean, std_one=self.std_one, max_one=self.max_one)

    def from_noise(self, noise) -> "torch.Tensor":
        """The fields made from a (B, 1, N, ..., N) float32 CUDA tensor of white noise, on the GPU."""
        from . import _device

        _device.require_cuda()
        u = self._device_filter(noise.contiguous())
        return _normalize_device(u.contiguous(), self.zero_mean, self.std_one, self.max_one)

    def device_batch(self, num_points: int, keys) -> "torch.Tensor":
        """The fields of `keys` (same noise draws as __call__), filtered on the GPU: (B, 1, N, ...)."""
        return self.from_noise(self.white_noise.device_batch(num_points, keys))


class GaussianRandomField(_NoiseFilterIC):
    """ic/_gaussian_random_field.py:17-93: white noise whose spectrum is multiplied by |k|^(-p/2)
    (scaled wavenumbers, 1 at k = 0), so that the power spectrum follows a power law of exponent p.
    On the GPU the filter is one ETDRK0 step of dt = 1 with L = -(p/2) log|k| (E = exp(L), built in
    FP64 by the plan) between rfftn and irfftn."""

    def __init__(self, num_spatial_dims: int, *, domain_extent: float = 1.0, powerlaw_exponent: float = 3.0,
                 zero_mean: bool = True, std_one: bool = False, max_one: bool = False):
        super().__init__(num_spatial_dims, domain_extent, zero_mean, std_one, max_one)
        self.powerlaw_exponent = powerlaw_exponent

    def _knorm(self, num_points, dtype):
        from .spectral import build_scaled_wavenumbers

        k = build_scaled_wavenumbers(self.num_spatial_dims, self.domain_extent, num_points).astype(dtype)
        return np.linalg.norm(k, axis=0, keepdims=True)

    def _host_filter(self, noise):
        from .spectral import space_indices

        D, N = self.num_spatial_dims, noise.shape[-1]
        kn = self._knorm(N, np.float32)
        with np.errstate(divide="ignore"):
            amp = np.power(kn, np.float32(-self.powerlaw_exponent / 2.0))
        amp.reshape(-1)[0] = 1.0
        hat = np.fft.rfftn(noise, axes=space_indices(D)) * amp
        return np.fft.irfftn(hat, s=(N,) * D, axes=space_indices(D)).astype(np.float32)

    def _device_filter(self, noise):
        from .etdrk import ETDRK0
        from .spectral import fft, ifft

        D, N = self.num_spatial_dims, noise.shape[-1]
        f = self._filters.get(N)
        if f is None:
            kn = self._knorm(N, np.float64)
            with np.errstate(divide="ignore"):
                L = -(self.powerlaw_exponent / 2.0) * np.log(kn)
            L.reshape(-1)[0] = 0.0
            f = self._filters[N] = ETDRK0(1.0, L.astype(np.complex128), num_points=N)
        hat = f._batched_step_fourier(fft(noise, num_spatial_dims=D))
        return ifft(hat, num_spatial_dims=D, num_points=N)


class DiffusedNoise(_NoiseFilterIC):
    """ic/_diffused_noise.py:15-76: white noise advanced by one Diffusion step of dt = 1 with
    diffusivity `intensity` (the spectrum decays like exp(-intensity |k|^2)), then normalised."""

    def __init__(self, num_spatial_dims: int, *, domain_extent: float = 1.0, intensity: float = 0.001,
                 zero_mean: bool = True, std_one: bool = False, max_one: bool = False):
        super().__init__(num_spatial_dims, domain_extent, zero_mean, std_one, max_one)
        self.intensity = intensity

    def _stepper(self, num_points):
        from .stepper import Diffusion

        st = self._filters.get(num_points)
        if st is None:
            st = self._filters[num_points] = Diffusion(self.num_spatial_dims, self.domain_extent, num_points, 1.0,
                                                       diffusivity=self.intensity)
        return st

    def _host_filter(self, noise):
        from .spectral import space_indices

        D, N = self.num_spatial_dims, noise.shape[-1]
        E = np.exp(self._stepper(N).linear_operator.real).astype(np.float32)
        hat = np.fft.rfftn(noise, axes=space_indices(D)) * E
        return np.fft.irfftn(hat, s=(N,) * D, axes=space_indices(D)).astype(np.float32)

    def _device_filter(self, noise):
        from ._utils import vmap

        return vmap(self._stepper(noise.shape[-1]))(noise)


def build_ic_set(ic_generator, *, num_points: int, num_samples: int, key: int = 0, device: bool = False):
    """_utils.py:316-348: stack of num_samples ICs; sample i uses seed key + i.
    device=True builds them on the GPU (generators with `device_batch`) and returns a CUDA tensor."""
    if device and hasattr(ic_generator, "device_batch"):
        return ic_generator.device_batch(num_points, range(key, key + num_samples))
    return np.stack([ic_generator(num_points, key=key + i) for i in range(num_samples)])
