"""Initial-condition generators (exponax/ic/*).

The reference draws its random fields with jax.random (threefry); those streams
are not reproduced.  Every generator here draws with NumPy's seeded PCG64 (per
integer key k, ``np.random.default_rng(k)``; sub-keys from
``np.random.SeedSequence``), and parity tests feed identical arrays to the GPU
path and the oracle.  The classes keep the reference's names, arguments and
normalisation rules.  The random-series and filtered-noise generators also
build their fields on the GPU (``device_batch``, ``build_ic_set(device=True)``,
``from_noise``); the closed-form ones (sine waves, Gaussian blobs,
discontinuities) are evaluated on the host grid as the reference evaluates them
on its grid.

``RandomAmplitudePhaseSeries`` is the benchmark workloads' recipe (random
amplitudes U(-1, 1) and phases U(0, 2 pi) of the modes |k_d| <= cutoff), which
the benchmark descriptions call a "random truncated Fourier series"; the reference's
``RandomTruncatedFourierSeries`` is low-pass-filtered white noise and is
provided under its own name with its own recipe.
"""

from __future__ import annotations

import numpy as np


def _device_series(num_spatial_dims, num_points, keys, draw, zero_mean, max_one, std_one=False):
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
    if zero_mean or max_one or std_one:
        check(lib.exgb_normalize_fields(st, B, N ** D, out.data_ptr(), int(zero_mean), int(std_one), int(max_one)),
              "normalize")
    return out


def _split_key(key, n):
    """n independent integer sub-keys of `key` (the role of jax.random.split)."""
    return [int(v) for v in np.random.SeedSequence(int(key)).generate_state(n)]


def _grid(num_spatial_dims, domain_extent, num_points):
    from ._utils import make_grid

    return make_grid(num_spatial_dims, domain_extent, num_points)


class BaseIC:
    """ic/_base_ic.py:35-52: an initial condition as a function of the grid x (D, N, ..., N) -> (1, N, ...)."""

    def __call__(self, x):
        raise NotImplementedError


class BaseRandomICGenerator:
    """ic/_base_ic.py:55-105: gen_ic_fun(key) draws an initial-condition function; calling the generator
    evaluates it on the grid of num_points points per axis over [0, domain_extent)."""

    num_spatial_dims: int
    domain_extent: float = 1.0

    def gen_ic_fun(self, *, key: int) -> BaseIC:
        raise NotImplementedError(
            "This random ic generator cannot represent its initial condition as a function. Directly evaluate it.")

    def __call__(self, num_points: int, *, key: int) -> np.ndarray:
        ic_fun = self.gen_ic_fun(key=key)
        return np.asarray(ic_fun(_grid(self.num_spatial_dims, self.domain_extent, num_points)), dtype=np.float32)


class SineWaves1d(BaseIC):
    """ic/_sine_waves_1d.py:10-79: sum_i a_i sin(k_i 2 pi / L x + phi_i) + offset, then optionally divided
    by its standard deviation or by max |u|."""

    def __init__(self, domain_extent, amplitudes, wavenumbers, phases, offset=0.0, std_one=False, max_one=False):
        if offset != 0.0 and std_one:
            raise ValueError("Cannot have non-zero offset and `std_one=True`.")
        if std_one and max_one:
            raise ValueError("Cannot have `std_one=True` and `max_one=True`.")
        if len(amplitudes) != len(wavenumbers) or len(wavenumbers) != len(phases):
            raise ValueError("The number of amplitudes, wavenumbers, and phases must be the same.")
        self.domain_extent = domain_extent
        self.amplitudes = tuple(float(a) for a in amplitudes)
        self.wavenumbers = tuple(float(k) for k in wavenumbers)
        self.phases = tuple(float(p) for p in phases)
        self.offset = float(offset)
        self.std_one = std_one
        self.max_one = max_one

    def __call__(self, x):
        x = np.asarray(x)
        if x.shape[0] != 1:
            raise ValueError("SineWaves1d only works in 1d.")
        xd = x.astype(np.float64)
        result = np.zeros_like(xd)
        for a, k, p in zip(self.amplitudes, self.wavenumbers, self.phases):
            result += a * np.sin(k * (2 * np.pi / self.domain_extent) * xd + p)
        result += self.offset
        if self.std_one:
            result = result / np.std(result)
        if self.max_one:
            result = result / np.max(np.abs(result))
        return result.astype(x.dtype if np.issubdtype(x.dtype, np.floating) else np.float32)


class RandomSineWaves1d(BaseRandomICGenerator):
    """ic/_sine_waves_1d.py:82-179: cutoff sine waves k = 1..cutoff with amplitudes and phases drawn
    uniformly from amplitude_range / phase_range and an offset from offset_range (drawn in that order
    from one PCG64 stream per key)."""

    def __init__(self, num_spatial_dims: int = 1, *, domain_extent: float = 1.0, cutoff: int = 5,
                 amplitude_range=(-1.0, 1.0), phase_range=(0.0, 2 * np.pi), offset_range=(0.0, 0.0),
                 std_one: bool = False, max_one: bool = False):
        if num_spatial_dims != 1:
            raise ValueError("RandomSineWaves1d only works in 1d.")
        if tuple(offset_range) != (0.0, 0.0) and std_one:
            raise ValueError("Cannot have non-zero offset and `std_one=True`.")
        if std_one and max_one:
            raise ValueError("Cannot have `std_one=True` and `max_one=True`.")
        self.num_spatial_dims = 1
        self.domain_extent = domain_extent
        self.cutoff = cutoff
        self.amplitude_range = tuple(amplitude_range)
        self.phase_range = tuple(phase_range)
        self.offset_range = tuple(offset_range)
        self.std_one = std_one
        self.max_one = max_one

    def _params(self, key):
        rng = np.random.default_rng(key)
        a = rng.uniform(self.amplitude_range[0], self.amplitude_range[1], self.cutoff)
        phi = rng.uniform(self.phase_range[0], self.phase_range[1], self.cutoff)
        offset = float(rng.uniform(self.offset_range[0], self.offset_range[1]))
        return a, phi, offset

    def gen_ic_fun(self, *, key: int) -> SineWaves1d:
        a, phi, offset = self._params(key)
        return SineWaves1d(self.domain_extent, a, np.arange(1, self.cutoff + 1), phi, offset=offset,
                           std_one=self.std_one, max_one=self.max_one)

    def __call__(self, num_points: int, *, key: int) -> np.ndarray:
        # the grid in FP64 (x = L i / N) rather than the float32 make_grid
        x = (self.domain_extent * np.arange(num_points) / num_points)[None, :]
        return self.gen_ic_fun(key=key)(x).astype(np.float32)

    def _draw(self, num_points):
        N = num_points

        def draw(key):
            a, phi, offset = self._params(key)
            # a sin(theta + phi) -> rfft coefficient N a e^{i phi} / (2 i) at k; the offset N c at k = 0
            idx = np.arange(0, self.cutoff + 1)
            z = np.concatenate([[N * offset + 0j], 0.5 * N * a * (np.sin(phi) - 1j * np.cos(phi))])
            return idx, z

        return draw

    def device_batch(self, num_points: int, keys) -> "torch.Tensor":
        """The fields of `keys` (same draws as __call__), built on the GPU: (B, 1, N)."""
        return _device_series(1, num_points, keys, self._draw(num_points), False, self.max_one, self.std_one)


class RandomAmplitudePhaseSeries:
    """The benchmark workloads' "random truncated Fourier series": one cosine per +-k pair of the
    modes |k_d| <= cutoff on every axis (the hypercube of ic/_truncated_fourier_series.py's low-pass)
    with amplitude U(-1, 1) and phase U(0, 2 pi), zero mean, optionally rescaled to max |u| = 1
    (normalize_ic, ic/_base_ic.py:18-32).  In 1D it is RandomSineWaves1d's series."""

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


class RandomTruncatedFourierSeries(BaseRandomICGenerator):
    """ic/_truncated_fourier_series.py:17-100: white noise (i.i.d. N(0, 1) on the grid) -> rfftn ->
    hypercube low-pass |k_d| <= cutoff -> the mean coefficient (index 0) set to an offset drawn from
    offset_range (the unnormalised rfftn coefficient, so the field's mean becomes offset / N^D) ->
    irfftn -> normalize_ic with zero_mean = (offset_range == (0, 0)).  Per key the noise and then the
    offset come from one PCG64 stream; device_batch / from_noise run the transforms on the GPU."""

    def __init__(self, num_spatial_dims: int, *, cutoff: int = 5, offset_range=(0.0, 0.0), std_one: bool = False,
                 max_one: bool = False):
        zero_mean = tuple(offset_range) == (0.0, 0.0)
        validate_normalization_options(zero_mean=zero_mean, std_one=std_one, max_one=max_one)
        self.num_spatial_dims = num_spatial_dims
        self.cutoff = cutoff
        self.offset_range = tuple(offset_range)
        self.std_one = std_one
        self.max_one = max_one
        self.white_noise = WhiteNoise(num_spatial_dims)
        self._tables = {}

    def _zero_mean(self):
        return self.offset_range == (0.0, 0.0)

    def _draws(self, num_points, key):
        rng = np.random.default_rng(key)
        noise = rng.standard_normal((1,) + (num_points,) * self.num_spatial_dims).astype(np.float32)
        offset = float(rng.uniform(self.offset_range[0], self.offset_range[1]))
        return noise, offset

    def _mask(self, num_points):
        from .spectral import low_pass_filter_mask

        return low_pass_filter_mask(self.num_spatial_dims, num_points, cutoff=self.cutoff, axis_separate=True)

    def __call__(self, num_points: int, *, key: int) -> np.ndarray:
        from .spectral import space_indices

        D = self.num_spatial_dims
        noise, offset = self._draws(num_points, key)
        hat = (np.fft.rfftn(noise, axes=space_indices(D)) * self._mask(num_points)).astype(np.complex64)
        hat.reshape(-1)[0] = offset
        u = np.fft.irfftn(hat, s=(num_points,) * D, axes=space_indices(D)).astype(np.float32)
        return normalize_ic(u, zero_mean=self._zero_mean(), std_one=self.std_one, max_one=self.max_one)

    def from_noise(self, noise, offsets=None) -> "torch.Tensor":
        """The fields made on the GPU from a (B, 1, N, ..., N) float32 CUDA tensor of white noise and B
        offsets (default 0): exgb_rfftn, the low-pass mask (exgb_mode_scale), the offsets written into the
        mean coefficients, exgb_irfftn, exgb_normalize_fields."""
        from . import _device
        from ._lib import check, load
        from .spectral import fft, ifft

        torch = _device.torch()
        _device.require_cuda()
        D, N = self.num_spatial_dims, noise.shape[-1]
        B = noise.shape[0]
        table = self._tables.get(N)
        if table is None:
            m = self._mask(N).reshape(-1).astype(np.complex64)
            table = self._tables[N] = torch.from_numpy(np.ascontiguousarray(m)).cuda()
        hat = fft(noise.contiguous(), num_spatial_dims=D).contiguous()
        check(load().exgb_mode_scale(_device.stream(), B, table.numel(), table.data_ptr(), hat.data_ptr(),
                                     hat.data_ptr()), "RandomTruncatedFourierSeries")
        off = torch.zeros(B, dtype=torch.complex64) if offsets is None else \
            torch.tensor(np.asarray(offsets, dtype=np.float32)).to(torch.complex64)
        hat.view(B, -1)[:, 0] = off.cuda()
        u = ifft(hat, num_spatial_dims=D, num_points=N).contiguous()
        return _normalize_device(u, self._zero_mean(), self.std_one, self.max_one)

    def device_batch(self, num_points: int, keys) -> "torch.Tensor":
        """The fields of `keys` (same draws as __call__), transformed on the GPU: (B, 1, N, ...)."""
        from . import _device

        torch = _device.torch()
        draws = [self._draws(num_points, int(k)) for k in keys]
        noise = torch.from_numpy(np.stack([d[0] for d in draws])).pin_memory().cuda(non_blocking=True)
        return self.from_noise(noise, [d[1] for d in draws])


class GaussianBlob:
    """ic/_gaussian_blob.py:12-72: exp(-(x - p)^T S^-1 (x - p) / 2) on the grid (1 minus it with
    one_complement)."""

    def __init__(self, position, covariance, *, one_complement: bool = False):
        self.position = np.asarray(position, dtype=np.float64)
        self.covariance = np.asarray(covariance, dtype=np.float64)
        self._inv_covariance = np.linalg.inv(self.covariance)
        self.one_complement = one_complement

    def __call__(self, x):
        x = np.asarray(x)
        D = x.shape[0]
        if D != self.position.shape[0]:
            raise ValueError(f"The position has {self.position.shape[0]} dimensions but the grid {D}")
        diff = x.astype(np.float64) - self.position.reshape((D,) + (1,) * D)
        q = np.einsum("i...,ij,j...->...", diff, self._inv_covariance, diff)
        blob = np.exp(-0.5 * q)[None]
        return (1.0 - blob) if self.one_complement else blob


class GaussianBlobs(BaseIC):
    """ic/_gaussian_blob.py:75-98: the mean of several blobs."""

    def __init__(self, blob_list):
        self.blob_list = tuple(blob_list)

    def __call__(self, x):
        return sum(b(x) for b in self.blob_list) / len(self.blob_list)


class RandomGaussianBlobs(BaseRandomICGenerator):
    """ic/_gaussian_blob.py:101-190: num_blobs blobs with positions U(position_range) L and diagonal
    variances U(variance_range) L per axis."""

    def __init__(self, num_spatial_dims: int, *, domain_extent: float = 1.0, num_blobs: int = 1,
                 position_range=(0.4, 0.6), variance_range=(0.005, 0.01), one_complement: bool = False):
        self.num_spatial_dims = num_spatial_dims
        self.domain_extent = domain_extent
        self.num_blobs = num_blobs
        self.position_range = tuple(position_range)
        self.variance_range = tuple(variance_range)
        self.one_complement = one_complement

    def gen_blob(self, *, key: int) -> GaussianBlob:
        rng = np.random.default_rng(key)
        D, L = self.num_spatial_dims, self.domain_extent
        position = rng.uniform(self.position_range[0] * L, self.position_range[1] * L, D)
        variances = rng.uniform(self.variance_range[0] * L, self.variance_range[1] * L, D)
        return GaussianBlob(position, np.diag(variances), one_complement=self.one_complement)

    def gen_ic_fun(self, *, key: int) -> GaussianBlobs:
        return GaussianBlobs([self.gen_blob(key=k) for k in _split_key(key, self.num_blobs)])


class Discontinuity:
    """ic/_discontinuities.py:10-27: value inside the open box lower < x_d < upper on every axis, 0 outside."""

    def __init__(self, lower_limits, upper_limits, value):
        self.lower_limits = tuple(float(v) for v in lower_limits)
        self.upper_limits = tuple(float(v) for v in upper_limits)
        self.value = float(value)

    def __call__(self, x):
        x = np.asarray(x)
        mask = np.ones_like(x[0:1], dtype=bool)
        for i, (lb, ub) in enumerate(zip(self.lower_limits, self.upper_limits)):
            mask = mask & (x[i:i + 1] > lb) & (x[i:i + 1] < ub)
        return np.where(mask, self.value, 0.0)


class Discontinuities(BaseIC):
    """ic/_discontinuities.py:30-75: the sum of boxes, then zero mean / std one / max one."""

    def __init__(self, discontinuity_list, *, zero_mean: bool = True, std_one: bool = False, max_one: bool = False):
        validate_normalization_options(zero_mean=zero_mean, std_one=std_one, max_one=max_one)
        self.discontinuity_list = tuple(discontinuity_list)
        self.zero_mean = zero_mean
        self.std_one = std_one
        self.max_one = max_one

    def __call__(self, x):
        ic = sum(d(x) for d in self.discontinuity_list)
        return normalize_ic(np.asarray(ic, dtype=np.float64), zero_mean=self.zero_mean, std_one=self.std_one,
                            max_one=self.max_one)


class RandomDiscontinuities(BaseRandomICGenerator):
    """ic/_discontinuities.py:78-160: num_discontinuities boxes with per-axis limits U(0, L) (sorted) and a
    value U(value_range)."""

    def __init__(self, num_spatial_dims: int, *, domain_extent: float = 1.0, num_discontinuities: int = 3,
                 value_range=(-1.0, 1.0), zero_mean: bool = False, std_one: bool = False, max_one: bool = False):
        validate_normalization_options(zero_mean=zero_mean, std_one=std_one, max_one=max_one)
        self.num_spatial_dims = num_spatial_dims
        self.domain_extent = domain_extent
        self.num_discontinuities = num_discontinuities
        self.value_range = tuple(value_range)
        self.zero_mean = zero_mean
        self.std_one = std_one
        self.max_one = max_one

    def gen_one_ic_fn(self, *, key: int) -> Discontinuity:
        rng = np.random.default_rng(key)
        lo, hi = [], []
        for _ in range(self.num_spatial_dims):
            l1, l2 = rng.uniform(0.0, self.domain_extent, 2)
            lo.append(min(l1, l2))
            hi.append(max(l1, l2))
        value = rng.uniform(self.value_range[0], self.value_range[1])
        return Discontinuity(lo, hi, value)

    def gen_ic_fun(self, *, key: int) -> Discontinuities:
        return Discontinuities([self.gen_one_ic_fn(key=k) for k in _split_key(key, self.num_discontinuities)],
                               zero_mean=self.zero_mean, std_one=self.std_one, max_one=self.max_one)


class MultiChannelIC:
    """ic/_multi_channel.py:11-33: the channels of several initial-condition functions, concatenated."""

    def __init__(self, initial_conditions):
        self.initial_conditions = tuple(initial_conditions)

    def __call__(self, x):
        return np.concatenate([np.asarray(ic(x)) for ic in self.initial_conditions], axis=0)


class RandomMultiChannelICGenerator:
    """ic/_multi_channel.py:36-96: one generator per channel, each with its own sub-key."""

    def __init__(self, ic_generators):
        self.ic_generators = tuple(ic_generators)
        self.num_spatial_dims = self.ic_generators[0].num_spatial_dims

    def gen_ic_fun(self, *, key: int) -> MultiChannelIC:
        ks = _split_key(key, len(self.ic_generators))
        return MultiChannelIC([g.gen_ic_fun(key=k) for g, k in zip(self.ic_generators, ks)])

    def __call__(self, num_points: int, *, key: int) -> np.ndarray:
        ks = _split_key(key, len(self.ic_generators))
        return np.concatenate([np.asarray(g(num_points, key=k)) for g, k in zip(self.ic_generators, ks)], axis=0)


class ScaledIC(BaseIC):
    """ic/_scaled.py:9-28: an initial-condition function times a constant."""

    def __init__(self, ic, *, scale: float):
        self.ic = ic
        self.scale = scale

    def __call__(self, x):
        return self.ic(x) * self.scale


class ScaledICGenerator(BaseRandomICGenerator):
    """ic/_scaled.py:31-70: a generator's fields times a constant."""

    def __init__(self, ic_gen, scale: float):
        self.ic_gen = ic_gen
        self.scale = scale
        self.num_spatial_dims = ic_gen.num_spatial_dims

    def gen_ic_fun(self, *, key: int) -> ScaledIC:
        return ScaledIC(self.ic_gen.gen_ic_fun(key=key), scale=self.scale)

    def __call__(self, num_points: int, *, key: int) -> np.ndarray:
        return self.ic_gen(num_points=num_points, key=key) * self.scale


class ClampingICGenerator(BaseRandomICGenerator):
    """ic/_clamping.py:9-49: a generator's fields shifted and scaled to span exactly `limits`."""

    def __init__(self, ic_gen, limits=(0, 1)):
        self.ic_gen = ic_gen
        self.limits = tuple(limits)
        self.num_spatial_dims = ic_gen.num_spatial_dims

    def __call__(self, num_points: int, *, key: int) -> np.ndarray:
        ic = np.asarray(self.ic_gen(num_points=num_points, key=key))
        above = ic - np.min(ic)
        unit = above / np.max(above)
        return unit * (self.limits[1] - self.limits[0]) + self.limits[0]


def build_ic_set(ic_generator, *, num_points: int, num_samples: int, key: int = 0, device: bool = False):
    """_utils.py:316-348: stack of num_samples ICs; sample i uses seed key + i.
    device=True builds them on the GPU (generators with `device_batch`) and returns a CUDA tensor."""
    if device and hasattr(ic_generator, "device_batch"):
        return ic_generator.device_batch(num_points, range(key, key + num_samples))
    return np.stack([ic_generator(num_points, key=key + i) for i in range(num_samples)])
