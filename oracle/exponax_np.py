"""NumPy restatement of exponax's ETDRK pseudo-spectral stepping path.

TEST INFRASTRUCTURE ONLY.  This module is the oracle the CUDA library is
checked against.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU
baseline leg of ``bench.py`` may import it; the product package never does.

It restates, in plain NumPy (``numpy.fft`` = pocketfft, the same algorithm
family as the DUCC backend the reference uses on CPU), the functions of
exponax 0.2.0 listed below.  Every function names the reference file:line it
follows (paths inside the exponax project).

Precision: every constructor takes ``dtype`` = ``"float32"`` (the reference's
default JAX configuration: float32 / complex64 everywhere, including the
phi-coefficient contour mean) or ``"float64"`` (stands in for a JAX run with
``jax_enable_x64``).  NumPy 2 keeps float32 through ``numpy.fft`` and treats
Python scalars as weakly typed (NEP 50), which matches JAX's promotion rules
for the mixed scalar/array expressions used here.

Parity pin: JAX is not importable where this oracle was written, so the
restatement is pinned against the reference's own known-answer tests, golden
mask arrays and published validation numbers (see tests/test_oracle_*.py),
not against live reference outputs.
"""

from __future__ import annotations

from itertools import product

import numpy as np

# --------------------------------------------------------------------------
# dtype helpers
# --------------------------------------------------------------------------


def _dt(dtype):
    """Return (real dtype, complex dtype) for "float32" / "float64"."""
    if dtype in ("float32", np.float32):
        return np.float32, np.complex64
    if dtype in ("float64", np.float64):
        return np.float64, np.complex128
    raise ValueError(f"unknown dtype {dtype!r}")


# --------------------------------------------------------------------------
# spectral helpers            exponax/_spectral.py
# --------------------------------------------------------------------------


def spatial_shape(num_spatial_dims, num_points):
    """_spectral.py:230-250"""
    return (num_points,) * num_spatial_dims


def wavenumber_shape(num_spatial_dims, num_points):
    """_spectral.py:253-275"""
    return (num_points,) * (num_spatial_dims - 1) + (num_points // 2 + 1,)


def space_indices(num_spatial_dims):
    """_spectral.py:212-227"""
    return tuple(range(-num_spatial_dims, 0))


def build_wavenumbers(num_spatial_dims, num_points, *, dtype="float32"):
    """_spectral.py:13-49: integer wavenumber grid; fftfreq on leading axes,
    rfftfreq on the last axis, 'ij' meshgrid."""
    rd, _ = _dt(dtype)
    right = np.fft.rfftfreq(num_points, 1 / num_points).astype(rd)
    other = np.fft.fftfreq(num_points, 1 / num_points).astype(rd)
    lists = [other] * (num_spatial_dims - 1) + [right]
    return np.stack(np.meshgrid(*lists, indexing="ij"))


def build_scaled_wavenumbers(num_spatial_dims, domain_extent, num_points, *, dtype="float32"):
    """_spectral.py:52-83: wavenumbers * 2*pi/L."""
    rd, _ = _dt(dtype)
    scale = 2 * np.pi / domain_extent
    return (scale * build_wavenumbers(num_spatial_dims, num_points, dtype=dtype)).astype(rd)


def build_derivative_operator(num_spatial_dims, domain_extent, num_points, *, dtype="float32"):
    """_spectral.py:86-115: 1j * scaled wavenumbers, shape (D, ..., N//2+1)."""
    _, cd = _dt(dtype)
    return (1j * build_scaled_wavenumbers(num_spatial_dims, domain_extent, num_points, dtype=dtype)).astype(cd)


def build_laplace_operator(derivative_operator, *, order=2):
    """_spectral.py:118-155: sum_d (ik_d)^order; order 0 gives ones."""
    if order % 2 != 0:
        raise ValueError("Order must be even.")
    if order == 0:
        return np.ones((1, *derivative_operator.shape[1:]), dtype=derivative_operator.dtype)
    return np.sum(derivative_operator**order, axis=0, keepdims=True)


def build_gradient_inner_product_operator(derivative_operator, velocity, *, order=1):
    """_spectral.py:158-209: sum_d c_d (ik_d)^order for odd order."""
    if order % 2 != 1:
        raise ValueError("Order must be odd.")
    velocity = np.asarray(velocity)
    if velocity.shape != (derivative_operator.shape[0],):
        raise ValueError(
            f"Expected velocity shape to be {derivative_operator.shape[0]}, got {velocity.shape}."
        )
    op = np.einsum("i,i...->...", velocity.astype(derivative_operator.real.dtype), derivative_operator**order)
    return op[None, ...].astype(derivative_operator.dtype)


def low_pass_filter_mask(num_spatial_dims, num_points, *, cutoff, axis_separate=True, dtype="float32"):
    """_spectral.py:278-342: keep |k_d| <= cutoff on every axis (inclusive).

    The comparison happens in the wavenumber dtype (the cutoff is a weakly
    typed Python float, as in JAX)."""
    rd, _ = _dt(dtype)
    wn = build_wavenumbers(num_spatial_dims, num_points, dtype=dtype)
    if axis_separate:
        mask = np.ones(wn.shape[1:], dtype=bool)
        for g in wn:
            mask = mask & (np.abs(g) <= rd(cutoff))
    else:
        mask = np.linalg.norm(wn, axis=0) <= rd(cutoff)
    return mask[None, ...]


def oddball_filter_mask(num_spatial_dims, num_points):
    """_spectral.py:345-400: removes the Nyquist mode for even N."""
    if num_points % 2 == 1:
        return np.ones((1, *wavenumber_shape(num_spatial_dims, num_points)), dtype=bool)
    nyquist_mode = num_points // 2 + 1
    mode_below_nyquist = nyquist_mode - 1
    return low_pass_filter_mask(num_spatial_dims, num_points, cutoff=mode_below_nyquist - 1, axis_separate=True)


def _build_scaling_array(num_spatial_dims, num_points, *, right_den, other_den, dtype="float32"):
    """_spectral.py:403-457"""
    rd, _ = _dt(dtype)
    right_wn = np.fft.rfftfreq(num_points, 1 / num_points)
    other_wn = np.fft.fftfreq(num_points, 1 / num_points)
    right = np.where(right_wn == 0, num_points, num_points / right_den)
    other = np.where(other_wn == 0, num_points, num_points / other_den)
    if num_points % 2 == 0:
        right = np.where(right_wn == num_points // 2, num_points, right)
        other = np.where(other_wn == -num_points // 2, num_points, other)
    lists = [other] * (num_spatial_dims - 1) + [right]
    return np.prod(np.stack(np.meshgrid(*lists, indexing="ij")), axis=0, keepdims=True).astype(rd)


def build_scaling_array(num_spatial_dims, num_points, *, mode, dtype="float32"):
    """_spectral.py:460-527"""
    if mode == "norm_compensation":
        return _build_scaling_array(num_spatial_dims, num_points, right_den=1, other_den=1, dtype=dtype)
    if mode == "reconstruction":
        return _build_scaling_array(num_spatial_dims, num_points, right_den=2, other_den=1, dtype=dtype)
    if mode == "coef_extraction":
        return _build_scaling_array(num_spatial_dims, num_points, right_den=2, other_den=2, dtype=dtype)
    raise ValueError("Invalid mode.")


def get_modes_slices(num_spatial_dims, num_points):
    """_spectral.py:530-611: positive/negative wavenumber blocks."""
    is_even = num_points % 2 == 0
    nyq = num_points // 2
    if is_even:
        left, right = slice(None, nyq), slice(-nyq, None)
    else:
        left, right = slice(None, nyq + 1), slice(-nyq, None)
    slices_ = [[slice(None, nyq + 1)]] + [[left, right] for _ in range(num_spatial_dims - 1)]
    out = [tuple([slice(None)] + list(reversed(p))) for p in product(*slices_)]
    return tuple(out)


def fft(field, *, num_spatial_dims=None):
    """_spectral.py:614-656: rfftn over the last D axes, norm='backward'."""
    if num_spatial_dims is None:
        num_spatial_dims = field.ndim - 1
    return np.fft.rfftn(field, axes=space_indices(num_spatial_dims))


def ifft(field_hat, *, num_spatial_dims=None, num_points=None):
    """_spectral.py:659-721: irfftn with s=(N,)*D over the last D axes."""
    if num_spatial_dims is None:
        num_spatial_dims = field_hat.ndim - 1
    if num_points is None:
        if num_spatial_dims >= 2:
            num_points = field_hat.shape[-2]
        else:
            raise ValueError("num_points must be provided if num_spatial_dims == 1.")
    return np.fft.irfftn(
        field_hat,
        s=spatial_shape(num_spatial_dims, num_points),
        axes=space_indices(num_spatial_dims),
    )


def derivative(field, domain_extent, *, order=1):
    """_spectral.py:724-791"""
    C, D, N = field.shape[0], field.ndim - 1, field.shape[-1]
    dtype = "float64" if field.dtype == np.float64 else "float32"
    op = build_derivative_operator(D, domain_extent, N, dtype=dtype) ** order
    fh = fft(field, num_spatial_dims=D)
    dh = op * fh if C == 1 else fh[:, None] * op[None, ...]
    return ifft(dh, num_spatial_dims=D, num_points=N)


def make_incompressible(field):
    """_spectral.py:794-863"""
    D, N = field.ndim - 1, field.shape[-1]
    if field.shape[0] != D:
        raise ValueError("the number of channels must match the number of spatial dimensions")
    dtype = "float64" if field.dtype == np.float64 else "float32"
    d = build_derivative_operator(D, 1.0, N, dtype=dtype)
    uh = fft(field, num_spatial_dims=D)
    div = np.sum(d * uh, axis=0, keepdims=True)
    lap = build_laplace_operator(d)
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = np.where(lap == 0, 1.0, 1.0 / lap)
    return ifft(uh - d * (inv * div), num_spatial_dims=D, num_points=N)


def get_fourier_coefficients(state, *, scaling_compensation_mode="coef_extraction", round=5):
    """_spectral.py:1033-1172 (np.round: round half to even, like jnp.round)"""
    dtype = "float64" if state.dtype == np.float64 else "float32"
    hat = fft(state)
    if scaling_compensation_mode is not None:
        hat = hat / build_scaling_array(state.ndim - 1, state.shape[-1], mode=scaling_compensation_mode, dtype=dtype)
    if round is not None:
        hat = np.round(hat, round)
    return hat


def wrap_bc(u):
    """_utils.py:65-89"""
    return np.pad(u, ((0, 0),) + ((0, 1),) * (u.ndim - 1), mode="wrap")


def stack_sub_trajectories(trj, sub_len):
    """_utils.py:257-313 for one array trajectory (n, ...)."""
    n = trj.shape[0]
    if sub_len > n:
        raise ValueError("n must be smaller than or equal to the number of time steps in trj")
    return np.stack([trj[i:i + sub_len] for i in range(n - sub_len + 1)])


def make_grid(num_spatial_dims, domain_extent, num_points, *, full=False, zero_centered=False, dtype="float32"):
    """_utils.py:10-62"""
    rd, _ = _dt(dtype)
    if full:
        g = np.linspace(0, domain_extent, num_points + 1, endpoint=True)
    else:
        g = np.linspace(0, domain_extent, num_points, endpoint=False)
    if zero_centered:
        g = g - domain_extent / 2
    return np.stack(np.meshgrid(*([g] * num_spatial_dims), indexing="ij")).astype(rd)


def get_spectrum(state, *, power=True, radial_binning="sum"):
    """_spectral.py:866-1030: radially binned power (or amplitude) spectrum."""
    D = state.ndim - 1
    N = state.shape[-1]
    dtype = "float64" if state.dtype == np.float64 else "float32"
    rd, _ = _dt(dtype)
    absval = np.abs(fft(state, num_spatial_dims=D))
    magnitude = absval / build_scaling_array(D, N, mode="reconstruction", dtype=dtype)
    if power:
        q = 0.5 * magnitude * (absval / build_scaling_array(D, N, mode="norm_compensation", dtype=dtype))
    else:
        q = magnitude
    q = q.astype(rd)
    if D == 1:
        return q
    wn = build_wavenumbers(D, N, dtype=dtype)
    wn1 = build_wavenumbers(1, N, dtype=dtype)
    norm = np.linalg.norm(wn, axis=0)
    dk = wn1[0, 1] - wn1[0, 0]
    out = np.zeros((state.shape[0], wn1.shape[-1]), dtype=rd)
    for i, k in enumerate(wn1[0]):
        m = (norm >= k - dk / 2) & (norm < k + dk / 2)
        for c in range(state.shape[0]):
            if radial_binning == "average":
                out[c, i] = np.nanmean(q[c][m]) if m.any() else np.nan
            else:
                out[c, i] = np.nansum(q[c][m])
    return out


# --------------------------------------------------------------------------
# nonlinear functions          exponax/nonlin_fun/*
# --------------------------------------------------------------------------


class BaseNonlinearFun:
    """nonlin_fun/_base.py:9-159: dealiasing mask with cutoff
    dealiasing_fraction*(N//2) - 1 (inclusive, per axis); pre-mask before every
    ifft, post-mask after every fft."""

    def __init__(self, num_spatial_dims, num_points, *, dealiasing_fraction=None, dtype="float32"):
        self.num_spatial_dims = num_spatial_dims
        self.num_points = num_points
        self.dtype = dtype
        self.rd, self.cd = _dt(dtype)
        if dealiasing_fraction is None:
            self.dealiasing_mask = None
        else:
            nyquist_mode = (num_points // 2) + 1
            highest_resolved_mode = nyquist_mode - 1
            start_of_aliased_modes = dealiasing_fraction * highest_resolved_mode
            self.dealiasing_mask = low_pass_filter_mask(
                num_spatial_dims, num_points, cutoff=start_of_aliased_modes - 1, dtype=dtype
            )

    def dealias(self, u_hat):
        """_base.py:73-97"""
        if self.dealiasing_mask is None:
            raise ValueError("Nonlinear function was set up without dealiasing")
        return self.dealiasing_mask * u_hat

    def fft(self, u):
        """_base.py:99-116 (post-dealiasing)"""
        u_hat = fft(u, num_spatial_dims=self.num_spatial_dims)
        if self.dealiasing_mask is not None:
            u_hat = self.dealiasing_mask * u_hat
        return u_hat

    def ifft(self, u_hat):
        """_base.py:118-137 (pre-dealiasing)"""
        if self.dealiasing_mask is not None:
            u_hat = self.dealiasing_mask * u_hat
        return ifft(u_hat, num_spatial_dims=self.num_spatial_dims, num_points=self.num_points)


class ZeroNonlinearFun(BaseNonlinearFun):
    """nonlin_fun/_zero.py:7-38"""

    def __init__(self, num_spatial_dims, num_points, *, dtype="float32"):
        super().__init__(num_spatial_dims, num_points, dtype=dtype)

    def __call__(self, u_hat):
        return np.zeros_like(u_hat)


class ConvectionNonlinearFun(BaseNonlinearFun):
    """nonlin_fun/_convection.py:7-245 (four variants)."""

    def __init__(self, num_spatial_dims, num_points, *, derivative_operator, dealiasing_fraction=2 / 3,
                 scale=1.0, single_channel=False, conservative=False, dtype="float32"):
        self.derivative_operator = derivative_operator
        self.scale = scale
        self.single_channel = single_channel
        self.conservative = conservative
        super().__init__(num_spatial_dims, num_points, dealiasing_fraction=dealiasing_fraction, dtype=dtype)

    def _multi_channel_conservative_eval(self, u_hat):
        """_convection.py:104-138: -b/2 sum_j ik_j F[u_i u_j]"""
        if u_hat.shape[0] != self.num_spatial_dims:
            raise ValueError("Number of channels in u_hat should match number of spatial dimensions")
        u = self.ifft(u_hat)
        outer = u[None, :] * u[:, None]
        outer_hat = self.fft(outer)
        conv = 0.5 * np.sum(self.derivative_operator[None, :] * outer_hat, axis=1)
        return -self.scale * conv

    def _multi_channel_nonconservative_eval(self, u_hat):
        """_convection.py:140-171: -b F[sum_j u_j d_j u_i]"""
        if u_hat.shape[0] != self.num_spatial_dims:
            raise ValueError("Number of channels in u_hat should match number of spatial dimensions")
        u = self.ifft(u_hat)
        nabla_u = self.ifft(self.derivative_operator[None, :] * u_hat[:, None])
        conv_u = np.sum(u[None, :] * nabla_u, axis=1)
        return -self.scale * self.fft(conv_u)

    def _single_channel_conservative_eval(self, u_hat):
        """_convection.py:173-202: -b/2 (sum_d ik_d) F[u^2]"""
        u = self.ifft(u_hat)
        u_sq_hat = self.fft(u**2)
        sum_ops = np.sum(self.derivative_operator, axis=0, keepdims=True)
        return -self.scale * (0.5 * sum_ops * u_sq_hat)

    def _single_channel_nonconservative_eval(self, u_hat):
        """_convection.py:204-231: -b F[u (sum_d d_d u)]"""
        u = self.ifft(u_hat)
        nabla_u = self.ifft(self.derivative_operator * u_hat)
        conv_u = np.sum(u * nabla_u, axis=0, keepdims=True)
        return -self.scale * self.fft(conv_u)

    def __call__(self, u_hat):
        """_convection.py:233-245"""
        if self.single_channel:
            if self.conservative:
                return self._single_channel_conservative_eval(u_hat)
            return self._single_channel_nonconservative_eval(u_hat)
        if self.conservative:
            return self._multi_channel_conservative_eval(u_hat)
        return self._multi_channel_nonconservative_eval(u_hat)


class GradientNormNonlinearFun(BaseNonlinearFun):
    """nonlin_fun/_gradient_norm.py:8-101: -b/2 F[|grad u|^2 - mean]"""

    def __init__(self, num_spatial_dims, num_points, *, derivative_operator, dealiasing_fraction,
                 zero_mode_fix=True, scale=1.0, dtype="float32"):
        super().__init__(num_spatial_dims, num_points, dealiasing_fraction=dealiasing_fraction, dtype=dtype)
        self.derivative_operator = derivative_operator
        self.zero_mode_fix = zero_mode_fix
        self.scale = scale

    def __call__(self, u_hat):
        grad_hat = self.derivative_operator[None, :] * u_hat[:, None]
        grad = self.ifft(grad_hat)
        gn2 = np.sum(grad**2, axis=1)
        if self.zero_mode_fix:
            axes = tuple(range(1, gn2.ndim))
            gn2 = gn2 - np.mean(gn2, axis=axes, keepdims=True)
        return -self.scale * (0.5 * self.fft(gn2))


class PolynomialNonlinearFun(BaseNonlinearFun):
    """nonlin_fun/_polynomial.py:6-76: F[sum_k c_k u^k]"""

    def __init__(self, num_spatial_dims, num_points, *, dealiasing_fraction, coefficients, dtype="float32"):
        super().__init__(num_spatial_dims, num_points, dealiasing_fraction=dealiasing_fraction, dtype=dtype)
        self.coefficients = tuple(coefficients)

    def __call__(self, u_hat):
        u = self.ifft(u_hat)
        u_power = 1.0
        u_nonlin = 0.0
        for c in self.coefficients:
            u_nonlin = u_nonlin + c * u_power
            u_power = u_power * u
        u_nonlin = np.broadcast_to(np.asarray(u_nonlin, dtype=self.rd), u.shape)
        return self.fft(u_nonlin)


class GeneralNonlinearFun(BaseNonlinearFun):
    """nonlin_fun/_general_nonlinear.py:9-119: quadratic + single-channel
    conservative convection + gradient norm (note the sign flips at :90, :101)."""

    def __init__(self, num_spatial_dims, num_points, *, derivative_operator, dealiasing_fraction,
                 scale_list=(0.0, -1.0, 0.0), zero_mode_fix=True, dtype="float32"):
        if len(scale_list) != 3:
            raise ValueError("The scale list must have exactly 3 elements")
        self.square = PolynomialNonlinearFun(num_spatial_dims, num_points, dealiasing_fraction=dealiasing_fraction,
                                             coefficients=[0.0, 0.0, scale_list[0]], dtype=dtype)
        self.convection = ConvectionNonlinearFun(num_spatial_dims, num_points, derivative_operator=derivative_operator,
                                                 dealiasing_fraction=dealiasing_fraction, scale=-scale_list[1],
                                                 single_channel=True, conservative=True, dtype=dtype)
        self.gradient_norm = GradientNormNonlinearFun(num_spatial_dims, num_points,
                                                      derivative_operator=derivative_operator,
                                                      dealiasing_fraction=dealiasing_fraction,
                                                      scale=-scale_list[2], zero_mode_fix=zero_mode_fix, dtype=dtype)
        super().__init__(num_spatial_dims, num_points, dealiasing_fraction=dealiasing_fraction, dtype=dtype)

    def __call__(self, u_hat):
        return self.square(u_hat) + self.convection(u_hat) + self.gradient_norm(u_hat)


class VorticityConvection2d(BaseNonlinearFun):
    """nonlin_fun/_vorticity_convection.py:8-99: psi = inv_lap * omega with
    inv_lap(k=0) = 1 (:76); u = +d_y psi, v = -d_x psi; -b F[u w_x + v w_y]."""

    def __init__(self, num_spatial_dims, num_points, *, convection_scale=1.0, derivative_operator,
                 dealiasing_fraction, dtype="float32"):
        if num_spatial_dims != 2:
            raise ValueError(f"Expected num_spatial_dims = 2, got {num_spatial_dims}.")
        super().__init__(num_spatial_dims, num_points, dealiasing_fraction=dealiasing_fraction, dtype=dtype)
        self.convection_scale = convection_scale
        self.derivative_operator = derivative_operator
        lap = build_laplace_operator(derivative_operator, order=2)
        with np.errstate(divide="ignore", invalid="ignore"):
            self.inv_laplacian = np.where(lap == 0, 1.0, 1 / lap).astype(self.cd)

    def __call__(self, u_hat):
        w_hat = u_hat
        psi_hat = self.inv_laplacian * w_hat
        uu_hat = +self.derivative_operator[1:2] * psi_hat
        vv_hat = -self.derivative_operator[0:1] * psi_hat
        wx_hat = self.derivative_operator[0:1] * w_hat
        wy_hat = self.derivative_operator[1:2] * w_hat
        uu = self.ifft(uu_hat)
        vv = self.ifft(vv_hat)
        wx = self.ifft(wx_hat)
        wy = self.ifft(wy_hat)
        conv = uu * wx + vv * wy
        return -self.convection_scale * self.fft(conv)


class VorticityConvection2dKolmogorov(VorticityConvection2d):
    """nonlin_fun/_vorticity_convection.py:102-182: adds
    -k*gamma*coef_extraction_scaling at (k_x=0, k_y=k), unmasked."""

    def __init__(self, num_spatial_dims, num_points, *, convection_scale=1.0, injection_mode=4,
                 injection_scale=1.0, derivative_operator, dealiasing_fraction, dtype="float32"):
        super().__init__(num_spatial_dims, num_points, convection_scale=convection_scale,
                         derivative_operator=derivative_operator, dealiasing_fraction=dealiasing_fraction,
                         dtype=dtype)
        wn = build_wavenumbers(num_spatial_dims, num_points, dtype=dtype)
        m = (wn[0] == 0) & (wn[1] == injection_mode)
        self.injection = np.where(
            m,
            -injection_mode * injection_scale * build_scaling_array(num_spatial_dims, num_points,
                                                                    mode="coef_extraction", dtype=dtype),
            0.0,
        ).astype(self.rd)

    def __call__(self, u_hat):
        return super().__call__(u_hat) + self.injection


class Leray(BaseNonlinearFun):
    """nonlin_fun/_leray.py:8-136: u - ik (inv_lap (ik . u)) with inv_lap(0)=0."""

    def __init__(self, num_spatial_dims, num_points, *, derivative_operator, order=2, dtype="float32"):
        super().__init__(num_spatial_dims, num_points, dtype=dtype)
        lap = build_laplace_operator(derivative_operator, order=order)
        with np.errstate(divide="ignore", invalid="ignore"):
            self.inv_laplacian = np.where(lap != 0, 1.0 / lap, 0.0).astype(self.cd)
        self.derivative_operator = derivative_operator

    def __call__(self, u_hat):
        div = np.sum(self.derivative_operator * u_hat, axis=0, keepdims=True)
        p = -self.inv_laplacian * div
        return u_hat + self.derivative_operator * p


def _cross3(a, b):
    """nonlin_fun/_projected_convection.py:9-16"""
    return np.stack([a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]], axis=0)


class ProjectedConvection3d(BaseNonlinearFun):
    """nonlin_fun/_projected_convection.py:19-136: P F[u x (curl u)]."""

    def __init__(self, num_spatial_dims, num_points, *, derivative_operator, dealiasing_fraction=2 / 3,
                 dtype="float32"):
        if num_spatial_dims != 3:
            raise ValueError("ProjectedConvection3d only supports 3 spatial dimensions.")
        super().__init__(num_spatial_dims, num_points, dealiasing_fraction=dealiasing_fraction, dtype=dtype)
        self.derivative_operator = derivative_operator
        self.leray = Leray(num_spatial_dims, num_points, derivative_operator=derivative_operator, dtype=dtype)

    def __call__(self, u_hat):
        curl_hat = _cross3(self.derivative_operator, u_hat)
        curl = self.ifft(curl_hat)
        vel = self.ifft(u_hat)
        conv = _cross3(vel, curl)
        return self.leray(self.fft(conv))


class ProjectedConvection3dKolmogorov(ProjectedConvection3d):
    """nonlin_fun/_projected_convection.py:139-226: forcing gamma*scaling at
    (0, k, 0) on the first velocity channel."""

    def __init__(self, num_spatial_dims, num_points, *, injection_mode=4, injection_scale=1.0,
                 derivative_operator, dealiasing_fraction, dtype="float32"):
        super().__init__(num_spatial_dims, num_points, derivative_operator=derivative_operator,
                         dealiasing_fraction=dealiasing_fraction, dtype=dtype)
        wn = build_wavenumbers(num_spatial_dims, num_points, dtype=dtype)
        m = (wn[0] == 0) & (wn[1] == injection_mode) & (wn[2] == 0)
        single = np.where(m, injection_scale * build_scaling_array(num_spatial_dims, num_points,
                                                                   mode="coef_extraction", dtype=dtype), 0.0)
        z = np.zeros_like(single)
        self.injection = np.concatenate([single, z, z], axis=0).astype(self.rd)

    def __call__(self, u_hat):
        return super().__call__(u_hat) + self.injection


# --------------------------------------------------------------------------
# ETDRK integrators             exponax/etdrk/*
# --------------------------------------------------------------------------


def roots_of_unity(M, *, dtype="float32"):
    """etdrk/_utils.py:9-23: exp(2 pi i (j - 1/2) / M), j = 1..M."""
    _, cd = _dt(dtype)
    rd, _ = _dt(dtype)
    j = np.arange(1, M + 1).astype(rd)
    return np.exp((2j * np.pi * (j - 0.5) / M).astype(cd)).astype(cd)


class BaseETDRK:
    """etdrk/_base_etdrk.py:15-80: _exp_term = exp(dt * L)."""

    def __init__(self, dt, linear_operator):
        self.dt = dt
        self.cd = linear_operator.dtype
        self.rd = linear_operator.real.dtype
        self._exp_term = np.exp(dt * linear_operator).astype(self.cd)


def _contour_means(linear_operator, dt, num_circle_points, circle_radius, fns):
    """Kassam-Trefethen contour mean used by etdrk/_etdrk_1..4 (real part only,
    accumulated over the roots in order, as jax.lax.scan does)."""
    cd = linear_operator.dtype
    dtype = "float64" if cd == np.complex128 else "float32"
    roots = roots_of_unity(num_circle_points, dtype=dtype)
    L_dt = (linear_operator * dt).astype(cd)
    sums = [np.zeros(L_dt.shape, dtype=L_dt.real.dtype) for _ in fns]
    with np.errstate(all="ignore"):
        for r in roots:
            lr = (circle_radius * r + L_dt).astype(cd)
            exp_lr = np.exp(lr)
            exp_lr_half = np.exp(lr / 2)
            for i, f in enumerate(fns):
                sums[i] = sums[i] + f(lr, exp_lr, exp_lr_half).real
    return [(dt * (s / num_circle_points)).astype(L_dt.real.dtype) for s in sums]


class ETDRK0(BaseETDRK):
    """etdrk/_etdrk_0.py:6-34"""

    def __init__(self, dt, linear_operator):
        super().__init__(dt, linear_operator)

    def step_fourier(self, u_hat):
        return self._exp_term * u_hat


class ETDRK1(BaseETDRK):
    """etdrk/_etdrk_1.py:10-82"""

    def __init__(self, dt, linear_operator, nonlinear_fun, *, num_circle_points=16, circle_radius=1.0):
        super().__init__(dt, linear_operator)
        self._nonlinear_fun = nonlinear_fun
        (self._coef_1,) = _contour_means(linear_operator, dt, num_circle_points, circle_radius,
                                         [lambda lr, e, eh: (e - 1) / lr])

    def step_fourier(self, u_hat):
        return self._exp_term * u_hat + self._coef_1 * self._nonlinear_fun(u_hat)


class ETDRK2(BaseETDRK):
    """etdrk/_etdrk_2.py:10-102"""

    def __init__(self, dt, linear_operator, nonlinear_fun, *, num_circle_points=16, circle_radius=1.0):
        super().__init__(dt, linear_operator)
        self._nonlinear_fun = nonlinear_fun
        self._coef_1, self._coef_2 = _contour_means(
            linear_operator, dt, num_circle_points, circle_radius,
            [lambda lr, e, eh: (e - 1) / lr, lambda lr, e, eh: (e - 1 - lr) / lr**2])

    def step_fourier(self, u_hat):
        n0 = self._nonlinear_fun(u_hat)
        s1 = self._exp_term * u_hat + self._coef_1 * n0
        n1 = self._nonlinear_fun(s1)
        return s1 + self._coef_2 * (n1 - n0)


class ETDRK3(BaseETDRK):
    """etdrk/_etdrk_3.py:10-212"""

    def __init__(self, dt, linear_operator, nonlinear_fun, *, num_circle_points=16, circle_radius=1.0):
        super().__init__(dt, linear_operator)
        self._nonlinear_fun = nonlinear_fun
        self._half_exp_term = np.exp(0.5 * dt * linear_operator).astype(self.cd)
        (self._coef_1, self._coef_2, self._coef_3, self._coef_4, self._coef_5) = _contour_means(
            linear_operator, dt, num_circle_points, circle_radius,
            [
                lambda lr, e, eh: (eh - 1) / lr,
                lambda lr, e, eh: (e - 1) / lr,
                lambda lr, e, eh: (-4 - lr + e * (4 - 3 * lr + lr**2)) / lr**3,
                lambda lr, e, eh: (4.0 * (2.0 + lr + e * (-2 + lr))) / lr**3,
                lambda lr, e, eh: (-4 - 3 * lr - lr**2 + e * (4 - lr)) / lr**3,
            ])

    def step_fourier(self, u_hat):
        n0 = self._nonlinear_fun(u_hat)
        s1 = self._half_exp_term * u_hat + self._coef_1 * n0
        n1 = self._nonlinear_fun(s1)
        s2 = self._exp_term * u_hat + self._coef_2 * (2 * n1 - n0)
        n2 = self._nonlinear_fun(s2)
        return self._exp_term * u_hat + self._coef_3 * n0 + self._coef_4 * n1 + self._coef_5 * n2


class ETDRK4(BaseETDRK):
    """etdrk/_etdrk_4.py:10-224 (Cox-Matthews; coef_2 = coef_3 = coef_1)."""

    def __init__(self, dt, linear_operator, nonlinear_fun, *, num_circle_points=16, circle_radius=1.0):
        super().__init__(dt, linear_operator)
        self._nonlinear_fun = nonlinear_fun
        self._half_exp_term = np.exp(0.5 * dt * linear_operator).astype(self.cd)
        (self._coef_1, self._coef_4, self._coef_5, self._coef_6) = _contour_means(
            linear_operator, dt, num_circle_points, circle_radius,
            [
                lambda lr, e, eh: (eh - 1) / lr,
                lambda lr, e, eh: (-4 - lr + e * (4 - 3 * lr + lr**2)) / lr**3,
                lambda lr, e, eh: (2 + lr + e * (-2 + lr)) / lr**3,
                lambda lr, e, eh: (-4 - 3 * lr - lr**2 + e * (4 - lr)) / lr**3,
            ])
        self._coef_2 = self._coef_1
        self._coef_3 = self._coef_1

    def step_fourier(self, u_hat):
        n0 = self._nonlinear_fun(u_hat)
        s1 = self._half_exp_term * u_hat + self._coef_1 * n0
        n1 = self._nonlinear_fun(s1)
        s2 = self._half_exp_term * u_hat + self._coef_2 * n1
        n2 = self._nonlinear_fun(s2)
        s3 = self._half_exp_term * s1 + self._coef_3 * (2 * n2 - n0)
        n3 = self._nonlinear_fun(s3)
        return (self._exp_term * u_hat + self._coef_4 * n0 + self._coef_5 * 2 * (n1 + n2)
                + self._coef_6 * n3)


# --------------------------------------------------------------------------
# steppers                     exponax/_base_stepper.py, exponax/stepper/*
# --------------------------------------------------------------------------


class BaseStepper:
    """_base_stepper.py:17-271"""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, num_channels, order,
                 num_circle_points=16, circle_radius=1.0, dtype="float32"):
        self.num_spatial_dims = num_spatial_dims
        self.domain_extent = domain_extent
        self.num_points = num_points
        self.dt = dt
        self.num_channels = num_channels
        self.dx = domain_extent / num_points
        self.dtype = dtype
        self.rd, self.cd = _dt(dtype)
        deriv = build_derivative_operator(num_spatial_dims, domain_extent, num_points, dtype=dtype)
        lin = np.asarray(self._build_linear_operator(deriv)).astype(self.cd)
        ws = wavenumber_shape(num_spatial_dims, num_points)
        if lin.shape not in ((1,) + ws, (num_channels,) + ws):
            raise ValueError(
                f"Expected linear operator to have shape {(1,) + ws} or {(num_channels,) + ws}, got {lin.shape}."
            )
        self.linear_operator = lin
        self.nonlinear_fun = self._build_nonlinear_fun(deriv)
        kw = dict(num_circle_points=num_circle_points, circle_radius=circle_radius)
        if order == 0:
            self._integrator = ETDRK0(dt, lin)
        elif order == 1:
            self._integrator = ETDRK1(dt, lin, self.nonlinear_fun, **kw)
        elif order == 2:
            self._integrator = ETDRK2(dt, lin, self.nonlinear_fun, **kw)
        elif order == 3:
            self._integrator = ETDRK3(dt, lin, self.nonlinear_fun, **kw)
        elif order == 4:
            self._integrator = ETDRK4(dt, lin, self.nonlinear_fun, **kw)
        else:
            raise NotImplementedError(f"Order {order} not implemented.")

    def step(self, u):
        """_base_stepper.py:201-220"""
        u_hat = fft(u, num_spatial_dims=self.num_spatial_dims)
        return ifft(self.step_fourier(u_hat), num_spatial_dims=self.num_spatial_dims, num_points=self.num_points)

    def step_fourier(self, u_hat):
        """_base_stepper.py:222-239"""
        return self._integrator.step_fourier(u_hat)

    def __call__(self, u):
        """_base_stepper.py:241-271"""
        expected = (self.num_channels,) + spatial_shape(self.num_spatial_dims, self.num_points)
        if u.shape != expected:
            raise ValueError(f"Expected shape {expected}, got {u.shape}. For batched operation use vmap.")
        return self.step(u)


def _dt_of(self):
    return dict(dtype=self.dtype)


class KuramotoSivashinsky(BaseStepper):
    """stepper/_kuramoto_sivashinsky.py:8-168 (gradient-norm form)."""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, gradient_norm_scale=1.0,
                 second_order_scale=1.0, fourth_order_scale=1.0, dealiasing_fraction=2 / 3, order=2,
                 num_circle_points=16, circle_radius=1.0, dtype="float32"):
        self.gradient_norm_scale = gradient_norm_scale
        self.second_order_scale = second_order_scale
        self.fourth_order_scale = fourth_order_scale
        self.dealiasing_fraction = dealiasing_fraction
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=1, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius, dtype=dtype)

    def _build_linear_operator(self, d):
        return (-self.second_order_scale * build_laplace_operator(d, order=2)
                - self.fourth_order_scale * build_laplace_operator(d, order=4))

    def _build_nonlinear_fun(self, d):
        return GradientNormNonlinearFun(self.num_spatial_dims, self.num_points, derivative_operator=d,
                                        dealiasing_fraction=self.dealiasing_fraction, zero_mode_fix=True,
                                        scale=self.gradient_norm_scale, dtype=self.dtype)


class KuramotoSivashinskyConservative(BaseStepper):
    """stepper/_kuramoto_sivashinsky.py:171-315 (convection form)."""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, convection_scale=1.0,
                 second_order_scale=1.0, fourth_order_scale=1.0, single_channel=False, conservative=True,
                 dealiasing_fraction=2 / 3, order=2, num_circle_points=16, circle_radius=1.0, dtype="float32"):
        self.convection_scale = convection_scale
        self.second_order_scale = second_order_scale
        self.fourth_order_scale = fourth_order_scale
        self.single_channel = single_channel
        self.conservative = conservative
        self.dealiasing_fraction = dealiasing_fraction
        nc = 1 if single_channel else num_spatial_dims
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=nc, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius, dtype=dtype)

    def _build_linear_operator(self, d):
        return (-self.second_order_scale * build_laplace_operator(d, order=2)
                - self.fourth_order_scale * build_laplace_operator(d, order=4))

    def _build_nonlinear_fun(self, d):
        return ConvectionNonlinearFun(self.num_spatial_dims, self.num_points, derivative_operator=d,
                                      dealiasing_fraction=self.dealiasing_fraction, scale=self.convection_scale,
                                      single_channel=self.single_channel, conservative=self.conservative,
                                      dtype=self.dtype)


class Burgers(BaseStepper):
    """stepper/_burgers.py:8-155"""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, diffusivity=0.1, convection_scale=1.0,
                 single_channel=False, conservative=False, order=2, dealiasing_fraction=2 / 3,
                 num_circle_points=16, circle_radius=1.0, dtype="float32"):
        self.diffusivity = diffusivity
        self.convection_scale = convection_scale
        self.single_channel = single_channel
        self.conservative = conservative
        self.dealiasing_fraction = dealiasing_fraction
        nc = 1 if single_channel else num_spatial_dims
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=nc, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius, dtype=dtype)

    def _build_linear_operator(self, d):
        return self.diffusivity * build_laplace_operator(d)

    def _build_nonlinear_fun(self, d):
        return ConvectionNonlinearFun(self.num_spatial_dims, self.num_points, derivative_operator=d,
                                      dealiasing_fraction=self.dealiasing_fraction, scale=self.convection_scale,
                                      single_channel=self.single_channel, conservative=self.conservative,
                                      dtype=self.dtype)


class KortewegDeVries(BaseStepper):
    """stepper/_korteweg_de_vries.py:13-216"""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, convection_scale=-6.0, diffusivity=0.0,
                 dispersivity=1.0, hyper_diffusivity=0.01, advect_over_diffuse=False, diffuse_over_diffuse=False,
                 single_channel=False, conservative=False, order=2, dealiasing_fraction=2 / 3,
                 num_circle_points=16, circle_radius=1.0, dtype="float32"):
        self.convection_scale = convection_scale
        self.diffusivity = diffusivity
        self.dispersivity = dispersivity
        self.hyper_diffusivity = hyper_diffusivity
        self.advect_over_diffuse = advect_over_diffuse
        self.diffuse_over_diffuse = diffuse_over_diffuse
        self.single_channel = single_channel
        self.conservative = conservative
        self.dealiasing_fraction = dealiasing_fraction
        nc = 1 if single_channel else num_spatial_dims
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=nc, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius, dtype=dtype)

    def _build_linear_operator(self, d):
        vel = self.dispersivity * np.ones(self.num_spatial_dims)
        lap = build_laplace_operator(d, order=2)
        diff = self.diffusivity * lap
        if self.advect_over_diffuse:
            disp = -build_gradient_inner_product_operator(d, vel, order=1) * lap
        else:
            disp = -build_gradient_inner_product_operator(d, vel, order=3)
        if self.diffuse_over_diffuse:
            hyp = -self.hyper_diffusivity * lap * lap
        else:
            hyp = -self.hyper_diffusivity * build_laplace_operator(d, order=4)
        return diff + disp + hyp

    def _build_nonlinear_fun(self, d):
        return ConvectionNonlinearFun(self.num_spatial_dims, self.num_points, derivative_operator=d,
                                      dealiasing_fraction=self.dealiasing_fraction, scale=self.convection_scale,
                                      single_channel=self.single_channel, conservative=self.conservative,
                                      dtype=self.dtype)


class NavierStokesVorticity(BaseStepper):
    """stepper/_navier_stokes.py:13-153: L = nu*Lap + drag."""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, diffusivity=0.01,
                 vorticity_convection_scale=1.0, drag=0.0, order=2, dealiasing_fraction=2 / 3,
                 num_circle_points=16, circle_radius=1.0, dtype="float32"):
        if num_spatial_dims != 2:
            raise ValueError(f"Expected num_spatial_dims = 2, got {num_spatial_dims}. "
                             "For 3D, use NavierStokesVelocity instead.")
        self.diffusivity = diffusivity
        self.vorticity_convection_scale = vorticity_convection_scale
        self.drag = drag
        self.dealiasing_fraction = dealiasing_fraction
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=1, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius, dtype=dtype)

    def _build_linear_operator(self, d):
        return self.diffusivity * build_laplace_operator(d, order=2) + self.drag * build_laplace_operator(d, order=0)

    def _build_nonlinear_fun(self, d):
        return VorticityConvection2d(self.num_spatial_dims, self.num_points,
                                     convection_scale=self.vorticity_convection_scale, derivative_operator=d,
                                     dealiasing_fraction=self.dealiasing_fraction, dtype=self.dtype)


class KolmogorovFlowVorticity(BaseStepper):
    """stepper/_navier_stokes.py:156-327"""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, diffusivity=0.001, convection_scale=1.0,
                 drag=-0.1, injection_mode=4, injection_scale=1.0, order=2, dealiasing_fraction=2 / 3,
                 num_circle_points=16, circle_radius=1.0, dtype="float32"):
        if num_spatial_dims != 2:
            raise ValueError(f"Expected num_spatial_dims = 2, got {num_spatial_dims}. "
                             "For 3D, use KolmogorovFlowVelocity instead.")
        self.diffusivity = diffusivity
        self.convection_scale = convection_scale
        self.drag = drag
        self.injection_mode = injection_mode
        self.injection_scale = injection_scale
        self.dealiasing_fraction = dealiasing_fraction
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=1, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius, dtype=dtype)

    def _build_linear_operator(self, d):
        return self.diffusivity * build_laplace_operator(d, order=2) + self.drag * build_laplace_operator(d, order=0)

    def _build_nonlinear_fun(self, d):
        return VorticityConvection2dKolmogorov(self.num_spatial_dims, self.num_points,
                                               convection_scale=self.convection_scale,
                                               injection_mode=self.injection_mode,
                                               injection_scale=self.injection_scale, derivative_operator=d,
                                               dealiasing_fraction=self.dealiasing_fraction, dtype=self.dtype)


class NavierStokesVelocity(BaseStepper):
    """stepper/_navier_stokes.py:330-463"""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, diffusivity=0.01, drag=0.0, order=2,
                 dealiasing_fraction=2 / 3, num_circle_points=16, circle_radius=1.0, dtype="float32"):
        if num_spatial_dims != 3:
            raise ValueError(f"Expected num_spatial_dims = 3, got {num_spatial_dims}. "
                             "For 2D, use NavierStokesVorticity instead.")
        self.diffusivity = diffusivity
        self.drag = drag
        self.dealiasing_fraction = dealiasing_fraction
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=3, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius, dtype=dtype)

    def _build_linear_operator(self, d):
        return self.diffusivity * build_laplace_operator(d, order=2) + self.drag * build_laplace_operator(d, order=0)

    def _build_nonlinear_fun(self, d):
        return ProjectedConvection3d(self.num_spatial_dims, self.num_points, derivative_operator=d,
                                     dealiasing_fraction=self.dealiasing_fraction, dtype=self.dtype)


class KolmogorovFlowVelocity(BaseStepper):
    """stepper/_navier_stokes.py:466-598"""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, diffusivity=0.01, drag=0.0,
                 injection_mode=4, injection_scale=1.0, order=2, dealiasing_fraction=2 / 3,
                 num_circle_points=16, circle_radius=1.0, dtype="float32"):
        if num_spatial_dims != 3:
            raise ValueError(f"Expected num_spatial_dims = 3, got {num_spatial_dims}. "
                             "For 2D, use KolmogorovFlowVorticity instead.")
        self.diffusivity = diffusivity
        self.drag = drag
        self.injection_mode = injection_mode
        self.injection_scale = injection_scale
        self.dealiasing_fraction = dealiasing_fraction
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=3, order=order,
                         num_circle_points=num_circle_points, circle_radius=circle_radius, dtype=dtype)

    def _build_linear_operator(self, d):
        return self.diffusivity * build_laplace_operator(d, order=2) + self.drag * build_laplace_operator(d, order=0)

    def _build_nonlinear_fun(self, d):
        return ProjectedConvection3dKolmogorov(self.num_spatial_dims, self.num_points,
                                               injection_mode=self.injection_mode,
                                               injection_scale=self.injection_scale, derivative_operator=d,
                                               dealiasing_fraction=self.dealiasing_fraction, dtype=self.dtype)


class _LinearStepper(BaseStepper):
    def _build_nonlinear_fun(self, d):
        return ZeroNonlinearFun(self.num_spatial_dims, self.num_points, dtype=self.dtype)


class Advection(_LinearStepper):
    """stepper/_advection.py:13-104: L = -c . ik (ETDRK0)."""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, velocity=1.0, dtype="float32"):
        if np.isscalar(velocity):
            velocity = np.ones(num_spatial_dims) * velocity
        self.velocity = np.asarray(velocity)
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=1, order=0, dtype=dtype)

    def _build_linear_operator(self, d):
        return -build_gradient_inner_product_operator(d, self.velocity, order=1)


def _diffusivity_matrix(num_spatial_dims, diffusivity):
    """stepper/_diffusion.py:84-89"""
    if np.isscalar(diffusivity):
        return np.diag(np.ones(num_spatial_dims)) * diffusivity
    diffusivity = np.asarray(diffusivity)
    if diffusivity.ndim == 1:
        return np.diag(diffusivity)
    return diffusivity


class Diffusion(_LinearStepper):
    """stepper/_diffusion.py:12-122: L = sum_ij A_ij (ik_i)(ik_j) (ETDRK0)."""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, diffusivity=0.01, dtype="float32"):
        self.diffusivity = _diffusivity_matrix(num_spatial_dims, diffusivity)
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=1, order=0, dtype=dtype)

    def _build_linear_operator(self, d):
        outer = d[:, None] * d[None, :]
        return np.einsum("ij,ij...->...", self.diffusivity.astype(d.real.dtype), outer)[None, ...]


class AdvectionDiffusion(_LinearStepper):
    """stepper/_advection_diffusion.py:107-128"""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, velocity=1.0, diffusivity=0.01,
                 dtype="float32"):
        if np.isscalar(velocity):
            velocity = np.ones(num_spatial_dims) * velocity
        self.velocity = np.asarray(velocity)
        self.diffusivity = _diffusivity_matrix(num_spatial_dims, diffusivity)
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=1, order=0, dtype=dtype)

    def _build_linear_operator(self, d):
        outer = d[:, None] * d[None, :]
        diff = np.einsum("ij,ij...->...", self.diffusivity.astype(d.real.dtype), outer)[None, ...]
        adv = -build_gradient_inner_product_operator(d, self.velocity, order=1)
        return adv + diff


class Dispersion(_LinearStepper):
    """stepper/_dispersion.py:102-117"""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, dispersivity=1.0,
                 advect_on_diffusion=False, dtype="float32"):
        if np.isscalar(dispersivity):
            dispersivity = np.ones(num_spatial_dims) * dispersivity
        self.dispersivity = np.asarray(dispersivity)
        self.advect_on_diffusion = advect_on_diffusion
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=1, order=0, dtype=dtype)

    def _build_linear_operator(self, d):
        if self.advect_on_diffusion:
            return build_gradient_inner_product_operator(d, self.dispersivity, order=1) * build_laplace_operator(d)
        return build_gradient_inner_product_operator(d, self.dispersivity, order=3)


class HyperDiffusion(_LinearStepper):
    """stepper/_hyper_diffusion.py:95-110"""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, hyper_diffusivity=0.0001,
                 diffuse_on_diffuse=False, dtype="float32"):
        self.hyper_diffusivity = hyper_diffusivity
        self.diffuse_on_diffuse = diffuse_on_diffuse
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=1, order=0, dtype=dtype)

    def _build_linear_operator(self, d):
        if self.diffuse_on_diffuse:
            lap = build_laplace_operator(d)
            return -self.hyper_diffusivity * lap * lap
        return -self.hyper_diffusivity * build_laplace_operator(d, order=4)


class Wave(_LinearStepper):
    """stepper/_wave.py:8-197: h_tt = c^2 Lap h as the first-order system (h, v = h_t), stepped in the
    diagonalising variables w = i c |k| h (|k| guarded to 1 at k = 0), pos/neg = (w +- v)/sqrt(2) with
    the ETDRK0 factors exp(+-i c |k| dt), transformed back; the mean mode gets h += dt v."""

    def __init__(self, num_spatial_dims, domain_extent, num_points, dt, *, speed_of_sound=1.0, dtype="float32"):
        self.speed_of_sound = speed_of_sound
        self.wavenumber_norm = np.linalg.norm(
            build_scaled_wavenumbers(num_spatial_dims, domain_extent, num_points, dtype=dtype), axis=0, keepdims=True)
        super().__init__(num_spatial_dims, domain_extent, num_points, dt, num_channels=2, order=0, dtype=dtype)

    def _build_linear_operator(self, d):
        val = 1j * self.speed_of_sound * self.wavenumber_norm
        return np.concatenate((val, -val), axis=0)

    def _guard(self):
        return np.where(self.wavenumber_norm == 0, 1.0, self.wavenumber_norm).astype(self.wavenumber_norm.dtype)

    def _forward_transform(self, u_hat):
        """stepper/_wave.py:130-150"""
        h_hat, v_hat = u_hat[0:1], u_hat[1:2]
        w_hat = 1j * self.speed_of_sound * self._guard() * h_hat
        pos = (1 / np.sqrt(2)) * (w_hat + v_hat)
        neg = (1 / np.sqrt(2)) * (w_hat - v_hat)
        return np.concatenate([pos, neg], axis=0).astype(self.cd)

    def _inverse_transform(self, waves_hat):
        """stepper/_wave.py:152-160"""
        pos, neg = waves_hat[0:1], waves_hat[1:2]
        w_hat = (1 / np.sqrt(2)) * (pos + neg)
        v_hat = (1 / np.sqrt(2)) * (pos - neg)
        h_hat = w_hat / (1j * self.speed_of_sound * self._guard())
        return np.concatenate([h_hat, v_hat], axis=0).astype(self.cd)

    def step_fourier(self, u_hat):
        """stepper/_wave.py:175-197"""
        nxt = self._inverse_transform(self._integrator.step_fourier(self._forward_transform(u_hat)))
        dc = (0,) * self.num_spatial_dims
        nxt[(0,) + dc] += self.dt * u_hat[(1,) + dc]
        return nxt


class Poisson:
    """_poisson.py:14-128: -inv(Lap^(order/2)) f with a zero mean mode."""

    def __init__(self, num_spatial_dims, domain_extent, num_points, *, order=2, dtype="float32"):
        self.num_spatial_dims = num_spatial_dims
        self.num_points = num_points
        d = build_derivative_operator(num_spatial_dims, domain_extent, num_points, dtype=dtype)
        op = build_laplace_operator(d, order=order)
        with np.errstate(divide="ignore", invalid="ignore"):
            self._inv_operator = np.where(op == 0, 0.0, 1 / op).astype(op.dtype)

    def step_fourier(self, f_hat):
        return -self._inv_operator * f_hat

    def __call__(self, f):
        f_hat = fft(f, num_spatial_dims=self.num_spatial_dims)
        return ifft(self.step_fourier(f_hat), num_spatial_dims=self.num_spatial_dims, num_points=self.num_points)


# --------------------------------------------------------------------------
# time loops                    exponax/_utils.py, exponax/_repeated_stepper.py
# --------------------------------------------------------------------------


def rollout(stepper_fn, n, *, include_init=False, takes_aux=False, constant_aux=True):
    """_utils.py:92-186: stack of n successive states; with takes_aux the
    callable is (u0, aux) and stepper_fn(u, aux_t), aux_t = aux (constant_aux)
    or aux[t] (:137-163)."""

    def run(u0, aux=None):
        u = u0
        out = [u0] if include_init else []
        for t in range(n):
            if takes_aux:
                u = stepper_fn(u, aux if constant_aux else aux[t])
            else:
                u = stepper_fn(u)
            out.append(u)
        return np.stack(out)

    return run


def repeat(stepper_fn, n, *, takes_aux=False, constant_aux=True):
    """_utils.py:189-254: final state after n steps (aux as in rollout, :212-229)."""

    def run(u0, aux=None):
        u = u0
        for t in range(n):
            if takes_aux:
                u = stepper_fn(u, aux if constant_aux else aux[t])
            else:
                u = stepper_fn(u)
        return u

    return run


class ForcedStepper:
    """_forced_stepper.py:7-108: u_t = Lu + N(u) + f by splitting: one explicit
    Euler substep with the forcing, then the wrapped stepper."""

    def __init__(self, stepper):
        self.stepper = stepper

    def step(self, u, f):
        """:44-65"""
        return self.stepper.step(u + self.stepper.dt * f)

    def step_fourier(self, u_hat, f_hat):
        """:67-87"""
        return self.stepper.step_fourier(u_hat + self.stepper.dt * f_hat)

    def __call__(self, u, f):
        """:89-108"""
        return self.step(u, f)


class RepeatedStepper:
    """_repeated_stepper.py:9-139: n substeps kept in Fourier space."""

    def __init__(self, stepper, num_sub_steps):
        self.stepper = stepper
        self.num_sub_steps = num_sub_steps
        self.dt = stepper.dt * num_sub_steps
        self.num_spatial_dims = stepper.num_spatial_dims
        self.num_points = stepper.num_points
        self.num_channels = stepper.num_channels

    def step_fourier(self, u_hat):
        return repeat(self.stepper.step_fourier, self.num_sub_steps)(u_hat)

    def step(self, u):
        u_hat = fft(u, num_spatial_dims=self.num_spatial_dims)
        return ifft(self.step_fourier(u_hat), num_spatial_dims=self.num_spatial_dims, num_points=self.num_points)

    def __call__(self, u):
        expected = (self.num_channels,) + spatial_shape(self.num_spatial_dims, self.num_points)
        if u.shape != expected:
            raise ValueError(f"Expected shape {expected}, got {u.shape}.")
        return self.step(u)


# --------------------------------------------------------------------------
# resolution mapping and metrics
# --------------------------------------------------------------------------


class FourierInterpolator:
    """_interpolation.py:22-112: Re sum (rfftn(state) / reconstruction scaling) exp(i k . x) per channel."""

    def __init__(self, state, *, domain_extent=1.0):
        self.num_spatial_dims = state.ndim - 1
        self.num_points = state.shape[-1]
        dtype = "float64" if state.dtype == np.float64 else "float32"
        self.state_hat_scaled = fft(state, num_spatial_dims=self.num_spatial_dims) / build_scaling_array(
            self.num_spatial_dims, self.num_points, mode="reconstruction", dtype=dtype)
        self.wavenumbers = build_scaled_wavenumbers(self.num_spatial_dims, domain_extent, self.num_points, dtype=dtype)

    def __call__(self, x):
        D = self.num_spatial_dims
        xb = np.asarray(x, dtype=self.wavenumbers.dtype).reshape((D,) + (1,) * D)
        e = np.exp(np.sum(1j * self.wavenumbers * xb, axis=0))[None]
        return np.real(np.sum((self.state_hat_scaled * e).reshape(self.state_hat_scaled.shape[0], -1), axis=1))


def map_between_resolutions(state, new_num_points, *, oddball_zero=True):
    """_interpolation.py:195-285"""
    D = state.ndim - 1
    old = state.shape[-1]
    C = state.shape[0]
    if old == new_num_points:
        return state
    dtype = "float64" if state.dtype == np.float64 else "float32"
    old_hat = fft(state, num_spatial_dims=D) / build_scaling_array(D, old, mode="norm_compensation", dtype=dtype)
    if new_num_points > old and old % 2 == 0 and oddball_zero:
        old_hat = old_hat * oddball_filter_mask(D, old)
    new_hat = np.zeros((C,) + wavenumber_shape(D, new_num_points), dtype=old_hat.dtype)
    for sl in get_modes_slices(D, min(old, new_num_points)):
        new_hat[sl] = old_hat[sl]
    new_hat = new_hat * build_scaling_array(D, new_num_points, mode="norm_compensation", dtype=dtype)
    if old > new_num_points and new_num_points % 2 == 0 and oddball_zero:
        new_hat = new_hat * oddball_filter_mask(D, new_num_points)
    return ifft(new_hat, num_spatial_dims=D, num_points=new_num_points)


def validate_normalization_options(*, zero_mean, std_one, max_one):
    """ic/_base_ic.py:8-13"""
    if not zero_mean and std_one:
        raise ValueError("Cannot have `zero_mean=False` and `std_one=True`.")
    if std_one and max_one:
        raise ValueError("Cannot have `std_one=True` and `max_one=True`.")


def normalize_ic(ic, *, zero_mean=True, std_one=False, max_one=False):
    """ic/_base_ic.py:18-32: mean over all entries, then std (population) or max |u|."""
    if zero_mean:
        ic = ic - np.mean(ic)
    if std_one:
        ic = ic / np.std(ic)
    if max_one:
        ic = ic / np.max(np.abs(ic))
    return ic


def truncated_fourier_series_from_noise(noise, *, num_spatial_dims, cutoff=5, offset=0.0, zero_mean=True,
                                        std_one=False, max_one=False):
    """ic/_truncated_fourier_series.py:65-100 on a given white-noise field (1, N, ..., N): rfftn, the
    hypercube low-pass |k_d| <= cutoff, the first coefficient set to `offset`, irfftn, normalize_ic."""
    D = num_spatial_dims
    N = noise.shape[-1]
    dtype = "float64" if noise.dtype == np.float64 else "float32"
    hat = fft(noise, num_spatial_dims=D) * low_pass_filter_mask(D, N, cutoff=cutoff, axis_separate=True, dtype=dtype)
    shape = hat.shape
    hat = hat.reshape(-1)
    hat[0] = offset
    ic = ifft(hat.reshape(shape), num_spatial_dims=D, num_points=N)
    return normalize_ic(ic, zero_mean=zero_mean, std_one=std_one, max_one=max_one)


def gaussian_random_field_from_noise(noise, *, num_spatial_dims, domain_extent=1.0, powerlaw_exponent=3.0,
                                     zero_mean=True, std_one=False, max_one=False):
    """ic/_gaussian_random_field.py:60-93 applied to a given white-noise field (1, N, ..., N):
    rfftn, times |k|^(-p/2) of the scaled wavenumbers (1 at k = 0), irfftn, normalize_ic."""
    D = num_spatial_dims
    N = noise.shape[-1]
    dtype = "float64" if noise.dtype == np.float64 else "float32"
    noise_hat = fft(noise, num_spatial_dims=D)
    k = build_scaled_wavenumbers(D, domain_extent, N, dtype=dtype)
    knorm = np.linalg.norm(k, axis=0, keepdims=True)
    with np.errstate(divide="ignore"):
        amp = np.power(knorm, -powerlaw_exponent / 2.0)
    amp = amp.reshape(-1)
    amp[0] = 1.0
    amp = amp.reshape(knorm.shape)
    ic = ifft(noise_hat * amp, num_spatial_dims=D, num_points=N)
    return normalize_ic(ic, zero_mean=zero_mean, std_one=std_one, max_one=max_one)


def diffused_noise_from_noise(noise, *, num_spatial_dims, domain_extent=1.0, intensity=0.001, zero_mean=True,
                              std_one=False, max_one=False):
    """ic/_diffused_noise.py:60-76 applied to a given white-noise field: one Diffusion step of
    dt = 1 with diffusivity = intensity, then normalize_ic."""
    N = noise.shape[-1]
    dtype = "float64" if noise.dtype == np.float64 else "float32"
    st = Diffusion(num_spatial_dims, domain_extent, N, 1.0, diffusivity=intensity, dtype=dtype)
    return normalize_ic(st(noise), zero_mean=zero_mean, std_one=std_one, max_one=max_one)


def nRMSE(u_pred, u_ref, *, domain_extent=1.0):
    """metrics/_spatial.py:537-586 via spatial_norm(mode='normalized') :84-200:
    per-channel ratio of L2 norms, summed over channels."""
    D = u_pred.ndim - 1
    N = u_pred.shape[-1]
    scale = (domain_extent / N) ** D
    tot = 0.0
    for c in range(u_pred.shape[0]):
        num = np.sqrt(scale * np.sum(np.abs(u_pred[c] - u_ref[c]) ** 2))
        den = np.sqrt(scale * np.sum(np.abs(u_ref[c]) ** 2))
        tot = tot + num / den
    return tot


def spatial_aggregator(state_no_channel, *, num_spatial_dims=None, domain_extent=1.0, num_points=None,
                       inner_exponent=2.0, outer_exponent=None):
    """metrics/_spatial.py:8-83: (scale * sum |u|^p)^q, scale = (L/N)^D."""
    if num_spatial_dims is None:
        num_spatial_dims = state_no_channel.ndim
    if num_points is None:
        num_points = state_no_channel.shape[-1]
    if outer_exponent is None:
        outer_exponent = 1 / inner_exponent
    scale = (domain_extent / num_points) ** num_spatial_dims
    return (scale * np.sum(np.abs(state_no_channel) ** inner_exponent)) ** outer_exponent


def spatial_norm(state, state_ref=None, *, mode="absolute", domain_extent=1.0, inner_exponent=2.0,
                 outer_exponent=None):
    """metrics/_spatial.py:86-195: per-channel aggregations (absolute / normalized / symmetric), summed."""
    if state_ref is None:
        if mode in ("normalized", "symmetric"):
            raise ValueError(f"mode '{mode}' requires state_ref")
        diff = state
    else:
        diff = state - state_ref
    kw = dict(domain_extent=domain_extent, inner_exponent=inner_exponent, outer_exponent=outer_exponent)
    dn = np.array([spatial_aggregator(d, **kw) for d in diff])
    if mode == "normalized":
        return np.sum(dn / np.array([spatial_aggregator(r, **kw) for r in state_ref]))
    if mode == "symmetric":
        sn = np.array([spatial_aggregator(x, **kw) for x in state])
        rn = np.array([spatial_aggregator(r, **kw) for r in state_ref])
        return np.sum(2 * dn / (sn + rn))
    return np.sum(dn)


def _spatial_metric(mode, p, q):
    def metric(u_pred, u_ref=None, *, domain_extent=1.0):
        return spatial_norm(u_pred, u_ref, mode=mode, domain_extent=domain_extent, inner_exponent=p,
                            outer_exponent=q)
    return metric


# metrics/_spatial.py:198-634
MAE = _spatial_metric("absolute", 1.0, 1.0)
nMAE = _spatial_metric("normalized", 1.0, 1.0)
sMAE = _spatial_metric("symmetric", 1.0, 1.0)
MSE = _spatial_metric("absolute", 2.0, 1.0)
nMSE = _spatial_metric("normalized", 2.0, 1.0)
sMSE = _spatial_metric("symmetric", 2.0, 1.0)
RMSE = _spatial_metric("absolute", 2.0, 0.5)
sRMSE = _spatial_metric("symmetric", 2.0, 0.5)


def fourier_aggregator(state_no_channel, *, num_spatial_dims=None, domain_extent=1.0, num_points=None,
                       inner_exponent=2.0, outer_exponent=None, low=None, high=None, derivative_order=None):
    """metrics/_fourier.py:15-140"""
    if num_spatial_dims is None:
        num_spatial_dims = state_no_channel.ndim
    if num_points is None:
        num_points = state_no_channel.shape[-1]
    if outer_exponent is None:
        outer_exponent = 1 / inner_exponent
    dtype = "float64" if state_no_channel.dtype == np.float64 else "float32"
    uh = fft(state_no_channel, num_spatial_dims=num_spatial_dims)
    uh = np.where(np.abs(uh) < 1e-5, np.zeros_like(uh), uh)
    if low is not None or high is not None:
        low = 0 if low is None else low
        high = (num_points // 2) + 1 if high is None else high
        low_mask = low_pass_filter_mask(num_spatial_dims, num_points, cutoff=low - 1, dtype=dtype)
        high_mask = low_pass_filter_mask(num_spatial_dims, num_points, cutoff=high, dtype=dtype)
        uh = uh * (np.invert(low_mask) & high_mask)[0]
    if derivative_order is not None:
        d = build_derivative_operator(num_spatial_dims, domain_extent, num_points, dtype=dtype)
        comps = uh * d ** derivative_order
    else:
        comps = uh[None]
    recon = build_scaling_array(num_spatial_dims, num_points, mode="reconstruction", dtype=dtype)[0]
    scale = (domain_extent / num_points) ** num_spatial_dims
    return np.sum([(scale * np.sum(np.abs(c) ** inner_exponent / recon)) ** outer_exponent for c in comps])


def fourier_norm(state, state_ref=None, *, mode="absolute", domain_extent=1.0, inner_exponent=2.0,
                 outer_exponent=None, low=None, high=None, derivative_order=None):
    """metrics/_fourier.py:143-235"""
    if state_ref is None:
        if mode == "normalized":
            raise ValueError("mode 'normalized' requires state_ref")
        diff = state
    else:
        diff = state - state_ref
    kw = dict(domain_extent=domain_extent, inner_exponent=inner_exponent, outer_exponent=outer_exponent, low=low,
              high=high, derivative_order=derivative_order)
    dn = np.array([fourier_aggregator(x, **kw) for x in diff])
    if mode == "normalized":
        return np.sum(dn / np.array([fourier_aggregator(r, **kw) for r in state_ref]))
    return np.sum(dn)


def _fourier_metric(mode, p, q):
    def metric(u_pred, u_ref=None, *, domain_extent=1.0, low=None, high=None, derivative_order=None):
        return fourier_norm(u_pred, u_ref, mode=mode, domain_extent=domain_extent, inner_exponent=p,
                            outer_exponent=q, low=low, high=high, derivative_order=derivative_order)
    return metric


# metrics/_fourier.py:238-592
fourier_MAE = _fourier_metric("absolute", 1.0, 1.0)
fourier_nMAE = _fourier_metric("normalized", 1.0, 1.0)
fourier_MSE = _fourier_metric("absolute", 2.0, 1.0)
fourier_nMSE = _fourier_metric("normalized", 2.0, 1.0)
fourier_RMSE = _fourier_metric("absolute", 2.0, 0.5)
fourier_nRMSE = _fourier_metric("normalized", 2.0, 0.5)


def _h1(fm):
    def metric(u_pred, u_ref=None, *, domain_extent=1.0, low=None, high=None):
        kw = dict(domain_extent=domain_extent, low=low, high=high)
        return fm(u_pred, u_ref, derivative_order=None, **kw) + fm(u_pred, u_ref, derivative_order=1, **kw)
    return metric


# metrics/_derivative.py:13-368: the Fourier metric plus that of the first derivative
H1_MAE = _h1(fourier_MAE)
H1_nMAE = _h1(fourier_nMAE)
H1_MSE = _h1(fourier_MSE)
H1_nMSE = _h1(fourier_nMSE)
H1_RMSE = _h1(fourier_RMSE)
H1_nRMSE = _h1(fourier_nRMSE)


def correlation(u_pred, u_ref):
    """metrics/_correlation.py:33-60: channel-mean of normalised inner products."""
    vals = []
    for c in range(u_pred.shape[0]):
        a = u_pred[c] / np.linalg.norm(u_pred[c])
        b = u_ref[c] / np.linalg.norm(u_ref[c])
        vals.append(np.dot(a.ravel(), b.ravel()))
    return np.mean(vals)
