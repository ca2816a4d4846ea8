// exgb_util.cu -- small device helpers behind the Python surface:
//   exgb_axpy             out = x + alpha y (ForcedStepper's explicit forcing
//                         substep, reference _forced_stepper.py:64-65, :86-87)
//   exgb_scatter_modes    zero `count` Fourier fields and write per-field
//                         values at fixed mode positions (random-series ICs)
//   exgb_normalize_fields subtract the mean, then divide by the standard deviation or by max |u|, per field
//                         (reference ic/_base_ic.py:18-32, normalize_ic)
//   exgb_mode_scale       multiply Fourier fields by a per-mode complex table (Poisson.step_fourier,
//                         reference _poisson.py:67-82)
//   exgb_mode_mix2        per-mode real 2x2 map of two-channel Fourier fields, repeated (Wave,
//                         reference stepper/_wave.py)
//   exgb_spectral_derivative, exgb_make_incompressible
//                         spectral.derivative and spectral.make_incompressible in Fourier space
//                         (reference _spectral.py:724-863)
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "exgb_internal.h"

namespace exgb {
namespace {

__global__ void axpy_kernel(int64_t n, float alpha, const float* __restrict__ x, const float* __restrict__ y,
                            float* out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = fmaf(alpha, y[i], x[i]);
}

__global__ void scatter_kernel(int64_t count, int64_t field_elems, int nmodes, const int64_t* __restrict__ idx,
                               const float2* __restrict__ vals, float2* hat) {
  const int64_t n = count * nmodes;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t f = i / nmodes;
    const int m = (int)(i - f * nmodes);
    hat[f * field_elems + idx[m]] = vals[i];
  }
}

// one CTA per field: the mean, then (std_one) the population standard deviation or (max_one)
// max |u - mean|, then (u - mean) * scale with the mean subtracted only when zero_mean -- normalize_ic
// (ic/_base_ic.py:18-32) in its order; std_one without zero_mean divides by the standard deviation
// alone, as SineWaves1d does (ic/_sine_waves_1d.py:72-77).  FP32 sums with Kahan compensation.
__device__ __forceinline__ float block_total(float v, float* red) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) red[w] = v;
  __syncthreads();
  KahanSum t;
  for (int i = 0; i < nw; ++i) t.add(red[i]);
  __syncthreads();  // red may be reused by the caller
  return t.s;
}

__global__ void __launch_bounds__(256) normalize_kernel(int64_t n, float* u, int zero_mean, int std_one,
                                                        int max_one) {
  float* p = u + (int64_t)blockIdx.x * n;
  __shared__ float red[8];
  __shared__ float redf[8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  KahanSum s;
  if (zero_mean || std_one)
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s.add(p[i]);
  const float fmean = block_total(s.s, red) / (float)n;
  const float mean = zero_mean ? fmean : 0.f;
  float inv = 1.f;
  if (std_one) {
    KahanSum q;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
      const float d = p[i] - fmean;
      q.add(d * d);
    }
    const float sd = sqrtf(block_total(q.s, red) / (float)n);
    if (sd > 0.f) inv = 1.f / sd;
  }
  float mx = 0.f;
  if (max_one)
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) mx = fmaxf(mx, fabsf(p[i] - mean));
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (lane == 0) redf[w] = mx;
  __syncthreads();
  float m = 0.f;
  for (int i = 0; i < nw; ++i) m = fmaxf(m, redf[i]);
  if (max_one && m > 0.f) inv = 1.f / m;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) p[i] = (p[i] - mean) * inv;
}

// out[f][r] = table[r] * in[f][r] over count fields of `per` complex modes
__global__ void mode_scale_kernel(int64_t count, int64_t per, const float2* __restrict__ table,
                                  const float2* __restrict__ in, float2* __restrict__ out) {
  const int64_t n = count * per;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = cmul(__ldg(table + i % per), in[i]);
}

// Two-channel fields (h, v) per sample: (h, v) <- M(r) (h, v) nsteps times, M real [4][per] row-major
// per mode (m00, m01, m10, m11), state in registers between steps
__global__ void mode_mix2_kernel(int64_t count, int64_t per, const float* __restrict__ mat,
                                 const float2* __restrict__ in, float2* __restrict__ out, int nsteps) {
  const int64_t n = count * per;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i / per, r = i - b * per;
    const float m00 = __ldg(mat + r), m01 = __ldg(mat + per + r);
    const float m10 = __ldg(mat + 2 * per + r), m11 = __ldg(mat + 3 * per + r);
    const int64_t o = b * 2 * per + r;
    float2 h = in[o], v = in[o + per];
    for (int s = 0; s < nsteps; ++s) {
      const float2 h2 = make_float2(fmaf(m00, h.x, m01 * v.x), fmaf(m00, h.y, m01 * v.y));
      v = make_float2(fmaf(m10, h.x, m11 * v.x), fmaf(m10, h.y, m11 * v.y));
      h = h2;
    }
    out[o] = h;
    out[o + per] = v;
  }
}

// signed integer wavenumbers of rfftn mode r of an (N..., N/2+1) field with D axes ('ij', rfftfreq last)
__device__ __forceinline__ void mode_wavenumbers(int D, int N, int64_t r, int (&k)[3]) {
  const int M = N / 2 + 1;
  k[0] = k[1] = k[2] = 0;
  k[D - 1] = (int)(r % M);
  int64_t rest = r / M;
  for (int a = D - 2; a >= 0; --a) {
    const int i = (int)(rest % N);
    rest /= N;
    k[a] = (i <= (N - 1) / 2) ? i : i - N;
  }
}

// (i k)^order u^ for every axis: out[f][d][r] = (i kscale k_d)^order in[f][r] (spectral.derivative,
// reference _spectral.py:724-791); the integer power is taken by repeated multiplication
__global__ void derivative_kernel(int D, int N, int64_t count, int64_t per, int order, float kscale,
                                  const float2* __restrict__ in, float2* __restrict__ out) {
  const int64_t n = count * per;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t f = i / per, r = i - f * per;
    int k[3];
    mode_wavenumbers(D, N, r, k);
    const float2 u = in[i];
    for (int d = 0; d < D; ++d) {
      const float2 ik = make_float2(0.f, kscale * (float)k[d]);
      float2 m = make_float2(1.f, 0.f);
      for (int q = 0; q < order; ++q) m = cmul(m, ik);
      out[(f * D + d) * per + r] = cmul(m, u);
    }
  }
}

// Leray projection of count samples of D velocity spectra (make_incompressible, _spectral.py:794-863):
// div = sum_d i k_d u_d, p = div / Lap (1 / Lap taken as 1 where Lap = 0), u_d -= i k_d p
__global__ void incompressible_kernel(int D, int N, int64_t count, int64_t per, float kscale,
                                      const float2* __restrict__ in, float2* __restrict__ out) {
  const int64_t n = count * per;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i / per, r = i - b * per;
    int k[3];
    mode_wavenumbers(D, N, r, k);
    float ks[3];
    float lap = 0.f;
    float2 div = make_float2(0.f, 0.f);
    for (int d = 0; d < D; ++d) {
      ks[d] = kscale * (float)k[d];
      lap -= ks[d] * ks[d];
      const float2 u = in[(b * D + d) * per + r];
      div = cadd(div, make_float2(-ks[d] * u.y, ks[d] * u.x));
    }
    const float il = (lap == 0.f) ? 1.f : 1.f / lap;
    const float2 pp = cscale(div, il);
    for (int d = 0; d < D; ++d) {
      const float2 u = in[(b * D + d) * per + r];
      out[(b * D + d) * per + r] = csub(u, make_float2(-ks[d] * pp.y, ks[d] * pp.x));
    }
  }
}

int grid_for(int64_t n) { return (int)std::min<int64_t>((n + 255) / 256, 152 * 16); }

}  // namespace
}  // namespace exgb

using namespace exgb;

extern "C" int exgb_axpy(void* stream, int64_t n, float alpha, const float* x, const float* y, float* out) {
  if (n < 0) return fail(EXGB_EINVAL, "exgb_axpy: negative size");
  if (n == 0) return EXGB_OK;
  if (!x || !y || !out) return fail(EXGB_EINVAL, "exgb_axpy: NULL pointer");
  axpy_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(n, alpha, x, y, out);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

extern "C" int exgb_scatter_modes(void* stream, int64_t count, int64_t field_elems, int nmodes, const int64_t* idx,
                                  const void* vals, void* hat) {
  if (!idx || !vals || !hat) return fail(EXGB_EINVAL, "exgb_scatter_modes: NULL pointer");
  if (count < 0 || field_elems <= 0 || nmodes < 0) return fail(EXGB_EINVAL, "exgb_scatter_modes: bad size");
  cudaStream_t st = (cudaStream_t)stream;
  EXGB_CUDA(cudaMemsetAsync(hat, 0, sizeof(float2) * (size_t)(count * field_elems), st));
  if (count == 0 || nmodes == 0) return EXGB_OK;
  scatter_kernel<<<grid_for(count * nmodes), 256, 0, st>>>(count, field_elems, nmodes, idx, (const float2*)vals,
                                                          (float2*)hat);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

extern "C" int exgb_normalize_fields(void* stream, int64_t count, int64_t n, float* u, int zero_mean, int std_one,
                                     int max_one) {
  if (count < 0 || n <= 0) return fail(EXGB_EINVAL, "exgb_normalize_fields: bad size");
  if (std_one && max_one) return fail(EXGB_EINVAL, "Cannot have `std_one=True` and `max_one=True`.");
  if (count == 0) return EXGB_OK;
  if (!u) return fail(EXGB_EINVAL, "exgb_normalize_fields: NULL pointer");
  if (count > 2147483647LL) return fail(EXGB_EINVAL, "exgb_normalize_fields: too many fields for one launch");
  normalize_kernel<<<(unsigned)count, 256, 0, (cudaStream_t)stream>>>(n, u, zero_mean, std_one, max_one);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

extern "C" int exgb_mode_scale(void* stream, int64_t count, int64_t per, const void* table, const void* in,
                               void* out) {
  if (count < 0 || per <= 0) return fail(EXGB_EINVAL, "exgb_mode_scale: bad size");
  if (count == 0) return EXGB_OK;
  if (!table || !in || !out) return fail(EXGB_EINVAL, "exgb_mode_scale: NULL pointer");
  mode_scale_kernel<<<grid_for(count * per), 256, 0, (cudaStream_t)stream>>>(
      count, per, (const float2*)table, (const float2*)in, (float2*)out);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

extern "C" int exgb_mode_mix2(void* stream, int64_t count, int64_t per, const float* mat, const void* in, void* out,
                              int nsteps) {
  if (count < 0 || per <= 0 || nsteps < 0) return fail(EXGB_EINVAL, "exgb_mode_mix2: bad size");
  if (count == 0) return EXGB_OK;
  if (!mat || !in || !out) return fail(EXGB_EINVAL, "exgb_mode_mix2: NULL pointer");
  mode_mix2_kernel<<<grid_for(count * per), 256, 0, (cudaStream_t)stream>>>(
      count, per, mat, (const float2*)in, (float2*)out, nsteps);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

static int64_t modes_per_field(int D, int N) {
  int64_t per = N / 2 + 1;
  for (int d = 0; d < D - 1; ++d) per *= N;
  return per;
}

extern "C" int exgb_spectral_derivative(void* stream, int num_spatial_dims, int num_points, int64_t count,
                                        int order, float domain_extent, const void* in, void* out) {
  const int D = num_spatial_dims, N = num_points;
  if (D < 1 || D > 3 || N < 1) return fail(EXGB_ESHAPE, "exgb_spectral_derivative: 1 to 3 axes of N >= 1 points");
  if (count < 0 || order < 0 || !(domain_extent > 0.f)) return fail(EXGB_EINVAL, "exgb_spectral_derivative: bad arguments");
  if (count == 0) return EXGB_OK;
  if (!in || !out) return fail(EXGB_EINVAL, "exgb_spectral_derivative: NULL pointer");
  const int64_t per = modes_per_field(D, N);
  const float ks = (float)(2.0 * 3.14159265358979323846 / (double)domain_extent);
  derivative_kernel<<<grid_for(count * per), 256, 0, (cudaStream_t)stream>>>(D, N, count, per, order, ks,
                                                                             (const float2*)in, (float2*)out);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

extern "C" int exgb_make_incompressible(void* stream, int num_spatial_dims, int num_points, int64_t count,
                                        const void* in, void* out) {
  const int D = num_spatial_dims, N = num_points;
  if (D < 1 || D > 3 || N < 1) return fail(EXGB_ESHAPE, "exgb_make_incompressible: 1 to 3 axes of N >= 1 points");
  if (count < 0) return fail(EXGB_EINVAL, "exgb_make_incompressible: negative count");
  if (count == 0) return EXGB_OK;
  if (!in || !out) return fail(EXGB_EINVAL, "exgb_make_incompressible: NULL pointer");
  const int64_t per = modes_per_field(D, N);
  // the projection does not depend on the domain extent: the reference evaluates it with L = 1
  const float ks = (float)(2.0 * 3.14159265358979323846);
  incompressible_kernel<<<grid_for(count * per), 256, 0, (cudaStream_t)stream>>>(D, N, count, per, ks,
                                                                                 (const float2*)in, (float2*)out);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}
