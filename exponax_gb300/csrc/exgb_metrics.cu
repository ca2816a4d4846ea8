// exgb_metrics.cu -- evaluation kernels on device fields: the radially binned
// power / amplitude spectrum (reference _spectral.py:866-1030, get_spectrum),
// the per-field sums behind nRMSE (metrics/_spatial.py:537-586) and
// correlation (metrics/_correlation.py:33-60), and the p-norm aggregations of
// the spatial, Fourier and H1 metric families (metrics/_spatial.py,
// _fourier.py, _derivative.py).
//
// Spectrum of one field from its rfftn (N..., N/2+1 modes):
//   power:      q = 0.5 * (|u^| / recon) * (|u^| / norm)
//   amplitude:  q = |u^| / recon
// with norm = N^D on every mode and recon = N^D / 2 on the rfft-axis modes
// 0 < k < N/2 (N^D on k = 0 and, for even N, k = N/2) -- the reference's
// "reconstruction" / "norm_compensation" scaling arrays, evaluated in FP32.
// 1D: q itself.  D >= 2: bin i in [0, N/2] sums (or averages) the q of the
// modes whose integer wavenumber norm r = sqrt(sum k_d^2) (FP32) satisfies
// i - 1/2 <= r < i + 1/2; NaN values are skipped as nansum / nanmean do, an
// empty bin averages to NaN.  Summation order differs from the reference
// (shared-memory atomics), so results agree to FP32 rounding, not bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "exgb_internal.h"

namespace exgb {

namespace {

constexpr int SPEC_THREADS = 256;
constexpr int SPEC_MAX_BINS = 2049;  // N <= 4096

__global__ void __launch_bounds__(SPEC_THREADS) spectrum_kernel(int D, int N, int64_t modes_per_field, int per_field_ctas,
                                                                 const float2* __restrict__ hat, float* sums,
                                                                 int* counts, int power) {
  extern __shared__ float s_bins[];  // [nb] sums, then [nb] counts as int
  const int M = N / 2 + 1;
  const int nb = M;
  int* s_cnt = reinterpret_cast<int*>(s_bins + nb);
  const int field = blockIdx.x / per_field_ctas;
  const int part = blockIdx.x % per_field_ctas;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    s_bins[i] = 0.f;
    s_cnt[i] = 0;
  }
  __syncthreads();
  const float nd = (D == 1) ? (float)N : (D == 2) ? (float)N * (float)N : (float)N * (float)N * (float)N;
  const float2* f = hat + (int64_t)field * modes_per_field;
  const int64_t chunk = (modes_per_field + per_field_ctas - 1) / per_field_ctas;
  const int64_t m0 = (int64_t)part * chunk;
  const int64_t m1 = min(modes_per_field, m0 + chunk);
  for (int64_t m = m0 + threadIdx.x; m < m1; m += blockDim.x) {
    const int kl = (int)(m % M);  // rfft axis
    int64_t rest = m / M;
    float r2 = (float)kl * (float)kl;
    for (int d = 0; d < D - 1; ++d) {
      const int idx = (int)(rest % N);
      rest /= N;
      const int k = (idx <= (N - 1) / 2) ? idx : idx - N;  // fftfreq
      r2 += (float)k * (float)k;
    }
    const bool full = (kl == 0) || (N % 2 == 0 && kl == N / 2);
    const float recon = full ? nd : nd / 2.f;
    const float2 v = f[m];
    const float a = hypotf(v.x, v.y);
    const float mag = a / recon;
    const float q = power ? 0.5f * mag * (a / nd) : mag;
    if (D == 1) {
      sums[(int64_t)field * nb + kl] = q;
      continue;
    }
    if (isnan(q)) continue;
    const float r = sqrtf(r2);
    int b = (int)floorf(r + 0.5f);
    if (r < (float)b - 0.5f) --b;
    if (r >= (float)b + 0.5f) ++b;
    if (b < 0 || b >= nb) continue;
    atomicAdd(&s_bins[b], q);
    atomicAdd(&s_cnt[b], 1);
  }
  __syncthreads();
  if (D == 1) return;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    if (s_cnt[i]) {
      atomicAdd(&sums[(int64_t)field * nb + i], s_bins[i]);
      atomicAdd(&counts[(int64_t)field * nb + i], s_cnt[i]);
    }
  }
}

__global__ void spectrum_average_kernel(int64_t n, float* sums, const int* counts) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) sums[i] = counts[i] ? sums[i] / (float)counts[i] : nanf("");
}

// Block sum of K per-thread values (K <= 4, blockDim.x <= 256); thread k < K gets the total of value k.
template <int K>
__device__ __forceinline__ void block_sum(float (&v)[K], float* red /* [K][8] */) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int q = 0; q < K; ++q) {
    for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_xor_sync(0xffffffffu, v[q], o);
    if (lane == 0) red[q * 8 + w] = v[q];
  }
  __syncthreads();
  if (threadIdx.x < K) {
    KahanSum t;
    for (int i = 0; i < nw; ++i) t.add(red[threadIdx.x * 8 + i]);
#pragma unroll
    for (int q = 0; q < K; ++q)
      if (q == (int)threadIdx.x) v[q] = t.s;
  }
}

// per field: sum (a-b)^2, sum b^2, sum a b, sum a^2 (one CTA per field)
__global__ void __launch_bounds__(256) field_sums_kernel(int64_t n, const float* __restrict__ a,
                                                         const float* __restrict__ b, double* out) {
  const float* pa = a + (int64_t)blockIdx.x * n;
  const float* pb = b + (int64_t)blockIdx.x * n;
  KahanSum s[4];
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    const float x = pa[i], y = pb[i];
    const float d = x - y;
    s[0].add(d * d);
    s[1].add(y * y);
    s[2].add(x * y);
    s[3].add(x * x);
  }
  __shared__ float red[4 * 8];
  float v[4] = {s[0].s, s[1].s, s[2].s, s[3].s};
  block_sum<4>(v, red);
#pragma unroll
  for (int q = 0; q < 4; ++q)
    if (q == (int)threadIdx.x) out[(int64_t)blockIdx.x * 4 + q] = (double)v[q];
}

__device__ __forceinline__ float pow_abs(float x, float p) {
  x = fabsf(x);
  return p == 1.f ? x : p == 2.f ? x * x : powf(x, p);
}

// One CTA per field of n floats: out[3 f + 0..2] = sum |a - b|^p, sum |a|^p, sum |b|^p
// (b == nullptr: the difference is a itself and the last sum is 0) -- the aggregations behind
// spatial_norm (metrics/_spatial.py:8-195), accumulated in FP64.
__global__ void __launch_bounds__(256) field_pnorms_kernel(int64_t n, const float* __restrict__ a,
                                                           const float* __restrict__ b, float p, double* out) {
  __shared__ float red[3 * 8];
  const float* fa = a + (int64_t)blockIdx.x * n;
  const float* fb = b ? b + (int64_t)blockIdx.x * n : nullptr;
  KahanSum s[3];
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    const float x = fa[i];
    const float y = fb ? fb[i] : 0.f;
    s[0].add(pow_abs(fb ? x - y : x, p));
    s[1].add(pow_abs(x, p));
    s[2].add(pow_abs(y, p));
  }
  float v[3] = {s[0].s, s[1].s, s[2].s};
  block_sum<3>(v, red);
#pragma unroll
  for (int q = 0; q < 3; ++q)
    if (q == (int)threadIdx.x) out[3 * (int64_t)blockIdx.x + q] = (double)v[q];
}

// One CTA per rfftn field (N..., N/2+1 modes): the sums of fourier_aggregator
// (metrics/_fourier.py:15-140): coefficients with |c| < 1e-5 dropped, the band
// low <= max_d |k_d| <= high kept (low_pass_filter_mask(low - 1) inverted, and
// low_pass_filter_mask(high)), each |c|^p divided by the "reconstruction" scaling
// (N^D, halved on the rfft-axis modes 0 < k < N/2).  With a derivative order a >= 0
// the sum is split per axis d and weighted by |2 pi k_d / L|^(a p) (the magnitude of
// (i k_d)^a); otherwise out has one sum per field.
__global__ void __launch_bounds__(256) fourier_pnorms_kernel(int D, int N, int64_t per, const float2* __restrict__ hat,
                                                             float p, float alpha, int use_deriv, int low, int high,
                                                             float kscale, double* out) {
  __shared__ float red[3 * 8];
  const int M = N / 2 + 1;
  const float2* h = hat + (int64_t)blockIdx.x * per;
  KahanSum s[3];
  float full = 1.f;
  for (int d = 0; d < D; ++d) full *= (float)N;
  for (int64_t r = threadIdx.x; r < per; r += blockDim.x) {
    const float2 c = h[r];
    const float m = sqrtf(c.x * c.x + c.y * c.y);
    if (m < 1e-5f) continue;
    int k[3] = {0, 0, 0};
    const int kl = (int)(r % M);
    k[D - 1] = kl;
    int64_t rest = r / M;
    for (int a = D - 2; a >= 0; --a) {
      const int i = (int)(rest % N);
      rest /= N;
      k[a] = (i <= (N - 1) / 2) ? i : i - N;
    }
    int kmax = 0;
    for (int a = 0; a < D; ++a) kmax = max(kmax, abs(k[a]));
    if (kmax < low || kmax > high) continue;
    const bool halve = kl != 0 && !((N % 2) == 0 && kl == N / 2);
    const float base = pow_abs(m, p) / (halve ? 0.5f * full : full);
    if (!use_deriv) {
      s[0].add(base);
    } else {
      for (int a = 0; a < D; ++a) s[a].add(base * powf(kscale * (float)abs(k[a]), alpha * p));
    }
  }
  float v[3] = {s[0].s, s[1].s, s[2].s};
  block_sum<3>(v, red);
  const int nout = use_deriv ? D : 1;
  for (int q = 0; q < 3; ++q)
    if (q == (int)threadIdx.x && q < nout) out[(int64_t)blockIdx.x * nout + q] = (double)v[q];
}

}  // namespace
}  // namespace exgb

using namespace exgb;

extern "C" int exgb_field_pnorms(void* stream, int64_t count, int64_t n, const float* a, const float* b, float p,
                                 double* out) {
  if (!a || !out) return fail(EXGB_EINVAL, "exgb_field_pnorms: NULL pointer");
  if (count < 0 || n < 0) return fail(EXGB_EINVAL, "exgb_field_pnorms: negative size");
  if (!(p > 0.f)) return fail(EXGB_EINVAL, "exgb_field_pnorms: the exponent must be positive");
  if (count == 0) return EXGB_OK;
  field_pnorms_kernel<<<(unsigned)count, 256, 0, (cudaStream_t)stream>>>(n, a, b, p, out);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

extern "C" int exgb_fourier_pnorms(void* stream, int num_spatial_dims, int num_points, int64_t count,
                                   const void* u_hat, float p, float derivative_order, int low, int high,
                                   float domain_extent, double* out) {
  const int D = num_spatial_dims, N = num_points;
  if (!u_hat || !out) return fail(EXGB_EINVAL, "exgb_fourier_pnorms: NULL pointer");
  if (D < 1 || D > 3 || N < 1) return fail(EXGB_ESHAPE, "exgb_fourier_pnorms: 1 to 3 axes of N >= 1 points");
  if (count < 0) return fail(EXGB_EINVAL, "exgb_fourier_pnorms: negative count");
  if (!(p > 0.f) || !(domain_extent > 0.f)) return fail(EXGB_EINVAL, "exgb_fourier_pnorms: bad exponent or extent");
  if (count == 0) return EXGB_OK;
  int64_t per = N / 2 + 1;
  for (int d = 0; d < D - 1; ++d) per *= N;
  const int use_deriv = derivative_order >= 0.f ? 1 : 0;
  const float kscale = (float)(2.0 * 3.14159265358979323846 / (double)domain_extent);
  fourier_pnorms_kernel<<<(unsigned)count, 256, 0, (cudaStream_t)stream>>>(
      D, N, per, (const float2*)u_hat, p, use_deriv ? derivative_order : 0.f, use_deriv, low, high, kscale, out);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

extern "C" int exgb_spectrum(void* stream, int num_spatial_dims, int num_points, int64_t count, const void* u_hat,
                             float* out, int power, int average) {
  const int D = num_spatial_dims, N = num_points;
  if (!u_hat || !out) return fail(EXGB_EINVAL, "exgb_spectrum: NULL pointer");
  if (D < 1 || D > 3) return fail(EXGB_ESHAPE, "exgb_spectrum: num_spatial_dims must be 1, 2 or 3");
  if (N < 2 || N / 2 + 1 > SPEC_MAX_BINS) return fail(EXGB_ESHAPE, "exgb_spectrum: num_points out of range");
  if (count < 0) return fail(EXGB_EINVAL, "exgb_spectrum: negative count");
  if (count == 0) return EXGB_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const int M = N / 2 + 1;
  int64_t modes = M;
  for (int d = 0; d < D - 1; ++d) modes *= N;
  const int64_t nout = count * M;
  int* counts = nullptr;
  if (D > 1) {
    EXGB_CUDA(cudaMemsetAsync(out, 0, sizeof(float) * nout, st));
    EXGB_CUDA(cudaMallocAsync(&counts, sizeof(int) * nout, st));
    EXGB_CUDA(cudaMemsetAsync(counts, 0, sizeof(int) * nout, st));
  }
  const int per = (int)std::max<int64_t>(1, std::min<int64_t>(64, modes / (16 * SPEC_THREADS)));
  const size_t smem = (size_t)M * (sizeof(float) + sizeof(int));
  spectrum_kernel<<<(unsigned)(count * per), SPEC_THREADS, smem, st>>>(D, N, modes, per, (const float2*)u_hat, out,
                                                                      counts, power);
  EXGB_CUDA(cudaGetLastError());
  if (D > 1) {
    if (average) {
      spectrum_average_kernel<<<(unsigned)((nout + 255) / 256), 256, 0, st>>>(nout, out, counts);
      EXGB_CUDA(cudaGetLastError());
    }
    EXGB_CUDA(cudaFreeAsync(counts, st));
  }
  return EXGB_OK;
}

extern "C" int exgb_field_sums(void* stream, int64_t count, int64_t n, const float* a, const float* b, double* out) {
  if (!a || !b || !out) return fail(EXGB_EINVAL, "exgb_field_sums: NULL pointer");
  if (count < 0 || n < 0) return fail(EXGB_EINVAL, "exgb_field_sums: negative size");
  if (count == 0) return EXGB_OK;
  field_sums_kernel<<<(unsigned)count, 256, 0, (cudaStream_t)stream>>>(n, a, b, out);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}
