// exgb_fftnd.cu -- batched real FFTs over the last D axes (rfftn / irfftn
// with the reference's conventions), the spectral re-sampling of
// map_between_resolutions, and a grow-only device workspace.
//
// Layout: rows are contiguous; two real rows are packed into one complex
// FFT (z = a + i b) and separated afterwards.  Leading axes are transformed
// by a strided complex FFT kernel that loads tiles of TI contiguous
// positions (coalesced 8*TI-byte segments per element row).
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "exgb_internal.h"

namespace exgb {

// ---------------------------------------------------------------- workspace
// Grow-only buffers per device: 0 = inverse-transform intermediate,
// 1 = re-sampling spectra / 1D work items, 2 = Fourier state of the
// physical-space entry points, 3 = rollout frame, 4 = 3D stage buffers.  Growing
// calls cudaFree/cudaMalloc (device-synchronising); the steady state does
// not allocate.
static std::mutex g_ws_mu;
static void* g_ws[128] = {nullptr};
static size_t g_ws_bytes[128] = {0};

void* workspace(size_t bytes, int slot_offset = 0) {
  int dev = 0;
  cudaGetDevice(&dev);
  const int slot = (dev % 16) * 8 + slot_offset;
  std::lock_guard<std::mutex> lk(g_ws_mu);
  if (g_ws_bytes[slot] < bytes) {
    if (g_ws[slot]) cudaFree(g_ws[slot]);
    g_ws[slot] = nullptr;
    g_ws_bytes[slot] = 0;
    void* p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
    g_ws[slot] = p;
    g_ws_bytes[slot] = bytes;
  }
  return g_ws[slot];
}

static inline size_t smem_optin_limit() {
  static size_t lim = 0;
  if (!lim) {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    lim = (size_t)v;
  }
  return lim;
}

// ---------------------------------------------------------------- row r2c
// Each CTA transforms `pairs` pairs of real rows (2*pairs rows).
__global__ void rfft_rows_kernel(FftPlan fp, const float2* __restrict__ tw, int64_t rows, int pairs,
                                 const float* __restrict__ in, float2* __restrict__ out) {
  extern __shared__ float2 smem[];
  const int n = fp.n, M = n / 2 + 1;
  float2* buf0 = smem;
  float2* buf1 = smem + (size_t)pairs * n;
  const int64_t row0 = (int64_t)blockIdx.x * pairs * 2;
  for (int t = threadIdx.x; t < pairs * n; t += blockDim.x) {
    const int p = t / n, x = t - p * n;
    const int64_t ra = row0 + 2 * p, rb = ra + 1;
    const float a = ra < rows ? in[ra * n + x] : 0.f;
    const float b = rb < rows ? in[rb * n + x] : 0.f;
    buf0[t] = make_float2(a, b);
  }
  __syncthreads();
  float2* res = (fp.npass & 1) ? buf1 : buf0;
  block_fft<false>(fp, buf0, buf1, LinMap{res, n}, pairs, tw, threadIdx.x, blockDim.x, BlockSync{});
  for (int t = threadIdx.x; t < pairs * M; t += blockDim.x) {
    const int p = t / M, k = t - p * M;
    const int64_t ra = row0 + 2 * p, rb = ra + 1;
    float2 P, Q;
    unpack_pair(res[p * n + k], res[p * n + (k == 0 ? 0 : n - k)], P, Q);
    if (ra < rows) out[ra * M + k] = P;
    if (rb < rows) out[rb * M + k] = Q;
  }
}

// ---------------------------------------------------------------- row c2r
__global__ void irfft_rows_kernel(FftPlan fp, const float2* __restrict__ tw, int64_t rows, int pairs,
                                  const float2* __restrict__ in, float* __restrict__ out, float scale) {
  extern __shared__ float2 smem[];
  const int n = fp.n, M = n / 2 + 1;
  float2* buf0 = smem;
  float2* buf1 = smem + (size_t)pairs * n;
  const int64_t row0 = (int64_t)blockIdx.x * pairs * 2;
  const bool even = (n % 2) == 0;
  for (int t = threadIdx.x; t < pairs * n; t += blockDim.x) {
    const int p = t / n, k = t - p * n;
    const int64_t ra = row0 + 2 * p, rb = ra + 1;
    const bool ext = k >= M;
    const int kk = ext ? n - k : k;
    const bool real_only = (k == 0) || (even && k == n / 2);
    const float2 a = ra < rows ? in[ra * M + kk] : make_float2(0.f, 0.f);
    const float2 b = rb < rows ? in[rb * M + kk] : make_float2(0.f, 0.f);
    buf0[t] = pack_pair(a, b, ext, real_only);
  }
  __syncthreads();
  float2* res = (fp.npass & 1) ? buf1 : buf0;
  block_fft<true>(fp, buf0, buf1, LinMap{res, n}, pairs, tw, threadIdx.x, blockDim.x, BlockSync{});
  for (int t = threadIdx.x; t < pairs * n; t += blockDim.x) {
    const int p = t / n, x = t - p * n;
    const int64_t ra = row0 + 2 * p, rb = ra + 1;
    const float2 z = res[t];
    if (ra < rows) out[ra * n + x] = z.x * scale;
    if (rb < rows) out[rb * n + x] = z.y * scale;
  }
}

// ---------------------------------------------------------------- strided axis c2c
// Element k of the sequence at (o, i) lives at o*outer_stride + i + k*es.
// CTA (blockIdx.x = tile of TI inner positions, blockIdx.y = outer).
template <bool INV>
__global__ void cfft_axis_kernel(FftPlan fp, const float2* __restrict__ tw, int64_t outer_stride, int64_t inner,
                                 int64_t es, int TI, const float2* in, float2* out, float scale) {
  extern __shared__ float2 smem[];
  const int n = fp.n;
  float2* buf0 = smem;
  float2* buf1 = smem + (size_t)TI * n;
  const int64_t o = blockIdx.y;
  const int64_t i0 = (int64_t)blockIdx.x * TI;
  const int ti = (inner - i0) < (int64_t)TI ? (int)(inner - i0) : TI;
  const float2* src = in + o * outer_stride + i0;
  for (int t = threadIdx.x; t < TI * n; t += blockDim.x) {
    const int k = t / TI, ii = t - k * TI;
    buf0[ii * n + k] = ii < ti ? src[(int64_t)k * es + ii] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  float2* res = (fp.npass & 1) ? buf1 : buf0;
  block_fft<INV>(fp, buf0, buf1, LinMap{res, n}, TI, tw, threadIdx.x, blockDim.x, BlockSync{});
  float2* dst = out + o * outer_stride + i0;
  for (int t = threadIdx.x; t < TI * n; t += blockDim.x) {
    const int k = t / TI, ii = t - k * TI;
    if (ii < ti) dst[(int64_t)k * es + ii] = cscale(res[ii * n + k], scale);
  }
}

static int set_smem(const void* fn, size_t bytes) {
  if (bytes > 48 * 1024) {
    if (bytes > smem_optin_limit()) return fail(EXGB_EUNSUPPORTED, "transform does not fit in shared memory");
    EXGB_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  }
  return EXGB_OK;
}

static int pairs_for(int n) { return std::max(1, 2048 / n); }

int launch_rfft1d(cudaStream_t st, const FftPlan& fp, const float2* tw, int64_t rows, const float* in, float2* out) {
  if (rows <= 0) return EXGB_OK;
  const int pairs = pairs_for(fp.n);
  const size_t smem = sizeof(float2) * 2 * pairs * fp.n;
  int rc = set_smem((const void*)rfft_rows_kernel, smem);
  if (rc) return rc;
  const int64_t blocks = (rows + 2 * pairs - 1) / (2 * pairs);
  rfft_rows_kernel<<<(unsigned)blocks, 256, smem, st>>>(fp, tw, rows, pairs, in, out);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

int launch_irfft1d(cudaStream_t st, const FftPlan& fp, const float2* tw, int64_t rows, const float2* in, float* out,
                   float scale) {
  if (rows <= 0) return EXGB_OK;
  const int pairs = pairs_for(fp.n);
  const size_t smem = sizeof(float2) * 2 * pairs * fp.n;
  int rc = set_smem((const void*)irfft_rows_kernel, smem);
  if (rc) return rc;
  const int64_t blocks = (rows + 2 * pairs - 1) / (2 * pairs);
  irfft_rows_kernel<<<(unsigned)blocks, 256, smem, st>>>(fp, tw, rows, pairs, in, out, scale);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

int launch_cfft_axis(cudaStream_t st, const FftPlan& fp, const float2* tw, bool inverse, int64_t outer,
                     int64_t outer_stride, int64_t inner, int64_t es, const float2* in, float2* out, float scale) {
  if (outer <= 0 || inner <= 0) return EXGB_OK;
  int TI = std::max(1, std::min(16, 4096 / fp.n));
  const size_t smem = sizeof(float2) * 2 * (size_t)TI * fp.n;
  const void* fn = inverse ? (const void*)cfft_axis_kernel<true> : (const void*)cfft_axis_kernel<false>;
  int rc = set_smem(fn, smem);
  if (rc) return rc;
  dim3 grid((unsigned)((inner + TI - 1) / TI), (unsigned)outer);
  if (outer > 65535) return fail(EXGB_EUNSUPPORTED, "too many outer sequences for one launch");
  if (inverse)
    cfft_axis_kernel<true><<<grid, 256, smem, st>>>(fp, tw, outer_stride, inner, es, TI, in, out, scale);
  else
    cfft_axis_kernel<false><<<grid, 256, smem, st>>>(fp, tw, outer_stride, inner, es, TI, in, out, scale);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

// ---------------------------------------------------------------- transform plans cache
struct TfCache {
  int n = 0;
  FftPlan fp{};
  float2* tw = nullptr;
};
static std::mutex g_tf_mu;
static TfCache g_tf[64];

static int get_tf(int n, const FftPlan** fp, const float2** tw) {
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(g_tf_mu);
  int freeslot = -1;
  for (int i = 0; i < 64; ++i) {
    if (g_tf[i].n == n + (dev << 20)) {
      *fp = &g_tf[i].fp;
      *tw = g_tf[i].tw;
      return EXGB_OK;
    }
    if (g_tf[i].n == 0 && freeslot < 0) freeslot = i;
  }
  if (freeslot < 0) return fail(EXGB_EUNSUPPORTED, "too many distinct transform sizes");
  TfCache& c = g_tf[freeslot];
  if (!make_fft_plan(n, &c.fp)) return fail(EXGB_ENOTFACTORABLE, "N must be a product of 2, 3 and 5");
  int rc = build_twiddles(n, &c.tw);
  if (rc) return rc;
  c.n = n + (dev << 20);
  *fp = &c.fp;
  *tw = c.tw;
  return EXGB_OK;
}

int rfftn_impl(cudaStream_t st, int D, int N, int64_t count, const float* in, float2* out) {
  const FftPlan* fp;
  const float2* tw;
  int rc = get_tf(N, &fp, &tw);
  if (rc) return rc;
  const int M = N / 2 + 1;
  if (D == 1) return launch_rfft1d(st, *fp, tw, count, in, out);
  if (D == 2) {
    rc = launch_rfft1d(st, *fp, tw, count * N, in, out);
    if (rc) return rc;
    return launch_cfft_axis(st, *fp, tw, false, count, (int64_t)N * M, M, M, out, out, 1.f);
  }
  if (D == 3) {
    const int64_t plane = (int64_t)N * M;
    rc = launch_rfft1d(st, *fp, tw, count * N * N, in, out);
    if (rc) return rc;
    rc = launch_cfft_axis(st, *fp, tw, false, count * N, plane, M, M, out, out, 1.f);
    if (rc) return rc;
    return launch_cfft_axis(st, *fp, tw, false, count, plane * N, plane, plane, out, out, 1.f);
  }
  return fail(EXGB_EUNSUPPORTED, "num_spatial_dims must be 1, 2 or 3");
}

int irfftn_impl(cudaStream_t st, int D, int N, int64_t count, const float2* in, float* out) {
  const FftPlan* fp;
  const float2* tw;
  int rc = get_tf(N, &fp, &tw);
  if (rc) return rc;
  const int M = N / 2 + 1;
  if (D == 1) return launch_irfft1d(st, *fp, tw, count, in, out, 1.f / (float)N);
  if (D == 2) {
    float2* tmp = (float2*)workspace(sizeof(float2) * (size_t)count * N * M, 0);
    if (!tmp) return fail(EXGB_ENOMEM, "workspace allocation failed");
    rc = launch_cfft_axis(st, *fp, tw, true, count, (int64_t)N * M, M, M, in, tmp, 1.f);
    if (rc) return rc;
    return launch_irfft1d(st, *fp, tw, count * N, tmp, out, 1.f / ((float)N * (float)N));
  }
  if (D == 3) {
    const int64_t plane = (int64_t)N * M;
    float2* tmp = (float2*)workspace(sizeof(float2) * (size_t)count * N * plane, 0);
    if (!tmp) return fail(EXGB_ENOMEM, "workspace allocation failed");
    rc = launch_cfft_axis(st, *fp, tw, true, count, plane * N, plane, plane, in, tmp, 1.f);
    if (rc) return rc;
    rc = launch_cfft_axis(st, *fp, tw, true, count * N, plane, M, M, tmp, tmp, 1.f);
    if (rc) return rc;
    return launch_irfft1d(st, *fp, tw, count * N * N, tmp, out, 1.f / ((float)N * (float)N * (float)N));
  }
  return fail(EXGB_EUNSUPPORTED, "num_spatial_dims must be 1, 2 or 3");
}

// ---------------------------------------------------------------- map_between_resolutions
// Gathers the new half-spectrum from the old one (_interpolation.py:195-285):
// blocks of get_modes_slices(D, min(N_old, N_new)) are copied, rescaled by
// (N_new/N_old)^D, and the Nyquist planes are zeroed as the oddball masks do.
__device__ __forceinline__ int src_index_axis(int k_new, int n_new, int n_old, int nmin) {
  // leading (fftfreq) axis: returns old index or -1 if not copied
  const int half = nmin / 2;
  const bool even = (nmin % 2) == 0;
  const int pos_hi = even ? half : half + 1;  // positive block [0, pos_hi)
  if (k_new < pos_hi) return k_new < n_old ? k_new : -1;
  const int neg = k_new - n_new;  // negative wavenumber in the new grid
  if (neg >= -half && neg < 0) return n_old + neg;
  return -1;
}

// signed wavenumber of index i on an fftfreq axis of n points
__device__ __forceinline__ int fftfreq_k(int i, int n) { return (i <= (n - 1) / 2) ? i : i - n; }

// true if a mode touches the Nyquist plane of an even n-point grid on any axis
// (oddball_filter_mask, _spectral.py:345-400): |k| = n/2 on a leading axis or
// k = n/2 on the last (rfftfreq) axis
__device__ __forceinline__ bool on_nyquist(int D, const int (&k)[3], int kl, int n) {
  if (kl >= n / 2) return true;
  for (int a = 0; a < D - 1; ++a)
    if (k[a] >= n / 2 || k[a] <= -n / 2) return true;
  return false;
}

__global__ void resample_kernel(int D, int n_old, int n_new, int64_t count, const float2* __restrict__ in,
                                float2* __restrict__ out, float scale, int zero_old_nyq, int zero_new_nyq) {
  const int Mo = n_old / 2 + 1, Mn = n_new / 2 + 1;
  const int nmin = min(n_old, n_new);
  int64_t per = Mn, per_old = Mo;
  for (int a = 0; a < D - 1; ++a) {
    per *= n_new;
    per_old *= n_old;
  }
  const int64_t total = per * count;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = t / per;
    int64_t r = t - c * per;
    const int kl = (int)(r % Mn);  // last (rfftfreq) axis
    r /= Mn;
    // leading axes, innermost first: new index, old source index, signed wavenumbers
    int kn[3] = {0, 0, 0}, ko[3] = {0, 0, 0};
    int64_t src = kl;
    int64_t stride = Mo;
    bool ok = kl <= nmin / 2;
    for (int a = D - 2; a >= 0 && ok; --a) {
      const int i = (int)(r % n_new);
      r /= n_new;
      const int si = src_index_axis(i, n_new, n_old, nmin);
      ok = si >= 0;
      kn[a] = fftfreq_k(i, n_new);
      ko[a] = fftfreq_k(si, n_old);
      src += (int64_t)si * stride;
      stride *= n_old;
    }
    // oddball masks: Nyquist of the old grid (upscaling) / new grid (downscaling)
    if (ok && zero_old_nyq && on_nyquist(D, ko, kl, n_old)) ok = false;
    if (ok && zero_new_nyq && on_nyquist(D, kn, kl, n_new)) ok = false;
    out[t] = ok ? cscale(in[c * per_old + src], scale) : make_float2(0.f, 0.f);
  }
}

// FourierInterpolator.__call__ (_interpolation.py:22-112) at P points: one warp per point,
// u_c(x) = Re sum_modes c_scaled[c][mode] exp(i (k_0 x_0 + ... + k_{D-1} x_{D-1})) with the
// scaled wavenumbers k_d = 2 pi n_d / L ('ij' grid, rfftfreq on the last axis).  The phase is
// summed over the axes in FP32 in axis order and exp taken by sincosf, as the reference forms
// exp(sum_d i k_d x_d); the per-lane partial sums are FP32, combined by a warp reduction.
__global__ void __launch_bounds__(256) fourier_interp_kernel(int D, int N, int C, int64_t per,
                                                             const float2* __restrict__ coef, float kscale,
                                                             int64_t P, const float* __restrict__ x,
                                                             float* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t pt = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (pt >= P) return;  // whole warps exit together (P indexes warps)
  const int M = N / 2 + 1;
  float xs[3] = {0.f, 0.f, 0.f};
  for (int d = 0; d < D; ++d) xs[d] = x[pt * D + d];
  constexpr int kMaxC = 8;
  for (int c0 = 0; c0 < C; c0 += kMaxC) {
    const int nc = min(kMaxC, C - c0);
    float acc[kMaxC];
    for (int c = 0; c < kMaxC; ++c) acc[c] = 0.f;
    for (int64_t r = lane; r < per; r += 32) {
      int k[3] = {0, 0, 0};
      k[D - 1] = (int)(r % M);
      int64_t rest = r / M;
      for (int a = D - 2; a >= 0; --a) {
        const int i = (int)(rest % N);
        rest /= N;
        k[a] = (i <= (N - 1) / 2) ? i : i - N;
      }
      float th = 0.f;
      for (int a = 0; a < D; ++a) th += (kscale * (float)k[a]) * xs[a];
      float sn, cs;
      sincosf(th, &sn, &cs);
      for (int c = 0; c < nc; ++c) {
        const float2 v = coef[(int64_t)(c0 + c) * per + r];
        acc[c] += v.x * cs - v.y * sn;
      }
    }
    for (int c = 0; c < nc; ++c) {
      float v = acc[c];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) out[pt * C + c0 + c] = v;
    }
  }
}

}  // namespace exgb

using namespace exgb;

extern "C" {

int exgb_fourier_interp(void* stream, int num_spatial_dims, int num_points, int num_channels, const void* coef,
                        float domain_extent, int64_t num_queries, const float* x, float* out) {
  const int D = num_spatial_dims, N = num_points, C = num_channels;
  if (D < 1 || D > 3 || N < 1 || C < 1) return fail(EXGB_ESHAPE, "exgb_fourier_interp: bad shape");
  if (num_queries < 0 || !(domain_extent > 0.f)) return fail(EXGB_EINVAL, "exgb_fourier_interp: bad arguments");
  if (num_queries == 0) return EXGB_OK;
  if (!coef || !x || !out) return fail(EXGB_EINVAL, "exgb_fourier_interp: NULL pointer");
  int64_t per = N / 2 + 1;
  for (int d = 0; d < D - 1; ++d) per *= N;
  const float kscale = (float)(2.0 * 3.14159265358979323846 / (double)domain_extent);
  const int64_t threads = num_queries * 32;
  const int64_t blocks = (threads + 255) / 256;
  if (blocks > 2147483647LL) return fail(EXGB_EINVAL, "exgb_fourier_interp: too many query points");
  fourier_interp_kernel<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(D, N, C, per, (const float2*)coef, kscale,
                                                                           num_queries, x, out);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}


int exgb_rfftn(void* stream, int num_spatial_dims, int num_points, int64_t count, const float* in, void* out) {
  if (count < 0) return fail(EXGB_EINVAL, "negative count");
  if (count == 0) return EXGB_OK;
  if (!in || !out) return fail(EXGB_EINVAL, "NULL pointer");
  return rfftn_impl((cudaStream_t)stream, num_spatial_dims, num_points, count, in, (float2*)out);
}

int exgb_irfftn(void* stream, int num_spatial_dims, int num_points, int64_t count, const void* in, float* out) {
  if (count < 0) return fail(EXGB_EINVAL, "negative count");
  if (count == 0) return EXGB_OK;
  if (!in || !out) return fail(EXGB_EINVAL, "NULL pointer");
  return irfftn_impl((cudaStream_t)stream, num_spatial_dims, num_points, count, (const float2*)in, out);
}

int exgb_map_between_resolutions(void* stream, int D, int n_old, int n_new, int64_t count, const float* in,
                                 float* out, int oddball_zero) {
  if (D < 1 || D > 3) return fail(EXGB_EINVAL, "num_spatial_dims must be 1, 2 or 3");
  if (n_old < 1 || n_new < 1 || count < 0) return fail(EXGB_EINVAL, "bad sizes");
  if (count == 0) return EXGB_OK;
  if (!in || !out) return fail(EXGB_EINVAL, "NULL pointer");
  cudaStream_t st = (cudaStream_t)stream;
  size_t pts_old = (size_t)n_old, pts_new = (size_t)n_new;  // grid points per field
  size_t so = (size_t)(n_old / 2 + 1), sn = (size_t)(n_new / 2 + 1);  // modes per field
  for (int d = 1; d < D; ++d) {
    pts_old *= n_old;
    pts_new *= n_new;
    so *= n_old;
    sn *= n_new;
  }
  if (n_old == n_new) {
    EXGB_CUDA(cudaMemcpyAsync(out, in, sizeof(float) * (size_t)count * pts_old, cudaMemcpyDeviceToDevice, st));
    return EXGB_OK;
  }
  so *= (size_t)count;
  sn *= (size_t)count;
  // slot 1 holds the old spectrum; the new spectrum goes to slot 2 (irfftn_impl uses slot 0 for its
  // intermediate in 2D and 3D)
  float2* a = (float2*)workspace(sizeof(float2) * so, 1);
  if (!a) return fail(EXGB_ENOMEM, "workspace allocation failed");
  int rc = rfftn_impl(st, D, n_old, count, in, a);
  if (rc) return rc;
  float2* b = (float2*)workspace(sizeof(float2) * sn, 2);
  if (!b) return fail(EXGB_ENOMEM, "workspace allocation failed");
  double ratio = 1.0;
  for (int d = 0; d < D; ++d) ratio *= (double)n_new / (double)n_old;
  const float scale = (float)ratio;
  const int zo = (n_new > n_old) && (n_old % 2 == 0) && oddball_zero;
  const int zn = (n_old > n_new) && (n_new % 2 == 0) && oddball_zero;
  const int64_t total = (int64_t)sn;
  const int th = 256;
  const unsigned blocks = (unsigned)std::min<int64_t>((total + th - 1) / th, 65535);
  resample_kernel<<<blocks, th, 0, st>>>(D, n_old, n_new, count, a, b, scale, zo, zn);
  EXGB_CUDA(cudaGetLastError());
  return irfftn_impl(st, D, n_new, count, b, out);
}

}  // extern "C"
