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
#include <cmath>
#include <complex>
#include <mutex>
#include <string>
#include <vector>

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

// ---------------------------------------------------------------- transform descriptors
// A length-n transform along one axis is taken one of three ways:
//   direct     n = 2^a 3^b 5^c and a sequence fits one CTA's shared memory: Stockham passes
//   Bluestein  any other n with a smooth L >= 2n - 1 that fits: the chirp-z identity
//                X_k = c_k sum_j (x_j c_j) conj(c_(k-j)),   c_j = exp(-i pi j^2 / n)
//              (inverse: conjugate chirps), a circular convolution of length L computed as
//              a forward and an inverse length-L Stockham transform around a product with
//              the precomputed spectrum of the chirp; the chirps are evaluated in FP64 from
//              j^2 mod 2n and rounded once
//   four-step  smooth n too long for one CTA (1D only): n = n1 n2, length-n1 transforms over
//              j1 (stride n2), twiddles w_n^(k1 j2), length-n2 transforms over j2 (contiguous);
//              X[k1 + n1 k2] ends at k1 n2 + k2 and the real packing reads it transposed
enum TfKind { TF_DIRECT = 0, TF_BLUESTEIN = 1, TF_FOURSTEP = 2 };

struct Blue {
  int L;
  FftPlan fp;            // length L
  const float2* tw;      // L twiddles exp(-2 pi i m / L)
  const float2* chirp;   // c_j, j < n
  const float2* bhat;    // chirp spectrum for the direction in use, 1/L folded in
};

struct Tf {
  int key = 0;  // n + (device << 20); 0 = free
  int n = 0, kind = TF_DIRECT;
  FftPlan fp{};            // direct: length n; Bluestein: length L; four-step: length n1
  float2* tw = nullptr;
  int L = 0;               // Bluestein
  float2* chirp = nullptr;
  float2* bhat = nullptr;  // [2][L]: forward (FFT_L of conj c), inverse (FFT_L of c), each / L
  int n1 = 0, n2 = 0;      // four-step
  FftPlan fp2{};
  float2* tw2 = nullptr;
  float2* twn = nullptr;   // exp(-2 pi i m / n), m < n
  Blue blue(bool inv) const {
    Blue b;
    b.L = L;
    b.fp = fp;
    b.tw = tw;
    b.chirp = chirp;
    b.bhat = bhat + (inv ? L : 0);
    return b;
  }
};

// chirp factor of position j for the transform direction (conjugated for the inverse)
template <bool INV>
__device__ __forceinline__ float2 chirp_at(const Blue& b, int j) {
  const float2 c = b.chirp[j];
  return INV ? cconj(c) : c;
}

// Circular convolution with the chirp of `count` sequences (stride L) that sit premultiplied and
// zero-padded in buf0: forward transform, product with the chirp spectrum, inverse transform.
// Returns the buffer holding the result (stride L); a barrier follows every step.
__device__ float2* blue_conv(const Blue& b, float2* buf0, float2* buf1, int count, int tid, int nthr) {
  float2* r1 = result_buf(b.fp, buf0, buf1);
  block_fft<false>(b.fp, buf0, buf1, LinMap{r1, b.L}, count, b.tw, tid, nthr, BlockSync{});
  for (int t = tid; t < count * b.L; t += nthr) {
    const int m = t - (t / b.L) * b.L;
    r1[t] = cmul(r1[t], __ldg(b.bhat + m));
  }
  __syncthreads();
  float2* o = (r1 == buf0) ? buf1 : buf0;
  float2* r2 = result_buf(b.fp, r1, o);
  block_fft<true>(b.fp, r1, o, LinMap{r2, b.L}, count, b.tw, tid, nthr, BlockSync{});
  return r2;
}

// ---------------------------------------------------------------- row r2c
// Each CTA transforms `pairs` pairs of real rows (2*pairs rows) of length n, two rows packed as
// a + i b; S = n (direct) or L (Bluestein) is the shared-memory stride of one sequence.
template <bool BLUE>
__global__ void rfft_rows_kernel(int n, FftPlan fp, const float2* __restrict__ tw, Blue bl, int64_t rows, int pairs,
                                 const float* __restrict__ in, float2* __restrict__ out) {
  extern __shared__ float2 smem[];
  const int M = n / 2 + 1;
  const int S = BLUE ? bl.L : n;
  float2* buf0 = smem;
  float2* buf1 = smem + (size_t)pairs * S;
  const int64_t row0 = (int64_t)blockIdx.x * pairs * 2;
  for (int t = threadIdx.x; t < pairs * S; t += blockDim.x) {
    const int p = t / S, x = t - p * S;
    float2 v = make_float2(0.f, 0.f);
    if (x < n) {
      const int64_t ra = row0 + 2 * p, rb = ra + 1;
      v.x = ra < rows ? in[ra * n + x] : 0.f;
      v.y = rb < rows ? in[rb * n + x] : 0.f;
      if (BLUE) v = cmul(v, chirp_at<false>(bl, x));
    }
    buf0[t] = v;
  }
  __syncthreads();
  float2* res;
  if (BLUE) {
    res = blue_conv(bl, buf0, buf1, pairs, threadIdx.x, blockDim.x);
  } else {
    res = result_buf(fp, buf0, buf1);
    block_fft<false>(fp, buf0, buf1, LinMap{res, n}, pairs, tw, threadIdx.x, blockDim.x, BlockSync{});
  }
  for (int t = threadIdx.x; t < pairs * M; t += blockDim.x) {
    const int p = t / M, k = t - p * M;
    const int64_t ra = row0 + 2 * p, rb = ra + 1;
    const int kn = k == 0 ? 0 : n - k;
    float2 zk = res[p * S + k], znk = res[p * S + kn];
    if (BLUE) {
      zk = cmul(zk, chirp_at<false>(bl, k));
      znk = cmul(znk, chirp_at<false>(bl, kn));
    }
    float2 P, Q;
    unpack_pair(zk, znk, P, Q);
    if (ra < rows) out[ra * M + k] = P;
    if (rb < rows) out[rb * M + k] = Q;
  }
}

// ---------------------------------------------------------------- row c2r
template <bool BLUE>
__global__ void irfft_rows_kernel(int n, FftPlan fp, const float2* __restrict__ tw, Blue bl, int64_t rows, int pairs,
                                  const float2* __restrict__ in, float* __restrict__ out, float scale) {
  extern __shared__ float2 smem[];
  const int M = n / 2 + 1;
  const int S = BLUE ? bl.L : n;
  float2* buf0 = smem;
  float2* buf1 = smem + (size_t)pairs * S;
  const int64_t row0 = (int64_t)blockIdx.x * pairs * 2;
  const bool even = (n % 2) == 0;
  for (int t = threadIdx.x; t < pairs * S; t += blockDim.x) {
    const int p = t / S, k = t - p * S;
    float2 v = make_float2(0.f, 0.f);
    if (k < n) {
      const int64_t ra = row0 + 2 * p, rb = ra + 1;
      const bool ext = k >= M;
      const int kk = ext ? n - k : k;
      const bool real_only = (k == 0) || (even && k == n / 2);
      const float2 a = ra < rows ? in[ra * M + kk] : make_float2(0.f, 0.f);
      const float2 b = rb < rows ? in[rb * M + kk] : make_float2(0.f, 0.f);
      v = pack_pair(a, b, ext, real_only);
      if (BLUE) v = cmul(v, chirp_at<true>(bl, k));
    }
    buf0[t] = v;
  }
  __syncthreads();
  float2* res;
  if (BLUE) {
    res = blue_conv(bl, buf0, buf1, pairs, threadIdx.x, blockDim.x);
  } else {
    res = result_buf(fp, buf0, buf1);
    block_fft<true>(fp, buf0, buf1, LinMap{res, n}, pairs, tw, threadIdx.x, blockDim.x, BlockSync{});
  }
  for (int t = threadIdx.x; t < pairs * n; t += blockDim.x) {
    const int p = t / n, x = t - p * n;
    const int64_t ra = row0 + 2 * p, rb = ra + 1;
    float2 z = res[p * S + x];
    if (BLUE) z = cmul(z, chirp_at<true>(bl, x));
    if (ra < rows) out[ra * n + x] = z.x * scale;
    if (rb < rows) out[rb * n + x] = z.y * scale;
  }
}

// ---------------------------------------------------------------- strided axis c2c
// Element k of the sequence at (o, i) lives at o*outer_stride + i + k*es.
// CTA (blockIdx.x = tile of TI inner positions, blockIdx.y + y0 = outer).
template <bool INV, bool BLUE>
__global__ void cfft_axis_kernel(int n, FftPlan fp, const float2* __restrict__ tw, Blue bl, int64_t outer_stride,
                                 int64_t inner, int64_t es, int TI, int64_t y0, const float2* in, float2* out,
                                 float scale) {
  extern __shared__ float2 smem[];
  const int S = BLUE ? bl.L : n;
  float2* buf0 = smem;
  float2* buf1 = smem + (size_t)TI * S;
  const int64_t o = (int64_t)blockIdx.y + y0;
  const int64_t i0 = (int64_t)blockIdx.x * TI;
  const int ti = (inner - i0) < (int64_t)TI ? (int)(inner - i0) : TI;
  const float2* src = in + o * outer_stride + i0;
  for (int t = threadIdx.x; t < TI * n; t += blockDim.x) {
    const int k = t / TI, ii = t - k * TI;
    float2 v = ii < ti ? src[(int64_t)k * es + ii] : make_float2(0.f, 0.f);
    if (BLUE) v = cmul(v, chirp_at<INV>(bl, k));
    buf0[ii * S + k] = v;
  }
  if (BLUE)
    for (int t = threadIdx.x; t < TI * (S - n); t += blockDim.x) {
      const int ii = t / (S - n), k = n + (t - ii * (S - n));
      buf0[ii * S + k] = make_float2(0.f, 0.f);
    }
  __syncthreads();
  float2* res;
  if (BLUE) {
    res = blue_conv(bl, buf0, buf1, TI, threadIdx.x, blockDim.x);
  } else {
    res = result_buf(fp, buf0, buf1);
    block_fft<INV>(fp, buf0, buf1, LinMap{res, n}, TI, tw, threadIdx.x, blockDim.x, BlockSync{});
  }
  float2* dst = out + o * outer_stride + i0;
  for (int t = threadIdx.x; t < TI * n; t += blockDim.x) {
    const int k = t / TI, ii = t - k * TI;
    if (ii < ti) {
      float2 v = res[ii * S + k];
      if (BLUE) v = cmul(v, chirp_at<INV>(bl, k));
      dst[(int64_t)k * es + ii] = cscale(v, scale);
    }
  }
}

// ---------------------------------------------------------------- four-step pieces (1D, long n)
// rows of n2 contiguous elements, row r = s n1 + k1: multiply by w_n^(-+ k1 j2), transform over j2
template <bool INV>
__global__ void rows_twiddle_fft_kernel(FftPlan fp2, const float2* __restrict__ tw2, const float2* __restrict__ twn,
                                        int n1, int64_t nrows, int cnt, float2* data) {
  extern __shared__ float2 smem[];
  const int n2 = fp2.n;
  float2* buf0 = smem;
  float2* buf1 = smem + (size_t)cnt * n2;
  const int64_t r0 = (int64_t)blockIdx.x * cnt;
  for (int t = threadIdx.x; t < cnt * n2; t += blockDim.x) {
    const int rr = t / n2, j2 = t - rr * n2;
    const int64_t row = r0 + rr;
    float2 v = make_float2(0.f, 0.f);
    if (row < nrows) {
      const int k1 = (int)(row % n1);
      float2 w = __ldg(twn + (int64_t)k1 * j2);  // k1 j2 < n1 n2 = n
      if (INV) w.y = -w.y;
      v = cmul(data[row * n2 + j2], w);
    }
    buf0[t] = v;
  }
  __syncthreads();
  float2* res = result_buf(fp2, buf0, buf1);
  block_fft<INV>(fp2, buf0, buf1, LinMap{res, n2}, cnt, tw2, threadIdx.x, blockDim.x, BlockSync{});
  for (int t = threadIdx.x; t < cnt * n2; t += blockDim.x) {
    const int rr = t / n2;
    const int64_t row = r0 + rr;
    if (row < nrows) data[row * n2 + (t - rr * n2)] = res[t];
  }
}

// pairs of real rows -> complex sequences z = a + i b (forward), or half spectra -> the full
// packed spectrum pack_pair(A~, B~) (inverse), natural order
__global__ void pack_rows_kernel(int n, int64_t rows, int64_t seqs, const float* __restrict__ in, float2* z) {
  const int64_t total = seqs * n;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = t / n, x = t - s * n;
    const int64_t ra = 2 * s, rb = ra + 1;
    z[t] = make_float2(in[ra * n + x], rb < rows ? in[rb * n + x] : 0.f);
  }
}
__global__ void pack_spectra_kernel(int n, int64_t rows, int64_t seqs, const float2* __restrict__ in, float2* z) {
  const int M = n / 2 + 1;
  const bool even = (n % 2) == 0;
  const int64_t total = seqs * n;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = t / n;
    const int k = (int)(t - s * n);
    const int64_t ra = 2 * s, rb = ra + 1;
    const bool ext = k >= M;
    const int kk = ext ? n - k : k;
    const bool real_only = (k == 0) || (even && k == n / 2);
    const float2 a = in[ra * M + kk];
    const float2 b = rb < rows ? in[rb * M + kk] : make_float2(0.f, 0.f);
    z[t] = pack_pair(a, b, ext, real_only);
  }
}
// the four-step output holds X[k1 + n1 k2] at k1 n2 + k2
__device__ __forceinline__ int64_t fourstep_at(int64_t k, int n1, int n2) { return (k % n1) * n2 + k / n1; }

__global__ void unpack_spectra_kernel(int n, int n1, int n2, int64_t rows, int64_t seqs, const float2* __restrict__ z,
                                      float2* __restrict__ out) {
  const int M = n / 2 + 1;
  const int64_t total = seqs * M;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = t / M;
    const int k = (int)(t - s * M);
    const float2* zs = z + s * n;
    const float2 zk = zs[fourstep_at(k, n1, n2)];
    const float2 znk = zs[fourstep_at(k == 0 ? 0 : n - k, n1, n2)];
    float2 P, Q;
    unpack_pair(zk, znk, P, Q);
    const int64_t ra = 2 * s, rb = ra + 1;
    out[ra * M + k] = P;
    if (rb < rows) out[rb * M + k] = Q;
  }
}
__global__ void unpack_rows_kernel(int n, int n1, int n2, int64_t rows, int64_t seqs, const float2* __restrict__ z,
                                   float* __restrict__ out, float scale) {
  const int64_t total = seqs * n;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = t / n, x = t - s * n;
    const float2 v = z[s * n + fourstep_at(x, n1, n2)];
    const int64_t ra = 2 * s, rb = ra + 1;
    out[ra * n + x] = v.x * scale;
    if (rb < rows) out[rb * n + x] = v.y * scale;
  }
}

static int set_smem(const void* fn, size_t bytes) {
  if (bytes > 48 * 1024) {
    if (bytes > smem_optin_limit()) return fail(EXGB_EUNSUPPORTED, "transform does not fit in shared memory");
    EXGB_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  }
  return EXGB_OK;
}

// sequences per CTA of the row kernels (stride S elements each)
static int pairs_for(int S) { return std::max(1, 2048 / S); }

static unsigned flat_grid(int64_t n) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 65535));
}

// Complex length-n transforms of `seqs` contiguous sequences, four-step, in place.
static int fourstep_c2c(cudaStream_t st, const Tf& tf, bool inverse, int64_t seqs, float2* z);

// longest sequence one CTA transforms directly (two buffers of n complex values)
static int direct_max_n() { return (int)(smem_optin_limit() / (2 * sizeof(float2))); }

static int launch_rows(cudaStream_t st, const Tf& tf, bool inverse, int64_t rows, const float* in_r,
                       const float2* in_c, float2* out_c, float* out_r, float scale) {
  if (rows <= 0) return EXGB_OK;
  const int n = tf.n;
  if (tf.kind == TF_FOURSTEP) {
    const int64_t seqs = (rows + 1) / 2;
    float2* z = (float2*)workspace(sizeof(float2) * (size_t)seqs * n, 7);
    if (!z) return fail(EXGB_ENOMEM, "workspace allocation failed");
    if (!inverse) {
      pack_rows_kernel<<<flat_grid(seqs * n), 256, 0, st>>>(n, rows, seqs, in_r, z);
    } else {
      pack_spectra_kernel<<<flat_grid(seqs * n), 256, 0, st>>>(n, rows, seqs, in_c, z);
    }
    EXGB_CUDA(cudaGetLastError());
    int rc = fourstep_c2c(st, tf, inverse, seqs, z);
    if (rc) return rc;
    if (!inverse) {
      unpack_spectra_kernel<<<flat_grid(seqs * (n / 2 + 1)), 256, 0, st>>>(n, tf.n1, tf.n2, rows, seqs, z, out_c);
    } else {
      unpack_rows_kernel<<<flat_grid(seqs * n), 256, 0, st>>>(n, tf.n1, tf.n2, rows, seqs, z, out_r, scale);
    }
    EXGB_CUDA(cudaGetLastError());
    return EXGB_OK;
  }
  const bool blue = tf.kind == TF_BLUESTEIN;
  const int S = blue ? tf.L : n;
  const int pairs = pairs_for(S);
  const size_t smem = sizeof(float2) * 2 * pairs * (size_t)S;
  const Blue bl = blue ? tf.blue(inverse) : Blue{};
  const void* fn = !inverse ? (blue ? (const void*)rfft_rows_kernel<true> : (const void*)rfft_rows_kernel<false>)
                            : (blue ? (const void*)irfft_rows_kernel<true> : (const void*)irfft_rows_kernel<false>);
  int rc = set_smem(fn, smem);
  if (rc) return rc;
  const int64_t blocks = (rows + 2 * pairs - 1) / (2 * pairs);
  if (blocks > 2147483647LL) return fail(EXGB_EUNSUPPORTED, "too many rows for one launch");
  if (!inverse) {
    if (blue)
      rfft_rows_kernel<true><<<(unsigned)blocks, 256, smem, st>>>(n, tf.fp, tf.tw, bl, rows, pairs, in_r, out_c);
    else
      rfft_rows_kernel<false><<<(unsigned)blocks, 256, smem, st>>>(n, tf.fp, tf.tw, bl, rows, pairs, in_r, out_c);
  } else {
    if (blue)
      irfft_rows_kernel<true><<<(unsigned)blocks, 256, smem, st>>>(n, tf.fp, tf.tw, bl, rows, pairs, in_c, out_r,
                                                                  scale);
    else
      irfft_rows_kernel<false><<<(unsigned)blocks, 256, smem, st>>>(n, tf.fp, tf.tw, bl, rows, pairs, in_c, out_r,
                                                                   scale);
  }
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

// Strided complex transforms along one axis: `outer` x `inner` sequences (see cfft_axis_kernel);
// direct or Bluestein, launched in slices of at most 65535 outer indices.
static int launch_axis(cudaStream_t st, const Tf& tf, bool inverse, int64_t outer, int64_t outer_stride,
                       int64_t inner, int64_t es, const float2* in, float2* out, float scale) {
  if (outer <= 0 || inner <= 0) return EXGB_OK;
  if (tf.kind == TF_FOURSTEP) return fail(EXGB_EUNSUPPORTED, "axes this long are transformed only in 1D");
  const bool blue = tf.kind == TF_BLUESTEIN;
  const int S = blue ? tf.L : tf.n;
  const int TI = std::max(1, std::min(16, 4096 / S));
  const size_t smem = sizeof(float2) * 2 * (size_t)TI * S;
  const Blue bl = blue ? tf.blue(inverse) : Blue{};
  const void* fn = inverse ? (blue ? (const void*)cfft_axis_kernel<true, true> : (const void*)cfft_axis_kernel<true, false>)
                           : (blue ? (const void*)cfft_axis_kernel<false, true> : (const void*)cfft_axis_kernel<false, false>);
  int rc = set_smem(fn, smem);
  if (rc) return rc;
  const int64_t gx = (inner + TI - 1) / TI;
  if (gx > 2147483647LL) return fail(EXGB_EUNSUPPORTED, "too many inner sequences for one launch");
  for (int64_t y0 = 0; y0 < outer; y0 += 65535) {
    dim3 grid((unsigned)gx, (unsigned)std::min<int64_t>(65535, outer - y0));
#define EXGB_AXIS_LAUNCH(I, B) \
  cfft_axis_kernel<I, B><<<grid, 256, smem, st>>>(tf.n, tf.fp, tf.tw, bl, outer_stride, inner, es, TI, y0, in, out, scale)
    if (inverse) {
      if (blue) EXGB_AXIS_LAUNCH(true, true);
      else EXGB_AXIS_LAUNCH(true, false);
    } else {
      if (blue) EXGB_AXIS_LAUNCH(false, true);
      else EXGB_AXIS_LAUNCH(false, false);
    }
#undef EXGB_AXIS_LAUNCH
    EXGB_CUDA(cudaGetLastError());
  }
  return EXGB_OK;
}

static int fourstep_c2c(cudaStream_t st, const Tf& tf, bool inverse, int64_t seqs, float2* z) {
  const int n = tf.n, n1 = tf.n1, n2 = tf.n2;
  // (1) length-n1 transforms over j1 (element j = n2 j1 + j2): n2 sequences of stride n2 per row
  Tf t1;
  t1.n = n1;
  t1.kind = TF_DIRECT;
  t1.fp = tf.fp;
  t1.tw = tf.tw;
  int rc = launch_axis(st, t1, inverse, seqs, n, n2, n2, z, z, 1.f);
  if (rc) return rc;
  // (2) twiddles and length-n2 transforms over j2
  const int cnt = std::max(1, 2048 / n2);
  const size_t smem = sizeof(float2) * 2 * (size_t)cnt * n2;
  const void* fn = inverse ? (const void*)rows_twiddle_fft_kernel<true> : (const void*)rows_twiddle_fft_kernel<false>;
  rc = set_smem(fn, smem);
  if (rc) return rc;
  const int64_t nrows = seqs * n1;
  const int64_t blocks = (nrows + cnt - 1) / cnt;
  if (inverse)
    rows_twiddle_fft_kernel<true><<<(unsigned)blocks, 256, smem, st>>>(tf.fp2, tf.tw2, tf.twn, n1, nrows, cnt, z);
  else
    rows_twiddle_fft_kernel<false><<<(unsigned)blocks, 256, smem, st>>>(tf.fp2, tf.tw2, tf.twn, n1, nrows, cnt, z);
  EXGB_CUDA(cudaGetLastError());
  (void)n;
  return EXGB_OK;
}

int launch_rfft1d(cudaStream_t st, const FftPlan& fp, const float2* tw, int64_t rows, const float* in, float2* out) {
  Tf tf;
  tf.n = fp.n;
  tf.fp = fp;
  tf.tw = (float2*)tw;
  return launch_rows(st, tf, false, rows, in, nullptr, out, nullptr, 1.f);
}

int launch_irfft1d(cudaStream_t st, const FftPlan& fp, const float2* tw, int64_t rows, const float2* in, float* out,
                   float scale) {
  Tf tf;
  tf.n = fp.n;
  tf.fp = fp;
  tf.tw = (float2*)tw;
  return launch_rows(st, tf, true, rows, nullptr, in, nullptr, out, scale);
}

int launch_cfft_axis(cudaStream_t st, const FftPlan& fp, const float2* tw, bool inverse, int64_t outer,
                     int64_t outer_stride, int64_t inner, int64_t es, const float2* in, float2* out, float scale) {
  Tf tf;
  tf.n = fp.n;
  tf.fp = fp;
  tf.tw = (float2*)tw;
  return launch_axis(st, tf, inverse, outer, outer_stride, inner, es, in, out, scale);
}

// ---------------------------------------------------------------- transform descriptors cache
static bool smooth235(int n) {
  if (n < 2) return false;
  for (int p : {2, 3, 5})
    while (n % p == 0) n /= p;
  return n == 1;
}

// FP64 complex FFT of a smooth length on the host (recursive decimation in time), for the chirp
// spectra of the Bluestein transforms.
static void host_fft(std::vector<std::complex<double>>& a) {
  const size_t n = a.size();
  if (n <= 1) return;
  size_t p = 2;
  while (n % p) ++p;
  const size_t m = n / p;
  std::vector<std::vector<std::complex<double>>> sub(p, std::vector<std::complex<double>>(m));
  for (size_t j = 0; j < m; ++j)
    for (size_t r = 0; r < p; ++r) sub[r][j] = a[j * p + r];
  for (size_t r = 0; r < p; ++r) host_fft(sub[r]);
  for (size_t k = 0; k < n; ++k) {
    std::complex<double> acc = 0.0;
    for (size_t r = 0; r < p; ++r) {
      const double ang = -2.0 * M_PI * (double)((r * k) % n) / (double)n;
      acc += sub[r][k % m] * std::complex<double>(std::cos(ang), std::sin(ang));
    }
    a[k] = acc;
  }
}

static int upload(const std::vector<float2>& h, float2** d) {
  EXGB_CUDA(cudaMalloc(d, sizeof(float2) * h.size()));
  EXGB_CUDA(cudaMemcpy(*d, h.data(), sizeof(float2) * h.size(), cudaMemcpyHostToDevice));
  return EXGB_OK;
}

static int build_tf(int n, Tf& c) {
  c.n = n;
  const int dmax = direct_max_n();
  if (smooth235(n) && n <= dmax) {
    c.kind = TF_DIRECT;
    if (!make_fft_plan(n, &c.fp)) return fail(EXGB_ENOTFACTORABLE, "cannot plan a transform of this length");
    return build_twiddles(n, &c.tw);
  }
  if (smooth235(n)) {
    // four-step: n1 the largest divisor <= sqrt(n), both factors short enough for one CTA
    int n1 = 1;
    for (int d = 2; (int64_t)d * d <= n; ++d)
      if (n % d == 0) n1 = d;
    const int n2 = n / n1;
    if (n1 < 2 || n2 > dmax) return fail(EXGB_EUNSUPPORTED, "transform length too long for this build");
    c.kind = TF_FOURSTEP;
    c.n1 = n1;
    c.n2 = n2;
    if (!make_fft_plan(n1, &c.fp) || !make_fft_plan(n2, &c.fp2))
      return fail(EXGB_ENOTFACTORABLE, "cannot plan the four-step factors");
    int rc = build_twiddles(n1, &c.tw);
    if (rc) return rc;
    rc = build_twiddles(n2, &c.tw2);
    if (rc) return rc;
    return build_twiddles(n, &c.twn);
  }
  // Bluestein: the smallest smooth L >= 2n - 1
  int L = 2 * n - 1;
  while (!smooth235(L)) ++L;
  if (L > dmax)
    return fail(EXGB_ENOTFACTORABLE, "N with a prime factor above 5 is supported up to about " +
                                         std::to_string((dmax + 1) / 2) + " points per axis (got " +
                                         std::to_string(n) + ")");
  c.kind = TF_BLUESTEIN;
  c.L = L;
  if (!make_fft_plan(L, &c.fp)) return fail(EXGB_ENOTFACTORABLE, "cannot plan the Bluestein length");
  int rc = build_twiddles(L, &c.tw);
  if (rc) return rc;
  std::vector<std::complex<double>> cz(n);
  for (int j = 0; j < n; ++j) {
    const long long q = ((long long)j * j) % (2LL * n);  // exp(-i pi j^2 / n) has period 2n in j^2
    const double ang = -M_PI * (double)q / (double)n;
    cz[j] = std::complex<double>(std::cos(ang), std::sin(ang));
  }
  std::vector<float2> hc(n);
  for (int j = 0; j < n; ++j) hc[j] = make_float2((float)cz[j].real(), (float)cz[j].imag());
  rc = upload(hc, &c.chirp);
  if (rc) return rc;
  // forward kernel b_m = conj(c_m), inverse kernel c_m, on m in (-n, n), circularly wrapped to L
  std::vector<float2> hb(2 * (size_t)L);
  for (int dir = 0; dir < 2; ++dir) {
    std::vector<std::complex<double>> b(L, 0.0);
    for (int m = 0; m < n; ++m) {
      const std::complex<double> v = dir == 0 ? std::conj(cz[m]) : cz[m];
      b[m] = v;
      if (m > 0) b[L - m] = v;
    }
    host_fft(b);
    for (int m = 0; m < L; ++m)
      hb[(size_t)dir * L + m] = make_float2((float)(b[m].real() / L), (float)(b[m].imag() / L));
  }
  return upload(hb, &c.bhat);
}

static std::mutex g_tf_mu;
static Tf g_tf[64];

static int get_tf(int n, const Tf** out) {
  if (n < 2) return fail(EXGB_EINVAL, "transforms need at least 2 points per axis");
  int dev = 0;
  cudaGetDevice(&dev);
  const int key = n + (dev << 20);
  std::lock_guard<std::mutex> lk(g_tf_mu);
  int freeslot = -1;
  for (int i = 0; i < 64; ++i) {
    if (g_tf[i].key == key) {
      *out = &g_tf[i];
      return EXGB_OK;
    }
    if (g_tf[i].key == 0 && freeslot < 0) freeslot = i;
  }
  if (freeslot < 0) return fail(EXGB_EUNSUPPORTED, "too many distinct transform sizes");
  Tf c;
  const int rc = build_tf(n, c);
  if (rc) {
    cudaFree(c.tw);
    cudaFree(c.chirp);
    cudaFree(c.bhat);
    cudaFree(c.tw2);
    cudaFree(c.twn);
    return rc;
  }
  c.key = key;
  g_tf[freeslot] = c;
  *out = &g_tf[freeslot];
  return EXGB_OK;
}

// Transform of length n available on this device (the lengths rfftn/irfftn accept).
int transform_supported(int n) {
  const Tf* tf;
  return get_tf(n, &tf);
}

int rfftn_impl(cudaStream_t st, int D, int N, int64_t count, const float* in, float2* out) {
  const Tf* tf;
  int rc = get_tf(N, &tf);
  if (rc) return rc;
  const int M = N / 2 + 1;
  if (D == 1) return launch_rows(st, *tf, false, count, in, nullptr, out, nullptr, 1.f);
  if (D == 2) {
    rc = launch_rows(st, *tf, false, count * N, in, nullptr, out, nullptr, 1.f);
    if (rc) return rc;
    return launch_axis(st, *tf, false, count, (int64_t)N * M, M, M, out, out, 1.f);
  }
  if (D == 3) {
    const int64_t plane = (int64_t)N * M;
    rc = launch_rows(st, *tf, false, count * N * N, in, nullptr, out, nullptr, 1.f);
    if (rc) return rc;
    rc = launch_axis(st, *tf, false, count * N, plane, M, M, out, out, 1.f);
    if (rc) return rc;
    return launch_axis(st, *tf, false, count, plane * N, plane, plane, out, out, 1.f);
  }
  return fail(EXGB_EUNSUPPORTED, "num_spatial_dims must be 1, 2 or 3");
}

int irfftn_impl(cudaStream_t st, int D, int N, int64_t count, const float2* in, float* out) {
  const Tf* tf;
  int rc = get_tf(N, &tf);
  if (rc) return rc;
  const int M = N / 2 + 1;
  if (D == 1) return launch_rows(st, *tf, true, count, nullptr, in, nullptr, out, 1.f / (float)N);
  if (D == 2) {
    float2* tmp = (float2*)workspace(sizeof(float2) * (size_t)count * N * M, 0);
    if (!tmp) return fail(EXGB_ENOMEM, "workspace allocation failed");
    rc = launch_axis(st, *tf, true, count, (int64_t)N * M, M, M, in, tmp, 1.f);
    if (rc) return rc;
    return launch_rows(st, *tf, true, count * N, nullptr, tmp, nullptr, out, 1.f / ((float)N * (float)N));
  }
  if (D == 3) {
    const int64_t plane = (int64_t)N * M;
    float2* tmp = (float2*)workspace(sizeof(float2) * (size_t)count * N * plane, 0);
    if (!tmp) return fail(EXGB_ENOMEM, "workspace allocation failed");
    rc = launch_axis(st, *tf, true, count, plane * N, plane, plane, in, tmp, 1.f);
    if (rc) return rc;
    rc = launch_axis(st, *tf, true, count * N, plane, M, M, tmp, tmp, 1.f);
    if (rc) return rc;
    return launch_rows(st, *tf, true, count * N * N, nullptr, tmp, nullptr, out,
                       1.f / ((float)N * (float)N * (float)N));
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
