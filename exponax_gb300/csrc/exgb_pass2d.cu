// exgb_pass2d.cu -- 2D ETDRK stages of the staged nonlinearities in three fused passes per stage.
//
// The staged N-D path (exgb_ndgen.cu) spends five kernels and about a dozen HBM passes on a stage:
// derive, inverse transform (two axis passes), pointwise, forward transform (two axis passes),
// combine.  In 2D the same arithmetic (exgb_ndops.cuh, one definition for both paths) runs here in
// three passes, each reading and writing global memory once:
//   pass 1  per tile of ky columns: the NI derived spectra of every mode of the columns (pre-mask),
//           inverse transforms along kx in shared memory            -> W[f][ky][x]
//   pass 2  per tile of rows x: for each of the NI fields the c2r transform along y (two real rows
//           packed in one complex transform, 1/N^2 folded in), the pointwise products, the r2c
//           transforms of the NF products (packed in pairs)          -> Hq[f][ky][x], ky <= K
//   pass 3  per tile of ky columns: forward transforms along x, post-mask and multipliers
//           (combine), the ETDRK stage update of every channel of the mode
// Only the Kc = K + 1 columns inside the dealiasing mask (all N/2 + 1 without a mask) take part;
// the columns above it feel the linear part alone (the post-mask zeroes their nonlinear term), so
// they are advanced by E once per step in a separate elementwise kernel with the same c2r projection.
// State and stage buffers are column-major per sample ([c][ky][kx], the coefficient tables of such
// plans share the layout), filled and emptied by transposes at the call boundary.
//
// Reference: nonlin_fun/_base.py:73-137 (pre-mask before every inverse transform, post-mask after
// every forward transform), the nonlinear functions named in exgb_ndops.cuh, etdrk/_etdrk_1..4.py.
#include <cuda_runtime.h>

#include <algorithm>

#include "exgb_internal.h"
#include "exgb_ndops.cuh"
#include "exgb_regfft.cuh"
#include "exgb_stage.cuh"

namespace exgb {

void* workspace(size_t bytes, int slot_offset);

namespace p2d {

using ndg::Geo;
using ndg::MAXC;
using ndg::Prog;

struct Args {
  PlanDev P;
  Geo g;
  Prog p;
  FftPlan fp;          // length N
  const float2* tw;    // N twiddles
  int N, M, K, Kc;     // Kc = columns that enter the nonlinear term
  int TY, TX, TY3;     // columns per pass-1 CTA, rows per pass-2 CTA, columns per pass-3 CTA
  int64_t plane;       // M * N modes per channel
  StageBufs sb;        // [s][c][ky][kx]
  int64_t sstride;     // C * plane
  const float2* xin;   // stage input (sb.U, sb.S or sb.S1)
  float2* W;           // [s][f < NI][x][ky < Kc]
  float2* Hq;          // [s][f < NF][x][ky < Kc]
  int stage;           // ETDRK stage, -1: nonlinear term only
  float2* nout;        // nonlinear term, natural layout [s][c][kx][ky] (stage -1)
};

__device__ __forceinline__ int sgn_of(int i, int N) { return (i <= (N - 1) / 2) ? i : i - N; }

// ---- pass 1: derived spectra of TY columns, inverse transforms along kx
__global__ void __launch_bounds__(256) pass1_kernel(const Args a) {
  extern __shared__ float2 sm1[];
  const int N = a.N, NI = a.p.NI, TY = a.TY;
  const int64_t s = blockIdx.y;
  const int ky0 = blockIdx.x * TY;
  const int ty = min(TY, a.Kc - ky0);
  const int count = NI * TY;  // sequence (f, t) at (f * TY + t) * N
  float2* buf0 = sm1;
  float2* buf1 = sm1 + (size_t)count * N;
  const float2* xs = a.xin + s * a.sstride;
  for (int e = threadIdx.x; e < TY * N; e += blockDim.x) {
    const int t = e / N, kx = e - t * N;
    if (t < ty) {
      const int ky = ky0 + t;
      const int k[3] = {sgn_of(kx, N), ky, 0};
      const bool m = abs(k[0]) <= a.K && ky <= a.K;
      ndg::derive_mode(a.g, a.p, k, m, xs + (int64_t)ky * N + kx, a.plane, buf0 + (size_t)t * N + kx,
                       (int64_t)TY * N);
    } else {
      for (int f = 0; f < NI; ++f) buf0[((size_t)f * TY + t) * N + kx] = make_float2(0.f, 0.f);
    }
  }
  __syncthreads();
  float2* res = result_buf(a.fp, buf0, buf1);
  block_fft<true>(a.fp, buf0, buf1, LinMap{res, N}, count, a.tw, threadIdx.x, blockDim.x, BlockSync{});
  float2* W = a.W + s * (int64_t)NI * a.Kc * N;
  // consecutive threads: consecutive columns of one row x (TY * 8 contiguous bytes)
  for (int e = threadIdx.x; e < count * N; e += blockDim.x) {
    const int t = e % TY, r = e / TY;
    const int x = r % N, f = r / N;
    if (t < ty) W[((int64_t)f * N + x) * a.Kc + ky0 + t] = res[((size_t)f * TY + t) * N + x];
  }
}

// ---- pass 2: c2r along y, pointwise products, r2c along y, for TX rows
__global__ void __launch_bounds__(256) pass2_kernel(const Args a) {
  extern __shared__ float2 sm2[];
  const int N = a.N, NI = a.p.NI, NF = a.p.NF, TX = a.TX, Kc = a.Kc;
  const int M = N / 2 + 1;
  const bool even = (N & 1) == 0;
  const int64_t s = blockIdx.y;
  const int x0 = blockIdx.x * TX;
  const int tx = min(TX, N - x0);
  const int NP = (NI > NF ? NI : NF) * TX / 2;  // complex sequences of the larger transform set
  float2* buf0 = sm2;
  float2* buf1 = sm2 + (size_t)NP * N;
  float* phys = reinterpret_cast<float*>(sm2 + 2 * (size_t)NP * N);  // [NI * TX][N]
  float* prod = phys + (size_t)NI * TX * N;                           // [NF * TX][N]
  const float2* W = a.W + s * (int64_t)NI * Kc * N;
  // c2r inputs: sequence j packs real rows q = 2j, 2j + 1 (q = f * TX + xx)
  const int ni = NI * TX / 2;
  for (int e = threadIdx.x; e < ni * N; e += blockDim.x) {
    const int j = e / N, k = e - j * N;
    const bool ext = k >= M;
    const int kk = ext ? N - k : k;
    const bool real_only = (k == 0) || (even && k == N / 2);
    float2 va = make_float2(0.f, 0.f), vb = va;
    if (kk < Kc) {
      const int qa = 2 * j, qb = 2 * j + 1;
      const int fa = qa / TX, xa = qa - fa * TX, fb = qb / TX, xb = qb - fb * TX;
      if (xa < tx) va = W[((int64_t)fa * N + x0 + xa) * Kc + kk];
      if (xb < tx) vb = W[((int64_t)fb * N + x0 + xb) * Kc + kk];
    }
    buf0[e] = pack_pair(va, vb, ext, real_only);
  }
  __syncthreads();
  float2* res = result_buf(a.fp, buf0, buf1);
  block_fft<true>(a.fp, buf0, buf1, LinMap{res, N}, ni, a.tw, threadIdx.x, blockDim.x, BlockSync{});
  const float inv = 1.f / ((float)N * (float)N);
  for (int e = threadIdx.x; e < ni * N; e += blockDim.x) {
    const int j = e / N, y = e - j * N;
    const float2 z = res[e];
    phys[(size_t)(2 * j) * N + y] = z.x * inv;
    phys[(size_t)(2 * j + 1) * N + y] = z.y * inv;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < TX * N; e += blockDim.x) {
    const int xx = e / N, y = e - xx * N;
    float in[ndg::kMaxNI];
    ndg::load_point(phys + (size_t)xx * N + y, (int64_t)TX * N, NI, in);
    ndg::pointwise_point_reg(a.g, a.p, in, prod + (size_t)xx * N + y, (int64_t)TX * N);
  }
  __syncthreads();
  // r2c: sequence j packs product rows 2j, 2j + 1 (row index q = f * TX + xx)
  const int nf = NF * TX / 2;
  for (int e = threadIdx.x; e < nf * N; e += blockDim.x) {
    const int j = e / N, y = e - j * N;
    buf0[e] = make_float2(prod[(size_t)(2 * j) * N + y], prod[(size_t)(2 * j + 1) * N + y]);
  }
  __syncthreads();
  res = result_buf(a.fp, buf0, buf1);
  block_fft<false>(a.fp, buf0, buf1, LinMap{res, N}, nf, a.tw, threadIdx.x, blockDim.x, BlockSync{});
  float2* Hq = a.Hq + s * (int64_t)NF * Kc * N;
  for (int e = threadIdx.x; e < nf * Kc; e += blockDim.x) {
    const int j = e / Kc, k = e - j * Kc;
    float2 P, Q;
    unpack_pair(res[(size_t)j * N + k], res[(size_t)j * N + (k == 0 ? 0 : N - k)], P, Q);
    const int qa = 2 * j, qb = 2 * j + 1;
    const int fa = qa / TX, xa = qa - fa * TX, fb = qb / TX, xb = qb - fb * TX;
    if (xa < tx) Hq[((int64_t)fa * N + x0 + xa) * Kc + k] = P;
    if (xb < tx) Hq[((int64_t)fb * N + x0 + xb) * Kc + k] = Q;
  }
}

// ---- pass 3: forward transforms along x, combine, ETDRK stage update
__global__ void __launch_bounds__(256) pass3_kernel(const Args a) {
  extern __shared__ float2 sm3[];
  const int N = a.N, NF = a.p.NF, TY = a.TY, C = a.g.C;
  const int64_t s = blockIdx.y;
  const int ky0 = blockIdx.x * TY;
  const int ty = min(TY, a.Kc - ky0);
  const int count = NF * TY;
  float2* buf0 = sm3;
  float2* buf1 = sm3 + (size_t)count * N;
  const float2* Hq = a.Hq + s * (int64_t)NF * a.Kc * N;
  for (int e = threadIdx.x; e < count * N; e += blockDim.x) {
    const int t = e % TY, r = e / TY;
    const int x = r % N, f = r / N;
    buf0[((size_t)f * TY + t) * N + x] = t < ty ? Hq[((int64_t)f * N + x) * a.Kc + ky0 + t] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  float2* res = result_buf(a.fp, buf0, buf1);
  block_fft<false>(a.fp, buf0, buf1, LinMap{res, N}, count, a.tw, threadIdx.x, blockDim.x, BlockSync{});
  for (int e = threadIdx.x; e < ty * N; e += blockDim.x) {
    const int t = e / N, kx = e - t * N;
    const int ky = ky0 + t;
    const int k[3] = {sgn_of(kx, N), ky, 0};
    const bool m = abs(k[0]) <= a.K && ky <= a.K;
    float2 nv[MAXC];
    ndg::combine_mode(a.P, a.g, a.p, k, m, res + (size_t)t * N + kx, (int64_t)TY * N, nv);
    const int64_t r = (int64_t)ky * N + kx;  // column-major mode index
    if (a.stage < 0) {
      float2* o = a.nout + s * a.sstride + (int64_t)kx * a.M + ky;
#pragma unroll
      for (int c = 0; c < MAXC; ++c)
        if (c < C) o[c * a.plane] = nv[c];
      continue;
    }
    // every channel's stage loads in flight together (compile-time channel indices keep nv in registers)
    int64_t so[MAXC], co[MAXC];
#pragma unroll
    for (int c = 0; c < MAXC; ++c) {
      const int cc = c < C ? c : 0;
      so[c] = s * a.sstride + cc * a.plane + r;
      co[c] = (a.P.lin_ch == 1 ? 0 : (int64_t)cc * a.plane) + r;
    }
    stage_upd_channels<MAXC>(a.P, a.sb, C, so, co, a.stage, nv);
  }
}

// ---- the same passes with register (group) FFTs for N = 64, 128, 256, 512: T lanes of a warp hold a
// length-N sequence (E points each, lane l at positions l + T j), one shared-memory transpose per
// transform and no block barrier inside a transform (exgb_regfft.cuh)
template <int N>
struct RegPass {
  static constexpr int E = RegCfg<N>::E, T = RegCfg<N>::T;
  static constexpr int TS = tile_stride<E, T>();
  // every pass keeps each sequence in a slot of SLOT float2 that also serves as its transform's
  // transpose tile (the sequence is in registers meanwhile); at N = 512, where a lane holds 32 points
  // (about 90-128 registers), CTAs of 128 threads (5 per SM against 2 of 256: 2.06e10 -> 2.21e10
  // DOF-steps/s on Kolmogorov 512^2)
  static constexpr int SLOT = N > TS ? N : TS;
  static constexpr int THREADS = N >= 512 ? 128 : 256, NG = THREADS / T;
  static constexpr int THREADS2 = N >= 512 ? 128 : 256, NG2 = THREADS2 / T;
  // float2 offsets: twiddles, then the pass's slots
  static constexpr int TWL = 0, FREE13 = N;
};

template <int N>
__device__ __forceinline__ void load_twl(float2* twl, const float2* __restrict__ tw) {
  constexpr int T = RegCfg<N>::T;
  for (int t = threadIdx.x; t < N; t += blockDim.x) {
    const int k1 = t / T, ll = t % T;
    twl[t] = __ldg(tw + ((ll * k1) % N));  // w_N^(l k1), [k1][l]
  }
}

template <int N>
__device__ __forceinline__ unsigned group_mask() {
  constexpr int T = RegCfg<N>::T;
  const int lane = threadIdx.x & 31;
  return (T == 32) ? 0xffffffffu : (((1u << T) - 1u) << (lane & ~(T - 1)));
}

// `count` sequences of N complex values in slots buf + q * SLOT, transformed in place by the groups;
// a sequence's slot is its transpose tile once the group holds the sequence in registers
template <int N, bool INV>
__device__ __forceinline__ void groups_fft(float2* buf, int count, const float2* twl) {
  using R = RegPass<N>;
  const int gi = threadIdx.x / R::T, l = threadIdx.x % R::T;
  const unsigned gmask = group_mask<N>();
  for (int q = gi; q < count; q += R::NG) {
    float2* slot = buf + (size_t)q * R::SLOT;
    float2 v[R::E];
#pragma unroll
    for (int j = 0; j < R::E; ++j) v[j] = slot[l + R::T * j];
    __syncwarp(gmask);  // every lane holds its points before the slot becomes the tile
    group_fft<R::E, R::T, INV>(v, l, slot, twl, gmask);
#pragma unroll
    for (int j = 0; j < R::E; ++j) slot[l + R::T * j] = v[j];
  }
}

template <int N>
__global__ void __launch_bounds__(RegPass<N>::THREADS) pass1_reg_kernel(const Args a) {
  using R = RegPass<N>;
  constexpr int SL = R::SLOT;
  extern __shared__ __align__(16) float2 smr1[];
  float2* twl = smr1 + R::TWL;
  float2* buf = smr1 + R::FREE13;  // [NI * TY][SLOT]
  const int NI = a.p.NI, TY = a.TY;
  const int64_t s = blockIdx.y;
  const int ky0 = blockIdx.x * TY;
  const int ty = min(TY, a.Kc - ky0);
  load_twl<N>(twl, a.tw);
  const float2* xs = a.xin + s * a.sstride;
  // kU modes per thread at a time, their channel loads issued together
  constexpr int kU = 4;
  static_assert(MAXC == 3, "the channel accessor below picks among 3 registers");
  const int C = a.g.C;
  const int64_t fstride = (int64_t)TY * SL;
  for (int e0 = threadIdx.x; e0 < TY * N; e0 += kU * (int)blockDim.x) {
    float2 xv[kU][MAXC];
    int kk[kU][3];
    bool mk[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const int e = e0 + u * (int)blockDim.x;
      const int ee = e < TY * N ? e : e0;
      const int t = ee / N, kx = ee - t * N;
      const int ky = ky0 + t;
      kk[u][0] = sgn_of(kx, N);
      kk[u][1] = ky;
      kk[u][2] = 0;
      mk[u] = t < ty && abs(kk[u][0]) <= a.K && ky <= a.K;
#pragma unroll
      for (int c = 0; c < MAXC; ++c)
        xv[u][c] = (mk[u] && c < C) ? xs[(int64_t)ky * N + kx + (int64_t)c * a.plane] : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const int e = e0 + u * (int)blockDim.x;
      if (e >= TY * N) break;
      const int t = e / N, kx = e - t * N;
      float2* o = buf + (size_t)t * SL + kx;
      if (t < ty) {
        ndg::derive_mode_xo(
            a.g, a.p, kk[u], mk[u], [&](int c) { return c == 0 ? xv[u][0] : (c == 1 ? xv[u][1] : xv[u][2]); },
            [&](int i, float2 v) { o[i * fstride] = v; });
      } else {
        for (int f = 0; f < NI; ++f) o[f * fstride] = make_float2(0.f, 0.f);
      }
    }
  }
  __syncthreads();
  groups_fft<N, true>(buf, NI * TY, twl);
  __syncthreads();
  float2* W = a.W + s * (int64_t)NI * a.Kc * N;
  for (int e = threadIdx.x; e < NI * TY * N; e += blockDim.x) {
    const int t = e % TY, r = e / TY;
    const int x = r % N, f = r / N;
    if (t < ty) W[((int64_t)f * N + x) * a.Kc + ky0 + t] = buf[((size_t)f * TY + t) * SL + x];
  }
}

// Pass 2 keeps everything in sequence slots of SLOT float2: slot j first serves as the transpose tile
// of the c2r transform of real rows 2j, 2j + 1 (q = f * TX + xx, built from global W in registers),
// then holds those two rows as floats ([0, N) and [N, 2N)); the pointwise products overwrite the
// rows of their first NF fields in place (one thread per grid point), and the r2c transform of product
// rows 2j, 2j + 1 runs in slot j again (rows to registers, slot as tile, spectrum back to the slot).
// (at N = 512 capped to 102 registers for 5 CTAs per SM: 96 without spills, 128 uncapped)
template <int N>
__global__ void __launch_bounds__(RegPass<N>::THREADS2, (N >= 512 ? 5 : 3)) pass2_reg_kernel(const Args a) {
  using R = RegPass<N>;
  constexpr int E = R::E, T = R::T, M = N / 2 + 1, SL = R::SLOT;
  extern __shared__ __align__(16) float2 smr2[];
  float2* twl = smr2 + R::TWL;
  float2* slots = smr2 + R::FREE13;  // [max(NI, NF) * TX / 2][SLOT]
  const int NI = a.p.NI, NF = a.p.NF, TX = a.TX, Kc = a.Kc;
  const int64_t s = blockIdx.y;
  const int x0 = blockIdx.x * TX;
  const int tx = min(TX, N - x0);
  load_twl<N>(twl, a.tw);
  __syncthreads();
  const int gi = threadIdx.x / T, l = threadIdx.x % T;
  const unsigned gmask = group_mask<N>();
  const float2* W = a.W + s * (int64_t)NI * Kc * N;
  const float inv = 1.f / ((float)N * (float)N);
  // c2r: sequence j packs rows qa = 2j, qb = 2j + 1, gathered straight from W
  const int ni = NI * TX / 2;
  for (int j = gi; j < ni; j += R::NG2) {
    const int qa = 2 * j, qb = qa + 1;
    const int fa = qa / TX, xa = qa - fa * TX, fb = qb / TX, xb = qb - fb * TX;
    const float2* wa = W + ((int64_t)fa * N + x0 + xa) * Kc;
    const float2* wb = W + ((int64_t)fb * N + x0 + xb) * Kc;
    float2* slot = slots + (size_t)j * SL;
    float2 v[E];
#pragma unroll
    for (int jj = 0; jj < E; ++jj) {
      const int k = l + T * jj;
      const bool ext = k >= M;
      const int kk = ext ? N - k : k;
      const bool real_only = (k == 0) || (k == N / 2);
      float2 va = make_float2(0.f, 0.f), vb = va;
      if (kk < Kc) {
        if (xa < tx) va = wa[kk];
        if (xb < tx) vb = wb[kk];
      }
      v[jj] = pack_pair(va, vb, ext, real_only);
    }
    group_fft<E, T, true>(v, l, slot, twl, gmask);
    float* rows = reinterpret_cast<float*>(slot);
#pragma unroll
    for (int jj = 0; jj < E; ++jj) {
      const int y = l + T * jj;
      rows[y] = v[jj].x * inv;
      rows[N + y] = v[jj].y * inv;
    }
  }
  __syncthreads();
  // row q at float offset (q / 2) * 2 SL + (q % 2) N; with TX even, field f of point xx sits
  // f * TX * SL floats after field 0
  const int64_t fs = (int64_t)TX * SL;
  for (int e = threadIdx.x; e < TX * N; e += blockDim.x) {
    const int xx = e / N, y = e - xx * N;
    float* base = reinterpret_cast<float*>(slots) + (size_t)(xx >> 1) * 2 * SL + (xx & 1) * N + y;
    float in[ndg::kMaxNI];
    ndg::load_point(base, fs, NI, in);
    ndg::pointwise_point_reg(a.g, a.p, in, base, fs);
  }
  __syncthreads();
  // r2c: sequence j packs product rows 2j, 2j + 1, in place in slot j
  const int nf = NF * TX / 2;
  for (int j = gi; j < nf; j += R::NG2) {
    float2* slot = slots + (size_t)j * SL;
    const float* rows = reinterpret_cast<const float*>(slot);
    float2 v[E];
#pragma unroll
    for (int jj = 0; jj < E; ++jj) {
      const int y = l + T * jj;
      v[jj] = make_float2(rows[y], rows[N + y]);
    }
    __syncwarp(gmask);  // every lane holds its points before the slot becomes the tile
    group_fft<E, T, false>(v, l, slot, twl, gmask);
#pragma unroll
    for (int jj = 0; jj < E; ++jj) slot[l + T * jj] = v[jj];
  }
  __syncthreads();
  float2* Hq = a.Hq + s * (int64_t)NF * Kc * N;
  for (int e = threadIdx.x; e < nf * Kc; e += blockDim.x) {
    const int j = e / Kc, k = e - j * Kc;
    const float2* zb = slots + (size_t)j * SL;
    float2 P, Q;
    unpack_pair(zb[k], zb[k == 0 ? 0 : N - k], P, Q);
    const int qa = 2 * j, qb = qa + 1;
    const int fa = qa / TX, xa = qa - fa * TX, fb = qb / TX, xb = qb - fb * TX;
    if (xa < tx) Hq[((int64_t)fa * N + x0 + xa) * Kc + k] = P;
    if (xb < tx) Hq[((int64_t)fb * N + x0 + xb) * Kc + k] = Q;
  }
}

template <int N>
__global__ void __launch_bounds__(RegPass<N>::THREADS) pass3_reg_kernel(const Args a) {
  using R = RegPass<N>;
  constexpr int SL = R::SLOT;
  extern __shared__ __align__(16) float2 smr3[];
  float2* twl = smr3 + R::TWL;
  float2* buf = smr3 + R::FREE13;  // [NF * TY3][SLOT]
  const int NF = a.p.NF, TY = a.TY3, C = a.g.C;
  const int64_t s = blockIdx.y;
  const int ky0 = blockIdx.x * TY;
  const int ty = min(TY, a.Kc - ky0);
  load_twl<N>(twl, a.tw);
  const float2* Hq = a.Hq + s * (int64_t)NF * a.Kc * N;
  for (int e = threadIdx.x; e < NF * TY * N; e += blockDim.x) {
    const int t = e % TY, r = e / TY;
    const int x = r % N, f = r / N;
    buf[((size_t)f * TY + t) * SL + x] = t < ty ? Hq[((int64_t)f * N + x) * a.Kc + ky0 + t] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  groups_fft<N, false>(buf, NF * TY, twl);
  __syncthreads();
  for (int e = threadIdx.x; e < ty * N; e += blockDim.x) {
    const int t = e / N, kx = e - t * N;
    const int ky = ky0 + t;
    const int k[3] = {sgn_of(kx, N), ky, 0};
    const bool m = abs(k[0]) <= a.K && ky <= a.K;
    float2 nv[MAXC];
    ndg::combine_mode(a.P, a.g, a.p, k, m, buf + (size_t)t * SL + kx, (int64_t)TY * SL, nv);
    const int64_t r = (int64_t)ky * N + kx;
    if (a.stage < 0) {
      float2* o = a.nout + s * a.sstride + (int64_t)kx * a.M + ky;
#pragma unroll
      for (int c = 0; c < MAXC; ++c)
        if (c < C) o[c * a.plane] = nv[c];
      continue;
    }
    // every channel's stage loads in flight together (compile-time channel indices keep nv in registers)
    int64_t so[MAXC], co[MAXC];
#pragma unroll
    for (int c = 0; c < MAXC; ++c) {
      const int cc = c < C ? c : 0;
      so[c] = s * a.sstride + cc * a.plane + r;
      co[c] = (a.P.lin_ch == 1 ? 0 : (int64_t)cc * a.plane) + r;
    }
    stage_upd_channels<MAXC>(a.P, a.sb, C, so, co, a.stage, nv);
  }
}

// natural [s][c][kx][ky] <-> column-major [s][c][ky][kx] for the columns ky < ncol (32 x 32 tiles)
__global__ void transpose_kernel(const float2* __restrict__ in, float2* __restrict__ out, int N, int M, int ncol,
                                 int64_t fields, int to_cols) {
  __shared__ float2 tile[32][33];
  const int64_t f = blockIdx.z;
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;  // bx over kx, by over ky
  const int64_t plane = (int64_t)N * M;
  const float2* src = in + f * plane;
  float2* dst = out + f * plane;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    if (to_cols) {
      const int kx = bx + j, ky = by + threadIdx.x;
      if (kx < N && ky < ncol) tile[j][threadIdx.x] = src[(int64_t)kx * M + ky];
    } else {
      const int ky = by + j, kx = bx + threadIdx.x;
      if (kx < N && ky < ncol) tile[threadIdx.x][j] = src[(int64_t)ky * N + kx];
    }
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    if (to_cols) {
      const int ky = by + j, kx = bx + threadIdx.x;
      if (kx < N && ky < ncol) dst[(int64_t)ky * N + kx] = tile[threadIdx.x][j];
    } else {
      const int kx = bx + j, ky = by + threadIdx.x;
      if (kx < N && ky < ncol) dst[(int64_t)kx * M + ky] = tile[j][threadIdx.x];
    }
  }
}

// c2r projection of a step's physical round trip on the column-major state: ky = 0 and (N even)
// ky = N/2 columns, v(kx) <- (v(kx) + conj(v(-kx))) / 2, one thread per {kx, N - kx} pair
__global__ void project_cols_kernel(float2* __restrict__ U, int N, int M, int Kc, int64_t fields) {
  const int half = N / 2 + 1;
  const int64_t total = fields * 2 * half;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t f = t / (2 * half);
    const int rr = (int)(t - f * 2 * half);
    const int col = rr / half, kx = rr - col * half;
    const int ky = col == 0 ? 0 : N / 2;
    if (col == 1 && ((N & 1) || ky >= Kc)) continue;  // no Nyquist column, or it is a linear column
    const int kx2 = (N - kx) % N;
    float2* c = U + f * (int64_t)N * M + (int64_t)ky * N;
    const float2 v1 = c[kx], v2 = c[kx2];
    const float2 pv = make_float2(0.5f * (v1.x + v2.x), 0.5f * (v1.y - v2.y));
    c[kx] = pv;
    c[kx2] = cconj(pv);
  }
}

// The columns above the mask (ky >= Kc): nsteps of u <- E u (what every ETDRK order gives with a zero
// nonlinear term), with the projection on ky = N/2; natural layout in and out.  One thread per
// {kx, N - kx} pair.  E is column-major [lin_ch][ky][kx].
__global__ void linear_cols_kernel(const float2* __restrict__ E, int lin_ch, int C, int N, int M, int Kc,
                                   int64_t fields, const float2* __restrict__ in, float2* __restrict__ out,
                                   int nsteps, int project, int zero) {
  const int half = N / 2 + 1;
  const int ncol = M - Kc;
  const int64_t total = fields * (int64_t)ncol * half;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t f = t / ((int64_t)ncol * half);
    const int rr = (int)(t - f * (int64_t)ncol * half);
    const int ky = Kc + rr / half, kx = rr % half;
    const int kx2 = (kx == 0) ? 0 : N - kx;
    if (kx2 < kx) continue;
    const int64_t base = f * (int64_t)N * M;
    if (zero) {
      out[base + (int64_t)kx * M + ky] = make_float2(0.f, 0.f);
      out[base + (int64_t)kx2 * M + ky] = make_float2(0.f, 0.f);
      continue;
    }
    const int c = (int)(f % C);
    const float2* Et = E + (lin_ch == 1 ? 0 : (int64_t)c * N * M) + (int64_t)ky * N;
    const float2 e1 = Et[kx], e2 = Et[kx2];
    float2 v1 = in[base + (int64_t)kx * M + ky], v2 = in[base + (int64_t)kx2 * M + ky];
    const bool proj = project && (ky == 0 || ((N & 1) == 0 && ky == N / 2));
    for (int st = 0; st < nsteps; ++st) {
      v1 = cmul(e1, v1);
      v2 = cmul(e2, v2);
      if (proj) {
        const float2 pv = make_float2(0.5f * (v1.x + v2.x), 0.5f * (v1.y - v2.y));
        v1 = pv;
        v2 = cconj(pv);
      }
    }
    out[base + (int64_t)kx * M + ky] = v1;
    if (kx2 != kx) out[base + (int64_t)kx2 * M + ky] = v2;
  }
}

static unsigned grid_for(int64_t n, int sm) {
  const int64_t b = (n + 255) / 256;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)sm * 32));
}

// shared memory of the three passes for tile sizes TY, TX
static size_t smem1(int NI, int TY, int N) { return sizeof(float2) * 2 * (size_t)NI * TY * N; }
static size_t smem2(int NI, int NF, int TX, int N) {
  const size_t np = (size_t)std::max(NI, NF) * TX / 2;
  return sizeof(float2) * 2 * np * N + sizeof(float) * (size_t)(NI + NF) * TX * N;
}
static size_t smem3(int NF, int TY, int N) { return sizeof(float2) * 2 * (size_t)NF * TY * N; }

static size_t smem_limit() {
  static int lim = 0;
  if (!lim) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&lim, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  }
  return (size_t)lim;
}

// tiles: about 2048 complex values per transform set, within half the shared memory
static void tiles(int NI, int NF, int N, int& TY, int& TX) {
  const size_t cap = smem_limit() / 2;
  TY = std::max(1, 2048 / (std::max(NI, NF) * N));
  while (TY > 1 && std::max(smem1(NI, TY, N), smem3(NF, TY, N)) > cap) --TY;
  TX = std::max(2, 2 * (4096 / (std::max(NI, NF) * N) / 2));
  while (TX > 2 && smem2(NI, NF, TX, N) > cap) TX -= 2;
}

// register-FFT passes: tile sizes and shared memory (bytes) for N in {64, 128, 256, 512}
template <int N>
struct RegSizes {
  using R = RegPass<N>;
  static size_t s1(int NI, int TY) { return sizeof(float2) * ((size_t)R::FREE13 + (size_t)NI * TY * R::SLOT); }
  static size_t s2(int NI, int NF, int TX) {
    return sizeof(float2) * ((size_t)R::FREE13 + (size_t)std::max(NI, NF) * TX / 2 * R::SLOT);
  }
  static size_t s3(int NF, int TY3) { return sizeof(float2) * ((size_t)R::FREE13 + (size_t)NF * TY3 * R::SLOT); }
};

template <int N>
static bool reg_tiles(int NI, int NF, int& TY, int& TX, int& TY3) {
  const size_t cap = smem_limit() - 1024;
  // columns per pass-1 CTA: 4 (2 at N = 512, where 128-thread CTAs take one sequence per group)
  TY = N >= 512 ? 2 : 4;
  TX = 4;
  TY3 = std::max(4, std::min(16, RegPass<N>::NG / std::max(1, NF)));  // one sequence per group
  while (TY > 1 && RegSizes<N>::s1(NI, TY) > cap / 2) --TY;
  while (TX > 2 && RegSizes<N>::s2(NI, NF, TX) > cap / 2) TX -= 2;
  while (TY3 > 1 && RegSizes<N>::s3(NF, TY3) > cap / 2) --TY3;
  return RegSizes<N>::s1(NI, TY) <= cap && RegSizes<N>::s2(NI, NF, TX) <= cap && RegSizes<N>::s3(NF, TY3) <= cap;
}

template <int N>
static int set_reg_attrs(const Args& a) {
  EXGB_CUDA(cudaFuncSetAttribute(pass1_reg_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)RegSizes<N>::s1(a.p.NI, a.TY)));
  EXGB_CUDA(cudaFuncSetAttribute(pass2_reg_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)RegSizes<N>::s2(a.p.NI, a.p.NF, a.TX)));
  EXGB_CUDA(cudaFuncSetAttribute(pass3_reg_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)RegSizes<N>::s3(a.p.NF, a.TY3)));
  return EXGB_OK;
}

template <int N>
static void launch_reg(const Args& a, int64_t n, cudaStream_t st) {
  constexpr int TH = RegPass<N>::THREADS, TH2 = RegPass<N>::THREADS2;
  const unsigned c1 = (unsigned)((a.Kc + a.TY - 1) / a.TY), c3 = (unsigned)((a.Kc + a.TY3 - 1) / a.TY3);
  const unsigned r2 = (unsigned)((N + a.TX - 1) / a.TX);
  pass1_reg_kernel<N><<<dim3(c1, (unsigned)n), TH, RegSizes<N>::s1(a.p.NI, a.TY), st>>>(a);
  pass2_reg_kernel<N><<<dim3(r2, (unsigned)n), TH2, RegSizes<N>::s2(a.p.NI, a.p.NF, a.TX), st>>>(a);
  pass3_reg_kernel<N><<<dim3(c3, (unsigned)n), TH, RegSizes<N>::s3(a.p.NF, a.TY3), st>>>(a);
}

}  // namespace p2d

using namespace p2d;

// Can the three-pass path step this 2D staged plan?  N = 2^a 3^b 5^c with the pass-2 tile of two rows
// within one CTA's shared memory.
bool pass2d_supported(int D, int N, int NI, int NF) {
  if (D != 2 || N < 2 || NI < 1 || NF < 1) return false;
  FftPlan fp;
  if (!make_fft_plan(N, &fp)) return false;
  return std::max(p2d::smem1(NI, 1, N), std::max(p2d::smem2(NI, NF, 2, N), p2d::smem3(NF, 1, N))) <=
         p2d::smem_limit() - 1024;
}

int pass2d_run(const exgb_plan* plan, const Geo& g0, const Prog& prog, cudaStream_t st, const float2* in, float2* out,
               int64_t batch, int nsteps, int project, int nonlinear_only) {
  const PlanDev& P = plan->dev;
  const int N = P.N, M = P.M, C = P.C;
  const int K = std::min(P.kmax, N / 2);
  const int Kc = std::min(M, K + 1);
  const int sm = plan->sm_count;
  const int64_t plane = (int64_t)N * M;
  if (batch == 0) return EXGB_OK;
  if (!nonlinear_only && nsteps == 0) {
    if (in != out) EXGB_CUDA(cudaMemcpyAsync(out, in, sizeof(float2) * batch * C * plane, cudaMemcpyDeviceToDevice, st));
    return EXGB_OK;
  }
  Args a{};
  a.P = P;
  a.g = g0;
  a.p = prog;
  a.fp = P.fft;
  a.tw = P.tw;
  a.N = N;
  a.M = M;
  a.K = K;
  a.Kc = Kc;
  // register-FFT passes at N = 64, 128, 256, 512, shared-memory Stockham passes otherwise
  bool reg = false;
  switch (N) {
    case 64: reg = reg_tiles<64>(prog.NI, prog.NF, a.TY, a.TX, a.TY3); break;
    case 128: reg = reg_tiles<128>(prog.NI, prog.NF, a.TY, a.TX, a.TY3); break;
    case 256: reg = reg_tiles<256>(prog.NI, prog.NF, a.TY, a.TX, a.TY3); break;
    case 512: reg = reg_tiles<512>(prog.NI, prog.NF, a.TY, a.TX, a.TY3); break;
    default: break;
  }
  if (!reg) {
    tiles(prog.NI, prog.NF, N, a.TY, a.TX);
    a.TY3 = a.TY;
  }
  a.plane = plane;
  a.sstride = (int64_t)C * plane;
  const int nb = stage_nbufs(P.order);
  const size_t per_sample = sizeof(float2) * ((size_t)(nonlinear_only ? 1 : nb) * C * plane +
                                              (size_t)(prog.NI + prog.NF) * Kc * N);
  const int64_t cb = std::max<int64_t>(1, std::min<int64_t>(batch, (int64_t)((size_t)(1u << 30) / per_sample)));
  char* ws = (char*)workspace(per_sample * (size_t)cb, 5);
  if (!ws) return fail(EXGB_ENOMEM, "workspace allocation failed");
  const size_t s1 = smem1(prog.NI, a.TY, N), s2 = smem2(prog.NI, prog.NF, a.TX, N), s3 = smem3(prog.NF, a.TY, N);
  if (reg) {
    int rc = EXGB_OK;
    switch (N) {
      case 64: rc = set_reg_attrs<64>(a); break;
      case 128: rc = set_reg_attrs<128>(a); break;
      case 256: rc = set_reg_attrs<256>(a); break;
      default: rc = set_reg_attrs<512>(a); break;
    }
    if (rc) return rc;
  } else {
    EXGB_CUDA(cudaFuncSetAttribute(pass1_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s1));
    EXGB_CUDA(cudaFuncSetAttribute(pass2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s2));
    EXGB_CUDA(cudaFuncSetAttribute(pass3_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s3));
  }
  const int ycols = (Kc + a.TY - 1) / a.TY, xrows = (N + a.TX - 1) / a.TX;
  for (int64_t b0 = 0; b0 < batch; b0 += cb) {
    const int64_t n = std::min<int64_t>(cb, batch - b0);
    if (n * C > 65535) return fail(EXGB_EUNSUPPORTED, "too many fields for one launch");
    const float2* src = in + b0 * a.sstride;
    float2* dst = out + b0 * a.sstride;
    float2* q = (float2*)ws;
    const int64_t fsz = a.sstride * n;
    a.sb = stage_bufs(q, nonlinear_only ? 1 : P.order, fsz);
    q += (int64_t)(nonlinear_only ? 1 : nb) * fsz;
    a.W = q;
    q += (int64_t)prog.NI * Kc * N * n;
    a.Hq = q;
    // a.sb.U = column-major copy of the masked columns
    {
      dim3 grid((N + 31) / 32, (Kc + 31) / 32, (unsigned)(n * C));
      transpose_kernel<<<grid, dim3(32, 8), 0, st>>>(src, a.sb.U, N, M, Kc, n * C, 1);
    }
    const int nst = nonlinear_only ? 1 : P.order;
    const int Q = nonlinear_only ? 1 : nsteps * P.order;
    for (int qq = 0; qq < Q; ++qq) {
      const int stage = qq % nst;
      a.stage = nonlinear_only ? -1 : stage;
      a.nout = nonlinear_only ? dst : nullptr;
      a.xin = (stage == 0) ? a.sb.U : (P.order == 4 && stage == 1) ? a.sb.S1 : a.sb.S;
      if (reg) {
        switch (N) {
          case 64: launch_reg<64>(a, n, st); break;
          case 128: launch_reg<128>(a, n, st); break;
          case 256: launch_reg<256>(a, n, st); break;
          default: launch_reg<512>(a, n, st); break;
        }
      } else {
        pass1_kernel<<<dim3(ycols, (unsigned)n), 256, s1, st>>>(a);
        pass2_kernel<<<dim3(xrows, (unsigned)n), 256, s2, st>>>(a);
        pass3_kernel<<<dim3(ycols, (unsigned)n), 256, s3, st>>>(a);
      }
      if (!nonlinear_only && stage == nst - 1 && project)
        project_cols_kernel<<<grid_for(n * C * 2 * (N / 2 + 1), sm), 256, 0, st>>>(a.sb.U, N, M, Kc, n * C);
      EXGB_CUDA(cudaGetLastError());
    }
    if (!nonlinear_only) {
      dim3 grid((N + 31) / 32, (Kc + 31) / 32, (unsigned)(n * C));
      transpose_kernel<<<grid, dim3(32, 8), 0, st>>>(a.sb.U, dst, N, M, Kc, n * C, 0);
    }
    if (Kc < M)
      linear_cols_kernel<<<grid_for(n * C * (int64_t)(M - Kc) * (N / 2 + 1), sm), 256, 0, st>>>(
          P.E, P.lin_ch, C, N, M, Kc, n * C, src, dst, nsteps, project, nonlinear_only);
    EXGB_CUDA(cudaGetLastError());
  }
  return EXGB_OK;
}

}  // namespace exgb
