// exgb_pass3d.cu -- 3D ETDRK stages (projected convection + Leray, and the nonlinearities of the
// staged N-D path) in three fused passes per stage, for N = 32, 64 and 128.
//
// The 3D counterpart of exgb_pass2d.cu: the rfft axis z takes the role of the 2D column index.
//   pass 1  per (kz plane, derived field): the field's spectrum on the plane (pre-mask, exgb_ndops.cuh),
//           2D inverse transform over (kx, ky) in shared memory          -> W[f][kz][x][y]
//   pass 2  per (x, tile of y): for each of the NI fields the c2r transform along z (two lines packed
//           in one complex transform, 1/N^3 folded in), the pointwise products (the cross product u x
//           curl u for projected convection), the r2c transforms of the NF products -> Hq[f][kz][x][y]
//   pass 3  per (kz plane, product field): 2D forward transform in place in Hq, then one elementwise
//           kernel over the Kc planes: post-mask, multipliers (Leray projection and forcing for
//           projected convection) and the ETDRK stage update (Hq still in L2)
// Only the Kc = K + 1 planes inside the dealiasing mask take part; the planes above it feel the linear
// part alone and are advanced by E once per step from the input in one elementwise kernel.  State and
// stage buffers are plane-major ([c][kz][kx][ky], kz < Kc), the coefficient tables of such plans
// plane-major over all N/2 + 1 planes; transposes at the call boundary.  Transforms are register
// (group) FFTs (exgb_regfft.cuh).
//
// Reference: nonlin_fun/_projected_convection.py:114-226, _leray.py:114-136, nonlin_fun/_base.py:73-137,
// the nonlinear functions named in exgb_ndops.cuh, etdrk/_etdrk_1..4.py.
#include <cuda_runtime.h>

#include <algorithm>

#include "exgb_internal.h"
#include "exgb_ndops.cuh"
#include "exgb_regfft.cuh"
#include "exgb_stage.cuh"

namespace exgb {

void* workspace(size_t bytes, int slot_offset);

namespace p3d {

using ndg::Geo;
using ndg::MAXC;
using ndg::Prog;

struct Args {
  PlanDev P;
  Geo g;
  Prog p;
  const float2* tw;  // N twiddles
  int N, M, K, Kc;
  int TY;            // y lines per pass-2 CTA
  int64_t pl;        // N * N modes of a plane
  int64_t cstride;   // Kc * pl: one channel of the plane-major state
  int64_t sstride;   // C * cstride
  int64_t tstride;   // M * pl: one coefficient set (plane-major tables)
  StageBufs sb;
  const float2* xin;
  float2* W;         // [s][f < NI][kz < Kc][x][y]
  float2* Hq;        // [s][f < NF][kz < Kc][x][y]
  int stage;         // -1: nonlinear term only, written to nout (natural layout [s][c][kx][ky][kz])
  float2* nout;
  int sm;            // SM count (grid of the elementwise kernels)
};

__device__ __forceinline__ int sgn_of(int i, int N) { return (i <= (N - 1) / 2) ? i : i - N; }

template <int N>
struct Cfg {
  static constexpr int E = RegCfg<N>::E, T = RegCfg<N>::T;
  static constexpr int THREADS = 256, NG = THREADS / T;
  // pass 2: up to N = 64, 24 transform groups, one per line pair of projected convection's 6 fields
  // x 8 lines (32 groups left a quarter idle: 32^3 +10 %, 64^3 +2 %); 32 at N = 128 (24: -6 %)
  static constexpr int NG2 = N <= 64 ? 24 : 32, THREADS2 = NG2 * T;
  static constexpr int TS = tile_stride<E, T>();
  static constexpr int SLOT = N > TS ? N : TS;  // pass 2: a pair of lines, also its transform's tile
  static constexpr int PS = N + 1;  // padded row stride of a plane in shared memory
  static constexpr int PLANE = N * PS;
  // float2 offsets: twiddles, transpose tiles, then the pass's planes / buffers
  static constexpr int TWL = 0, TILES = N, FREE = N + NG * TS;
};

template <int N>
__device__ __forceinline__ void load_twl(float2* twl, const float2* __restrict__ tw) {
  constexpr int T = RegCfg<N>::T;
  for (int t = threadIdx.x; t < N; t += blockDim.x) {
    const int k1 = t / T, ll = t % T;
    twl[t] = __ldg(tw + ((ll * k1) % N));
  }
}

template <int N>
__device__ __forceinline__ unsigned group_mask() {
  constexpr int T = RegCfg<N>::T;
  const int lane = threadIdx.x & 31;
  return (T == 32) ? 0xffffffffu : (((1u << T) - 1u) << (lane & ~(T - 1)));
}

// Transforms of the lines of a plane in shared memory (rows kx, row stride PS), in place: ROWS along
// the second index (line r at plane[r PS + x]), otherwise along the first (line c at plane[x PS + c]).
// K >= 0 takes only the lines with |signed index| <= K (the others are zero, or their outputs are not
// needed); K < 0 takes all N.  When the plane has at least two lines per transform group, a group
// takes two lines at once (group_fft_x2), so that the lines of a plane need half the rounds.
template <int N, bool INV, bool ROWS>
__device__ __forceinline__ void plane_fft(float2* plane, float2* tiles, const float2* twl, int K) {
  using R = Cfg<N>;
  constexpr bool kPair = N >= 2 * R::NG;
  const int gi = threadIdx.x / R::T, l = threadIdx.x % R::T;
  const unsigned gmask = group_mask<N>();
  float2* tile = tiles + (size_t)gi * R::TS;
  const int nl = (K >= 0 && 2 * K + 1 < N) ? 2 * K + 1 : N;
  auto line = [&](int q) { return q <= (nl - 1) / 2 || nl == N ? q : q + (N - nl); };
  auto at = [&](int ln, int j) -> float2& {
    return ROWS ? plane[(size_t)ln * R::PS + l + R::T * j] : plane[(size_t)(l + R::T * j) * R::PS + ln];
  };
  if constexpr (kPair) {
    for (int q = 2 * gi; q < nl; q += 2 * R::NG) {
      const int a = line(q);
      float2 v[R::E];
#pragma unroll
      for (int j = 0; j < R::E; ++j) v[j] = at(a, j);
      if (q + 1 < nl) {
        const int b = line(q + 1);
        float2 w[R::E];
#pragma unroll
        for (int j = 0; j < R::E; ++j) w[j] = at(b, j);
        group_fft_x2<R::E, R::T, INV>(v, w, l, tile, twl, gmask);
#pragma unroll
        for (int j = 0; j < R::E; ++j) at(b, j) = w[j];
      } else {
        group_fft<R::E, R::T, INV>(v, l, tile, twl, gmask);
      }
#pragma unroll
      for (int j = 0; j < R::E; ++j) at(a, j) = v[j];
    }
  } else {
    for (int q = gi; q < nl; q += R::NG) {
      const int a = line(q);
      float2 v[R::E];
#pragma unroll
      for (int j = 0; j < R::E; ++j) v[j] = at(a, j);
      group_fft<R::E, R::T, INV>(v, l, tile, twl, gmask);
#pragma unroll
      for (int j = 0; j < R::E; ++j) at(a, j) = v[j];
    }
  }
}

// ---- pass 1: one derived field on one kz plane (derived by consecutive threads over consecutive
// modes, into shared memory), 2D inverse over (kx, ky)
template <int N>
__global__ void __launch_bounds__(Cfg<N>::THREADS) pass1_3d_kernel(const Args a) {
  using R = Cfg<N>;
  extern __shared__ __align__(16) float2 sp1[];
  float2* twl = sp1 + R::TWL;
  float2* plane = sp1 + R::FREE;
  const int kz = blockIdx.x, f = blockIdx.y;
  const int64_t s = blockIdx.z;
  load_twl<N>(twl, a.tw);
  const float2* xs = a.xin + s * a.sstride + (int64_t)kz * a.pl;
  // kU modes per thread at a time: their channel loads are issued together, and only field f of the
  // derived spectra is kept (in a register, not a runtime-indexed local array)
  constexpr int kU = 4;
  static_assert(MAXC == 3, "the channel accessor below picks among 3 registers");
  const int C = a.g.C;
  for (int e0 = threadIdx.x; e0 < N * N; e0 += kU * (int)blockDim.x) {
    float2 xv[kU][MAXC];
    int kk[kU][3];
    bool mk[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const int e = e0 + u * (int)blockDim.x;
      const int ee = e < N * N ? e : e0;
      const int kx = ee / N, ky = ee - kx * N;
      kk[u][0] = sgn_of(kx, N);
      kk[u][1] = sgn_of(ky, N);
      kk[u][2] = kz;
      mk[u] = abs(kk[u][0]) <= a.K && abs(kk[u][1]) <= a.K && kz <= a.K;
#pragma unroll
      for (int c = 0; c < MAXC; ++c)
        xv[u][c] = (mk[u] && c < C) ? xs[ee + (int64_t)c * a.cstride] : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const int e = e0 + u * (int)blockDim.x;
      if (e >= N * N) break;
      float2 r = make_float2(0.f, 0.f);
      ndg::derive_mode_xo(
          a.g, a.p, kk[u], mk[u], [&](int c) { return c == 0 ? xv[u][0] : (c == 1 ? xv[u][1] : xv[u][2]); },
          [&](int i, float2 v) {
            if (i == f) r = v;
          });
      plane[(size_t)(e / N) * R::PS + (e % N)] = r;
    }
  }
  __syncthreads();
  plane_fft<N, true, true>(plane, sp1 + R::TILES, twl, a.K);  // rows |kx| > K are zero
  __syncthreads();
  plane_fft<N, true, false>(plane, sp1 + R::TILES, twl, -1);
  __syncthreads();
  float2* W = a.W + ((s * a.p.NI + f) * a.Kc + kz) * a.pl;
  for (int e = threadIdx.x; e < N * N; e += blockDim.x) W[e] = plane[(size_t)(e / N) * R::PS + (e % N)];
}

// ---- pass 2: lines along z at (x, y0 .. y0 + TY): c2r, pointwise, r2c.  The W values of the tile
// are staged in shared memory first (runs of TY consecutive y per (field, kz)); each pair of lines
// has a slot of SLOT float2 that is the transpose tile of its c2r transform, then holds the two
// physical lines, then (products overwritten in place) the pair's r2c transform and spectrum; the
// spectra leave as runs of TY consecutive y again.
template <int N>
__global__ void __launch_bounds__(Cfg<N>::THREADS2, (N == 32 ? 16 : N == 64 ? 8 : 4)) pass2_3d_kernel(const Args a) {
  using R = Cfg<N>;
  constexpr int E = R::E, T = R::T, M = N / 2 + 1, SL = R::SLOT;
  extern __shared__ __align__(16) float2 sp2[];
  const int NI = a.p.NI, NF = a.p.NF, TY = a.TY, Kc = a.Kc;
  float2* twl = sp2 + R::TWL;
  float2* wt = sp2 + N;                            // [NI][Kc][TY]
  float2* slots = wt + (size_t)NI * Kc * TY;       // [max(NI, NF) * TY / 2][SLOT]
  const int x = blockIdx.x / (N / TY), y0 = (blockIdx.x % (N / TY)) * TY;
  const int64_t s = blockIdx.y;
  load_twl<N>(twl, a.tw);
  // element (f, kz) of line (x, y) in W / Hq: ((s NI + f) Kc + kz) pl + x N + y
  const float2* W = a.W + s * (int64_t)NI * Kc * a.pl + (int64_t)x * N + y0;
#pragma unroll 4
  for (int e = threadIdx.x; e < NI * Kc * TY; e += blockDim.x) {
    const int yy = e % TY, r = e / TY;  // r = f Kc + kz
    wt[e] = W[(int64_t)r * a.pl + yy];
  }
  __syncthreads();
  const int gi = threadIdx.x / T, l = threadIdx.x % T;
  const unsigned gmask = group_mask<N>();
  const float inv = 1.f / ((float)N * (float)N * (float)N);
  const int ni = NI * TY / 2;
  for (int j = gi; j < ni; j += R::NG2) {
    const int qa = 2 * j, qb = qa + 1;
    const int fa = qa / TY, ya = qa - fa * TY, fb = qb / TY, yb = qb - fb * TY;
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
        va = wt[((size_t)fa * Kc + kk) * TY + ya];
        vb = wt[((size_t)fb * Kc + kk) * TY + yb];
      }
      v[jj] = pack_pair(va, vb, ext, real_only);
    }
    group_fft<E, T, true>(v, l, slot, twl, gmask);
    float* rows = reinterpret_cast<float*>(slot);
#pragma unroll
    for (int jj = 0; jj < E; ++jj) {
      const int z = l + T * jj;
      rows[z] = v[jj].x * inv;
      rows[N + z] = v[jj].y * inv;
    }
  }
  __syncthreads();
  // line q = f TY + yy at float offset (q / 2) 2 SL + (q % 2) N: field f of line yy is f TY SL floats on
  const int64_t fs = (int64_t)TY * SL;
  for (int e = threadIdx.x; e < TY * N; e += blockDim.x) {
    const int yy = e / N, z = e - yy * N;
    float* base = reinterpret_cast<float*>(slots) + (size_t)(yy >> 1) * 2 * SL + (yy & 1) * N + z;
    if (a.p.op == ndg::OP_PROJ3D) {  // u x (curl u): six loads, no guarded ones (measured 2 % faster)
      const float w0 = base[0], w1 = base[fs], w2 = base[2 * fs];
      const float v0 = base[3 * fs], v1 = base[4 * fs], v2 = base[5 * fs];
      base[0] = v1 * w2 - v2 * w1;
      base[fs] = v2 * w0 - v0 * w2;
      base[2 * fs] = v0 * w1 - v1 * w0;
      continue;
    }
    float in[ndg::kMaxNI];
    ndg::load_point(base, fs, NI, in);
    ndg::pointwise_point_reg(a.g, a.p, in, base, fs);
  }
  __syncthreads();
  const int nf = NF * TY / 2;
  for (int j = gi; j < nf; j += R::NG2) {
    float2* slot = slots + (size_t)j * SL;
    const float* rows = reinterpret_cast<const float*>(slot);
    float2 v[E];
#pragma unroll
    for (int jj = 0; jj < E; ++jj) {
      const int z = l + T * jj;
      v[jj] = make_float2(rows[z], rows[N + z]);
    }
    __syncwarp(gmask);  // every lane holds its points before the slot becomes the tile
    group_fft<E, T, false>(v, l, slot, twl, gmask);
#pragma unroll
    for (int jj = 0; jj < E; ++jj) slot[l + T * jj] = v[jj];
  }
  __syncthreads();
  float2* Hq = a.Hq + s * (int64_t)NF * Kc * a.pl + (int64_t)x * N + y0;
  for (int e = threadIdx.x; e < NF * Kc * TY; e += blockDim.x) {
    const int yy = e % TY, r = e / TY;  // r = f Kc + k
    const int f = r / Kc, k = r - f * Kc;
    const int q = f * TY + yy;
    const float2* zb = slots + (size_t)(q >> 1) * SL;
    float2 P, Q;
    unpack_pair(zb[k], zb[k == 0 ? 0 : N - k], P, Q);
    Hq[(int64_t)r * a.pl + yy] = (q & 1) ? Q : P;
  }
}

// ---- pass 3a: 2D forward transform of one product field on one kz plane, in place in Hq; rows go
// from global memory straight into the registers of their transform group
template <int N>
__global__ void __launch_bounds__(Cfg<N>::THREADS) pass3_3d_kernel(const Args a) {
  using R = Cfg<N>;
  extern __shared__ __align__(16) float2 sp3[];
  float2* twl = sp3 + R::TWL;
  float2* plane = sp3 + R::FREE;
  const int kz = blockIdx.x, f = blockIdx.y;
  const int64_t s = blockIdx.z;
  load_twl<N>(twl, a.tw);
  __syncthreads();
  const int gi = threadIdx.x / R::T, l = threadIdx.x % R::T;
  const unsigned gmask = group_mask<N>();
  float2* tile = sp3 + R::TILES + (size_t)gi * R::TS;
  float2* H = a.Hq + ((s * a.p.NF + f) * a.Kc + kz) * a.pl;
  for (int kx = gi; kx < N; kx += R::NG) {
    float2 v[R::E];
#pragma unroll
    for (int j = 0; j < R::E; ++j) v[j] = H[kx * N + l + R::T * j];
    group_fft<R::E, R::T, false>(v, l, tile, twl, gmask);
#pragma unroll
    for (int j = 0; j < R::E; ++j) plane[(size_t)kx * R::PS + l + R::T * j] = v[j];
  }
  __syncthreads();
  plane_fft<N, false, false>(plane, sp3 + R::TILES, twl, a.K);  // the combine reads |ky| <= K only
  __syncthreads();
  for (int e = threadIdx.x; e < N * N; e += blockDim.x) H[e] = plane[(size_t)(e / N) * R::PS + (e % N)];
}

// ---- pass 3b: post-mask, multipliers and the ETDRK stage update of every mode of the Kc planes
// (Hq was written by pass 3a just before and is read from L2)
__global__ void __launch_bounds__(256, 5) combine_planes_kernel(const Args a, int64_t n) {
  const int N = a.N, C = a.g.C, NF = a.p.NF;
  const int64_t per = a.Kc * a.pl;
  const int64_t total = n * per;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = t / per, r = t - s * per;  // r = kz pl + kx N + ky
    const int kz = (int)(r / a.pl);
    const int e = (int)(r - (int64_t)kz * a.pl);
    const int kx = e / N, ky = e - kx * N;
    const int k[3] = {sgn_of(kx, N), sgn_of(ky, N), kz};
    const bool m = abs(k[0]) <= a.K && abs(k[1]) <= a.K && kz <= a.K;
    float2 nv[MAXC];
    ndg::combine_mode(a.P, a.g, a.p, k, m, a.Hq + s * NF * per + r, per, nv);
    if (a.stage < 0) {
      float2* o = a.nout + s * (int64_t)C * a.tstride + (int64_t)e * a.M + kz;
#pragma unroll
      for (int c = 0; c < MAXC; ++c)
        if (c < C) o[c * a.tstride] = nv[c];
      continue;
    }
    // every channel's stage loads in flight together (compile-time channel indices keep nv in registers)
    int64_t so[MAXC], co[MAXC];
#pragma unroll
    for (int c = 0; c < MAXC; ++c) {
      const int cc = c < C ? c : 0;
      so[c] = s * a.sstride + cc * a.cstride + r;
      co[c] = (a.P.lin_ch == 1 ? 0 : (int64_t)cc * a.tstride) + r;
    }
    stage_upd_channels<MAXC>(a.P, a.sb, C, so, co, a.stage, nv);
  }
}

// natural [f][kx][ky][kz] (rows kx N + ky, M columns) <-> plane-major [f][kz][kx][ky] for kz < ncol;
// `cols_stride` = elements per field on the plane-major side
__global__ void transpose3_kernel(const float2* __restrict__ in, float2* __restrict__ out, int64_t rows, int M,
                                  int ncol, int64_t cols_stride, int to_cols) {
  __shared__ float2 tile[32][33];
  const int64_t f = blockIdx.z;
  const int64_t br = (int64_t)blockIdx.x * 32;
  const int bc = blockIdx.y * 32;
  const int64_t nat = rows * M;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    if (to_cols) {
      const int64_t r = br + j;
      const int c = bc + threadIdx.x;
      if (r < rows && c < ncol) tile[j][threadIdx.x] = in[f * nat + r * M + c];
    } else {
      const int c = bc + j;
      const int64_t r = br + threadIdx.x;
      if (r < rows && c < ncol) tile[threadIdx.x][j] = in[f * cols_stride + (int64_t)c * rows + r];
    }
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    if (to_cols) {
      const int c = bc + j;
      const int64_t r = br + threadIdx.x;
      if (r < rows && c < ncol) out[f * cols_stride + (int64_t)c * rows + r] = tile[threadIdx.x][j];
    } else {
      const int64_t r = br + j;
      const int c = bc + threadIdx.x;
      if (r < rows && c < ncol) out[f * nat + r * M + c] = tile[j][threadIdx.x];
    }
  }
}

// c2r projection of a step's round trip on the plane-major state: planes kz = 0 and (N even, inside the
// mask) kz = N/2, v(kx, ky) <- (v(kx, ky) + conj(v(-kx, -ky))) / 2; one thread per pair
__global__ void project_planes_kernel(float2* __restrict__ U, int N, int Kc, int64_t cstride, int64_t fields) {
  const int64_t pl = (int64_t)N * N;
  const int64_t total = fields * 2 * pl;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t f = t / (2 * pl);
    const int64_t rr = t - f * 2 * pl;
    const int which = (int)(rr / pl);
    const int64_t q = rr - which * pl;
    const int kz = which == 0 ? 0 : N / 2;
    if (which == 1 && ((N & 1) || kz >= Kc)) continue;
    const int kx = (int)(q / N), ky = (int)(q % N);
    const int64_t q2 = (int64_t)((N - kx) % N) * N + (N - ky) % N;
    if (q2 < q) continue;
    float2* base = U + f * cstride + (int64_t)kz * pl;
    const float2 v1 = base[q], v2 = base[q2];
    const float2 pv = make_float2(0.5f * (v1.x + v2.x), 0.5f * (v1.y - v2.y));
    base[q] = pv;
    base[q2] = cconj(pv);
  }
}

// planes above the mask (kz >= Kc): nsteps of u <- E u, projection on kz = N/2; natural layout in and
// out, E plane-major [lin_ch][kz][kx][ky]; one thread per {(kx, ky), (-kx, -ky)} pair
__global__ void linear_planes_kernel(const float2* __restrict__ E, int lin_ch, int C, int N, int M, int Kc,
                                     int64_t fields, const float2* __restrict__ in, float2* __restrict__ out,
                                     int nsteps, int project, int zero) {
  const int64_t pl = (int64_t)N * N;
  const int np = M - Kc;
  const int64_t total = fields * np * pl;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t f = t / (np * pl);
    const int64_t rr = t - f * np * pl;
    const int kz = Kc + (int)(rr / pl);
    const int64_t q = rr % pl;
    const int kx = (int)(q / N), ky = (int)(q % N);
    const int64_t q2 = (int64_t)((N - kx) % N) * N + (N - ky) % N;
    if (q2 < q) continue;
    const int64_t base = f * pl * M;
    const int64_t i1 = q * M + kz, i2 = q2 * M + kz;
    if (zero) {
      out[base + i1] = make_float2(0.f, 0.f);
      out[base + i2] = make_float2(0.f, 0.f);
      continue;
    }
    const int c = (int)(f % C);
    const float2* Et = E + (lin_ch == 1 ? 0 : (int64_t)c * M * pl) + (int64_t)kz * pl;
    const float2 e1 = Et[q], e2 = Et[q2];
    float2 v1 = in[base + i1], v2 = in[base + i2];
    const bool proj = project && ((N & 1) == 0 && kz == N / 2);
    for (int st = 0; st < nsteps; ++st) {
      v1 = cmul(e1, v1);
      v2 = cmul(e2, v2);
      if (proj) {
        const float2 pv = make_float2(0.5f * (v1.x + v2.x), 0.5f * (v1.y - v2.y));
        v1 = pv;
        v2 = cconj(pv);
      }
    }
    out[base + i1] = v1;
    if (q2 != q) out[base + i2] = v2;
  }
}

static unsigned grid_for(int64_t n, int sm) {
  const int64_t b = (n + 255) / 256;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)sm * 32));
}

template <int N>
struct Sizes {
  using R = Cfg<N>;
  static size_t s1() { return sizeof(float2) * ((size_t)R::FREE + R::PLANE); }
  static size_t s2(int NI, int NF, int TY, int Kc) {
    return sizeof(float2) * ((size_t)N + (size_t)NI * Kc * TY + (size_t)std::max(NI, NF) * TY / 2 * R::SLOT);
  }
  static size_t s3() { return s1(); }
};

static size_t smem_limit() {
  static int lim = 0;
  if (!lim) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&lim, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  }
  return (size_t)lim;
}

template <int N>
static int launch(Args& a, int64_t n, cudaStream_t st, bool set_attrs) {
  constexpr int TH = Cfg<N>::THREADS;
  const size_t s1 = Sizes<N>::s1(), s2 = Sizes<N>::s2(a.p.NI, a.p.NF, a.TY, a.Kc), s3 = Sizes<N>::s3();
  if (set_attrs) {
    EXGB_CUDA(cudaFuncSetAttribute(pass1_3d_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s1));
    EXGB_CUDA(cudaFuncSetAttribute(pass2_3d_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s2));
    EXGB_CUDA(cudaFuncSetAttribute(pass3_3d_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s3));
    return EXGB_OK;
  }
  pass1_3d_kernel<N><<<dim3(a.Kc, a.p.NI, (unsigned)n), TH, s1, st>>>(a);
  pass2_3d_kernel<N><<<dim3(N * (N / a.TY), (unsigned)n), Cfg<N>::THREADS2, s2, st>>>(a);
  pass3_3d_kernel<N><<<dim3(a.Kc, a.p.NF, (unsigned)n), TH, s3, st>>>(a);
  combine_planes_kernel<<<grid_for(n * a.Kc * a.pl, a.sm), 256, 0, st>>>(a, n);
  return EXGB_OK;
}

}  // namespace p3d

using namespace p3d;

// Can the three-pass 3D path step a plan of this size and these field counts?
bool pass3d_supported(int D, int N, int NI, int NF) {
  if (D != 3 || (N != 32 && N != 64 && N != 128) || NI < 1 || NF < 1 || NI > MAXC * 4 || NF > 2 * MAXC)
    return false;
  const size_t lim = smem_limit() - 1024;
  if (N == 32) return Sizes<32>::s1() <= lim && Sizes<32>::s2(NI, NF, 8, 17) <= lim;
  if (N == 64) return Sizes<64>::s1() <= lim && Sizes<64>::s2(NI, NF, 8, 33) <= lim;
  return Sizes<128>::s1() <= lim && Sizes<128>::s2(NI, NF, 8, 65) <= lim;
}

template <bool SET>
static int launch_n(int N, Args& a, int64_t n, cudaStream_t st) {
  switch (N) {
    case 32: return launch<32>(a, n, st, SET);
    case 64: return launch<64>(a, n, st, SET);
    default: return launch<128>(a, n, st, SET);
  }
}

int pass3d_run(const exgb_plan* plan, const Geo& g0, const Prog& prog, cudaStream_t st, const float2* in, float2* out,
               int64_t batch, int nsteps, int project, int nonlinear_only) {
  const PlanDev& P = plan->dev;
  const int N = P.N, M = P.M, C = P.C;
  const int K = std::min(P.kmax, N / 2);
  const int Kc = std::min(M, K + 1);
  const int sm = plan->sm_count;
  const int64_t pl = (int64_t)N * N;
  if (batch == 0) return EXGB_OK;
  if (!nonlinear_only && nsteps == 0) {
    if (in != out) EXGB_CUDA(cudaMemcpyAsync(out, in, sizeof(float2) * batch * C * pl * M, cudaMemcpyDeviceToDevice, st));
    return EXGB_OK;
  }
  Args a{};
  a.P = P;
  a.g = g0;
  a.p = prog;
  a.tw = P.tw;
  a.N = N;
  a.M = M;
  a.K = K;
  a.Kc = Kc;
  a.TY = 8;  // y lines per pass-2 CTA (16 measured no faster at 64^3)
  a.sm = sm;
  a.pl = pl;
  a.cstride = (int64_t)Kc * pl;
  a.sstride = (int64_t)C * a.cstride;
  a.tstride = (int64_t)M * pl;
  const int nb = stage_nbufs(P.order);
  const size_t per_sample = sizeof(float2) * ((size_t)(nonlinear_only ? 1 : nb) * a.sstride +
                                              (size_t)(prog.NI + prog.NF) * Kc * pl);
  const int64_t cb = std::max<int64_t>(1, std::min<int64_t>(batch, (int64_t)((size_t)(1u << 30) / per_sample)));
  char* ws = (char*)workspace(per_sample * (size_t)cb, 4);
  if (!ws) return fail(EXGB_ENOMEM, "workspace allocation failed");
  int rc = launch_n<true>(N, a, 0, st);
  if (rc) return rc;
  for (int64_t b0 = 0; b0 < batch; b0 += cb) {
    const int64_t n = std::min<int64_t>(cb, batch - b0);
    if (n * C > 65535) return fail(EXGB_EUNSUPPORTED, "too many fields for one launch");
    const float2* src = in + b0 * C * pl * M;
    float2* dst = out + b0 * C * pl * M;
    float2* q = (float2*)ws;
    const int64_t fsz = a.sstride * n;
    a.sb = stage_bufs(q, nonlinear_only ? 1 : P.order, fsz);
    q += (int64_t)(nonlinear_only ? 1 : nb) * fsz;
    a.W = q;
    q += (int64_t)prog.NI * Kc * pl * n;
    a.Hq = q;
    {
      dim3 grid((unsigned)((pl + 31) / 32), (Kc + 31) / 32, (unsigned)(n * C));
      transpose3_kernel<<<grid, dim3(32, 8), 0, st>>>(src, a.sb.U, pl, M, Kc, a.cstride, 1);
    }
    const int nst = nonlinear_only ? 1 : P.order;
    const int Q = nonlinear_only ? 1 : nsteps * P.order;
    for (int qq = 0; qq < Q; ++qq) {
      const int stage = qq % nst;
      a.stage = nonlinear_only ? -1 : stage;
      a.nout = nonlinear_only ? dst : nullptr;
      a.xin = (stage == 0) ? a.sb.U : (P.order == 4 && stage == 1) ? a.sb.S1 : a.sb.S;
      rc = launch_n<false>(N, a, n, st);
      if (rc) return rc;
      if (!nonlinear_only && stage == nst - 1 && project)
        project_planes_kernel<<<grid_for(n * C * 2 * pl, sm), 256, 0, st>>>(a.sb.U, N, Kc, a.cstride, n * C);
      EXGB_CUDA(cudaGetLastError());
    }
    if (!nonlinear_only) {
      dim3 grid((unsigned)((pl + 31) / 32), (Kc + 31) / 32, (unsigned)(n * C));
      transpose3_kernel<<<grid, dim3(32, 8), 0, st>>>(a.sb.U, dst, pl, M, Kc, a.cstride, 0);
    }
    if (Kc < M)
      linear_planes_kernel<<<grid_for(n * C * (int64_t)(M - Kc) * pl, sm), 256, 0, st>>>(
          P.E, P.lin_ch, C, N, M, Kc, n * C, src, dst, nsteps, project, nonlinear_only);
    EXGB_CUDA(cudaGetLastError());
  }
  return EXGB_OK;
}

}  // namespace exgb
