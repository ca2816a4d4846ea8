// exgb_tcdft2d.cu -- fused 2D vorticity ETDRK kernel whose transforms are
// dense DFT contractions on the tcgen05 tensor cores in split-BF16 form
// (three products hi.hi + hi.lo + lo.hi, FP32 accumulation in tensor memory).
// N = 128 (both axes), dealiasing cutoff K <= 47.
//
// Same step as vort2d_kernel (reference nonlin_fun/_vorticity_convection.py:
// 78-99 and :166-176 for the Kolmogorov injection; etdrk/_etdrk_1..4.py), one
// CTA per sample, persistent over the batch.  Only the kept modes
// (|k_full| <= K, k_half <= K) enter the nonlinear term, so every transform
// is a contraction over at most 2K+1 modes, and the cos/sin symmetry of the
// DFT halves both its length and its output count:
//
//   inverse, complex over the full axis (per half-axis column and field):
//     S_k = d_k + d_-k, D_k = d_k - d_-k;  E[i] = sum_k S_k cos(th k i),
//     O[i] = sum_k D_k sin(th k i);  g[i] = E + iO, g[N-i] = E - iO
//   inverse, c2r over the half axis (per full-axis row and field):
//     P[j] = sum_k w_k Re g_k cos(th k j), Q[j] = sum_k w_k Im g_k sin(th k j);
//     x[j] = P - Q, x[N-j] = P + Q          (w_0 = 1, w_k = 2)
//   forward, r2c over the half axis and complex over the full axis:
//     e_j = x_j + x_N-j, o_j = x_j - x_N-j;  C_m = sum_j e_j cos(th m j),
//     S_m = sum_j o_j sin(th m j);  X_m = C_m - i S_m, X_-m = C_m + i S_m
//
// with th = 2 pi / N.  The derived fields are d = i m(k) w^ with a real
// multiplier m (u: k_half/Lap, v: -k_full/Lap, wx: k_full, wy: k_half), odd
// or even in k_full, so S and D of every field come from the two spectra
// A+ = w^(k) + w^(-k) and A- = w^(k) - w^(-k), kept in shared memory.
// The constant matrices "Ai" (128 rows of cos/sin over the inverse modes)
// and "Af" (rows of cos/sin modes over e/o positions) are computed once on
// the host in FP64, split into hi/lo bf16 in the exact shared-memory layout
// and copied in at launch; rows are ordered so that the cos row and the sin
// row of one index sit 16 lanes apart in the same warp, and the
// +-combinations above are one warp shuffle.
//
// Per stage and sample: 4 x (inverse full axis, inverse half axis), the
// product u wx + v wy in registers, forward half axis, forward full axis,
// ETDRK stage update (exgb_stage.cuh) by all threads on mode pairs (k, -k)
// -- 10 MMA chains, all operands in shared memory, accumulators in 4 slots of
// 128 TMEM columns.  Modes outside the kept set evolve linearly (E^n, the c2r
// projection on the half-axis columns 0 and N/2) exactly as in the FP32 kernels.
// The complex helpers' scalar forms: in this kernel (SIMT work between MMA chains) they measured 2 %
// faster than the packed f32x2 ones the FFT kernels use (26.15 against 26.69 ms at kolmo128).
#define EXGB_SCALAR_COMPLEX 1
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "exgb_internal.h"
#include "exgb_stage.cuh"
#include "exgb_tc.cuh"

namespace exgb {
namespace tcd {

constexpr int N = 128;
constexpr int H = N / 2;
constexpr int M = N / 2 + 1;
constexpr int THREADS = 256;
constexpr int KMAX = 47;
constexpr int KI = 96;   // inverse contraction: [cos part, modes 0..47 | sin part, modes 0..47]
constexpr int KF = 128;  // forward contraction: [e_0 .. e_63 | e_64 | o_1 .. o_63]
constexpr int LD = 49;   // k_half stride of the A+- planes (odd: conflict-free row and column access)
// shared memory (bytes).  Af stores rows 0..95; the MMA also reads rows
// 96..127, which overlap the next tile (their outputs are never used).
constexpr uint32_t TILE_AI = 128 * KI * 2;
constexpr uint32_t TILE_AF = 96 * KF * 2;
constexpr uint32_t OFF_AI_HI = 0;
constexpr uint32_t OFF_AI_LO = OFF_AI_HI + TILE_AI;
constexpr uint32_t OFF_AF_HI = OFF_AI_LO + TILE_AI;
constexpr uint32_t OFF_AF_LO = OFF_AF_HI + TILE_AF;
constexpr uint32_t CONST_BYTES = OFF_AF_LO + TILE_AF;  // host-built image of the four constant tiles
constexpr uint32_t OFF_R = CONST_BYTES;
constexpr uint32_t TILE_B1 = 96 * KI * 2;   // inverse full-axis data: rows (part, half mode)
constexpr uint32_t TILE_A2 = 128 * KI * 2;  // inverse half-axis data: rows = full-axis positions
constexpr uint32_t TILE_B3 = 128 * KF * 2;  // forward half-axis data: rows = full-axis positions
constexpr uint32_t TILE_B4 = 96 * KF * 2;   // forward full-axis data: rows = Af rows of the half modes
constexpr uint32_t R_B1_HI = 0, R_B1_LO = TILE_B1;
constexpr uint32_t R_A2_HI = 2 * TILE_B1, R_A2_LO = 2 * TILE_B1 + TILE_A2;
constexpr uint32_t R_BYTES = 2 * TILE_B1 + 2 * TILE_A2;
constexpr uint32_t PLANE = 48 * LD * 4;     // one float plane [k_full 0..47][k_half]
constexpr uint32_t OFF_PM = OFF_R + R_BYTES;  // planes A+re, A+im, A-re, A-im
constexpr uint32_t OFF_IL = OFF_PM + 4 * PLANE;  // 1 / (N^2 Lap) on the kept modes [k_full][k_half]
constexpr uint32_t OFF_TAIL = OFF_IL + PLANE;     // mbarrier (8 B) and TMEM base address (4 B)
constexpr uint32_t SMEM_BYTES = OFF_TAIL + 16;
static_assert(2 * TILE_B3 <= R_BYTES && 2 * TILE_B4 <= R_BYTES, "region R too small");
static_assert(48u * N * 8u <= R_BYTES, "nonlinear-term buffer must fit region R");
static_assert(128 * KF * 2 - TILE_AF <= R_BYTES, "Af overflow rows must stay inside shared memory");
static_assert(CONST_BYTES % 16 == 0, "constant image is copied in 16-byte pieces");
constexpr long long WAIT_BUDGET = 4000000000LL;  // clock cycles (~2 s) before a wait gives up

struct Args {
  PlanDev P;
  const float2* in;
  float2* out;
  int64_t batch;
  int nsteps;
  int project;
  int nonlinear_only;
  float2* scratch;
  int64_t scratch_stride;
  const uint4* consts;
  int* status;
  long long first_wait_budget;  // budget of the launch's first MMA-completion wait
};

__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Inverse full-axis data of field F (0 u, 1 v, 2 wx, 3 wy): row n = part * 48
// + k_half, column k = [S_k (k < 48) | D_(k-48)].  S/D = i m (A+ or A-), the
// even fields (u, wy) taking A+ for S and the odd ones (v, wx) A- (the
// multiplier changes sign with k_full).  Values outside the kept set are 0.
// `il` holds 1 / (N^2 Lap) (u, v); wx and wy carry 1 / N^2 directly.
// Inverse full-axis data of field F (0 u, 1 v, 2 wx, 3 wy): row n = part * 48
// + k_half, column k = [S_k (k < 48) | D_(k-48)].  S/D = i m (A+ or A-), the
// even fields (u, wy) taking A+ for S and the odd ones (v, wx) A- (the
// multiplier changes sign with k_full).  Values outside the kept set are 0.
// `il` holds 1 / (N^2 Lap) (u, v); wx and wy carry 1 / N^2 directly.  One
// task = one 8-column chunk of both rows (re part, im part) of a k_half:
// i m A = (-m A.im, m A.re) shares the multiplier and the address.
template <int F>
__device__ __forceinline__ void build_b1(unsigned char* hi, unsigned char* lo, const float* pl, const float* il,
                                         int K, float ksc, float invNN, int tid) {
  constexpr bool odd = (F == 1 || F == 2);
  for (int t = tid; t < 48 * (KI / 8); t += THREADS) {
    const int c = t / 48, kh = t - c * 48;
    const bool dblk = c >= 6;
    const bool minus = (dblk != odd);
    const float* Pre = pl + (minus ? 2 : 0) * (int)(PLANE / 4);
    const float* Pim = Pre + PLANE / 4;
    float vr[8], vi[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) vr[j] = vi[j] = 0.f;
    if (kh <= K) {
      const float kys = ksc * (float)kh;
      const int kf0 = 8 * c - (dblk ? 48 : 0);
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int kf = kf0 + j;
        if (kf <= K) {
          const int o = kf * LD + kh;
          const float kxs = ksc * (float)kf;
          float m;
          if (F == 2) {
            m = kxs * invNN;
          } else if (F == 3) {
            m = kys * invNN;
          } else {
            m = (F == 0) ? kys * il[o] : -kxs * il[o];
          }
          vr[j] = -m * Pim[o];
          vi[j] = m * Pre[o];
        }
      }
    }
    tc::split8_store(vr, hi, lo, tc::kmaj_chunk(kh, c, KI));
    tc::split8_store(vi, hi, lo, tc::kmaj_chunk(48 + kh, c, KI));
  }
}

__global__ void __launch_bounds__(THREADS, 1) tcdft2d_kernel(const Args a) {
  extern __shared__ __align__(128) unsigned char sm[];
  uint64_t& s_mbar = *reinterpret_cast<uint64_t*>(sm + OFF_TAIL);
  uint32_t& s_tbase = *reinterpret_cast<uint32_t*>(sm + OFF_TAIL + 8);
  const PlanDev& P = a.P;
  const int K = min(P.kmax, KMAX);
  const int Kc = K + 1;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, q = warp & 3;
  const bool upper = warp >= 4;
  unsigned char* rg = sm + OFF_R;
  float* pl = reinterpret_cast<float*>(sm + OFF_PM);
  float* ilt = reinterpret_cast<float*>(sm + OFF_IL);
  float2* nvb = reinterpret_cast<float2*>(rg);  // nonlinear term [k_half][k_full index], region R
  const uint32_t sAiH = tc::smem_u32(sm + OFF_AI_HI), sAiL = tc::smem_u32(sm + OFF_AI_LO);
  const uint32_t sAfH = tc::smem_u32(sm + OFF_AF_HI), sAfL = tc::smem_u32(sm + OFF_AF_LO);
  const uint32_t sR = tc::smem_u32(rg);

  // ---- constant DFT tiles: host-built image, copied as is
  {
    uint4* dst = reinterpret_cast<uint4*>(sm);
    for (int t = tid; t < (int)(CONST_BYTES / 16); t += THREADS) dst[t] = __ldg(a.consts + t);
  }
  for (int t = tid; t < 48 * LD; t += THREADS) {
    const int kf = t / LD, kh = t - kf * LD;
    const float kxs = a.P.kscale * (float)kf, kys = a.P.kscale * (float)kh;
    const float lap = -(kxs * kxs + kys * kys);
    ilt[t] = (lap == 0.f) ? 0.f : __frcp_rn(lap) * (1.f / ((float)N * (float)N));
  }
  if (warp == 0) {
    tc::tmem_alloc(&s_tbase, 512);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(&s_mbar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc::fence_proxy_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = s_tbase;
  const uint32_t tl = tmem + ((uint32_t)(32 * q) << 16);  // this warp's TMEM lane quadrant

  const float invNN = 1.f / ((float)N * (float)N);
  const float negb = -P.conv_scale;
  const float ksc = P.kscale;
  const int nst = a.nonlinear_only ? 1 : P.order;
  const int Q = a.nonlinear_only ? 1 : a.nsteps * P.order;
  const StageBufs sb = stage_bufs(a.scratch + (int64_t)blockIdx.x * a.scratch_stride, P.order, (int64_t)Kc * N);
  const uint32_t idI1 = tc::idesc_bf16(128, 96), idI2 = tc::idesc_bf16(128, 128);
  const uint32_t idF1 = tc::idesc_bf16(128, 128), idF2 = tc::idesc_bf16(128, 96);
  uint32_t phase = 0;
  bool bad = false;

  auto sync_for_mma = [&]() {
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
  };
  bool first_wait = true;
  auto wait_mma = [&]() -> bool {
    const bool ok = tc::mbar_wait(&s_mbar, phase, first_wait ? a.first_wait_budget : WAIT_BUDGET);
    first_wait = false;
    phase ^= 1u;
    const int anybad = __syncthreads_or(!ok);
    tc::fence_after_sync();
    return anybad == 0;
  };
  auto b1 = [&](int f) {
    unsigned char* h = rg + R_B1_HI;
    unsigned char* l = rg + R_B1_LO;
    switch (f) {
      case 0: build_b1<0>(h, l, pl, ilt, K, ksc, invNN, tid); break;
      case 1: build_b1<1>(h, l, pl, ilt, K, ksc, invNN, tid); break;
      case 2: build_b1<2>(h, l, pl, ilt, K, ksc, invNN, tid); break;
      default: build_b1<3>(h, l, pl, ilt, K, ksc, invNN, tid); break;
    }
  };
  auto put_pm = [&](int kf, int kh, float2 s1, float2 s2) {
    const float2 ap = (kf == 0) ? s1 : cadd(s1, s2);
    const float2 am = (kf == 0) ? make_float2(0.f, 0.f) : csub(s1, s2);
    const int o = kf * LD + kh;
    pl[o] = ap.x;
    pl[PLANE / 4 + o] = ap.y;
    pl[2 * (PLANE / 4) + o] = am.x;
    pl[3 * (PLANE / 4) + o] = am.y;
  };

  // D1 (slot f) -> inverse half-axis data rows (full-axis position i), k = [w Re g | w Im g]
  auto build_a2 = [&](int f) {
    const bool sinl = lane >= 16;
    const int s = 16 * q + (lane & 15);
    const int iout = sinl ? (s == 0 ? H : N - s) : s;
    const bool eonly = (s == 0);
    const int b0 = upper ? 3 : 0;
    float re[32], im[32];
    tc::tmem_ld32x2(tl + 128u * f + 8u * b0, tl + 128u * f + 48u + 8u * b0, re, im);
#pragma unroll
    for (int bb = 0; bb < 3; ++bb) {
      const int b = b0 + bb;
      float gr[8], gi[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const float r0 = re[8 * bb + j], i0 = im[8 * bb + j];
        const float pre = __shfl_xor_sync(0xffffffffu, r0, 16);
        const float pim = __shfl_xor_sync(0xffffffffu, i0, 16);
        const float w = (b == 0 && j == 0) ? 1.f : 2.f;
        float r1, r2;
        if (eonly) {
          r1 = r0;
          r2 = i0;
        } else if (!sinl) {
          r1 = r0 - pim;  // E + i O
          r2 = i0 + pre;
        } else {
          r1 = pre + i0;  // E - i O
          r2 = pim - r0;
        }
        gr[j] = w * r1;
        gi[j] = w * r2;
      }
      tc::split8_store(gr, rg + R_A2_HI, rg + R_A2_LO, tc::kmaj_chunk(iout, b, KI));
      tc::split8_store(gi, rg + R_A2_HI, rg + R_A2_LO, tc::kmaj_chunk(iout, 6 + b, KI));
    }
  };

  for (int64_t smp = blockIdx.x; smp < a.batch && !bad; smp += gridDim.x) {
    const float2* uin = a.in + smp * (int64_t)N * M;
    float2* uout = a.out + smp * (int64_t)N * M;

    // ---- modes outside the kept set: linear part only (zero for the nonlinear term)
    for (int t = tid; t < M * (H + 1); t += THREADS) {
      const int kh = t / (H + 1), kx = t - kh * (H + 1);
      if (kh <= K && kx <= K) continue;
      const int kx2 = (kx == 0) ? 0 : N - kx;
      if (a.nonlinear_only) {
        uout[(int64_t)kx * M + kh] = make_float2(0.f, 0.f);
        uout[(int64_t)kx2 * M + kh] = make_float2(0.f, 0.f);
        continue;
      }
      float2 v1 = uin[(int64_t)kx * M + kh];
      float2 v2 = uin[(int64_t)kx2 * M + kh];
      const float2 E1 = __ldg(P.E + (int64_t)kh * N + kx);
      const float2 E2 = __ldg(P.E + (int64_t)kh * N + kx2);
      const bool proj = a.project && (kh == 0 || kh == H);
      for (int s = 0; s < a.nsteps; ++s) {
        v1 = cmul(E1, v1);
        v2 = cmul(E2, v2);
        if (proj) {
          const float2 pv = make_float2(0.5f * (v1.x + v2.x), 0.5f * (v1.y - v2.y));
          v1 = pv;
          v2 = cconj(pv);
        }
      }
      uout[(int64_t)kx * M + kh] = v1;
      if (kx2 != kx) uout[(int64_t)kx2 * M + kh] = v2;
    }
    // ---- kept modes, as pairs (k, -k) -> state and A+-
    for (int t = tid; t < Kc * Kc; t += THREADS) {
      const int kh = t / Kc, kf = t - kh * Kc;
      const int kfm = (N - kf) & (N - 1);
      const float2 x1 = uin[(int64_t)kf * M + kh];
      const float2 x2 = uin[(int64_t)kfm * M + kh];
      if (!a.nonlinear_only) {
        sb.U[(int64_t)kh * N + kf] = x1;
        sb.U[(int64_t)kh * N + kfm] = x2;
      }
      put_pm(kf, kh, x1, x2);
    }
    __syncthreads();

    for (int qq = 0; qq < Q && !bad; ++qq) {
      const int st = qq % nst;
      const bool last_of_step = (st == nst - 1);
      // ===== inverse transforms of the 4 derived fields; D2 of field f ends in TMEM slot f
      b1(0);
      sync_for_mma();
      if (tid == 0) {
        tc::fence_after_sync();
        tc::mma_split3(tmem, sAiH, sAiL, KI, sR + R_B1_HI, sR + R_B1_LO, KI, KI, idI1, false);
        tc::mma_commit(&s_mbar);
      }
      bad = !wait_mma();
      for (int f = 0; f < 4 && !bad; ++f) {
        build_a2(f);
        sync_for_mma();
        if (tid == 0) {
          tc::fence_after_sync();
          tc::mma_split3(tmem + 128u * f, sR + R_A2_HI, sR + R_A2_LO, KI, sAiH, sAiL, KI, KI, idI2, false);
        }
        if (f < 3) {
          b1(f + 1);  // B1 is free (its MMA completed); overlaps the MMA above
          sync_for_mma();
          if (tid == 0) {
            tc::fence_after_sync();
            tc::mma_split3(tmem + 128u * (f + 1), sAiH, sAiL, KI, sR + R_B1_HI, sR + R_B1_LO, KI, KI, idI1, false);
          }
        }
        if (tid == 0) tc::mma_commit(&s_mbar);
        bad = !wait_mma();
      }
      if (bad) break;

      // ===== product u wx + v wy at (i, j) and (i, N-j) -> forward half-axis data (e | o)
      {
        const int row = 32 * q + lane;
        const int c0 = upper ? 4 : 0;
        for (int c = c0; c < c0 + 4; ++c) {
          const uint32_t cc = 32u * (c >> 1) + 8u * (c & 1);
          float Pv[4][8], Qv[4][8];
          tc::tmem_ld8x4(tl + cc, tl + 128u + cc, tl + 256u + cc, tl + 384u + cc, Pv[0], Pv[1], Pv[2], Pv[3]);
          tc::tmem_ld8x4(tl + cc + 16u, tl + 144u + cc, tl + 272u + cc, tl + 400u + cc, Qv[0], Qv[1], Qv[2], Qv[3]);
          float e[8], o[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            float xs[4], xm[4];
#pragma unroll
            for (int f = 0; f < 4; ++f) {
              xs[f] = Pv[f][j] - Qv[f][j];
              xm[f] = Pv[f][j] + Qv[f][j];
            }
            const float ps = fmaf(xs[0], xs[2], xs[1] * xs[3]);
            const float pm = fmaf(xm[0], xm[2], xm[1] * xm[3]);
            e[j] = ps + pm;
            o[j] = ps - pm;
          }
          if (c == 0) {  // slot 0: column 0 is position 0, column 16 is position N/2
            e[0] = fmaf(Pv[0][0], Pv[2][0], Pv[1][0] * Pv[3][0]);
            o[0] = fmaf(Qv[0][0], Qv[2][0], Qv[1][0] * Qv[3][0]);
          }
          tc::split8_store(e, rg, rg + TILE_B3, tc::kmaj_chunk(row, c, KF));
          tc::split8_store(o, rg, rg + TILE_B3, tc::kmaj_chunk(row, 8 + c, KF));
        }
      }
      sync_for_mma();
      if (tid == 0) {
        tc::fence_after_sync();
        tc::mma_split3(tmem, sAfH, sAfL, KF, sR, sR + TILE_B3, KF, KF, idF1, false);
        tc::mma_commit(&s_mbar);
      }
      bad = !wait_mma();
      if (bad) break;

      // ===== D3 rows (half modes: Re, -Im) -> forward full-axis data (e | o over the full axis)
      if (q < 3) {
        const int row = 32 * q + lane;
        const int c0 = upper ? 4 : 0;
        for (int c = c0; c < c0 + 4; ++c) {
          float A[8], B[8];
          tc::tmem_ld8x2(tl + 8u * c, tl + 120u - 8u * c, A, B);
          const float X1 = tc::tmem_ld1(tl + (c == 0 ? 64u : 128u - 8u * c));
          float e[8], o[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const float mir = (j == 0) ? X1 : B[8 - j];
            e[j] = A[j] + mir;
            o[j] = A[j] - mir;
          }
          if (c == 0) {
            e[0] = A[0];
            o[0] = X1;
          }
          tc::split8_store(e, rg, rg + TILE_B4, tc::kmaj_chunk(row, c, KF));
          tc::split8_store(o, rg, rg + TILE_B4, tc::kmaj_chunk(row, 8 + c, KF));
        }
      }
      sync_for_mma();
      if (tid == 0) {
        tc::fence_after_sync();
        tc::mma_split3(tmem + 128u, sAfH, sAfL, KF, sR, sR + TILE_B4, KF, KF, idF2, false);
        tc::mma_commit(&s_mbar);
      }
      bad = !wait_mma();
      if (bad) break;

      // ===== D4 -> nonlinear term at the kept modes (region R, B4 is no longer read)
      if (q < 3) {
        const bool srow = lane >= 16;
        const int kf = 16 * q + (lane & 15);
        const bool active = kf <= K && !(srow && kf == 0);
        const int kfi = ((srow ? -kf : kf) + N) & (N - 1);
        const int b0 = upper ? 3 : 0;
        for (int b = b0; b < b0 + 3; ++b) {
          const uint32_t na = 32u * (b >> 1) + 8u * (b & 1);
          float Ca[8], Cb[8];
          tc::tmem_ld8x2(tl + 128u + na, tl + 128u + na + 16u, Ca, Cb);
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const float Pa = __shfl_xor_sync(0xffffffffu, Ca[j], 16);
            const float Pb = __shfl_xor_sync(0xffffffffu, Cb[j], 16);
            const int kh = 8 * b + j;
            const float2 Z = srow ? make_float2(Pa + Cb[j], Ca[j] - Pb) : make_float2(Ca[j] - Pb, -Cb[j] - Pa);
            if (active && kh <= K) {
              float2 nv = cscale(Z, negb);
              if (kh == P.inj_mode && kfi == 0) nv.x += P.inj_value;
              nvb[kh * N + kfi] = nv;
            }
          }
        }
      }
      tc::fence_before_sync();
      __syncthreads();
      // ===== ETDRK stage update on mode pairs (k, -k), all threads; next stage's A+-
      if (a.nonlinear_only) {
        for (int t = tid; t < Kc * Kc; t += THREADS) {
          const int kh = t / Kc, kf = t - kh * Kc;
          const int kfm = (N - kf) & (N - 1);
          uout[(int64_t)kf * M + kh] = nvb[kh * N + kf];
          uout[(int64_t)kfm * M + kh] = nvb[kh * N + kfm];
        }
      } else if (P.order == 2) {
        // ETDRK2 (etdrk/_etdrk_2.py:91-102), four mode pairs per thread with all loads issued first
        const int total = Kc * Kc;
        for (int t0 = tid; t0 < total; t0 += 4 * THREADS) {
          float2 n1[4], n2[4], x1[4], x2[4], y1[4], y2[4], e1[4], e2[4];
          float c1[4], c2[4];
          int kfv[4], khv[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const int t = min(t0 + u * THREADS, total - 1);
            const int kh = t / Kc, kf = t - kh * Kc;
            const int kfm = (N - kf) & (N - 1);
            const int64_t o1 = (int64_t)kh * N + kf, o2 = (int64_t)kh * N + kfm;
            khv[u] = kh;
            kfv[u] = kf;
            n1[u] = nvb[kh * N + kf];
            n2[u] = nvb[kh * N + kfm];
            if (st == 0) {
              x1[u] = sb.U[o1];
              x2[u] = sb.U[o2];
              e1[u] = __ldg(P.E + o1);
              e2[u] = __ldg(P.E + o2);
              c1[u] = __ldg(P.c[0] + o1);
              c2[u] = __ldg(P.c[0] + o2);
            } else {
              x1[u] = sb.S[o1];
              x2[u] = sb.S[o2];
              y1[u] = sb.N0[o1];
              y2[u] = sb.N0[o2];
              c1[u] = __ldg(P.c[1] + o1);
              c2[u] = __ldg(P.c[1] + o2);
            }
          }
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            if (t0 + u * THREADS >= total) break;
            const int kh = khv[u], kf = kfv[u];
            const int kfm = (N - kf) & (N - 1);
            const int64_t o1 = (int64_t)kh * N + kf, o2 = (int64_t)kh * N + kfm;
            float2 s1, s2;
            if (st == 0) {
              s1 = cadd(cmul(e1[u], x1[u]), cscale(n1[u], c1[u]));
              s2 = cadd(cmul(e2[u], x2[u]), cscale(n2[u], c2[u]));
              sb.N0[o1] = n1[u];
              sb.S[o1] = s1;
              if (kf > 0) {
                sb.N0[o2] = n2[u];
                sb.S[o2] = s2;
              } else {
                s2 = s1;
              }
            } else {
              s1 = cadd(x1[u], cscale(csub(n1[u], y1[u]), c1[u]));
              s2 = cadd(x2[u], cscale(csub(n2[u], y2[u]), c2[u]));
              if (kf == 0) s2 = s1;
              if (a.project && kh == 0) {
                // c2r projection of the step's physical round trip on the half-axis column 0
                const float2 pv = make_float2(0.5f * (s1.x + s2.x), 0.5f * (s1.y - s2.y));
                s1 = pv;
                s2 = cconj(pv);
              }
              sb.U[o1] = s1;
              if (kf > 0) sb.U[o2] = s2;
            }
            put_pm(kf, kh, s1, s2);
          }
        }
      } else {
        for (int t = tid; t < Kc * Kc; t += THREADS) {
          const int kh = t / Kc, kf = t - kh * Kc;
          const int kfm = (N - kf) & (N - 1);
          const int64_t o1 = (int64_t)kh * N + kf, o2 = (int64_t)kh * N + kfm;
          float2 s1 = stage_upd(P, sb, o1, st, nvb[kh * N + kf]);
          float2 s2 = (kf > 0) ? stage_upd(P, sb, o2, st, nvb[kh * N + kfm]) : s1;
          if (last_of_step && a.project && kh == 0) {
            // c2r projection of the step's physical round trip on the half-axis column 0
            const float2 pv = make_float2(0.5f * (s1.x + s2.x), 0.5f * (s1.y - s2.y));
            s1 = pv;
            s2 = cconj(pv);
            sb.U[o1] = s1;
            if (kf > 0) sb.U[o2] = s2;
          }
          put_pm(kf, kh, s1, s2);
        }
      }
      __syncthreads();
    }
    if (bad) break;

    // ---- kept modes -> output
    if (!a.nonlinear_only) {
      for (int t = tid; t < Kc * Kc; t += THREADS) {
        const int kh = t / Kc, kf = t - kh * Kc;
        const int kfm = (N - kf) & (N - 1);
        uout[(int64_t)kf * M + kh] = sb.U[(int64_t)kh * N + kf];
        uout[(int64_t)kfm * M + kh] = sb.U[(int64_t)kh * N + kfm];
      }
    }
    __syncthreads();
  }

  if (bad) {
    // let any MMA still in flight finish before the tensor memory is released
    tc::mbar_wait(&s_mbar, phase ^ 1u, WAIT_BUDGET);
    if (tid == 0) atomicExch(a.status, EXGB_ETIMEOUT);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 512);
}

// ---- host-side image of the constant tiles (FP64 angles, bf16 hi/lo, canonical K-major layout)
static uint16_t to_bf16(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  if ((u & 0x7fffffffu) > 0x7f800000u) return 0x7fc0;
  u += 0x7fffu + ((u >> 16) & 1u);  // round to nearest even
  return (uint16_t)(u >> 16);
}
static double from_bf16(uint16_t h) {
  const uint32_t u = (uint32_t)h << 16;
  float f;
  std::memcpy(&f, &u, 4);
  return (double)f;
}
static double cos2pi(long m) { return std::cos(2.0 * M_PI * (double)(m % N) / N); }
static double sin2pi(long m) { return std::sin(2.0 * M_PI * (double)(m % N) / N); }

// Ai[r][k]: rows r = 32 w + l, slot s = 16 w + (l & 15); l < 16: cos row of
// index s; l >= 16: sin row of index s (s >= 1) or the cos row of index N/2 (s = 0).
static double ai_val(int r, int k, int K) {
  const int w = r >> 5, l = r & 31, s = 16 * w + (l & 15);
  const bool sinl = l >= 16;
  if (!sinl || s == 0) {
    const int idx = sinl ? H : s;
    return (k < 48 && k <= K) ? cos2pi((long)k * idx) : 0.0;
  }
  const int kk = k - 48;
  return (k >= 48 && kk >= 1 && kk <= K) ? sin2pi((long)kk * s) : 0.0;
}
// Af[r][k]: rows r = 32 w + l (w < 3), mode m = 16 w + (l & 15); l < 16: cos
// row over e_0..e_64 (k = 0..64); l >= 16: sin row over o_1..o_63 (k = 65..127).
static double af_val(int r, int k, int K) {
  const int w = r >> 5, l = r & 31, m = 16 * w + (l & 15);
  if (m > K) return 0.0;
  if (l < 16) return k <= 64 ? cos2pi((long)m * k) : 0.0;
  if (m == 0 || k < 65) return 0.0;
  return sin2pi((long)m * (k - 64));
}
static void put_tile(std::vector<unsigned char>& img, uint32_t off_hi, uint32_t off_lo, int rows, int kdim, int K,
                     double (*val)(int, int, int)) {
  for (int r = 0; r < rows; ++r)
    for (int k = 0; k < kdim; ++k) {
      const double d = val(r, k, K);
      const uint16_t h = to_bf16((float)d);
      const uint16_t l = to_bf16((float)(d - from_bf16(h)));
      const uint32_t o = tc::kmaj_off(r, k, kdim);
      std::memcpy(&img[off_hi + o], &h, 2);
      std::memcpy(&img[off_lo + o], &l, 2);
    }
}

}  // namespace tcd

bool tcdft2d_supported(const exgb_plan* plan) {
  const PlanDev& P = plan->dev;
  return P.D == 2 && P.N == tcd::N && P.order >= 1 &&
         (P.kind == EXGB_NL_VORTICITY_2D || P.kind == EXGB_NL_VORTICITY_2D_KOLMOGOROV) && P.kmax >= 0 &&
         P.kmax <= tcd::KMAX && P.lin_ch == 1;
}

int tcdft2d_configure(exgb_plan* plan) {
  if (!tcdft2d_supported(plan))
    return fail(EXGB_EUNSUPPORTED,
                "split-BF16 tensor-core DFT: needs a 2D vorticity plan with N = 128, order >= 1 and a dealiasing "
                "cutoff <= 47");
  int dev = 0, major = 0;
  EXGB_CUDA(cudaGetDevice(&dev));
  EXGB_CUDA(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
  if (major != 10) return fail(EXGB_EUNSUPPORTED, "split-BF16 tensor-core DFT needs an sm_100-family GPU");
  EXGB_CUDA(cudaFuncSetAttribute(tcd::tcdft2d_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)tcd::SMEM_BYTES));
  const int K = std::min(plan->dev.kmax, tcd::KMAX);
  const size_t per = (size_t)stage_nbufs(plan->dev.order) * (K + 1) * tcd::N;
  if (!plan->d_tc_scratch) {
    std::vector<unsigned char> img(tcd::CONST_BYTES, 0);
    tcd::put_tile(img, tcd::OFF_AI_HI, tcd::OFF_AI_LO, 128, tcd::KI, K, tcd::ai_val);
    tcd::put_tile(img, tcd::OFF_AF_HI, tcd::OFF_AF_LO, 96, tcd::KF, K, tcd::af_val);
    const size_t scratch = sizeof(float2) * per * plan->sm_count;
    EXGB_CUDA(cudaMalloc(&plan->d_tc_scratch, scratch + tcd::CONST_BYTES));
    EXGB_CUDA(cudaMemcpy((unsigned char*)plan->d_tc_scratch + scratch, img.data(), img.size(),
                         cudaMemcpyHostToDevice));
    plan->tc_const_offset = scratch;
    EXGB_CUDA(cudaMalloc(&plan->d_status, sizeof(int)));
    EXGB_CUDA(cudaMemset(plan->d_status, 0, sizeof(int)));
  }
  plan->tc_scratch_per_cta = per;
  return EXGB_OK;
}

int tcdft2d_run(const exgb_plan* plan, cudaStream_t st, const float2* in, float2* out, int64_t batch, int nsteps,
                int project, int nonlinear_only) {
  if (batch <= 0) return EXGB_OK;
  tcd::Args a;
  a.P = plan->dev;
  a.in = in;
  a.out = out;
  a.batch = batch;
  a.nsteps = nsteps;
  a.project = project;
  a.nonlinear_only = nonlinear_only;
  a.scratch = (float2*)plan->d_tc_scratch;
  a.scratch_stride = (int64_t)plan->tc_scratch_per_cta;
  a.consts = reinterpret_cast<const uint4*>((const unsigned char*)plan->d_tc_scratch + plan->tc_const_offset);
  a.status = plan->d_status;
  a.first_wait_budget = plan->tc_first_wait_budget > 0 ? plan->tc_first_wait_budget : tcd::WAIT_BUDGET;
  const int grid = (int)std::min<int64_t>(batch, plan->sm_count);
  tcd::tcdft2d_kernel<<<grid, tcd::THREADS, tcd::SMEM_BYTES, st>>>(a);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

}  // namespace exgb
