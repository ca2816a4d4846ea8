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
// with th = 2 pi / N.  The matrices "Ai" (128 rows of cos/sin over the
// inverse modes) and "Af" (rows of cos/sin modes over e/o positions) live in
// shared memory as hi/lo bf16 pairs for the whole launch; rows are ordered
// so that the cos row and the sin row of one index sit 16 lanes apart in the
// same warp, and the +-combinations above are one warp shuffle.
//
// Per stage and sample: 4 x (inverse full axis, inverse half axis), the
// product u wx + v wy in registers, forward half axis, forward full axis,
// ETDRK stage update (exgb_stage.cuh) -- 10 MMA chains, all operands in
// shared memory, accumulators in 4 slots of 128 TMEM columns.
// Modes outside the kept set evolve linearly (E^n, the c2r projection on the
// half-axis columns 0 and N/2) exactly as in the FP32 kernels.
#include <cuda_runtime.h>

#include <algorithm>

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
constexpr int XS_LD = 48;
// shared memory (bytes).  Af stores rows 0..95; the MMA also reads rows
// 96..127, which overlap the next tile (their outputs are never used).
constexpr uint32_t TILE_AI = 128 * KI * 2;
constexpr uint32_t TILE_AF = 96 * KF * 2;
constexpr uint32_t OFF_AI_HI = 0;
constexpr uint32_t OFF_AI_LO = OFF_AI_HI + TILE_AI;
constexpr uint32_t OFF_AF_HI = OFF_AI_LO + TILE_AI;
constexpr uint32_t OFF_AF_LO = OFF_AF_HI + TILE_AF;
constexpr uint32_t OFF_R = OFF_AF_LO + TILE_AF;
constexpr uint32_t TILE_B1 = 96 * KI * 2;   // inverse full-axis data: rows (part, half mode)
constexpr uint32_t TILE_A2 = 128 * KI * 2;  // inverse half-axis data: rows = full-axis positions
constexpr uint32_t TILE_B3 = 128 * KF * 2;  // forward half-axis data: rows = full-axis positions
constexpr uint32_t TILE_B4 = 96 * KF * 2;   // forward full-axis data: rows = Af rows of the half modes
constexpr uint32_t R_B1_HI = 0, R_B1_LO = TILE_B1;
constexpr uint32_t R_A2_HI = 2 * TILE_B1, R_A2_LO = 2 * TILE_B1 + TILE_A2;
constexpr uint32_t R_BYTES = 2 * TILE_B1 + 2 * TILE_A2;
constexpr uint32_t OFF_X = OFF_R + R_BYTES;
constexpr uint32_t X_BYTES = (2 * KMAX + 1) * XS_LD * 8;
constexpr uint32_t SMEM_BYTES = OFF_X + X_BYTES;
static_assert(2 * TILE_B3 <= R_BYTES && 2 * TILE_B4 <= R_BYTES, "region R too small");
static_assert(128 * KF * 2 - TILE_AF <= R_BYTES, "Af overflow rows must stay inside shared memory");
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
  int* status;
};

// Ai[r][k]: rows r = 32 w + l, slot s = 16 w + (l & 15); l < 16: cos row of
// index s; l >= 16: sin row of index s (s >= 1) or the cos row of index N/2 (s = 0).
__device__ double ai_val(int r, int k, int K) {
  const int w = r >> 5, l = r & 31, s = 16 * w + (l & 15);
  const bool sinl = l >= 16;
  if (!sinl || s == 0) {
    const int idx = sinl ? H : s;
    return (k < 48 && k <= K) ? cospi(2.0 * ((k * idx) % N) / N) : 0.0;
  }
  const int kk = k - 48;
  return (k >= 48 && kk >= 1 && kk <= K) ? sinpi(2.0 * ((kk * s) % N) / N) : 0.0;
}

// Af[r][k]: rows r = 32 w + l (w < 3), mode m = 16 w + (l & 15); l < 16: cos
// row over e_0..e_64 (k = 0..64); l >= 16: sin row over o_1..o_63 (k = 65..127).
__device__ double af_val(int r, int k, int K) {
  const int w = r >> 5, l = r & 31, m = 16 * w + (l & 15);
  if (m > K) return 0.0;
  if (l < 16) return k <= 64 ? cospi(2.0 * ((m * k) % N) / N) : 0.0;
  if (m == 0 || k < 65) return 0.0;
  return sinpi(2.0 * ((m * (k - 64)) % N) / N);
}

__device__ __forceinline__ void split8d_store(const double (&v)[8], unsigned char* hi, unsigned char* lo, uint32_t off) {
  uint32_t h[4], q[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    uint32_t hh[2], ll[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const double d = v[2 * i + u];
      const __nv_bfloat16 b = __float2bfloat16_rn((float)d);
      const __nv_bfloat16 c = __float2bfloat16_rn((float)(d - (double)__bfloat162float(b)));
      hh[u] = __bfloat16_as_ushort(b);
      ll[u] = __bfloat16_as_ushort(c);
    }
    h[i] = hh[0] | (hh[1] << 16);
    q[i] = ll[0] | (ll[1] << 16);
  }
  *reinterpret_cast<uint4*>(hi + off) = make_uint4(h[0], h[1], h[2], h[3]);
  *reinterpret_cast<uint4*>(lo + off) = make_uint4(q[0], q[1], q[2], q[3]);
}

// derived field f of the vorticity spectrum X at (full mode kf, half mode kh), scaled by 1/N^2:
// 0: u^ = i k_half psi^, 1: v^ = -i k_full psi^, 2: wx^ = i k_full w^, 3: wy^ = i k_half w^,
// psi^ = w^ / Lap with 1/Lap = 1 at k = 0 (_vorticity_convection.py:76-92)
__device__ __forceinline__ float2 derived(int f, float2 X, float kxs, float kys, float invNN) {
  float2 r;
  if (f < 2) {
    const float lap = -(kxs * kxs + kys * kys);
    const float il = (lap == 0.f) ? 1.f : __frcp_rn(lap);
    const float2 psi = cscale(X, il);
    r = (f == 0) ? make_float2(-kys * psi.y, kys * psi.x) : make_float2(kxs * psi.y, -kxs * psi.x);
  } else {
    const float kk = (f == 2) ? kxs : kys;
    r = make_float2(-kk * X.y, kk * X.x);
  }
  return cscale(r, invNN);
}

__global__ void __launch_bounds__(THREADS, 1) tcdft2d_kernel(const Args a) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ __align__(8) uint64_t s_mbar;
  __shared__ uint32_t s_tbase;
  const PlanDev& P = a.P;
  const int K = min(P.kmax, KMAX);
  const int Kc = K + 1, NF = 2 * K + 1;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, q = warp & 3;
  const bool upper = warp >= 4;
  unsigned char* ai_hi = sm + OFF_AI_HI;
  unsigned char* ai_lo = sm + OFF_AI_LO;
  unsigned char* af_hi = sm + OFF_AF_HI;
  unsigned char* af_lo = sm + OFF_AF_LO;
  unsigned char* rg = sm + OFF_R;
  float2* Xs = reinterpret_cast<float2*>(sm + OFF_X);
  const uint32_t sAiH = tc::smem_u32(ai_hi), sAiL = tc::smem_u32(ai_lo);
  const uint32_t sAfH = tc::smem_u32(af_hi), sAfL = tc::smem_u32(af_lo);
  const uint32_t sR = tc::smem_u32(rg);

  // ---- constant DFT tiles (angles in FP64, split into bf16 hi/lo)
  for (int t = tid; t < 128 * (KI / 8); t += THREADS) {
    const int r = t / (KI / 8), c = t % (KI / 8);
    double v[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = ai_val(r, 8 * c + j, K);
    split8d_store(v, ai_hi, ai_lo, tc::kmaj_chunk(r, c, KI));
  }
  for (int t = tid; t < 96 * (KF / 8); t += THREADS) {
    const int r = t / (KF / 8), c = t % (KF / 8);
    double v[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = af_val(r, 8 * c + j, K);
    split8d_store(v, af_hi, af_lo, tc::kmaj_chunk(r, c, KF));
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
  auto wait_mma = [&]() -> bool {
    const bool ok = tc::mbar_wait(&s_mbar, phase, WAIT_BUDGET);
    phase ^= 1u;
    const int anybad = __syncthreads_or(!ok);
    tc::fence_after_sync();
    return anybad == 0;
  };

  // inverse full-axis data of field f: rows n = part * 48 + kh, k = [S_0..S_47 | D_0..D_47]
  auto build_b1 = [&](int f) {
    for (int t = tid; t < 96 * (KI / 8); t += THREADS) {
      const int c = t / 96, n = t - c * 96;
      const int part = n >= 48 ? 1 : 0;
      const int kh = n - 48 * part;
      float v[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) v[j] = 0.f;
      if (kh <= K) {
        const float kys = ksc * (float)kh;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int k = 8 * c + j;
          const bool dp = k >= 48;
          const int kf = dp ? k - 48 : k;
          if (kf <= K && !(dp && kf == 0)) {
            const float kxs = ksc * (float)kf;
            const float2 xp = derived(f, Xs[(kf + K) * XS_LD + kh], kxs, kys, invNN);
            float2 cmb = xp;
            if (kf > 0) {
              const float2 xm = derived(f, Xs[(K - kf) * XS_LD + kh], -kxs, kys, invNN);
              cmb = dp ? csub(xp, xm) : cadd(xp, xm);
            }
            v[j] = part ? cmb.y : cmb.x;
          }
        }
      }
      tc::split8_store(v, rg + R_B1_HI, rg + R_B1_LO, tc::kmaj_chunk(n, c, KI));
    }
  };

  // D1 (slot f) -> inverse half-axis data rows (full-axis position i), k = [w Re g | w Im g]
  auto build_a2 = [&](int f) {
    const bool sinl = lane >= 16;
    const int s = 16 * q + (lane & 15);
    const int iout = sinl ? (s == 0 ? H : N - s) : s;
    const bool eonly = (s == 0);
    const int b0 = upper ? 3 : 0;
    for (int b = b0; b < b0 + 3; ++b) {
      float re[8], im[8], gr[8], gi[8];
      tc::tmem_ld8(tl + 128u * f + 8u * b, re);
      tc::tmem_ld8(tl + 128u * f + 48u + 8u * b, im);
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const float pre = __shfl_xor_sync(0xffffffffu, re[j], 16);
        const float pim = __shfl_xor_sync(0xffffffffu, im[j], 16);
        const float w = (b == 0 && j == 0) ? 1.f : 2.f;
        float r1, r2;
        if (eonly) {
          r1 = re[j];
          r2 = im[j];
        } else if (!sinl) {
          r1 = re[j] - pim;  // E + i O
          r2 = im[j] + pre;
        } else {
          r1 = pre + im[j];  // E - i O
          r2 = pim - re[j];
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
    // ---- kept modes -> staging spectrum and state
    for (int t = tid; t < NF * Kc; t += THREADS) {
      const int fr = t / Kc, kh = t - fr * Kc;
      const int kfi = (fr - K + N) % N;
      const float2 v = uin[(int64_t)kfi * M + kh];
      Xs[fr * XS_LD + kh] = v;
      if (!a.nonlinear_only) sb.U[(int64_t)kh * N + kfi] = v;
    }
    __syncthreads();

    for (int qq = 0; qq < Q && !bad; ++qq) {
      const int st = qq % nst;
      const bool last_of_step = (st == nst - 1);
      // ===== inverse transforms of the 4 derived fields; D2 of field f ends in TMEM slot f
      build_b1(0);
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
          build_b1(f + 1);  // B1 is free (its MMA completed); overlaps the MMA above
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
#pragma unroll
          for (int f = 0; f < 4; ++f) {
            tc::tmem_ld8(tl + 128u * f + cc, Pv[f]);
            tc::tmem_ld8(tl + 128u * f + cc + 16u, Qv[f]);
          }
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
          tc::tmem_ld8(tl + 8u * c, A);
          tc::tmem_ld8(tl + 120u - 8u * c, B);
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

      // ===== D4 -> nonlinear term at the kept modes -> ETDRK stage update
      if (q < 3) {
        const bool srow = lane >= 16;
        const int kf = 16 * q + (lane & 15);
        const bool active = kf <= K && !(srow && kf == 0);
        const int kfs = srow ? -kf : kf;
        const int kfi = (kfs + N) % N;
        const int b0 = upper ? 3 : 0;
        for (int b = b0; b < b0 + 3; ++b) {
          const uint32_t na = 32u * (b >> 1) + 8u * (b & 1);
          float Ca[8], Cb[8];
          tc::tmem_ld8(tl + 128u + na, Ca);
          tc::tmem_ld8(tl + 128u + na + 16u, Cb);
          float2 res0 = make_float2(0.f, 0.f);
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const float Pa = __shfl_xor_sync(0xffffffffu, Ca[j], 16);
            const float Pb = __shfl_xor_sync(0xffffffffu, Cb[j], 16);
            const int kh = 8 * b + j;
            float2 Z;
            if (!srow) {
              Z = make_float2(Ca[j] - Pb, -Cb[j] - Pa);
            } else {
              Z = make_float2(Pa + Cb[j], Ca[j] - Pb);
            }
            if (active && kh <= K) {
              float2 nv = cscale(Z, negb);
              if (kh == P.inj_mode && kfs == 0) nv.x += P.inj_value;
              if (a.nonlinear_only) {
                uout[(int64_t)kfi * M + kh] = nv;
              } else {
                const float2 s = stage_upd(P, sb, (int64_t)kh * N + kfi, st, nv);
                Xs[(kfs + K) * XS_LD + kh] = s;
                if (j == 0) res0 = s;
              }
            }
          }
          if (b == 0 && last_of_step && a.project && !a.nonlinear_only) {
            // c2r projection of the step's physical round trip on the half-axis column 0
            const float2 other = make_float2(__shfl_xor_sync(0xffffffffu, res0.x, 16),
                                             __shfl_xor_sync(0xffffffffu, res0.y, 16));
            if (active) {
              const float2 mine = res0;
              const float2 a1 = srow ? other : mine;          // mode +kf
              const float2 a2 = (kf == 0) ? mine : (srow ? mine : other);  // mode -kf
              const float2 pv = make_float2(0.5f * (a1.x + a2.x), 0.5f * (a1.y - a2.y));
              const float2 val = srow ? cconj(pv) : pv;
              sb.U[kfi] = val;
              Xs[(kfs + K) * XS_LD] = val;
            }
          }
        }
      }
      tc::fence_before_sync();
      __syncthreads();
    }
    if (bad) break;

    // ---- kept modes -> output
    if (!a.nonlinear_only) {
      for (int t = tid; t < NF * Kc; t += THREADS) {
        const int fr = t / Kc, kh = t - fr * Kc;
        const int kfi = (fr - K + N) % N;
        uout[(int64_t)kfi * M + kh] = sb.U[(int64_t)kh * N + kfi];
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
    EXGB_CUDA(cudaMalloc(&plan->d_tc_scratch, sizeof(float2) * per * plan->sm_count));
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
  a.status = plan->d_status;
  const int grid = (int)std::min<int64_t>(batch, plan->sm_count);
  tcd::tcdft2d_kernel<<<grid, tcd::THREADS, tcd::SMEM_BYTES, st>>>(a);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

}  // namespace exgb
