// exgb_etdrk2d.cu -- fused multi-step ETDRK1..4 for the 2D vorticity
// formulation (NavierStokesVorticity / KolmogorovFlowVorticity), one
// thread-block cluster per sample.
//
// Reference: nonlin_fun/_vorticity_convection.py:78-99 (+ :178-182) for the
// nonlinearity, etdrk/_etdrk_1..4.py for the stage combinations,
// _spectral.py:614-721 for the transform conventions.
//
// Spectral layout: the Fourier state is (N, M = N/2+1), kx along the first
// axis, ky along the last (rfft) axis.  The 2/3 mask keeps |kx| <= K and
// ky <= K, so only Kc = K+1 ky-columns carry a nonlinear term.
//
// Work split inside a cluster of G CTAs:
//   * CTA g owns masked columns [g*Cl, min(Kc, (g+1)*Cl)) and physical rows
//     [g*Rl, min(N, (g+1)*Rl)), Rl = ceil(N/G) (the last CTA may own fewer).
//   * Column phase (per owned column, in batches of CB columns):
//       forward FFT along kx of the dealiased product (gathered from the
//       row owners' shared memory), -b scaling + forcing, ETDRK stage update
//       against the stage buffers (global scratch, L2-resident), and -- for
//       the next stage -- the four derived spectra
//         u^ = i k_y psi^, v^ = -i k_x psi^, wx^ = i k_x w^, wy^ = i k_y w^,
//         psi^ = w^ / Lap (1 at k = 0)
//       inverse-transformed along kx into `mixed` (distributed shared memory).
//   * Row phase (per owned row, batches of RB rows): gather the four mixed
//       rows over DSMEM, two complex inverse FFTs (u + i v, wx + i wy packed),
//       product u wx + v wy, one forward FFT per two rows (packed), keep
//       ky <= K into `prod` (local shared memory).
//   Two cluster barriers per ETDRK stage; the stage buffers never leave L2
//   while a cluster works on its sample; HBM sees the initial state and the
//   final state only.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>

#include "exgb_internal.h"

namespace cg = cooperative_groups;

namespace exgb {

constexpr int kMaxG = 16;

struct Args2D {
  PlanDev P;
  int G, Cl, Rl, CB, RB, Kc, Ul;
  int mixed_in_smem;
  const float2* in;   // (B, N, M) row-major
  float2* out;        // (B, N, M) row-major
  int64_t batch;
  int nsteps;
  int project;
  int nonlinear_only;
  float2* scratch;          // per-cluster stage buffers
  int64_t scratch_stride;   // float2 elements per cluster
  float2* gmixed;           // per-cluster mixed buffers when not in smem
  int64_t gmixed_stride;
};

struct Stage2D {
  float2 *U, *S1, *S, *N0, *N1, *N2;
};

__host__ __device__ __forceinline__ int nstage_bufs(int order) {
  return order <= 1 ? 1 : order == 2 ? 3 : order == 3 ? 4 : 6;
}

// ETDRK stage update at one mode; returns the next stage input (or the new
// state after the last stage).  Same formulas as the 1D epilogue.
__device__ __forceinline__ float2 stage2d(const PlanDev& P, const Stage2D& b, int64_t o, int64_t c, int stage,
                                          float2 nv) {
  switch (P.order) {
    case 1: {
      const float2 r = cadd(cmul(__ldg(P.E + c), b.U[o]), cscale(nv, __ldg(P.c[0] + c)));
      b.U[o] = r;
      return r;
    }
    case 2:
      if (stage == 0) {
        const float2 s = cadd(cmul(__ldg(P.E + c), b.U[o]), cscale(nv, __ldg(P.c[0] + c)));
        b.N0[o] = nv;
        b.S[o] = s;
        return s;
      } else {
        const float2 r = cadd(b.S[o], cscale(csub(nv, b.N0[o]), __ldg(P.c[1] + c)));
        b.U[o] = r;
        return r;
      }
    case 3:
      if (stage == 0) {
        const float2 s = cadd(cmul(__ldg(P.Eh + c), b.U[o]), cscale(nv, __ldg(P.c[0] + c)));
        b.N0[o] = nv;
        b.S[o] = s;
        return s;
      } else if (stage == 1) {
        const float2 t = csub(cscale(nv, 2.f), b.N0[o]);
        const float2 s = cadd(cmul(__ldg(P.E + c), b.U[o]), cscale(t, __ldg(P.c[1] + c)));
        b.N1[o] = nv;
        b.S[o] = s;
        return s;
      } else {
        float2 r = cmul(__ldg(P.E + c), b.U[o]);
        r = cadd(r, cscale(b.N0[o], __ldg(P.c[2] + c)));
        r = cadd(r, cscale(b.N1[o], __ldg(P.c[3] + c)));
        r = cadd(r, cscale(nv, __ldg(P.c[4] + c)));
        b.U[o] = r;
        return r;
      }
    default:  // 4
      if (stage == 0) {
        const float2 s = cadd(cmul(__ldg(P.Eh + c), b.U[o]), cscale(nv, __ldg(P.c[0] + c)));
        b.N0[o] = nv;
        b.S1[o] = s;
        return s;
      } else if (stage == 1) {
        const float2 s = cadd(cmul(__ldg(P.Eh + c), b.U[o]), cscale(nv, __ldg(P.c[0] + c)));
        b.N1[o] = nv;
        b.S[o] = s;
        return s;
      } else if (stage == 2) {
        const float2 t = csub(cscale(nv, 2.f), b.N0[o]);
        const float2 s = cadd(cmul(__ldg(P.Eh + c), b.S1[o]), cscale(t, __ldg(P.c[0] + c)));
        b.N2[o] = nv;
        b.S[o] = s;
        return s;
      } else {
        float2 r = cmul(__ldg(P.E + c), b.U[o]);
        r = cadd(r, cscale(b.N0[o], __ldg(P.c[3] + c)));
        r = cadd(r, cscale(cadd(b.N1[o], b.N2[o]), 2.f * __ldg(P.c[4] + c)));
        r = cadd(r, cscale(nv, __ldg(P.c[5] + c)));
        b.U[o] = r;
        return r;
      }
  }
}

// Output map of the column inverse FFT: sequence s = f * nc + c, element x
// -> mixed[(f * N + x) * Cl + cb0 + c].
struct MixedMap {
  float2* p;
  int nc, N, Cl, cb0;
  __device__ __forceinline__ float2& operator()(int s, int x) const {
    const int f = s / nc, c = s - f * nc;
    return p[(f * N + x) * Cl + cb0 + c];
  }
};

__device__ __forceinline__ int signed_k(int i, int N) { return (i <= (N - 1) / 2) ? i : i - N; }

__global__ void __launch_bounds__(512, 1) etdrk2d_kernel(const Args2D a) {
  cg::cluster_group cluster = cg::this_cluster();
  const int G = a.G;
  const int g = (int)cluster.block_rank();
  const int cid = (int)(blockIdx.x / G);
  const int ncl = (int)(gridDim.x / G);
  const PlanDev& P = a.P;
  const int N = P.N, M = P.M, K = a.Kc - 1, Kc = a.Kc;
  const int Cl = a.Cl, Rl = a.Rl, CB = a.CB, RB = a.RB;
  const int tid = threadIdx.x, nthr = blockDim.x;

  extern __shared__ __align__(16) float2 sm[];
  // shared memory carve-up (must match etdrk2d_configure)
  float2* tw = sm;
  float2* prod = tw + N;                         // Rl x Kc
  float2* colbuf = prod + (size_t)Rl * Kc;       // CB x N
  const int wlen = max(4 * CB * N, 2 * RB * N);
  float2* w0 = colbuf + (size_t)CB * N;
  float2* w1 = w0 + wlen;
  float2* mixed_local = w1 + wlen;               // 4 x N x Cl (when in smem)

  for (int t = tid; t < N; t += nthr) tw[t] = __ldg(P.tw + t);

  __shared__ float2* s_mixed[kMaxG];
  __shared__ float2* s_prod[kMaxG];
  if (tid < G) {
    if (a.mixed_in_smem) {
      s_mixed[tid] = cluster.map_shared_rank(mixed_local, tid);
    } else {
      s_mixed[tid] = a.gmixed + (int64_t)cid * a.gmixed_stride + (int64_t)tid * 4 * N * Cl;
    }
    s_prod[tid] = cluster.map_shared_rank(prod, tid);
  }
  float2* my_mixed = a.mixed_in_smem ? mixed_local : a.gmixed + (int64_t)cid * a.gmixed_stride + (int64_t)g * 4 * N * Cl;
  __syncthreads();

  const int col0 = g * Cl;
  const int ncols = max(0, min(Kc, col0 + Cl) - col0);
  const int row0 = g * Rl;
  const int myRl = max(0, min(Rl, N - row0));
  const float invNN = 1.f / ((float)N * (float)N);
  const float negb = -P.conv_scale;
  const int nst = a.nonlinear_only ? 1 : P.order;
  const int Q = a.nonlinear_only ? 1 : a.nsteps * P.order;
  const bool even = (N & 1) == 0;

  float2* sbase = a.scratch + (int64_t)cid * a.scratch_stride;
  Stage2D sb;
  {
    const int64_t colsz = (int64_t)Kc * N;
    float2* q = sbase;
    sb.U = q;
    q += colsz;
    sb.S1 = sb.S = sb.N0 = sb.N1 = sb.N2 = nullptr;
    if (P.order == 2) {
      sb.S = q; q += colsz;
      sb.N0 = q; q += colsz;
    } else if (P.order == 3) {
      sb.S = q; q += colsz;
      sb.N0 = q; q += colsz;
      sb.N1 = q; q += colsz;
    } else if (P.order == 4) {
      sb.S1 = q; q += colsz;
      sb.S = q; q += colsz;
      sb.N0 = q; q += colsz;
      sb.N1 = q; q += colsz;
      sb.N2 = q; q += colsz;
    }
  }

  for (int64_t smp = cid; smp < a.batch; smp += ncl) {
    const float2* uin = a.in + smp * (int64_t)N * M;
    float2* uout = a.out + smp * (int64_t)N * M;

    // ---- load owned masked columns into the state buffer (ky-major)
    for (int t = tid; t < ncols * N; t += nthr) {
      const int kx = t / ncols, c = t - kx * ncols;
      sb.U[(int64_t)(col0 + c) * N + kx] = uin[(int64_t)kx * M + col0 + c];
    }
    __syncthreads();

    // ---- prologue: derived spectra of stage 0 for all owned columns
    for (int cb0 = 0; cb0 < ncols; cb0 += CB) {
      const int nc = min(CB, ncols - cb0);
      for (int t = tid; t < nc * N; t += nthr) {
        const int c = t / N, kx = t - c * N;
        colbuf[t] = sb.U[(int64_t)(col0 + cb0 + c) * N + kx];
      }
      __syncthreads();
      // derive (shared code below, duplicated to keep the loop simple)
      for (int t = tid; t < 4 * nc * N; t += nthr) {
        const int s = t / N, kx = t - s * N;
        const int f = s / nc, c = s - f * nc;
        const int ky = col0 + cb0 + c;
        const int kxs_i = signed_k(kx, N);
        float2 r = make_float2(0.f, 0.f);
        if (kxs_i <= K && kxs_i >= -K) {
          const float2 w = colbuf[c * N + kx];
          const float kxs = P.kscale * (float)kxs_i, kys = P.kscale * (float)ky;
          const float lap = -(kxs * kxs + kys * kys);
          const float il = (lap == 0.f) ? 1.f : 1.f / lap;
          if (f == 0) r = make_float2(-kys * il * w.y, kys * il * w.x);        // i ky psi
          else if (f == 1) r = make_float2(kxs * il * w.y, -kxs * il * w.x);  // -i kx psi
          else if (f == 2) r = make_float2(-kxs * w.y, kxs * w.x);            // i kx w
          else r = make_float2(-kys * w.y, kys * w.x);                        // i ky w
          r = cscale(r, invNN);
        }
        w0[t] = r;
      }
      __syncthreads();
      block_fft<true>(P.fft, w0, w1, MixedMap{my_mixed, nc, N, Cl, cb0}, 4 * nc, tw, tid, nthr, BlockSync{});
    }

    for (int q = 0; q < Q; ++q) {
      const int st = q % nst;
      const bool last_of_step = (st == nst - 1);
      const bool last = (q == Q - 1);
      cluster.sync();  // mixed complete

      // ---------------- row phase
      for (int rb0 = 0; rb0 < myRl; rb0 += RB) {
        const int nr = min(RB, myRl - rb0);
        // gather, four elements per thread in flight: all loads (L2 or DSMEM) first, then the
        // shared-memory stores, so the loads of later elements do not wait behind earlier stores
        const int tot = nr * N;
        for (int t0 = tid; t0 < tot; t0 += 4 * nthr) {
          float2 L[4][4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const int t = t0 + u * nthr;
            L[u][0] = L[u][1] = L[u][2] = L[u][3] = make_float2(0.f, 0.f);
            if (t < tot) {
              const int r = t / N, k = t - r * N;
              const int x = row0 + rb0 + r;
              const int kk = k >= M ? N - k : k;
              if (kk <= K) {
                const int og = kk / Cl, c = kk - og * Cl;
                const float2* mb = s_mixed[og];
                L[u][0] = mb[(0 * N + x) * Cl + c];
                L[u][1] = mb[(1 * N + x) * Cl + c];
                L[u][2] = mb[(2 * N + x) * Cl + c];
                L[u][3] = mb[(3 * N + x) * Cl + c];
              }
            }
          }
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const int t = t0 + u * nthr;
            if (t < tot) {
              const int r = t / N, k = t - r * N;
              const bool ext = k >= M;
              const bool ro = (k == 0) || (even && k == N / 2);
              w0[(2 * r) * N + k] = pack_pair(L[u][0], L[u][1], ext, ro);
              w0[(2 * r + 1) * N + k] = pack_pair(L[u][2], L[u][3], ext, ro);
            }
          }
        }
        __syncthreads();
        float2* res = result_buf(P.fft, w0, w1);
        float2* oth = (res == w0) ? w1 : w0;
        block_fft<true>(P.fft, w0, w1, LinMap{res, N}, 2 * nr, tw, tid, nthr, BlockSync{});
        const int npair = (nr + 1) / 2;
        for (int t = tid; t < 2 * npair * N; t += nthr) {
          const int r = t / N, x = t - r * N;
          float p = 0.f;
          if (r < nr) {
            const float2 zu = res[(2 * r) * N + x];
            const float2 zw = res[(2 * r + 1) * N + x];
            p = fmaf(zu.x, zw.x, zu.y * zw.y);
          }
          reinterpret_cast<float*>(oth)[((r >> 1) * N + x) * 2 + (r & 1)] = p;
        }
        __syncthreads();
        float2* fres = result_buf(P.fft, oth, res);
        block_fft<false>(P.fft, oth, res, LinMap{fres, N}, npair, tw, tid, nthr, BlockSync{});
        for (int t = tid; t < npair * Kc; t += nthr) {
          const int j = t / Kc, ky = t - j * Kc;
          float2 A, B;
          unpack_pair(fres[j * N + ky], fres[j * N + (ky == 0 ? 0 : N - ky)], A, B);
          const int r = rb0 + 2 * j;
          prod[r * Kc + ky] = A;
          if (2 * j + 1 < nr) prod[(r + 1) * Kc + ky] = B;
        }
        __syncthreads();
      }
      cluster.sync();  // prod complete

      // ---------------- column phase
      for (int cb0 = 0; cb0 < ncols; cb0 += CB) {
        const int nc = min(CB, ncols - cb0);
        // gather the product columns (ky fixed, all x) from the row owners
        {
          const int tot = nc * N;
          for (int t0 = tid; t0 < tot; t0 += 4 * nthr) {
            float2 L[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
              const int t = t0 + u * nthr;
              L[u] = make_float2(0.f, 0.f);
              if (t < tot) {
                const int x = t / nc, c = t - x * nc;
                const int og = x / Rl, xr = x - og * Rl;
                L[u] = s_prod[og][xr * Kc + col0 + cb0 + c];
              }
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
              const int t = t0 + u * nthr;
              if (t < tot) {
                const int x = t / nc, c = t - x * nc;
                w0[c * N + x] = L[u];
              }
            }
          }
        }
        __syncthreads();
        float2* res = result_buf(P.fft, w0, w1);
        block_fft<false>(P.fft, w0, w1, LinMap{res, N}, nc, tw, tid, nthr, BlockSync{});
        for (int t = tid; t < nc * N; t += nthr) {
          const int c = t / N, kx = t - c * N;
          const int ky = col0 + cb0 + c;
          const int ks = signed_k(kx, N);
          float2 nv = make_float2(0.f, 0.f);
          if (ks <= K && ks >= -K) nv = cscale(res[t], negb);
          if (ky == P.inj_mode && kx == 0) nv.x += P.inj_value;
          const int64_t o = (int64_t)ky * N + kx;
          if (a.nonlinear_only) {
            uout[(int64_t)kx * M + ky] = nv;
          } else {
            colbuf[t] = stage2d(P, sb, o, o, st, nv);
          }
        }
        __syncthreads();
        if (!a.nonlinear_only && last_of_step && a.project) {
          // c2r projection of the step's physical round trip on ky = 0 (and
          // ky = N/2): Hermitian-symmetrise the column along kx
          for (int c = 0; c < nc; ++c) {
            const int ky = col0 + cb0 + c;
            if (ky == 0 || (even && ky == N / 2)) {
              float2 v[2];
              int idx[2];
              int cnt = 0;
              for (int kx = tid; kx < N && cnt < 2; kx += nthr) {
                const float2 a1 = colbuf[c * N + kx];
                const float2 a2 = colbuf[c * N + (kx == 0 ? 0 : N - kx)];
                v[cnt] = make_float2(0.5f * (a1.x + a2.x), 0.5f * (a1.y - a2.y));
                idx[cnt++] = kx;
              }
              // N <= 2*nthr is guaranteed by the configuration
              __syncthreads();
              for (int u = 0; u < cnt; ++u) {
                colbuf[c * N + idx[u]] = v[u];
                sb.U[(int64_t)ky * N + idx[u]] = v[u];
              }
              __syncthreads();
            }
          }
        }
        if (!last && !a.nonlinear_only) {
          for (int t = tid; t < 4 * nc * N; t += nthr) {
            const int s = t / N, kx = t - s * N;
            const int f = s / nc, c = s - f * nc;
            const int ky = col0 + cb0 + c;
            const int kxs_i = signed_k(kx, N);
            float2 r = make_float2(0.f, 0.f);
            if (kxs_i <= K && kxs_i >= -K) {
              const float2 w = colbuf[c * N + kx];
              const float kxs = P.kscale * (float)kxs_i, kys = P.kscale * (float)ky;
              const float lap = -(kxs * kxs + kys * kys);
              const float il = (lap == 0.f) ? 1.f : 1.f / lap;
              if (f == 0) r = make_float2(-kys * il * w.y, kys * il * w.x);
              else if (f == 1) r = make_float2(kxs * il * w.y, -kxs * il * w.x);
              else if (f == 2) r = make_float2(-kxs * w.y, kxs * w.x);
              else r = make_float2(-kys * w.y, kys * w.x);
              r = cscale(r, invNN);
            }
            w0[t] = r;
          }
          __syncthreads();
          block_fft<true>(P.fft, w0, w1, MixedMap{my_mixed, nc, N, Cl, cb0}, 4 * nc, tw, tid, nthr, BlockSync{});
        }
      }
    }

    // ---- store owned masked columns
    if (!a.nonlinear_only) {
      for (int t = tid; t < ncols * N; t += nthr) {
        const int kx = t / ncols, c = t - kx * ncols;
        uout[(int64_t)kx * M + col0 + c] = sb.U[(int64_t)(col0 + c) * N + kx];
      }
    }
    // ---- unmasked columns: linear part only (N^ = 0 there)
    {
      const int u0c = Kc + g * a.Ul;
      const int u1c = min(M, u0c + a.Ul);
      const int nuc = max(0, u1c - u0c);
      // one thread per (column, kx <= N/2) pair {kx, N-kx}
      const int half = N / 2 + 1;
      for (int t = tid; t < nuc * half; t += nthr) {
        const int c = t / half, kx = t - c * half;
        const int ky = u0c + c;
        const int kx2 = (kx == 0) ? 0 : N - kx;
        if (a.nonlinear_only) {
          uout[(int64_t)kx * M + ky] = make_float2(0.f, 0.f);
          uout[(int64_t)kx2 * M + ky] = make_float2(0.f, 0.f);
          continue;
        }
        float2 v1 = uin[(int64_t)kx * M + ky];
        float2 v2 = uin[(int64_t)kx2 * M + ky];
        // ky-major coefficient index
        const float2 E1 = __ldg(P.E + (int64_t)ky * N + kx);
        const float2 E2 = __ldg(P.E + (int64_t)ky * N + kx2);
        const bool proj = a.project && (ky == 0 || (even && ky == N / 2));
        for (int s = 0; s < a.nsteps; ++s) {
          v1 = cmul(E1, v1);
          v2 = cmul(E2, v2);
          if (proj) {
            const float2 pv = make_float2(0.5f * (v1.x + v2.x), 0.5f * (v1.y - v2.y));
            v1 = pv;
            v2 = cconj(pv);
          }
        }
        uout[(int64_t)kx * M + ky] = v1;
        if (kx2 != kx) uout[(int64_t)kx2 * M + ky] = v2;
      }
    }
    cluster.sync();  // all DSMEM reads of this sample done before reuse
  }
}

int etdrk2d_configure(exgb_plan* plan) {
  PlanDev& P = plan->dev;
  Plan2DConfig& c = plan->cfg2d;
  if (P.kmax < P.N / 2 && !getenv("EXGB_GENERIC_2D")) {
    const int rc = vort2d_configure(plan);
    if (rc == EXGB_OK) {
      c.variant = 1;
      return EXGB_OK;
    }
    if (rc != EXGB_EUNSUPPORTED) return rc;
  }
  c.variant = 0;
  const int N = P.N, M = P.M;
  const int K = std::min(P.kmax, N / 2);
  if (K < 0) return fail(EXGB_EUNSUPPORTED, "dealiasing mask removes every mode");
  const int Kc = K + 1;
  int dev = 0, lim = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&lim, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t limit = (size_t)lim - 1024;  // static shared memory headroom
  const int threads = N >= 128 ? 512 : 256;
  if (N > 2 * threads) return fail(EXGB_EUNSUPPORTED, "N too large for the 2D kernel in this build");
  // Candidates: cluster size G (the autotuner's choice, else EXGB_CLUSTER, else 1..8; a CTA owns
  // ceil(N/G) rows), columns (CB) and rows (RB) per transform batch (EXGB_2D_CB / EXGB_2D_RB, else
  // about twelve, eight or four points per thread per transform), mixed fields in distributed
  // shared memory or in a per-cluster global buffer.  The kernel waits at a block barrier after
  // every radix pass, so larger batches amortise the barriers: at 512^2 (Kolmogorov, 20 steps, per
  // sample and CTA-wave) twelve points per thread cost 0.70x and eight 0.75x the time of four; 256
  // threads instead of 512 were slower.  Choice: mixed fields in shared memory when any candidate
  // fits so, then the most SMs kept busy (co-resident clusters x G from the occupancy query, at
  // most the SM count) weighted by that batch efficiency, ties to the smaller cluster.
  const char* envG = getenv("EXGB_CLUSTER");
  const int wantG = plan->tune_cluster > 0 ? plan->tune_cluster : (envG ? atoi(envG) : 0);
  const char* envCB = getenv("EXGB_2D_CB");
  const char* envRB = getenv("EXGB_2D_RB");
  const int wantCB = envCB ? atoi(envCB) : 0;
  const int wantRB = envRB ? atoi(envRB) : 0;
  // the opt-in maximum (every generic 2D plan launches this kernel with its own footprint)
  EXGB_CUDA(cudaFuncSetAttribute(etdrk2d_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)limit));
  bool found = false;
  double best = -1.0;
  for (int mis = 1; mis >= 0 && !found; --mis) {
    for (int pts : {12, 8, 4}) {
      const double eff = pts == 12 ? 1.42 : pts == 8 ? 1.34 : 1.0;
      for (int G = 1; G <= 8; ++G) {
        if (wantG && wantG != G) continue;
        const int Rl = (N + G - 1) / G;
        if (Rl < 2 || (G - 1) * Rl >= N) continue;
        const int Cl = (Kc + G - 1) / G;
        int CB = std::max(1, std::min(Cl, wantCB > 0 ? wantCB : (threads * pts) / (4 * N)));
        int RB = std::max(2, std::min(Rl, wantRB > 0 ? wantRB : (threads * pts) / (2 * N)));
        RB += RB & 1;
        const size_t wlen = std::max((size_t)4 * CB * N, (size_t)2 * RB * N);
        size_t words = (size_t)N + (size_t)Rl * Kc + (size_t)CB * N + 2 * wlen;
        if (mis) words += (size_t)4 * N * Cl;
        const size_t bytes = words * sizeof(float2);
        if (bytes > limit) continue;
        cudaLaunchConfig_t q = {};
        cudaLaunchAttribute qa[1];
        qa[0].id = cudaLaunchAttributeClusterDimension;
        qa[0].val.clusterDim.x = G;
        qa[0].val.clusterDim.y = 1;
        qa[0].val.clusterDim.z = 1;
        q.gridDim = dim3(G * plan->sm_count, 1, 1);
        q.blockDim = dim3(threads, 1, 1);
        q.dynamicSmemBytes = bytes;
        q.attrs = qa;
        q.numAttrs = 1;
        int nq = 0;
        if (cudaOccupancyMaxActiveClusters(&nq, (void*)etdrk2d_kernel, &q) != cudaSuccess || nq <= 0) {
          cudaGetLastError();
          continue;
        }
        const double score = (double)std::min(nq * G, plan->sm_count) * eff;
        if (score > best * (1.0 + 1e-9)) {
          best = score;
          c.G = G;
          c.threads = threads;
          c.cols_per_cta = Cl;
          c.rows_per_cta = Rl;
          c.CB = CB;
          c.RB = RB;
          c.mixed_in_smem = mis;
          c.smem_bytes = bytes;
          found = true;
        }
      }
    }
  }
  if (!found) return fail(EXGB_EUNSUPPORTED, "2D configuration does not fit in shared memory");
  // co-resident clusters
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = c.G;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(c.G * plan->sm_count, 1, 1);
  cfg.blockDim = dim3(c.threads, 1, 1);
  cfg.dynamicSmemBytes = c.smem_bytes;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int ncl = 0;
  cudaError_t e = cudaOccupancyMaxActiveClusters(&ncl, (void*)etdrk2d_kernel, &cfg);
  if (e != cudaSuccess || ncl <= 0) {
    cudaGetLastError();
    ncl = std::max(1, plan->sm_count / c.G);
  }
  c.clusters = ncl;
  const size_t per = (size_t)nstage_bufs(P.order) * Kc * N;
  size_t mixed_per = c.mixed_in_smem ? 0 : (size_t)c.G * 4 * N * c.cols_per_cta;
  c.scratch_per_cluster = per + mixed_per;
  plan->scratch_bytes = sizeof(float2) * c.scratch_per_cluster * (size_t)ncl;
  EXGB_CUDA(cudaMalloc(&plan->d_scratch, plan->scratch_bytes));
  (void)M;
  return EXGB_OK;
}

int etdrk2d_run(const exgb_plan* plan, cudaStream_t st, const float2* in, float2* out, int64_t batch, int nsteps,
                int project, int nonlinear_only) {
  if (batch <= 0) return EXGB_OK;
  const Plan2DConfig& c = plan->cfg2d;
  if (plan->precision == 1) return tcdft2d_run(plan, st, in, out, batch, nsteps, project, nonlinear_only);
  if (c.variant == 1) return vort2d_run(plan, st, in, out, batch, nsteps, project, nonlinear_only);
  Args2D a;
  a.P = plan->dev;
  a.G = c.G;
  a.Cl = c.cols_per_cta;
  a.Rl = c.rows_per_cta;
  a.CB = c.CB;
  a.RB = c.RB;
  a.Kc = std::min(plan->dev.kmax, plan->dev.N / 2) + 1;
  a.Ul = (plan->dev.M - a.Kc + c.G - 1) / c.G;
  a.mixed_in_smem = c.mixed_in_smem;
  a.in = in;
  a.out = out;
  a.batch = batch;
  a.nsteps = nsteps;
  a.project = project;
  a.nonlinear_only = nonlinear_only;
  a.scratch = (float2*)plan->d_scratch;
  const size_t per = c.scratch_per_cluster;
  const size_t mixed_per = c.mixed_in_smem ? 0 : (size_t)c.G * 4 * plan->dev.N * c.cols_per_cta;
  a.scratch_stride = (int64_t)per;
  a.gmixed = c.mixed_in_smem ? nullptr : (float2*)plan->d_scratch + (per - mixed_per);
  a.gmixed_stride = (int64_t)per;
  const int ncl = (int)std::min<int64_t>(c.clusters, batch);
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = c.G;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(c.G * ncl, 1, 1);
  cfg.blockDim = dim3(c.threads, 1, 1);
  cfg.dynamicSmemBytes = c.smem_bytes;
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  EXGB_CUDA(cudaLaunchKernelEx(&cfg, etdrk2d_kernel, a));
  return EXGB_OK;
}

}  // namespace exgb
