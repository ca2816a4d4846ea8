// exgb_vort2d.cu -- register-FFT variant of the fused 2D vorticity ETDRK
// kernel for N in {64, 128, 256} (compile-time N).
//
// Same algorithm and cluster decomposition as etdrk2d_kernel
// (exgb_etdrk2d.cu; reference nonlin_fun/_vorticity_convection.py:78-99,
// etdrk/_etdrk_1..4.py), but every length-N transform is a group FFT of T
// lanes holding E points each (exgb_regfft.cuh): no block barrier inside a
// transform, compile-time index arithmetic, one shared-memory transpose per
// transform.  Lane l of a group always owns positions l + T j, so
//   * column inverse:  derived spectrum (registers) -> IFFT -> mixed[f][x][c]
//   * row phase:       gather over DSMEM -> 2 IFFTs -> product in registers
//                      -> pair two rows with a warp shuffle -> 1 FFT -> prod
//   * column forward:  gather prod over DSMEM -> FFT -> ETDRK stage update
// run without any intermediate layout change.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>

#include "exgb_internal.h"
#include "exgb_regfft.cuh"
#include "exgb_stage.cuh"

namespace cg = cooperative_groups;

namespace exgb {

struct ArgsV2 {
  PlanDev P;
  int G, Cl, Rl, Kc, KcP, Ul;
  const float2* in;
  float2* out;
  int64_t batch;
  int nsteps;
  int project;
  int nonlinear_only;
  float2* scratch;
  int64_t scratch_stride;
};

template <int N, int THREADS>
struct V2Layout {
  static constexpr int E = RegCfg<N>::E, T = RegCfg<N>::T;
  static constexpr int NG = THREADS / T;
  static constexpr int TS = tile_stride<E, T>();
  // Exchange buffers are laid out so that consecutive lanes (consecutive positions of one
  // transform) write consecutive addresses of the receiving CTA, 16 bytes at a time:
  //   derived fields  [pair][ky][row] x {field 2p, field 2p+1}   (float4 per entry)
  //   product spectra [row/2][column] x {row even, row odd}       (float4 per row pair)
  // The row strides are padded so that the local reads of one half-warp hit distinct banks:
  // padC (product / stage-input buffer, 8-byte reads) odd for groups of 16 lanes and = 2 (mod 16)
  // for groups of 8 (two groups, on neighbouring columns, per half-warp); padR (derived fields,
  // 16-byte reads, one group per quarter-warp phase) odd.
  __host__ __device__ static int padC(int v) { return T >= 16 ? (v | 1) : v + ((2 - v) & 15); }
  __host__ __device__ static int padR(int v) { return v | 1; }
  // float2 offsets
  __host__ __device__ static size_t twl() { return 0; }
  __host__ __device__ static size_t tiles() { return N; }
  __host__ __device__ static size_t colbuf() { return tiles() + (size_t)NG * TS; }
  // the product spectra received for the owned columns overwrite the stage input in place: the
  // stage input is consumed by the column inverse before the first cluster barrier of a stage
  __host__ __device__ static size_t prodr(int) { return colbuf(); }
  __host__ __device__ static size_t mixr(int Cl) { return prodr(Cl) + (size_t)N * padC(Cl); }
  __host__ __device__ static size_t maps(int Cl, int Rl, int Kc) { return mixr(Cl) + (size_t)4 * Kc * padR(Rl); }
  __host__ __device__ static size_t bytes(int Cl, int Rl, int Kc) {
    return sizeof(float2) * maps(Cl, Rl, Kc) + sizeof(int) * (size_t)(Kc + N);
  }
};

template <int N>
__device__ __forceinline__ int sgn_k(int i) {
  return (i <= (N - 1) / 2) ? i : i - N;
}

template <int N, int THREADS>
__global__ void __launch_bounds__(THREADS, (N == 64 ? 2 : 1)) vort2d_kernel(const ArgsV2 a) {
  using Lay = V2Layout<N, THREADS>;
  constexpr int E = Lay::E, T = Lay::T, NG = Lay::NG, TS = Lay::TS;
  constexpr int M = N / 2 + 1;
  cg::cluster_group cluster = cg::this_cluster();
  const int G = a.G;
  const int g = (int)cluster.block_rank();
  const int cid = (int)(blockIdx.x / G);
  const int ncl = (int)(gridDim.x / G);
  const PlanDev& P = a.P;
  const int Kc = a.Kc, K = Kc - 1, Cl = a.Cl, Rl = a.Rl;
  const int ClP = Lay::padC(Cl), RlP = Lay::padR(Rl);
  // stage input / product spectra of row (or kx) x in owned column c: rows interleaved in pairs
  auto cb = [ClP](int x, int c) { return ((x >> 1) * ClP + c) * 2 + (x & 1); };
  const int tid = threadIdx.x;
  const int gi = tid / T, l = tid % T;
  const int lane = tid & 31;
  const unsigned gmask = (T == 32) ? 0xffffffffu : (((1u << T) - 1u) << (lane & ~(T - 1)));

  extern __shared__ __align__(16) float2 sm[];
  float2* twl = sm + Lay::twl();
  float2* tile = sm + Lay::tiles() + (size_t)gi * TS;
  float2* colbuf = sm + Lay::colbuf();   // [kx][c]    owned columns (row stride ClP, shared with prodr)
  float2* prodr = sm + Lay::prodr(Cl);   // [x][c]     product spectra received for owned columns
  float4* mixr = reinterpret_cast<float4*>(sm + Lay::mixr(Cl));  // [pair][ky][r] derived fields of owned rows
  int* colmap = reinterpret_cast<int*>(sm + Lay::maps(Cl, Rl, Kc));  // ky -> (owner << 16) | column
  int* rowmap = colmap + Kc;                                          // x  -> (owner << 16) | row

  for (int t = tid; t < N; t += THREADS) {
    const int k1 = t / T, ll = t % T;
    twl[t] = __ldg(P.tw + ((ll * k1) % N));  // w_N^(l k1), [k1][l]
  }
  for (int kk = tid; kk < Kc; kk += THREADS) colmap[kk] = ((kk / Cl) << 16) | (kk % Cl);
  for (int x = tid; x < N; x += THREADS) rowmap[x] = ((x / Rl) << 16) | (x % Rl);
  __shared__ float4* s_mixr[16];
  __shared__ float2* s_prodr[16];
  if (tid < G) {
    s_mixr[tid] = cluster.map_shared_rank(mixr, tid);
    s_prodr[tid] = cluster.map_shared_rank(prodr, tid);
  }
  __syncthreads();

  const int col0 = g * Cl;
  const int ncols = max(0, min(Kc, col0 + Cl) - col0);
  const int row0 = g * Rl;
  const int Rg = max(0, min(Rl, N - row0));  // rows owned by this CTA (the last one may own fewer)
  const float invNN = 1.f / ((float)N * (float)N);
  const float negb = -P.conv_scale;
  const float ksc = P.kscale;
  const int nst = a.nonlinear_only ? 1 : P.order;
  const int Q = a.nonlinear_only ? 1 : a.nsteps * P.order;

  StageBufs sb;
  {
    float2* q = a.scratch + (int64_t)cid * a.scratch_stride;
    const int64_t colsz = (int64_t)Kc * N;
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

    // ---- owned masked columns -> state buffer and colbuf
    for (int t = tid; t < ncols * N; t += THREADS) {
      const int kx = t / ncols, c = t - kx * ncols;
      const float2 v = uin[(int64_t)kx * M + col0 + c];
      colbuf[cb(kx, c)] = v;
      sb.U[(int64_t)(col0 + c) * N + kx] = v;
    }
    __syncthreads();

    for (int q = 0; q < Q; ++q) {
      const int st = q % nst;
      const bool last_of_step = (st == nst - 1);
      // ================= column inverse: derived spectra -> IFFT -> pushed to the row owners
      // tasks = (column, pair): pair 0 -> (u^, v^) from psi^, pair 1 -> (wx^, wy^) from w^;
      // the two transforms of a pair are interleaved in one group
      for (int task = gi; task < 2 * ncols; task += NG) {
        const int pr = task / ncols, c = task - pr * ncols;
        const int ky = col0 + c;
        const float kys = ksc * (float)ky;
        float2 v[E], v2[E];
#pragma unroll
        for (int j = 0; j < E; ++j) {
          const int kx = l + T * j;
          const int ks = sgn_k<N>(kx);
          float2 r1 = make_float2(0.f, 0.f), r2 = r1;
          if (ks <= K && ks >= -K) {
            const float2 w = colbuf[cb(kx, c)];
            const float kxs = ksc * (float)ks;
            if (pr == 0) {
              const float lap = -(kxs * kxs + kys * kys);
              // 1/lap, 1 at k = 0: the hardware reciprocal (within 1 ulp) where registers allow; at
              // N = 256 the correctly rounded form measured faster under the 128-register cap
              float il = 1.f;
              if (lap != 0.f) {
                if constexpr (N == 256) {
                  il = __frcp_rn(lap);
                } else {
                  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(il) : "f"(lap));
                }
              }
              const float2 psi = cscale(w, il);
              r1 = make_float2(-kys * psi.y, kys * psi.x);   // u^  = i ky psi^
              r2 = make_float2(kxs * psi.y, -kxs * psi.x);   // v^  = -i kx psi^
            } else {
              r1 = make_float2(-kxs * w.y, kxs * w.x);       // wx^ = i kx w^
              r2 = make_float2(-kys * w.y, kys * w.x);       // wy^ = i ky w^
            }
            r1 = cscale(r1, invNN);
            r2 = cscale(r2, invNN);
          }
          v[j] = r1;
          v2[j] = r2;
        }
        group_fft_x2<E, T, true>(v, v2, l, tile, twl, gmask);
#pragma unroll
        for (int j = 0; j < E; ++j) {
          const int x = l + T * j;
          const int rm = rowmap[x];
          const int d = rm >> 16, xr = rm & 0xffff;
          s_mixr[d][(pr * Kc + ky) * RlP + xr] = make_float4(v[j].x, v[j].y, v2[j].x, v2[j].y);
        }
      }
      cluster.sync();  // derived fields delivered

      // ================= row phase: local gather -> 2 IFFTs -> product -> paired FFT -> pushed to column owners
      // product u wx + v wy of local row rr in registers (lane l owns positions l + T j)
      auto row_product = [&](int rr, float (&pj)[E]) {
        float2 z1[E], z2[E];
#pragma unroll
        for (int j = 0; j < E; ++j) {
          const int k = l + T * j;
          const bool ext = k > N / 2;
          const int kk = ext ? N - k : k;
          const bool ro = (k == 0) || (k == N / 2);
          float2 U = make_float2(0.f, 0.f), V = U, WX = U, WY = U;
          if (kk <= K) {
            const float4 uv = mixr[(0 * Kc + kk) * RlP + rr];
            const float4 wxy = mixr[(1 * Kc + kk) * RlP + rr];
            U = make_float2(uv.x, uv.y);
            V = make_float2(uv.z, uv.w);
            WX = make_float2(wxy.x, wxy.y);
            WY = make_float2(wxy.z, wxy.w);
          }
          z1[j] = pack_pair(U, V, ext, ro);
          z2[j] = pack_pair(WX, WY, ext, ro);
        }
        group_fft_x2<E, T, true>(z1, z2, l, tile, twl, gmask);
#pragma unroll
        for (int j = 0; j < E; ++j) pj[j] = fmaf(z1[j].x, z2[j].x, z1[j].y * z2[j].y);
      };
      // forward FFT of two rows packed as w = p_a + i p_b, unpacked and pushed to the column owners
      auto push_pair = [&](float2 (&w)[E], int r) {
        group_fft<E, T, false>(w, l, tile, twl, gmask);
        const int xa = row0 + r;
#pragma unroll
        for (int j = 0; j < E; ++j) {
          const float2 snd = w[E - 1 - j];
          float2 rcv;
          rcv.x = __shfl_sync(gmask, snd.x, (T - l) % T, T);
          rcv.y = __shfl_sync(gmask, snd.y, (T - l) % T, T);
          if (l == 0) rcv = w[(E - j) % E];
          const int k = l + T * j;
          if (k <= K) {
            float2 A, B;
            unpack_pair(w[j], rcv, A, B);
            const int cm = colmap[k];
            float2* dst = s_prodr[cm >> 16] + cb(xa, cm & 0xffff);  // xa is even: rows xa, xa + 1 adjacent
            if (r + 1 < Rg) {
              *reinterpret_cast<float4*>(dst) = make_float4(A.x, A.y, B.x, B.y);
            } else {
              dst[0] = A;
            }
          }
        }
      };
      // At N = 128 every cluster size that fits gives a CTA at most one row per group, and the
      // pair path below would only add register pressure, so it is compiled out there.
      constexpr bool kRowPairs = (N != 128);
      if (kRowPairs && Rg > NG) {
        // more rows than groups: each group takes a pair of rows (2 product evaluations, 1 FFT),
        // so no group waits through its neighbour's forward FFT
        for (int r0 = 0; r0 < Rg; r0 += 2 * NG) {
          const int r = r0 + 2 * gi;
          if (r < Rg) {
            float2 w[E];
            {
              float pa[E];
              row_product(r, pa);
              // park row r's product in row r's own (already consumed) derived-field slots, read by
              // no other group, instead of holding it in registers through the second transform
#pragma unroll
              for (int q = 0; q < E / 4; ++q)
                mixr[(q * T + l) * RlP + r] = make_float4(pa[4 * q], pa[4 * q + 1], pa[4 * q + 2], pa[4 * q + 3]);
            }
            {
              float pb[E];
              row_product(r + 1 < Rg ? r + 1 : r, pb);
#pragma unroll
              for (int q = 0; q < E / 4; ++q) {
                const float4 pa4 = mixr[(q * T + l) * RlP + r];
                w[4 * q] = make_float2(pa4.x, pb[4 * q]);
                w[4 * q + 1] = make_float2(pa4.y, pb[4 * q + 1]);
                w[4 * q + 2] = make_float2(pa4.z, pb[4 * q + 2]);
                w[4 * q + 3] = make_float2(pa4.w, pb[4 * q + 3]);
              }
            }
            push_pair(w, r);
          }
        }
      } else {
        // one row per group; neighbouring groups pair their rows through a warp shuffle
        for (int r0 = 0; r0 < Rg; r0 += NG) {
          const int r = r0 + gi;
          const bool valid = r < Rg;
          float pj[E];
          row_product(valid ? r : 0, pj);
          float2 w[E];
#pragma unroll
          for (int j = 0; j < E; ++j) {
            const float other = __shfl_xor_sync(0xffffffffu, pj[j], T);
            w[j] = make_float2(pj[j], other);
          }
          if ((gi & 1) == 0 && valid) push_pair(w, r);
        }
      }
      cluster.sync();  // product spectra delivered

      // ================= column forward FFT (local gather) -> raw N^ in colbuf
      for (int c = gi; c < ncols; c += NG) {
        const int ky = col0 + c;
        float2 v[E];
#pragma unroll
        for (int j = 0; j < E; ++j) v[j] = prodr[cb(l + T * j, c)];
        group_fft<E, T, false>(v, l, tile, twl, gmask);
#pragma unroll
        for (int j = 0; j < E; ++j) {
          const int kx = l + T * j;
          const int ks = sgn_k<N>(kx);
          float2 nv = make_float2(0.f, 0.f);
          if (ks <= K && ks >= -K) nv = cscale(v[j], negb);
          if (ky == P.inj_mode && kx == 0) nv.x += P.inj_value;
          colbuf[cb(kx, c)] = nv;
        }
      }
      __syncthreads();
      // ================= ETDRK stage update, all threads (latency-bound elementwise pass)
      if (a.nonlinear_only) {
        for (int t = tid; t < ncols * N; t += THREADS) {
          const int c = t / N, kx = t % N;
          uout[(int64_t)kx * M + col0 + c] = colbuf[cb(kx, c)];
        }
      } else {
        // kRU modes per thread at a time, their L2 loads in flight together
        constexpr int kRU = 4;
        for (int t0 = tid; t0 < ncols * N; t0 += kRU * THREADS) {
          int64_t o[kRU];
          bool ok[kRU];
          float2 nv[kRU];
          int ci[kRU];
#pragma unroll
          for (int j = 0; j < kRU; ++j) {
            const int t = t0 + j * THREADS;
            ok[j] = t < ncols * N;
            const int tt = ok[j] ? t : t0;
            const int c = tt / N, kx = tt % N;
            o[j] = (int64_t)(col0 + c) * N + kx;
            ci[j] = cb(kx, c);
            nv[j] = colbuf[ci[j]];
          }
          stage_upd_many<kRU>(P, sb, o, ok, st, nv);
#pragma unroll
          for (int j = 0; j < kRU; ++j)
            if (ok[j]) colbuf[ci[j]] = nv[j];
        }
      }
      if (!a.nonlinear_only) {
        if (last_of_step && a.project && col0 == 0 && ncols > 0) {
          // c2r projection of the step's physical round trip on ky = 0
          __syncthreads();
          for (int kx = tid; kx <= N / 2; kx += THREADS) {
            const int kx2 = (N - kx) % N;
            const float2 a1 = colbuf[cb(kx, 0)], a2 = colbuf[cb(kx2, 0)];
            const float2 pv = make_float2(0.5f * (a1.x + a2.x), 0.5f * (a1.y - a2.y));
            colbuf[cb(kx, 0)] = pv;
            colbuf[cb(kx2, 0)] = cconj(pv);
            sb.U[kx] = pv;
            sb.U[kx2] = cconj(pv);
          }
        }
      }
      __syncthreads();  // colbuf ready for the next inverse phase
    }

    // ---- store owned masked columns
    if (!a.nonlinear_only) {
      for (int t = tid; t < ncols * N; t += THREADS) {
        const int kx = t / ncols, c = t - kx * ncols;
        uout[(int64_t)kx * M + col0 + c] = sb.U[(int64_t)(col0 + c) * N + kx];
      }
    }
    // ---- unmasked columns: linear part only
    {
      const int u0c = Kc + g * a.Ul;
      const int u1c = min(M, u0c + a.Ul);
      const int nuc = max(0, u1c - u0c);
      constexpr int half = N / 2 + 1;
      for (int t = tid; t < nuc * half; t += THREADS) {
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
        const float2 E1 = __ldg(P.E + (int64_t)ky * N + kx);
        const float2 E2 = __ldg(P.E + (int64_t)ky * N + kx2);
        const bool proj = a.project && (ky == 0 || ky == N / 2);
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
    cluster.sync();
  }
}

template <int N, int THREADS>
static int v2_configure(exgb_plan* plan) {
  using Lay = V2Layout<N, THREADS>;
  PlanDev& P = plan->dev;
  Plan2DConfig& c = plan->cfg2d;
  const int K = std::min(P.kmax, N / 2 - 1);
  const int Kc = K + 1;
  int dev = 0, lim = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&lim, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t limit = (size_t)lim - 1024;
  const char* envG = getenv("EXGB_CLUSTER");
  const int wantG = plan->tune_cluster > 0 ? plan->tune_cluster : (envG ? atoi(envG) : 0);
  // Candidates: every cluster size whose shared memory fits; the automatic choice is the one that
  // keeps the most SMs busy (active clusters x G from the occupancy query: clusters must fit in one
  // GPC, so e.g. 6 can cover more SMs than 8), ties going to the smaller cluster.
  auto fn = vort2d_kernel<N, THREADS>;
  int bestG = 0, bestN = 0, bestSM = -1;
  size_t bestBytes = 0;
  int candN[9] = {0};
  size_t candBytes[9] = {0};
  cudaFree(plan->d_scratch_tail);
  plan->d_scratch_tail = nullptr;
  plan->cfg2d_tail = Plan2DConfig{};
  for (int G = 1; G <= 8; ++G) {
    if (wantG && wantG != G) continue;
    const int Cl = (Kc + G - 1) / G;
    const int Rl = 2 * ((N + 2 * G - 1) / (2 * G));  // even: row pairs never straddle two CTAs
    if (Rl < 2 || (G - 1) * Rl >= N) continue;
    const size_t bytes = Lay::bytes(Cl, Rl, Kc);
    if (bytes > limit) continue;
    EXGB_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = G;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(G * plan->sm_count, 1, 1);
    cfg.blockDim = dim3(THREADS, 1, 1);
    cfg.dynamicSmemBytes = bytes;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int ncl = 0;
    if (cudaOccupancyMaxActiveClusters(&ncl, (void*)fn, &cfg) != cudaSuccess || ncl <= 0) {
      cudaGetLastError();
      ncl = std::max(1, plan->sm_count / G);
    }
    candN[G] = ncl;
    candBytes[G] = bytes;
    if (ncl * G > bestSM) {
      bestSM = ncl * G;
      bestG = G;
      bestN = ncl;
      bestBytes = bytes;
    }
  }
  if (bestG > 0) {
    const int G = bestG;
    c.G = G;
    c.threads = THREADS;
    c.cols_per_cta = (Kc + G - 1) / G;
    c.rows_per_cta = 2 * ((N + 2 * G - 1) / (2 * G));
    c.CB = Kc | 1;  // padded ky stride of the derived-field receive buffer
    c.RB = 0;
    c.mixed_in_smem = 1;
    c.smem_bytes = bestBytes;
    // the opt-in maximum, not this plan's size: plans of the same N with other cluster sizes share
    // the kernel and launch with their own (larger or smaller) footprint
    EXGB_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)limit));
    c.clusters = bestN;
    const int nb = P.order <= 1 ? 1 : P.order == 2 ? 3 : P.order == 3 ? 4 : 6;
    c.scratch_per_cluster = (size_t)nb * Kc * N;
    plan->scratch_bytes = sizeof(float2) * c.scratch_per_cluster * (size_t)bestN;
    EXGB_CUDA(cudaMalloc(&plan->d_scratch, plan->scratch_bytes));
    // Partial last wave (N = 256): its samples run on the largest cluster size that fits, whose CTAs
    // own fewer rows and columns, so the wave ends sooner than one of the main configuration.  At
    // N = 128 (Kolmogorov, batch 1024: 13 waves of 76 clusters of 2 plus 36 samples) the 36 samples
    // on clusters of 4 took as long as a wave of 2 (36.38 against 36.32 ms), so 128 keeps one launch.
    int tG = 0;
    if (!wantG && N >= 256)
      for (int g2 = 8; g2 > G; --g2)
        if (candN[g2] > 0) {
          tG = g2;
          break;
        }
    if (tG) {
      Plan2DConfig& t = plan->cfg2d_tail;
      t = c;
      t.G = tG;
      t.cols_per_cta = (Kc + tG - 1) / tG;
      t.rows_per_cta = 2 * ((N + 2 * tG - 1) / (2 * tG));
      t.smem_bytes = candBytes[tG];
      t.clusters = candN[tG];
      EXGB_CUDA(cudaMalloc(&plan->d_scratch_tail, sizeof(float2) * t.scratch_per_cluster * (size_t)t.clusters));
    }
    return EXGB_OK;
  }
  return EXGB_EUNSUPPORTED;
}

template <int N, int THREADS>
static int v2_launch(const exgb_plan* plan, const Plan2DConfig& c, void* scratch, cudaStream_t st, const float2* in,
                     float2* out, int64_t batch, int nsteps, int project, int nonlinear_only) {
  ArgsV2 a;
  a.P = plan->dev;
  a.G = c.G;
  a.Cl = c.cols_per_cta;
  a.Rl = c.rows_per_cta;
  a.Kc = std::min(plan->dev.kmax, N / 2 - 1) + 1;
  a.KcP = c.CB;
  a.Ul = (N / 2 + 1 - a.Kc + c.G - 1) / c.G;
  a.in = in;
  a.out = out;
  a.batch = batch;
  a.nsteps = nsteps;
  a.project = project;
  a.nonlinear_only = nonlinear_only;
  a.scratch = (float2*)scratch;
  a.scratch_stride = (int64_t)c.scratch_per_cluster;
  const int ncl = (int)std::min<int64_t>(c.clusters, batch);
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = c.G;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(c.G * ncl, 1, 1);
  cfg.blockDim = dim3(THREADS, 1, 1);
  cfg.dynamicSmemBytes = c.smem_bytes;
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  EXGB_CUDA(cudaLaunchKernelEx(&cfg, vort2d_kernel<N, THREADS>, a));
  return EXGB_OK;
}

// Samples of the main configuration's partial last wave (when the tail configuration holds them
// all in one wave) go to a second launch with the tail configuration, on the same stream.
static int64_t v2_main_part(const exgb_plan* plan, int64_t batch) {
  const Plan2DConfig& c = plan->cfg2d;
  const Plan2DConfig& t = plan->cfg2d_tail;
  if (t.G <= 0 || !plan->d_scratch_tail || c.clusters <= 0) return batch;
  const int64_t r = batch % c.clusters;
  return (r > 0 && r <= t.clusters) ? batch - r : batch;
}

template <int N, int THREADS>
static int v2_run(const exgb_plan* plan, cudaStream_t st, const float2* in, float2* out, int64_t batch, int nsteps,
                  int project, int nonlinear_only) {
  const int64_t bm = v2_main_part(plan, batch);
  if (bm > 0) {
    const int rc = v2_launch<N, THREADS>(plan, plan->cfg2d, plan->d_scratch, st, in, out, bm, nsteps, project,
                                         nonlinear_only);
    if (rc) return rc;
  }
  if (bm < batch) {
    const int64_t off = bm * (int64_t)N * (N / 2 + 1);
    return v2_launch<N, THREADS>(plan, plan->cfg2d_tail, plan->d_scratch_tail, st, in + off, out + off, batch - bm,
                                 nsteps, project, nonlinear_only);
  }
  return EXGB_OK;
}

// Kernel launches one call of the register-FFT kernel makes for `batch` samples.
int vort2d_launches(const exgb_plan* plan, int64_t batch) {
  if (batch <= 0) return 0;
  const int64_t bm = v2_main_part(plan, batch);
  return (bm > 0 ? 1 : 0) + (bm < batch ? 1 : 0);
}

// Returns EXGB_EUNSUPPORTED when this N has no register-FFT variant.
int vort2d_configure(exgb_plan* plan) {
  switch (plan->dev.N) {
    case 64: return v2_configure<64, 256>(plan);
    case 128: return v2_configure<128, 512>(plan);
    case 256: return v2_configure<256, 512>(plan);
    default: return EXGB_EUNSUPPORTED;
  }
}

int vort2d_run(const exgb_plan* plan, cudaStream_t st, const float2* in, float2* out, int64_t batch, int nsteps,
               int project, int nonlinear_only) {
  if (batch <= 0) return EXGB_OK;
  switch (plan->dev.N) {
    case 64: return v2_run<64, 256>(plan, st, in, out, batch, nsteps, project, nonlinear_only);
    case 128: return v2_run<128, 512>(plan, st, in, out, batch, nsteps, project, nonlinear_only);
    case 256: return v2_run<256, 512>(plan, st, in, out, batch, nsteps, project, nonlinear_only);
    default: return fail(EXGB_EUNSUPPORTED, "no register-FFT variant for this N");
  }
}

}  // namespace exgb

namespace exgb {

// Launch of the register-FFT kernel on caller-provided scratch (no
// allocation): as many persistent clusters as `scratch_elems` float2 of
// stage buffers hold, at most the configured number.
template <int N, int THREADS>
static int v2_run_scratch(const exgb_plan* plan, cudaStream_t st, const float2* in, float2* out, int64_t batch,
                          int nsteps, int project, float2* scratch, size_t scratch_elems) {
  const Plan2DConfig& c = plan->cfg2d;
  const size_t fit = scratch_elems / c.scratch_per_cluster;
  if (fit < 1) return fail(EXGB_ENOMEM, "the static scratch array is smaller than one cluster's stage buffers");
  ArgsV2 a;
  a.P = plan->dev;
  a.G = c.G;
  a.Cl = c.cols_per_cta;
  a.Rl = c.rows_per_cta;
  a.Kc = std::min(plan->dev.kmax, N / 2 - 1) + 1;
  a.KcP = c.CB;
  a.Ul = (N / 2 + 1 - a.Kc + c.G - 1) / c.G;
  a.in = in;
  a.out = out;
  a.batch = batch;
  a.nsteps = nsteps;
  a.project = project;
  a.nonlinear_only = 0;
  a.scratch = scratch;
  a.scratch_stride = (int64_t)c.scratch_per_cluster;
  const int ncl = (int)std::min<int64_t>(std::min<int64_t>(c.clusters, (int64_t)fit), batch);
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = c.G;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(c.G * ncl, 1, 1);
  cfg.blockDim = dim3(THREADS, 1, 1);
  cfg.dynamicSmemBytes = c.smem_bytes;
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  EXGB_CUDA(cudaLaunchKernelEx(&cfg, vort2d_kernel<N, THREADS>, a));
  return EXGB_OK;
}

int vort2d_run_scratch(const exgb_plan* plan, cudaStream_t st, const float2* in, float2* out, int64_t batch,
                       int nsteps, int project, float2* scratch, size_t scratch_elems) {
  if (batch <= 0) return EXGB_OK;
  switch (plan->dev.N) {
    case 64: return v2_run_scratch<64, 256>(plan, st, in, out, batch, nsteps, project, scratch, scratch_elems);
    case 128: return v2_run_scratch<128, 512>(plan, st, in, out, batch, nsteps, project, scratch, scratch_elems);
    case 256: return v2_run_scratch<256, 512>(plan, st, in, out, batch, nsteps, project, scratch, scratch_elems);
    default: return fail(EXGB_EUNSUPPORTED, "no register-FFT variant for this N");
  }
}

}  // namespace exgb
