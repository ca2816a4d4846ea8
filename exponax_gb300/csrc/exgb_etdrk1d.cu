// exgb_etdrk1d.cu -- fused multi-step ETDRK0..4 for 1D pseudo-spectral
// problems, every state resident in shared memory for the whole rollout.
//
// One work item = m instances of one plan.  A CTA takes items from a device
// queue (atomicAdd on a head counter; no spin-waits anywhere), loads the m
// initial states (rfft), runs nsteps ETDRK steps and writes either the whole
// physical trajectory, the final physical state or the final Fourier state.
// Only the trajectory / final state touch HBM.
//
// Per nonlinear evaluation (reference: nonlin_fun/_convection.py:104-231,
// _gradient_norm.py:84-101, _polynomial.py:64-76, _general_nonlinear.py:111-119)
//   z = ifft(mask u^ + i mask ik u^)            one complex N-point FFT
//   p = u^2, q = beta u u_x + gamma (u_x^2 - zmf mean) + sum_k c_k u^k
//   Z = fft(p + i q)                             one complex N-point FFT
//   N^ = mask ( alpha ik P + Q )                 fused with the ETDRK stage update
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "exgb_internal.h"

namespace exgb {

void* workspace(size_t bytes, int slot_offset);
int irfftn_impl(cudaStream_t st, int D, int N, int64_t count, const float2* in, float* out);

enum : int {
  MODE_TRAJ = 0,      // physical in, trajectory out
  MODE_FINAL = 1,     // physical in, final physical state out
  MODE_FOURIER = 2,   // Fourier in, final Fourier state out
  MODE_NONLIN = 3,    // Fourier in, N(u^) out
  MODE_TRAJ_HAT = 4,  // physical in, trajectory of Fourier states out (one batched irfft afterwards)
};

struct Item1D {
  const PlanDev* plan;
  const void* in;   // float (physical) or float2 (Fourier), instance 0 of this item
  void* out;        // float or float2
  int m;            // instances
  int64_t in_stride, out_stride;  // elements (float or float2) between instances
};

__host__ __device__ inline int nbuf_for_order(int order) {
  return order <= 1 ? 1 : order == 2 ? 3 : order == 3 ? 4 : 6;
}

__device__ __forceinline__ float2 ldg2(const float2* p) { return __ldg(p); }

// Builds the packed inverse-transform input of the nonlinear evaluation
// for m instances from states X (stride M) into work (stride N).
__device__ void nl_pack(const PlanDev& P, const float2* X, int sx, float2* work, int m, int tid, int nthr) {
  const int N = P.N, M = P.M;
  const bool even = (N & 1) == 0;
  const float invN = 1.f / (float)N;
  for (int t = tid; t < m * N; t += nthr) {
    const int i = t / N, k = t - i * N;
    const bool ext = k >= M;
    const int kk = ext ? N - k : k;
    const bool ro = (k == 0) || (even && k == N / 2);
    float2 a = make_float2(0.f, 0.f), b = make_float2(0.f, 0.f);
    if (kk <= P.kmax) {
      a = X[i * sx + kk];
      if (P.needs_ux) {
        const float ks = P.kscale * (float)kk;  // ik u^ with k from rfftfreq
        b = make_float2(-ks * a.y, ks * a.x);
      }
    }
    work[t] = cscale(pack_pair(a, b, ext, ro), invN);
  }
}

// Pointwise products on the physical values z = u + i u_x (in place), with
// u_x^2 written to `sq` when the zero-mode fix needs its mean.
__device__ void nl_products(const PlanDev& P, float2* z, float* sq, int m, int tid, int nthr) {
  const int N = P.N;
  const bool zmf = P.gamma != 0.f && P.zero_mode_fix;
  for (int t = tid; t < m * N; t += nthr) {
    const float u = z[t].x, ux = z[t].y;
    float q = 0.f;
    if (P.beta != 0.f) q = fmaf(P.beta * u, ux, q);
    if (P.gamma != 0.f) q = fmaf(P.gamma * ux, ux, q);
    if (P.npoly > 0) {
      float pw = 1.f, acc = 0.f;
      for (int c = 0; c < P.npoly; ++c) {
        acc = fmaf(P.poly[c], pw, acc);
        pw *= u;
      }
      q += acc;
    }
    if (zmf) sq[t] = ux * ux;
    z[t] = make_float2(u * u, q);
  }
}

// Deterministic per-instance sums of sq (one warp per instance).
__device__ void nl_reduce(const float* sq, float* sums, int N, int m, int tid, int nthr) {
  const int warp = tid >> 5, lane = tid & 31, nw = nthr >> 5;
  for (int i = warp; i < m; i += nw) {
    float s = 0.f;
    for (int x = lane; x < N; x += 32) s += sq[i * N + x];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) sums[i] = s;
  }
}

struct Bufs {
  float2 *U, *S1, *S, *N0, *N1, *N2;
  float2 *w0, *w1;
  float* sums;
  const float2* tw;  // the item's twiddles: a shared-memory copy when it fits, else the plan's global table
};

// Stage epilogue: combine the fresh nonlinear value nv at mode k of instance
// i with the stored stages.  Reference stage formulas: etdrk/_etdrk_1.py:82,
// _etdrk_2.py:95-101, _etdrk_3.py:195-210, _etdrk_4.py:202-222.
__device__ __forceinline__ void stage_update(const PlanDev& P, const Bufs& b, int i, int k, int stage, float2 nv,
                                             int M, int ch_off) {
  const int o = i * M + k;
  const int c = ch_off + k;
  switch (P.order) {
    case 1: {
      const float2 E = ldg2(P.E + c);
      b.U[o] = cadd(cmul(E, b.U[o]), cscale(nv, __ldg(P.c[0] + c)));
    } break;
    case 2:
      if (stage == 0) {
        const float2 E = ldg2(P.E + c);
        b.N0[o] = nv;
        b.S[o] = cadd(cmul(E, b.U[o]), cscale(nv, __ldg(P.c[0] + c)));
      } else {
        b.U[o] = cadd(b.S[o], cscale(csub(nv, b.N0[o]), __ldg(P.c[1] + c)));
      }
      break;
    case 3:
      if (stage == 0) {
        b.N0[o] = nv;
        b.S[o] = cadd(cmul(ldg2(P.Eh + c), b.U[o]), cscale(nv, __ldg(P.c[0] + c)));
      } else if (stage == 1) {
        b.N1[o] = nv;
        const float2 t = csub(cscale(nv, 2.f), b.N0[o]);
        b.S[o] = cadd(cmul(ldg2(P.E + c), b.U[o]), cscale(t, __ldg(P.c[1] + c)));
      } else {
        float2 r = cmul(ldg2(P.E + c), b.U[o]);
        r = cadd(r, cscale(b.N0[o], __ldg(P.c[2] + c)));
        r = cadd(r, cscale(b.N1[o], __ldg(P.c[3] + c)));
        r = cadd(r, cscale(nv, __ldg(P.c[4] + c)));
        b.U[o] = r;
      }
      break;
    case 4:
      if (stage == 0) {
        b.N0[o] = nv;
        b.S1[o] = cadd(cmul(ldg2(P.Eh + c), b.U[o]), cscale(nv, __ldg(P.c[0] + c)));
      } else if (stage == 1) {
        b.N1[o] = nv;
        b.S[o] = cadd(cmul(ldg2(P.Eh + c), b.U[o]), cscale(nv, __ldg(P.c[0] + c)));
      } else if (stage == 2) {
        b.N2[o] = nv;
        const float2 t = csub(cscale(nv, 2.f), b.N0[o]);
        b.S[o] = cadd(cmul(ldg2(P.Eh + c), b.S1[o]), cscale(t, __ldg(P.c[0] + c)));
      } else {
        float2 r = cmul(ldg2(P.E + c), b.U[o]);
        r = cadd(r, cscale(b.N0[o], __ldg(P.c[3] + c)));
        r = cadd(r, cscale(cadd(b.N1[o], b.N2[o]), 2.f * __ldg(P.c[4] + c)));
        r = cadd(r, cscale(nv, __ldg(P.c[5] + c)));
        b.U[o] = r;
      }
      break;
    default:
      break;
  }
}

// The plan's device constants into shared memory, all threads copying 4-byte words.
__device__ __forceinline__ void copy_plan(PlanDev* dst, const PlanDev* __restrict__ src, int tid, int nthr) {
  static_assert(sizeof(PlanDev) % 4 == 0, "PlanDev is copied as 4-byte words");
  int* d = reinterpret_cast<int*>(dst);
  const int* s = reinterpret_cast<const int*>(src);
  for (int i = tid; i < (int)(sizeof(PlanDev) / 4); i += nthr) d[i] = s[i];
}

// First-pass source of the inverse transform of a nonlinear evaluation: element k of sequence i is
// what nl_pack would have stored (mask u^ + i mask ik u^, Hermitian extension, 1/N), computed from X.
struct PackSrc {
  const PlanDev* P;
  const float2* X;
  int sx;
  __device__ __forceinline__ float2 operator()(int i, int k) const {
    const int N = P->N, M = P->M;
    const bool ext = k >= M;
    const int kk = ext ? N - k : k;
    const bool ro = (k == 0) || ((N & 1) == 0 && k == N / 2);
    float2 a = make_float2(0.f, 0.f), b = make_float2(0.f, 0.f);
    if (kk <= P->kmax) {
      a = X[i * sx + kk];
      if (P->needs_ux) {
        const float ks = P->kscale * (float)kk;
        b = make_float2(-ks * a.y, ks * a.x);
      }
    }
    return cscale(pack_pair(a, b, ext, ro), P->rN);
  }
};

// Last-pass sink of that inverse transform: the physical value z = u + i u_x at x of sequence i
// becomes (u^2, q) as nl_products computes it, stored at res[i N + x].
struct ProductOut {
  const PlanDev* P;
  float2* res;
  struct Ref {
    const PlanDev* P;
    float2* p;
    __device__ __forceinline__ void operator=(float2 z) const {
      const float u = z.x, ux = z.y;
      float q = 0.f;
      if (P->beta != 0.f) q = fmaf(P->beta * u, ux, q);
      if (P->gamma != 0.f) q = fmaf(P->gamma * ux, ux, q);
      if (P->npoly > 0) {
        float pw = 1.f, acc = 0.f;
        for (int c = 0; c < P->npoly; ++c) {
          acc = fmaf(P->poly[c], pw, acc);
          pw *= u;
        }
        q += acc;
      }
      *p = make_float2(u * u, q);
    }
  };
  __device__ __forceinline__ Ref operator()(int i, int x) const { return Ref{P, res + i * P->N + x}; }
};

// ---- one-warp register transforms for the latency variant (one item per SM): N = A * B with
// A = A1 * A2 <= 32 and B = B1 * B2 <= A.  Lane l < A loads x[l + A j] (j < B), takes a length-B DFT
// in registers and the twiddle w_N^(l k1); a transpose through the output buffer (__syncwarp only);
// lane k1 < B then takes a length-A DFT over l in registers and writes X[k1 + B k2].  A whole
// transform is one barrier phase instead of one per radix pass.

// length R1 * R2 DFT in registers, in place: input x[n] in v[n], n = R2 n1 + n2; output X[k1 + R1 k2]
// in v[R2 k1 + k2].  The inner twiddles w_R^(n2 k1) = tw[tstep n2 k1] come from the N-point table
// (tstep = N / R).
template <int R1, int R2, bool INV>
__device__ __forceinline__ void lane_dft(float2 (&v)[R1 * R2], const float2* __restrict__ tw, int tstep) {
  if constexpr (R2 == 1) {
    dftR<R1, INV>(v);
  } else {
#pragma unroll
    for (int n2 = 0; n2 < R2; ++n2) {
      float2 t[R1];
#pragma unroll
      for (int n1 = 0; n1 < R1; ++n1) t[n1] = v[R2 * n1 + n2];
      dftR<R1, INV>(t);
#pragma unroll
      for (int k1 = 0; k1 < R1; ++k1) {
        float2 z = t[k1];
        if (n2 > 0 && k1 > 0) {
          float2 w = tw[tstep * n2 * k1];
          if (INV) w.y = -w.y;
          z = cmul(z, w);
        }
        v[R2 * k1 + n2] = z;
      }
    }
#pragma unroll
    for (int k1 = 0; k1 < R1; ++k1) {
      float2 t[R2];
#pragma unroll
      for (int n2 = 0; n2 < R2; ++n2) t[n2] = v[R2 * k1 + n2];
      dftR<R2, INV>(t);
#pragma unroll
      for (int k2 = 0; k2 < R2; ++k2) v[R2 * k1 + k2] = t[k2];
    }
  }
}

// One length-N transform by one warp, in -> out (in == out allowed); `out` also holds the transpose
// tile (N = A * B entries, row k1 rotated by k1 against bank conflicts).  No 1/N scaling.
template <int A1, int A2, int B1, int B2, bool INV>
__device__ __forceinline__ void warp_fft(const float2* in, float2* out, const float2* __restrict__ tw, int lane) {
  constexpr int A = A1 * A2, B = B1 * B2, N = A * B;
  static_assert(A <= 32 && B <= 32 && B <= A, "one warp, B <= A");
  float2 v[B];  // after the first DFT: X[q1 + B1 q2] in v[B2 q1 + q2]
  if (lane < A) {
#pragma unroll
    for (int j = 0; j < B; ++j) v[j] = in[lane + A * j];
    lane_dft<B1, B2, INV>(v, tw, N / B);
#pragma unroll
    for (int q1 = 0; q1 < B1; ++q1)
#pragma unroll
      for (int q2 = 0; q2 < B2; ++q2) {
        const int k1 = q1 + B1 * q2;
        if (k1 > 0) {
          float2 w = tw[lane * k1];
          if (INV) w.y = -w.y;
          v[B2 * q1 + q2] = cmul(v[B2 * q1 + q2], w);
        }
      }
  }
  __syncwarp();
  if (lane < A) {
#pragma unroll
    for (int q1 = 0; q1 < B1; ++q1)
#pragma unroll
      for (int q2 = 0; q2 < B2; ++q2) {
        const int k1 = q1 + B1 * q2;
        const int c = lane + k1;
        out[k1 * A + (c < A ? c : c - A)] = v[B2 * q1 + q2];
      }
  }
  __syncwarp();
  float2 u[A];
  if (lane < B) {
#pragma unroll
    for (int l = 0; l < A; ++l) {
      const int c = l + lane;
      u[l] = out[lane * A + (c < A ? c : c - A)];
    }
  }
  __syncwarp();
  if (lane < B) {
    lane_dft<A1, A2, INV>(u, tw, N / A);
#pragma unroll
    for (int q1 = 0; q1 < A1; ++q1)
#pragma unroll
      for (int q2 = 0; q2 < A2; ++q2) out[lane + B * (q1 + A1 * q2)] = u[A2 * q1 + q2];
  }
}

// Sizes with a one-warp transform (WN = N = A1 * A2 * B1 * B2); WN = 0: block Stockham passes.  Each size is
// a kernel instantiation of its own: one function holding several transforms' registers spills.
template <int WN>
struct WarpShape;
template <>
struct WarpShape<64> {
  static constexpr int A1 = 8, A2 = 1, B1 = 8, B2 = 1;
};
template <>
struct WarpShape<128> {
  static constexpr int A1 = 4, A2 = 4, B1 = 8, B2 = 1;
};
template <>
struct WarpShape<200> {  // 20 lanes x 10 points, then 10 lanes x 20 points
  static constexpr int A1 = 4, A2 = 5, B1 = 2, B2 = 5;
};
template <>
struct WarpShape<256> {  // 16 lanes x 16 points, twice
  static constexpr int A1 = 4, A2 = 4, B1 = 4, B2 = 4;
};

// m length-WN transforms in -> out (stride WN), one warp per sequence
template <int WN, bool INV>
__device__ __forceinline__ void warp_fft_many(const float2* in, float2* out, int m, const float2* __restrict__ tw,
                                              int tid, int nthr) {
  using S = WarpShape<WN>;
  const int lane = tid & 31;
  for (int i = tid >> 5; i < m; i += nthr >> 5) {
    warp_fft<S::A1, S::A2, S::B1, S::B2, INV>(in + (size_t)i * WN, out + (size_t)i * WN, tw, lane);
    __syncwarp();
  }
}

// One nonlinear evaluation of the m states X followed by the stage update
// (stage >= 0) or a plain store of N^ into X_out (stage < 0).
// fuse: pack fused into the first inverse pass and the products into the last (fewer barrier phases;
// the throughput choice when several work items share an SM).  Otherwise each elementwise step is a
// phase of its own spread over all threads (the latency choice for one small item per SM).
// WN != 0 (latency variant only, N == WN): each transform is one warp_fft phase.
template <bool fuse, int WN = 0, class Sync = BlockSync>
__device__ void nl_eval(const PlanDev& P, const Bufs& b, const float2* X, int m, int stage, float2* X_out,
                        int tid, int nthr, const Sync& sync = Sync{}) {
  static_assert(WN == 0 || !fuse, "warp transforms belong to the latency variant");
  const int N = P.N, M = P.M;
  const bool zmf = P.gamma != 0.f && P.zero_mode_fix;
  float2 *res, *other;
  if (fuse && !zmf) {  // compile-time fuse: each kernel carries one of the two paths
    res = io_result_buf(P.fft, b.w0, b.w1);
    other = (res == b.w0) ? b.w1 : b.w0;
    block_fft_io<true>(P.fft, PackSrc{&P, X, M}, b.w0, b.w1, ProductOut{&P, res}, m, b.tw, tid, nthr, sync);
  } else {
    // separate pack and product phases (the zero-mode fix also needs u_x^2 in a buffer of its own)
    nl_pack(P, X, M, b.w0, m, tid, nthr);
    sync();
    res = (P.fft.npass & 1) ? b.w1 : b.w0;
    other = (P.fft.npass & 1) ? b.w0 : b.w1;
    if constexpr (WN != 0) {
      warp_fft_many<WN, true>(b.w0, res, m, b.tw, tid, nthr);
      sync();
    } else {
      block_fft<true>(P.fft, b.w0, b.w1, LinMap{res, N}, m, b.tw, tid, nthr, sync);
    }
    nl_products(P, res, (float*)other, m, tid, nthr);
    sync();
    if (zmf) {
      nl_reduce((const float*)other, b.sums, N, m, tid, nthr);
      sync();
    }
  }
  // forward: input in res, passes ping-pong other <-> res
  float2* fres;
  if constexpr (WN != 0) {
    fres = res;
    warp_fft_many<WN, false>(res, fres, m, b.tw, tid, nthr);
    sync();
  } else {
    fres = io_result_buf(P.fft, other, res);
    block_fft_io<false>(P.fft, LinMap{res, N}, other, res, LinMap{fres, N}, m, b.tw, tid, nthr, sync);
  }
  for (int t = tid; t < m * M; t += nthr) {
    const int i = t / M, k = t - i * M;
    float2 nv = make_float2(0.f, 0.f);
    if (k <= P.kmax) {
      float2 Pk, Qk;
      unpack_pair(fres[i * N + k], fres[i * N + (k == 0 ? 0 : N - k)], Pk, Qk);
      if (P.needs_q) nv = Qk;
      if (P.alpha != 0.f) {
        const float ks = P.kscale * (float)k;
        // alpha * (i ks) * P
        nv = cadd(nv, make_float2(-P.alpha * ks * Pk.y, P.alpha * ks * Pk.x));
      }
      if (zmf && k == 0) nv.x -= P.gamma * b.sums[i];
    }
    if (stage < 0) X_out[t] = nv;
    else stage_update(P, b, i, k, stage, nv, M, 0);
  }
  sync();
}

// First-pass source of the trajectory output: instances 2p and 2p+1 packed as one complex sequence.
struct EmitSrc {
  const PlanDev* P;
  const float2* U;
  int m;
  __device__ __forceinline__ float2 operator()(int p, int k) const {
    const int N = P->N, M = P->M;
    const bool ext = k >= M;
    const int kk = ext ? N - k : k;
    const bool ro = (k == 0) || ((N & 1) == 0 && k == N / 2);
    const int ia = 2 * p, ib = 2 * p + 1;
    const float2 a = U[ia * M + kk];
    const float2 bb = ib < m ? U[ib * M + kk] : make_float2(0.f, 0.f);
    return cscale(pack_pair(a, bb, ext, ro), P->rN);
  }
};

// Last-pass sink of the trajectory output: the real and imaginary parts are the two instances' values.
struct EmitOut {
  float* out;
  int64_t stride;
  int m;
  struct Ref {
    float* a;
    float* b;
    __device__ __forceinline__ void operator=(float2 z) const {
      *a = z.x;
      if (b) *b = z.y;
    }
  };
  __device__ __forceinline__ Ref operator()(int p, int x) const {
    float* a = out + (int64_t)(2 * p) * stride + x;
    return Ref{a, (2 * p + 1 < m) ? a + stride : nullptr};
  }
};

// Physical output of m states (pairs packed in one complex FFT); with `fuse` the pack is the first
// pass's source and the global stores the last pass's sink, else each is a phase of its own.
template <bool fuse, class Sync = BlockSync>
__device__ void emit_phys(const PlanDev& P, const Bufs& b, int m, float* out, int64_t inst_stride, int tid,
                          int nthr, const Sync& sync = Sync{}) {
  const int pairs = (m + 1) / 2;
  if constexpr (fuse) {
    block_fft_io<true>(P.fft, EmitSrc{&P, b.U, m}, b.w0, b.w1, EmitOut{out, inst_stride, m}, pairs, b.tw, tid,
                       nthr, sync);
    return;
  }
  const int N = P.N;
  const EmitSrc src{&P, b.U, m};
  for (int t = tid; t < pairs * N; t += nthr) {
    const int p = t / N, k = t - p * N;
    b.w0[t] = src(p, k);
  }
  sync();
  float2* res = (P.fft.npass & 1) ? b.w1 : b.w0;
  block_fft<true>(P.fft, b.w0, b.w1, LinMap{res, N}, pairs, b.tw, tid, nthr, sync);
  for (int t = tid; t < pairs * N; t += nthr) {
    const int p = t / N, x = t - p * N;
    const float2 z = res[t];
    out[(int64_t)(2 * p) * inst_stride + x] = z.x;
    if (2 * p + 1 < m) out[(int64_t)(2 * p + 1) * inst_stride + x] = z.y;
  }
  sync();
}

// One work item (m instances of one plan) through all its steps, by the threads tid < nthr of a group
// that synchronises with `sync` (the whole block).  `sm`: the
// group's dynamic shared memory of smem_bytes; `gslot`: its global slot for state buffers that do not
// fit there (NULL when they always fit).
template <bool FUSE, int WN, class Sync>
__device__ void run_item(const Item1D& item, const PlanDev& P, float2* sm, int smem_bytes, float* sums,
                         float2* gslot, int nsteps, int mode, int project, int include_init, int tid, int nthr,
                         const Sync& sync) {
  const int N = P.N, M = P.M, m = item.m;
  // carve shared memory: the ETDRK state buffers and the two work buffers when the item fits in the
  // launch's reservation; otherwise the state buffers live in this CTA's global slot (L2-resident)
  // and only the work buffers in shared memory (the work queue reserves what keeps 3 CTAs per SM)
  Bufs b;
  const size_t state_elems = (size_t)nbuf_for_order(P.order) * m * M, work_elems = 2 * (size_t)m * N;
  const bool local = (state_elems + work_elems) * sizeof(float2) <= (size_t)smem_bytes;
  float2* q = local ? sm : gslot;
  b.U = q;
  q += m * M;
  b.S1 = b.S = b.N0 = b.N1 = b.N2 = nullptr;
  if (P.order == 2) {
    b.S = q; q += m * M;
    b.N0 = q; q += m * M;
  } else if (P.order == 3) {
    b.S = q; q += m * M;
    b.N0 = q; q += m * M;
    b.N1 = q; q += m * M;
  } else if (P.order == 4) {
    b.S1 = q; q += m * M;
    b.S = q; q += m * M;
    b.N0 = q; q += m * M;
    b.N1 = q; q += m * M;
    b.N2 = q; q += m * M;
  }
  if (!local) q = sm;
  b.w0 = q;
  q += m * N;
  b.w1 = q;
  q += m * N;
  b.sums = sums;
  // the twiddles go into the dynamic shared memory left over by this item (the launch reserves the
  // largest item's footprint, or room for them); the copy is complete at the barrier below
  if ((size_t)(q - sm + N) * sizeof(float2) <= (size_t)smem_bytes) {
    for (int i = tid; i < N; i += nthr) q[i] = __ldg(P.tw + i);
    b.tw = q;
  } else {
    b.tw = P.tw;
  }

  // ---- load initial state
  if (mode == MODE_TRAJ || mode == MODE_FINAL || mode == MODE_TRAJ_HAT) {
    const float* u0 = (const float*)item.in;
    const int pairs = (m + 1) / 2;
    for (int t = tid; t < pairs * N; t += nthr) {
      const int p = t / N, x = t - p * N;
      const float a = u0[(int64_t)(2 * p) * item.in_stride + x];
      const float bb = (2 * p + 1 < m) ? u0[(int64_t)(2 * p + 1) * item.in_stride + x] : 0.f;
      b.w0[t] = make_float2(a, bb);
      if (mode == MODE_TRAJ && include_init) {
        float* o = (float*)item.out;
        o[(int64_t)(2 * p) * item.out_stride + x] = a;
        if (2 * p + 1 < m) o[(int64_t)(2 * p + 1) * item.out_stride + x] = bb;
      }
    }
    sync();
    float2* res = (P.fft.npass & 1) ? b.w1 : b.w0;
    block_fft<false>(P.fft, b.w0, b.w1, LinMap{res, N}, pairs, b.tw, tid, nthr, sync);
    for (int t = tid; t < pairs * M; t += nthr) {
      const int p = t / M, k = t - p * M;
      float2 A, B;
      unpack_pair(res[p * N + k], res[p * N + (k == 0 ? 0 : N - k)], A, B);
      b.U[(2 * p) * M + k] = A;
      if (2 * p + 1 < m) b.U[(2 * p + 1) * M + k] = B;
    }
  } else {
    const float2* uh = (const float2*)item.in;
    for (int t = tid; t < m * M; t += nthr) {
      const int i = t / M, k = t - i * M;
      b.U[t] = uh[(int64_t)i * item.in_stride + k];
    }
  }
  sync();

  if (mode == MODE_TRAJ_HAT && include_init) {  // frame 0 (overwritten by the exact input afterwards)
    float2* o = (float2*)item.out;
    for (int t = tid; t < m * M; t += nthr) {
      const int i = t / M, k = t - i * M;
      o[(int64_t)i * item.out_stride + k] = b.U[t];
    }
  }

  // ---- time steps
  const int nstages = (P.order == 0 || P.kind == EXGB_NL_ZERO) ? 0 : P.order;
  for (int step = 0; step < nsteps; ++step) {
    if (nstages == 0) {
      for (int t = tid; t < m * M; t += nthr) {
        const int k = t % M;
        b.U[t] = cmul(ldg2(P.E + k), b.U[t]);
      }
      sync();
    } else {
      for (int s = 0; s < nstages; ++s) {
        const float2* X = (s == 0) ? b.U : (P.order == 4 && s == 1) ? b.S1 : b.S;
        nl_eval<FUSE, WN>(P, b, X, m, s, nullptr, tid, nthr, sync);
      }
    }
    if (project) {
      // c2r of the step's physical round trip drops Im at DC and Nyquist
      for (int i = tid; i < m; i += nthr) {
        b.U[i * M].y = 0.f;
        if ((N & 1) == 0) b.U[i * M + N / 2].y = 0.f;
      }
      sync();
    }
    if (mode == MODE_TRAJ) {
      float* o = (float*)item.out + (int64_t)(step + include_init) * N;
      emit_phys<FUSE>(P, b, m, o, item.out_stride, tid, nthr, sync);
    } else if (mode == MODE_TRAJ_HAT) {
      // the step's Fourier state; the batched inverse transform after the launch makes it physical
      float2* o = (float2*)item.out + (int64_t)(step + include_init) * M;
      for (int t = tid; t < m * M; t += nthr) {
        const int i = t / M, k = t - i * M;
        o[(int64_t)i * item.out_stride + k] = b.U[t];
      }
    }
  }

  // ---- final store
  if (mode == MODE_FINAL) {
    emit_phys<FUSE>(P, b, m, (float*)item.out, item.out_stride, tid, nthr, sync);
  } else if (mode == MODE_FOURIER) {
    float2* o = (float2*)item.out;
    for (int t = tid; t < m * M; t += nthr) {
      const int i = t / M, k = t - i * M;
      o[(int64_t)i * item.out_stride + k] = b.U[t];
    }
  }
}

// FUSE: the throughput variant (more items than SMs, 3 CTAs per SM); otherwise one CTA per SM, whose
// transforms are warp transforms when WN = N, block passes when WN = 0
template <bool FUSE, int WN>
__global__ void __launch_bounds__(256, FUSE ? 3 : 1) etdrk1d_kernel(const Item1D* __restrict__ items, int n_items,
                                                      int* __restrict__ head, int nsteps, int mode, int project,
                                                      int include_init, int smem_bytes, float2* gstate,
                                                      int64_t gstate_stride) {
  extern __shared__ __align__(16) float2 sm[];
  __shared__ PlanDev Ps;
  __shared__ int s_item;
  __shared__ float s_sums[64];
  const int tid = threadIdx.x, nthr = blockDim.x;
  for (;;) {
    if (tid == 0) s_item = atomicAdd(head, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= n_items) break;
    const Item1D item = items[it];
    copy_plan(&Ps, item.plan, tid, nthr);
    __syncthreads();
    run_item<FUSE, WN>(item, Ps, sm, smem_bytes, s_sums, gstate ? gstate + (int64_t)blockIdx.x * gstate_stride : nullptr,
                   nsteps, mode, project, include_init, tid, nthr, BlockSync{});
    __syncthreads();
  }
}

// Nonlinear-function-only kernel (exgb_nonlinear): one item, N^ written to out.
__global__ void __launch_bounds__(256) nonlin1d_kernel(const Item1D* __restrict__ items, int n_items) {
  extern __shared__ __align__(16) float2 sm[];
  __shared__ PlanDev Ps;
  __shared__ float s_sums[64];
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int it = blockIdx.x;
  if (it >= n_items) return;
  const Item1D item = items[it];
  copy_plan(&Ps, item.plan, tid, nthr);
  __syncthreads();
  const PlanDev& P = Ps;
  const int N = P.N, M = P.M, m = item.m;
  Bufs b{};
  b.U = sm;
  b.w0 = sm + m * M;
  b.w1 = b.w0 + m * N;
  b.sums = s_sums;
  b.tw = P.tw;
  const float2* uh = (const float2*)item.in;
  for (int t = tid; t < m * M; t += nthr) {
    const int i = t / M, k = t - i * M;
    b.U[t] = uh[(int64_t)i * item.in_stride + k];
  }
  __syncthreads();
  // results go back into U (the pack step has consumed it before the epilogue)
  nl_eval<false>(P, b, b.U, m, -1, b.U, tid, nthr);
  float2* o = (float2*)item.out;
  for (int t = tid; t < m * M; t += nthr) {
    const int i = t / M, k = t - i * M;
    o[(int64_t)i * item.out_stride + k] = b.U[t];
  }
}

// Shared memory a 1D CTA reserves when that keeps 3 CTAs of 256 threads per SM; items whose full
// footprint is larger keep their ETDRK state buffers in a per-CTA global slot (see etdrk1d_kernel).
constexpr size_t kQueueSmemCap = 72 * 1024;

static size_t smem_for(const PlanDev& P, int m, bool nonlin_only) {
  const int nb = nonlin_only ? 1 : nbuf_for_order(P.order);
  return sizeof(float2) * (size_t)m * ((size_t)nb * P.M + 2 * (size_t)P.N);
}

static int smem_limit() {
  static int lim = 0;
  if (!lim) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&lim, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  }
  return lim;
}

bool etdrk1d_fits(int N, int order) {
  PlanDev P{};
  P.N = N;
  P.M = N / 2 + 1;
  P.order = order;
  const size_t lim = (size_t)smem_limit() - 4096;
  const size_t work = sizeof(float2) * 2 * (size_t)N;
  return smem_for(P, 1, true) <= lim && (smem_for(P, 1, false) <= lim || work <= kQueueSmemCap);
}

// Items for `batch` instances of one plan, m instances per item.
static int choose_m(const PlanDev& P, int64_t batch, int sm_count, bool nonlin_only) {
  int m = std::max(1, 2048 / P.N);  // instances per item up to m N = 2048 (as the work queue)
  // spread small batches over the SMs first
  const int64_t per_sm = (batch + 2 * sm_count - 1) / (2 * (int64_t)sm_count);
  m = (int)std::max<int64_t>(1, std::min<int64_t>(m, per_sm));
  m = std::min(m, 64);
  while (m > 1 && smem_for(P, m, nonlin_only) > (size_t)smem_limit() - 4096) --m;
  return m;
}

using Kern1D = void (*)(const Item1D*, int, int*, int, int, int, int, int, float2*, int64_t);

// The kernel of a launch: the fused variant when there are more work items than SMs (throughput-
// bound, the fused elementwise steps pay); otherwise each SM runs one item at latency with separate
// all-thread elementwise phases, and with one-warp transforms when every item's N (n_uniform; 0 if
// the items differ) has one (one CTA of 256 threads, 3.79 -> 2.12 ms for 16 instances of N = 200 x
// 500 ETDRK2 steps).
static Kern1D kernel_1d(bool fuse, int n_uniform) {
  if (fuse) return etdrk1d_kernel<true, 0>;
  switch (n_uniform) {
    case 64: return etdrk1d_kernel<false, 64>;
    case 128: return etdrk1d_kernel<false, 128>;
    case 200: return etdrk1d_kernel<false, 200>;
    case 256: return etdrk1d_kernel<false, 256>;
    default: return etdrk1d_kernel<false, 0>;
  }
}

static int launch_items(const std::vector<Item1D>& items, size_t smem, cudaStream_t st, int nsteps, int mode,
                        int project, int include_init, int sm_count, bool nonlin_only, int n_uniform,
                        int threads = 256, size_t gstate_bytes = 0) {
  if (items.empty()) return EXGB_OK;
  {
    // the item list below is copied from host memory that is gone when a captured graph replays
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone)
      return fail(EXGB_EUNSUPPORTED,
                  "1D stepping through the per-call entry points cannot be captured in a CUDA graph (its work list "
                  "is copied from host memory); capture exgb_queue_launch of an exgb_queue_prepare'd queue instead");
  }
  if (smem > (size_t)smem_limit() - 2048)
    return fail(EXGB_EUNSUPPORTED, "1D state does not fit in shared memory (N too large for this build)");
  // items + queue head in one workspace region (slot 2+: keep the transform slots free)
  const size_t ib = sizeof(Item1D) * items.size();
  const size_t total = ib + 256;
  // workspace slot 1 may be shared with transforms issued earlier on the
  // same stream; stream order keeps that safe.
  char* ws = (char*)workspace(total, 1);
  if (!ws) return fail(EXGB_ENOMEM, "workspace allocation failed");
  int* head = (int*)(ws + ((ib + 127) / 128) * 128);
  EXGB_CUDA(cudaMemcpyAsync(ws, items.data(), ib, cudaMemcpyHostToDevice, st));
  EXGB_CUDA(cudaMemsetAsync(head, 0, sizeof(int), st));
  if (nonlin_only) {
    EXGB_CUDA(cudaFuncSetAttribute(nonlin1d_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    nonlin1d_kernel<<<(unsigned)items.size(), 256, smem, st>>>((const Item1D*)ws, (int)items.size());
  } else {
    const Kern1D kern = kernel_1d((int64_t)items.size() > (int64_t)sm_count, n_uniform);
    EXGB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 1;
    EXGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem));
    per_sm = std::max(1, per_sm);
    const int grid = (int)std::min<int64_t>((int64_t)items.size(), (int64_t)sm_count * per_sm);
    float2* gstate = nullptr;
    if (gstate_bytes) {
      gstate = (float2*)workspace(gstate_bytes * (size_t)grid, 6);
      if (!gstate) return fail(EXGB_ENOMEM, "workspace allocation failed");
    }
    kern<<<grid, threads, smem, st>>>((const Item1D*)ws, (int)items.size(), head, nsteps, mode, project,
                                      include_init, (int)smem, gstate, (int64_t)(gstate_bytes / sizeof(float2)));
  }
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

int etdrk1d_run(const exgb_plan* plan, cudaStream_t st, const float* u0_phys, const float2* u0_hat, float* out_phys,
                float2* out_hat, int64_t batch, int nsteps, int project, int emit_traj, int include_init,
                int nonlinear_only) {
  const PlanDev& P = plan->dev;
  if (batch <= 0) return EXGB_OK;
  int mode;
  if (nonlinear_only) mode = MODE_NONLIN;
  else if (u0_phys) mode = emit_traj ? MODE_TRAJ : MODE_FINAL;
  else mode = MODE_FOURIER;
  int m = choose_m(P, batch, plan->sm_count, nonlinear_only);
  if (plan->tune_items_per_cta > 0 && !nonlinear_only) {
    m = plan->tune_items_per_cta;
    while (m > 1 && smem_for(P, m, false) > (size_t)smem_limit() - 4096) --m;
  }
  const int T = nsteps + (include_init ? 1 : 0);
  // A trajectory with at most one item per SM (latency-bound: each SM steps one item) is written as
  // Fourier states and made physical by one batched inverse transform over all SMs afterwards, which
  // takes the per-step output transform off the items' critical path.
  float2* htraj = nullptr;
  if (mode == MODE_TRAJ && (batch + m - 1) / m <= (int64_t)plan->sm_count && T > 0) {
    htraj = (float2*)workspace(sizeof(float2) * (size_t)batch * T * P.M, 3);
    if (!htraj) return fail(EXGB_ENOMEM, "workspace allocation failed");
    mode = MODE_TRAJ_HAT;
  }
  std::vector<Item1D> items;
  for (int64_t b0 = 0; b0 < batch; b0 += m) {
    Item1D it{};
    it.plan = plan->d_dev;
    it.m = (int)std::min<int64_t>(m, batch - b0);
    if (mode == MODE_TRAJ || mode == MODE_FINAL || mode == MODE_TRAJ_HAT) {
      it.in = u0_phys + b0 * P.N;
      it.in_stride = P.N;
    } else {
      it.in = u0_hat + b0 * P.M;
      it.in_stride = P.M;
    }
    if (mode == MODE_TRAJ) {
      it.out = out_phys + b0 * (int64_t)T * P.N;
      it.out_stride = (int64_t)T * P.N;
    } else if (mode == MODE_TRAJ_HAT) {
      it.out = htraj + b0 * (int64_t)T * P.M;
      it.out_stride = (int64_t)T * P.M;
    } else if (mode == MODE_FINAL) {
      it.out = out_phys + b0 * P.N;
      it.out_stride = P.N;
    } else {
      it.out = out_hat + b0 * P.M;
      it.out_stride = P.M;
    }
    items.push_back(it);
  }
  // 256 unless tuned: fewer threads measured slower for small latency-bound items (N = 200, one
  // instance per CTA) and the autotuner picks 128 where it wins
  const int threads = plan->tune_threads_1d > 0 ? plan->tune_threads_1d : 256;
  // shared memory: as the work queue, at most kQueueSmemCap per CTA (3 CTAs per SM) when the items'
  // work buffers fit in it -- the state buffers then go to per-CTA global slots -- plus a copy of the
  // twiddles when that still fits
  size_t smem = smem_for(P, m, nonlinear_only), gstate_bytes = 0;
  if (!nonlinear_only) {
    const size_t work = sizeof(float2) * 2 * (size_t)m * P.N, tw = sizeof(float2) * (size_t)P.N;
    if (smem > kQueueSmemCap && work <= kQueueSmemCap) {
      gstate_bytes = smem - work;
      smem = work;
    }
    if (smem + tw <= kQueueSmemCap) smem += tw;
  }
  const int rc = launch_items(items, smem, st, nsteps, mode, project, include_init, plan->sm_count, nonlinear_only,
                              P.N, threads, gstate_bytes);
  if (rc || mode != MODE_TRAJ_HAT) return rc;
  const int rc2 = irfftn_impl(st, 1, P.N, batch * T, htraj, out_phys);
  if (rc2) return rc2;
  if (include_init)  // the initial frame is the input itself, not its round trip
    EXGB_CUDA(cudaMemcpy2DAsync(out_phys, sizeof(float) * (size_t)T * P.N, u0_phys, sizeof(float) * P.N,
                                sizeof(float) * P.N, (size_t)batch, cudaMemcpyDeviceToDevice, st));
  return EXGB_OK;
}

}  // namespace exgb

using namespace exgb;

namespace exgb {

// Groups consecutive instances of the same plan with evenly strided buffers
// into items of up to m instances and sorts the items longest first.
static int build_queue(const exgb_work_item* items, int64_t n_items, int nsteps, int include_init,
                       std::vector<Item1D>& sorted, size_t& smem, int& sm_count, size_t& gstate_bytes,
                       int& n_uniform) {
  if (n_items < 0 || (n_items > 0 && !items)) return fail(EXGB_EINVAL, "bad work item list");
  if (nsteps < 0) return fail(EXGB_EINVAL, "nsteps must be >= 0");
  const int T = nsteps + (include_init ? 1 : 0);
  std::vector<Item1D> its;
  std::vector<double> cost;
  smem = 0;
  gstate_bytes = 0;
  size_t full_max = 0;
  sm_count = 0;
  n_uniform = -1;
  for (int64_t i = 0; i < n_items;) {
    const exgb_plan* p = items[i].plan;
    if (!p || !items[i].u0 || !items[i].traj) return fail(EXGB_EINVAL, "work item with NULL plan or buffer");
    if (p->dev.D != 1 || p->staged || p->dev.fft.n == 0 || !etdrk1d_fits(p->dev.N, p->dev.order))
      return fail(EXGB_EUNSUPPORTED,
                  "the work queue runs 1D single-channel plans of N = 2^a 3^b 5^c that fit in one CTA");
    sm_count = p->sm_count;
    const int N = p->dev.N;
    n_uniform = (n_uniform == -1 || n_uniform == N) ? N : 0;
    const int mmax = std::min(64, std::max(1, 2048 / N));  // 2048 / N measured best (1024: -8 %, 4096: -22 %)
    int m = 1;
    while (m < mmax && i + m < n_items && items[i + m].plan == p &&
           items[i + m].u0 == items[i].u0 + (int64_t)m * N && items[i + m].traj == items[i].traj + (int64_t)m * T * N)
      ++m;
    Item1D it{};
    it.plan = p->d_dev;
    it.in = items[i].u0;
    it.in_stride = N;
    it.out = items[i].traj;
    it.out_stride = (int64_t)T * N;
    it.m = m;
    its.push_back(it);
    const double lg = std::log2((double)N);
    cost.push_back((double)m * N * lg * (p->dev.order + 1));
    full_max = std::max(full_max, smem_for(p->dev, m, false));
    const size_t full = smem_for(p->dev, m, false), work = sizeof(float2) * 2 * (size_t)m * N;
    if (full <= kQueueSmemCap) {
      smem = std::max(smem, full);
    } else {
      smem = std::max(smem, work);
      gstate_bytes = std::max(gstate_bytes, full - work);
    }
    i += m;
  }
  if (smem > kQueueSmemCap) {  // some item's work buffers alone exceed the cap: reserve full footprints
    smem = full_max;
    gstate_bytes = 0;
  }
  std::vector<size_t> idx(its.size());
  for (size_t k = 0; k < idx.size(); ++k) idx[k] = k;
  std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return cost[a] > cost[b]; });
  sorted.clear();
  sorted.reserve(its.size());
  for (size_t k : idx) sorted.push_back(its[k]);
  if (smem > (size_t)smem_limit() - 2048)
    return fail(EXGB_EUNSUPPORTED, "1D state does not fit in shared memory (N too large for this build)");
  return EXGB_OK;
}

}  // namespace exgb

struct exgb_queue {
  exgb::Item1D* d_items = nullptr;
  int* d_head = nullptr;
  int n_items = 0;
  size_t smem = 0;
  float2* d_gstate = nullptr;  // per-CTA global slots for the state buffers of the largest items
  size_t gstate_bytes = 0;     // per CTA
  int grid = 1;
  int sm_count = 1;
  int nsteps = 0;
  int include_init = 0;
  int n_uniform = 0;  // every item's N, or 0 if they differ (kernel_1d)
};

extern "C" int exgb_queue_rollout(const exgb_work_item* items, int64_t n_items, int32_t nsteps,
                                  int32_t include_init, void* stream) {
  if (n_items == 0) return EXGB_OK;
  std::vector<Item1D> sorted;
  size_t smem = 0, gstate_bytes = 0;
  int sm_count = 0, n_uniform = 0;
  const int rc = build_queue(items, n_items, nsteps, include_init, sorted, smem, sm_count, gstate_bytes, n_uniform);
  if (rc) return rc;
  return launch_items(sorted, smem, (cudaStream_t)stream, nsteps, MODE_TRAJ, 1, include_init, sm_count, false,
                      n_uniform, 256, gstate_bytes);
}

extern "C" int exgb_queue_prepare(const exgb_work_item* items, int64_t n_items, int32_t nsteps, int32_t include_init,
                                  exgb_queue** out) {
  if (!out) return fail(EXGB_EINVAL, "NULL argument");
  *out = nullptr;
  if (n_items < 1) return fail(EXGB_EINVAL, "empty work item list");
  std::vector<Item1D> sorted;
  size_t smem = 0, gstate_bytes = 0;
  int sm_count = 0, n_uniform = 0;
  int rc = build_queue(items, n_items, nsteps, include_init, sorted, smem, sm_count, gstate_bytes, n_uniform);
  if (rc) return rc;
  exgb_queue* q = new exgb_queue();
  q->n_items = (int)sorted.size();
  q->smem = smem;
  q->gstate_bytes = gstate_bytes;
  q->nsteps = nsteps;
  q->include_init = include_init ? 1 : 0;
  q->sm_count = sm_count;
  q->n_uniform = n_uniform;
  const Kern1D kern = kernel_1d(q->n_items > q->sm_count, q->n_uniform);
  cudaError_t e;
  if ((e = cudaMalloc(&q->d_items, sizeof(Item1D) * sorted.size())) != cudaSuccess ||
      (e = cudaMalloc(&q->d_head, sizeof(int))) != cudaSuccess ||
      (e = cudaMemcpy(q->d_items, sorted.data(), sizeof(Item1D) * sorted.size(), cudaMemcpyHostToDevice)) !=
          cudaSuccess ||
      (e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess) {
    exgb_queue_destroy(q);
    return cuda_fail(e, "exgb_queue_prepare");
  }
  int per_sm = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, smem) != cudaSuccess) per_sm = 1;
  q->grid = (int)std::min<int64_t>((int64_t)sorted.size(), (int64_t)sm_count * std::max(1, per_sm));
  if (gstate_bytes && (e = cudaMalloc(&q->d_gstate, gstate_bytes * (size_t)q->grid)) != cudaSuccess) {
    exgb_queue_destroy(q);
    return cuda_fail(e, "exgb_queue_prepare");
  }
  *out = q;
  return EXGB_OK;
}

extern "C" int exgb_queue_launch(exgb_queue* q, void* stream) {
  if (!q) return fail(EXGB_EINVAL, "NULL queue");
  cudaStream_t st = (cudaStream_t)stream;
  EXGB_CUDA(cudaMemsetAsync(q->d_head, 0, sizeof(int), st));
  const Kern1D kern = kernel_1d(q->n_items > q->sm_count, q->n_uniform);
  kern<<<q->grid, 256, q->smem, st>>>(q->d_items, q->n_items, q->d_head, q->nsteps, MODE_TRAJ, 1, q->include_init,
                                      (int)q->smem, q->d_gstate, (int64_t)(q->gstate_bytes / sizeof(float2)));
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

extern "C" int exgb_queue_destroy(exgb_queue* q) {
  if (!q) return EXGB_OK;
  cudaFree(q->d_items);
  cudaFree(q->d_head);
  cudaFree(q->d_gstate);
  delete q;
  return EXGB_OK;
}
