// exgb_stage.cuh -- ETDRK1..4 stage combinations of one Fourier mode, shared
// by the fused 2D kernels and the staged N-D path.  Reference: etdrk/_etdrk_1.py:78-82,
// _etdrk_2.py:91-102, _etdrk_3.py:191-212, _etdrk_4.py:198-224 (the
// coefficient tables are the real parts of the contour means, FP32).
// stage_upd: `o` indexes both the coefficient tables ([half-axis mode][full-axis
// mode]) and the per-CTA state buffers, which share that layout.
#pragma once

#include "exgb_internal.h"

namespace exgb {

struct StageBufs {
  float2 *U, *S1, *S, *N0, *N1, *N2;
};

// `o` indexes the state buffers, `c` the coefficient tables.
__device__ __forceinline__ float2 stage_upd_at(const PlanDev& P, const StageBufs& b, int64_t o, int64_t c, int stage,
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
    default:
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

__device__ __forceinline__ float2 stage_upd(const PlanDev& P, const StageBufs& b, int64_t o, int stage, float2 nv) {
  return stage_upd_at(P, b, o, o, stage, nv);
}

// R modes at once, each as stage_upd_at (o[j] indexes the state buffers, co[j] the coefficient
// tables; modes with ok[j] false are read at a valid index and not written).  All global loads of the R
// updates are issued before the first store, so their latencies overlap: in a loop of single updates
// the compiler must keep each mode's loads behind the previous mode's stores, which may alias them.
template <int R>
__device__ __forceinline__ void stage_upd_many_at(const PlanDev& P, const StageBufs& b, const int64_t (&o)[R],
                                                  const int64_t (&co)[R], const bool (&ok)[R], int stage,
                                                  float2 (&nv)[R]) {
  if (P.order == 1 || (P.order == 2 && stage == 0) || (P.order == 3 && stage == 0) ||
      (P.order == 4 && stage <= 1)) {
    // s = E' U + c0 nv with E' = E (orders 1, 2) or E_{h/2} (orders 3, 4)
    const float2* Ep = (P.order <= 2) ? P.E : P.Eh;
    float2 e[R], u[R];
    float k0[R];
#pragma unroll
    for (int j = 0; j < R; ++j) {
      e[j] = __ldg(Ep + co[j]);
      u[j] = b.U[o[j]];
      k0[j] = __ldg(P.c[0] + co[j]);
    }
    float2* Nd = (P.order == 1) ? nullptr : (P.order == 4 && stage == 1) ? b.N1 : b.N0;
    float2* Sd = (P.order == 1) ? b.U : (P.order == 4 && stage == 0) ? b.S1 : b.S;
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const float2 s = cadd(cmul(e[j], u[j]), cscale(nv[j], k0[j]));
      if (ok[j]) {
        if (Nd) Nd[o[j]] = nv[j];
        Sd[o[j]] = s;
      }
      nv[j] = s;
    }
  } else if (P.order == 2) {
    float2 sv[R], n0[R];
    float k1[R];
#pragma unroll
    for (int j = 0; j < R; ++j) {
      sv[j] = b.S[o[j]];
      n0[j] = b.N0[o[j]];
      k1[j] = __ldg(P.c[1] + co[j]);
    }
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const float2 r = cadd(sv[j], cscale(csub(nv[j], n0[j]), k1[j]));
      if (ok[j]) b.U[o[j]] = r;
      nv[j] = r;
    }
  } else if (P.order == 3 && stage == 1) {
    float2 e[R], u[R], n0[R];
    float k1[R];
#pragma unroll
    for (int j = 0; j < R; ++j) {
      e[j] = __ldg(P.E + co[j]);
      u[j] = b.U[o[j]];
      n0[j] = b.N0[o[j]];
      k1[j] = __ldg(P.c[1] + co[j]);
    }
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const float2 t = csub(cscale(nv[j], 2.f), n0[j]);
      const float2 s = cadd(cmul(e[j], u[j]), cscale(t, k1[j]));
      if (ok[j]) {
        b.N1[o[j]] = nv[j];
        b.S[o[j]] = s;
      }
      nv[j] = s;
    }
  } else if (P.order == 3) {
    float2 e[R], u[R], n0[R], n1[R];
    float k2[R], k3[R], k4[R];
#pragma unroll
    for (int j = 0; j < R; ++j) {
      e[j] = __ldg(P.E + co[j]);
      u[j] = b.U[o[j]];
      n0[j] = b.N0[o[j]];
      n1[j] = b.N1[o[j]];
      k2[j] = __ldg(P.c[2] + co[j]);
      k3[j] = __ldg(P.c[3] + co[j]);
      k4[j] = __ldg(P.c[4] + co[j]);
    }
#pragma unroll
    for (int j = 0; j < R; ++j) {
      float2 r = cmul(e[j], u[j]);
      r = cadd(r, cscale(n0[j], k2[j]));
      r = cadd(r, cscale(n1[j], k3[j]));
      r = cadd(r, cscale(nv[j], k4[j]));
      if (ok[j]) b.U[o[j]] = r;
      nv[j] = r;
    }
  } else if (stage == 2) {
    float2 e[R], s1[R], n0[R];
    float k0[R];
#pragma unroll
    for (int j = 0; j < R; ++j) {
      e[j] = __ldg(P.Eh + co[j]);
      s1[j] = b.S1[o[j]];
      n0[j] = b.N0[o[j]];
      k0[j] = __ldg(P.c[0] + co[j]);
    }
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const float2 t = csub(cscale(nv[j], 2.f), n0[j]);
      const float2 s = cadd(cmul(e[j], s1[j]), cscale(t, k0[j]));
      if (ok[j]) {
        b.N2[o[j]] = nv[j];
        b.S[o[j]] = s;
      }
      nv[j] = s;
    }
  } else {
    float2 e[R], u[R], n0[R], n1[R], n2[R];
    float k3[R], k4[R], k5[R];
#pragma unroll
    for (int j = 0; j < R; ++j) {
      e[j] = __ldg(P.E + co[j]);
      u[j] = b.U[o[j]];
      n0[j] = b.N0[o[j]];
      n1[j] = b.N1[o[j]];
      n2[j] = b.N2[o[j]];
      k3[j] = __ldg(P.c[3] + co[j]);
      k4[j] = __ldg(P.c[4] + co[j]);
      k5[j] = __ldg(P.c[5] + co[j]);
    }
#pragma unroll
    for (int j = 0; j < R; ++j) {
      float2 r = cmul(e[j], u[j]);
      r = cadd(r, cscale(n0[j], k3[j]));
      r = cadd(r, cscale(cadd(n1[j], n2[j]), 2.f * k4[j]));
      r = cadd(r, cscale(nv[j], k5[j]));
      if (ok[j]) b.U[o[j]] = r;
      nv[j] = r;
    }
  }
}

template <int R>
__device__ __forceinline__ void stage_upd_many(const PlanDev& P, const StageBufs& b, const int64_t (&o)[R],
                                               const bool (&ok)[R], int stage, float2 (&nv)[R]) {
  stage_upd_many_at<R>(P, b, o, o, ok, stage, nv);
}

// The stage update of one mode's C <= MC channels (state index so[c], coefficient index co[c]; entries
// c >= C must hold valid indices): one update for a single channel, otherwise every channel's loads
// issued together.
template <int MC>
__device__ __forceinline__ void stage_upd_channels(const PlanDev& P, const StageBufs& b, int C, const int64_t (&so)[MC],
                                                   const int64_t (&co)[MC], int stage, float2 (&nv)[MC]) {
  if (C == 1) {
    nv[0] = stage_upd_at(P, b, so[0], co[0], stage, nv[0]);
  } else {
    bool ok[MC];
#pragma unroll
    for (int c = 0; c < MC; ++c) ok[c] = c < C;
    stage_upd_many_at<MC>(P, b, so, co, ok, stage, nv);
  }
}

// Per-CTA state buffers (each `colsz` modes) of an ETDRK method of the given order.
__host__ __device__ __forceinline__ StageBufs stage_bufs(float2* q, int order, int64_t colsz) {
  StageBufs sb;
  sb.U = q;
  q += colsz;
  sb.S1 = sb.S = sb.N0 = sb.N1 = sb.N2 = nullptr;
  if (order == 2) {
    sb.S = q;
    sb.N0 = q + colsz;
  } else if (order == 3) {
    sb.S = q;
    sb.N0 = q + colsz;
    sb.N1 = q + 2 * colsz;
  } else if (order == 4) {
    sb.S1 = q;
    sb.S = q + colsz;
    sb.N0 = q + 2 * colsz;
    sb.N1 = q + 3 * colsz;
    sb.N2 = q + 4 * colsz;
  }
  return sb;
}

// number of state buffers stage_bufs lays out
__host__ __device__ constexpr int stage_nbufs(int order) {
  return order <= 1 ? 1 : order == 2 ? 3 : order == 3 ? 4 : 6;
}

}  // namespace exgb
