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
