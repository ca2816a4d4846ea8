// exgb_ndops.cuh -- the per-mode and per-point arithmetic of the nonlinear terms that the staged
// N-D paths evaluate (exgb_ndgen.cu: one kernel per step; exgb_pass2d.cu: three fused passes):
// the spectra the inverse transforms need (derive), the pointwise products (pointwise) and the
// post-masked combination of the forward spectra (combine).  Reference: nonlin_fun/_convection.py,
// _gradient_norm.py, _polynomial.py, _general_nonlinear.py, _vorticity_convection.py,
// stepper/reaction/*.py (each op below names its lines).
#pragma once

#include "exgb_internal.h"

namespace exgb {
namespace ndg {

constexpr int MAXC = 3;

enum Op {
  OP_CONV_MC_CONS = 0,  // -b/2 sum_j ik_j F[u_i u_j]          (_convection.py:104-138)
  OP_CONV_MC_NONCONS,   // -b F[sum_j u_j d_j u_i]              (_convection.py:140-171)
  OP_CONV_SC_CONS,      // -b/2 (sum_d ik_d) F[u^2]             (_convection.py:173-202)
  OP_CONV_SC_NONCONS,   // -b F[u sum_d d_d u]                  (_convection.py:204-231)
  OP_GRAD_NORM,         // -b/2 F[|grad u|^2 - mean]            (_gradient_norm.py:68-101)
  OP_POLY,              // F[sum_k c_k u^k]                     (_polynomial.py:56-76)
  OP_GENERAL,           // s0 F[u^2] + s1/2 (sum ik) F[u^2] + s2/2 F[|grad u|^2 - mean]
  OP_CAHN_HILLIARD,     // s Lap F[u^3]                         (_cahn_hilliard.py:31-45)
  OP_GRAY_SCOTT,        // F[f(1-u0) - u0 u1^2], F[-(f+k) u1 + u0 u1^2]  (_gray_scott.py:30-46)
  OP_BZ,                // F[u0 + u1 - u0 u1 - u0^2], F[u2 - u1 - u0 u1], F[u0 - u2]  (_belousov_zhabotinsky.py:33-51)
  OP_VORT,              // -b F[u w_x + v w_y], (u, v) = (d_y, -d_x) Lap^-1 w  (_vorticity_convection.py:78-99),
                        // + the Kolmogorov injection at (0, k)               (_vorticity_convection.py:166-176)
  OP_PROJ3D,            // P F[u x (curl u)], curl = i k x u^ (mask), P the Leray projection
                        // (_projected_convection.py:114-136, _leray.py:114-136) + the 3D Kolmogorov
                        // injection at (0, k, 0), first channel (_projected_convection.py:202-220)
};

struct Geo {
  int D, N, M, C, K;
  int64_t per;   // modes per field
  int64_t npts;  // grid points per field
  float ks;      // 2 pi / L
};

struct Prog {
  int op, NI, NF;
  float s0, s1, s2;  // combine scales
  float feed, kill;  // Gray-Scott rates (pointwise step)
  int zmf;
  int npoly;
  float poly[8];
};

// signed wavenumbers of mode r (leading axes fftfreq, last axis rfftfreq)
__device__ __forceinline__ void mode_of(const Geo& g, int64_t r, int (&k)[3]) {
  k[0] = k[1] = k[2] = 0;
  k[g.D - 1] = (int)(r % g.M);
  int64_t rest = r / g.M;
  for (int a = g.D - 2; a >= 0; --a) {
    const int i = (int)(rest % g.N);
    rest /= g.N;
    k[a] = (i <= (g.N - 1) / 2) ? i : i - g.N;
  }
}

__device__ __forceinline__ bool kept(const Geo& g, const int (&k)[3]) {
  bool m = true;
  for (int a = 0; a < g.D; ++a) m = m && (abs(k[a]) <= g.K);
  return m;
}

__device__ __forceinline__ float2 times_i(float d, float2 u) { return make_float2(-d * u.y, d * u.x); }


// index of the product u_i u_j (i <= j) among the C(C+1)/2 symmetric products
__device__ __forceinline__ int sym_index(int i, int j, int C) {
  if (i > j) {
    const int t = i;
    i = j;
    j = t;
  }
  return i * C - (i * (i - 1)) / 2 + (j - i);
}

// The NI spectra of mode k whose inverse transforms the pointwise step needs: channel c of the
// state at x[c * xs], field f written to w[f * ws]; m = inside the dealiasing mask (pre-mask).
// The derived spectra at one mode: channel c read as x(c), derived spectrum i written as w(i, value).
// Callers pass pointer accessors (derive_mode below) or registers loaded ahead, and a sink that
// stores every spectrum or keeps only the one they need (a runtime-indexed local array would live
// in local memory).
template <class X, class O>
__device__ __forceinline__ void derive_mode_xo(const Geo& g, const Prog& p, const int (&k)[3], bool m, const X& x,
                                               const O& w) {
  float d[3];
  for (int a = 0; a < 3; ++a) d[a] = g.ks * (float)k[a];
  const float2 z = make_float2(0.f, 0.f);
  switch (p.op) {
    case OP_CONV_MC_NONCONS:
      for (int c = 0; c < g.C; ++c) {
        const float2 u = m ? x(c) : z;
        w(c, u);
        for (int j = 0; j < g.D; ++j) w(g.C + c * g.D + j, times_i(d[j], u));
      }
      break;
    case OP_CONV_SC_NONCONS: {
      const float2 u = m ? x(0) : z;
      w(0, u);
      float s = 0.f;
      for (int j = 0; j < g.D; ++j) s += d[j];
      w(1, times_i(s, u));
    } break;
    case OP_GRAD_NORM:
      for (int c = 0; c < g.C; ++c) {
        const float2 u = m ? x(c) : z;
        for (int j = 0; j < g.D; ++j) w(c * g.D + j, times_i(d[j], u));
      }
      break;
    case OP_GENERAL: {
      const float2 u = m ? x(0) : z;
      w(0, u);
      for (int j = 0; j < g.D; ++j) w(1 + j, times_i(d[j], u));
    } break;
    case OP_VORT: {
      // stream function psi = w / Lap with 1/Lap = 1 at k = 0; u = i k_y psi, v = -i k_x psi,
      // w_x = i k_x w, w_y = i k_y w (k_x the leading axis, k_y the rfft axis)
      const float2 wv = m ? x(0) : z;
      const float lap = -(d[0] * d[0] + d[1] * d[1]);
      const float il = lap != 0.f ? 1.f / lap : 1.f;
      const float2 psi = cscale(wv, il);
      w(0, times_i(d[1], psi));
      w(1, times_i(-d[0], psi));
      w(2, times_i(d[0], wv));
      w(3, times_i(d[1], wv));
    } break;
    case OP_PROJ3D: {
      // w[0..2] = mask (i d x u^) (the curl), w[3..5] = mask u^
      const float2 u0 = m ? x(0) : z, u1 = m ? x(1) : z, u2 = m ? x(2) : z;
      const float2 a1 = make_float2(d[1] * u2.x - d[2] * u1.x, d[1] * u2.y - d[2] * u1.y);
      const float2 a2 = make_float2(d[2] * u0.x - d[0] * u2.x, d[2] * u0.y - d[0] * u2.y);
      const float2 a3 = make_float2(d[0] * u1.x - d[1] * u0.x, d[0] * u1.y - d[1] * u0.y);
      w(0, make_float2(-a1.y, a1.x));
      w(1, make_float2(-a2.y, a2.x));
      w(2, make_float2(-a3.y, a3.x));
      w(3, u0);
      w(4, u1);
      w(5, u2);
    } break;
    default:  // the masked state itself, one spectrum per channel
      for (int c = 0; c < g.C; ++c) w(c, m ? x(c) : z);
      break;
  }
}

__device__ __forceinline__ void derive_mode(const Geo& g, const Prog& p, const int (&k)[3], bool m,
                                            const float2* x, int64_t xs, float2* w, int64_t ws) {
  derive_mode_xo(
      g, p, k, m, [x, xs](int c) { return x[c * xs]; }, [w, ws](int i, float2 v) { w[i * ws] = v; });
}

constexpr int kMaxNI = MAXC + MAXC * 3;  // derived fields of a program, at most

template <int C, int D>
__device__ __forceinline__ void pw_mc_noncons(const float (&in)[kMaxNI], float* f, int64_t fs) {
#pragma unroll
  for (int i = 0; i < C; ++i) {
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < D; ++j) s += in[j] * in[C + i * D + j];
    f[i * fs] = s;
  }
}
template <int C>
__device__ __forceinline__ void pw_mc_cons(const float (&in)[kMaxNI], float* f, int64_t fs) {
  int o = 0;
#pragma unroll
  for (int i = 0; i < C; ++i)
#pragma unroll
    for (int j = i; j < C; ++j) f[(o++) * fs] = in[i] * in[j];
}
template <int C, int D>
__device__ __forceinline__ void pw_grad_norm(const float (&in)[kMaxNI], float* f, int64_t fs) {
#pragma unroll
  for (int c = 0; c < C; ++c) {
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < D; ++j) s += in[c * D + j] * in[c * D + j];
    f[c * fs] = s;
  }
}
#define EXGB_CD_DISPATCH(FN)                    \
  switch (g.C * 4 + g.D) {                      \
    case 5: FN<1, 1>(in, f, fs); break;         \
    case 6: FN<1, 2>(in, f, fs); break;         \
    case 7: FN<1, 3>(in, f, fs); break;         \
    case 9: FN<2, 1>(in, f, fs); break;         \
    case 10: FN<2, 2>(in, f, fs); break;        \
    case 11: FN<2, 3>(in, f, fs); break;        \
    case 13: FN<3, 1>(in, f, fs); break;        \
    case 14: FN<3, 2>(in, f, fs); break;        \
    default: FN<3, 3>(in, f, fs); break;        \
  }

// The NF products at one grid point from the NI physical values in[] (registers the caller loaded:
// every index below is a compile-time constant, the channel and dimension counts being dispatched to
// templates, so in[] never goes to local memory): field i written to f[i * fs].
__device__ __forceinline__ void pointwise_point_reg(const Geo& g, const Prog& p, const float (&in)[kMaxNI], float* f,
                                                    int64_t fs) {
  switch (p.op) {
    case OP_CONV_MC_CONS:
      if (g.C == 1) pw_mc_cons<1>(in, f, fs);
      else if (g.C == 2) pw_mc_cons<2>(in, f, fs);
      else pw_mc_cons<3>(in, f, fs);
      break;
    case OP_CONV_MC_NONCONS:
      EXGB_CD_DISPATCH(pw_mc_noncons)
      break;
    case OP_CONV_SC_CONS:
      f[0] = in[0] * in[0];
      break;
    case OP_CONV_SC_NONCONS:
      f[0] = in[0] * in[1];
      break;
    case OP_GRAD_NORM:
      EXGB_CD_DISPATCH(pw_grad_norm)
      break;
    case OP_POLY:
#pragma unroll
      for (int c = 0; c < MAXC; ++c) {
        if (c >= g.C) break;
        // sum_k c_k u^k with the powers accumulated as the reference does
        const float u = in[c];
        float pw = 1.f, acc = 0.f;
        for (int i = 0; i < p.npoly; ++i) {
          acc += p.poly[i] * pw;
          pw *= u;
        }
        f[c * fs] = acc;
      }
      break;
    case OP_GENERAL: {
      float s = 0.f;
#pragma unroll
      for (int j = 0; j < 3; ++j)
        if (j < g.D) s += in[1 + j] * in[1 + j];
      f[0] = in[0] * in[0];
      f[fs] = s;
    } break;
    case OP_CAHN_HILLIARD:
      f[0] = in[0] * in[0] * in[0];
      break;
    case OP_GRAY_SCOTT: {
      const float u0 = in[0], u1 = in[1];
      const float uvv = u0 * (u1 * u1);
      f[0] = p.feed * (1.f - u0) - uvv;
      f[fs] = -(p.feed + p.kill) * u1 + uvv;
    } break;
    case OP_VORT:
      f[0] = fmaf(in[0], in[2], in[1] * in[3]);
      break;
    case OP_PROJ3D: {  // velocity (in[3..5]) x curl (in[0..2])
      const float w0 = in[0], w1 = in[1], w2 = in[2], v0 = in[3], v1 = in[4], v2 = in[5];
      f[0] = v1 * w2 - v2 * w1;
      f[fs] = v2 * w0 - v0 * w2;
      f[2 * fs] = v0 * w1 - v1 * w0;
    } break;
    case OP_BZ: {
      const float u0 = in[0], u1 = in[1], u2 = in[2];
      const float u01 = u0 * u1;
      f[0] = u0 + u1 - u01 - u0 * u0;
      f[fs] = u2 - u1 - u01;
      f[2 * fs] = u0 - u2;
    } break;
  }
}
#undef EXGB_CD_DISPATCH

// The NI physical values at v[i * vs] into registers (then pointwise_point_reg may write its products
// over them in place).
__device__ __forceinline__ void load_point(const float* v, int64_t vs, int NI, float (&in)[kMaxNI]) {
#pragma unroll
  for (int i = 0; i < kMaxNI; ++i) in[i] = i < NI ? v[i * vs] : 0.f;
}


// N^ of every channel at mode k from the NF forward spectra h[f * hs] (post-mask m, derivative
// multipliers, scales); the Kolmogorov injection of the vorticity term included.
__device__ __forceinline__ void combine_mode(const PlanDev& P, const Geo& g, const Prog& p, const int (&k)[3], bool m,
                                             const float2* h, int64_t hs, float2 (&nv)[MAXC]) {
    float d[3];
    float dsum = 0.f, lap = 0.f;
    for (int a = 0; a < 3; ++a) {
      d[a] = g.ks * (float)k[a];
      if (a < g.D) {
        dsum += d[a];
        lap -= d[a] * d[a];
      }
    }
    const bool dc = (k[0] == 0 && k[1] == 0 && k[2] == 0);
    for (int c = 0; c < MAXC; ++c) nv[c] = make_float2(0.f, 0.f);
    if (m) {
      switch (p.op) {
        case OP_CONV_MC_CONS:
#pragma unroll
          for (int i = 0; i < MAXC; ++i) {  // compile-time channel indices keep nv in registers
            if (i >= g.C) break;
            float2 acc = make_float2(0.f, 0.f);
            for (int j = 0; j < g.D; ++j) acc = cadd(acc, times_i(d[j], h[(sym_index(i, j, g.C)) * hs]));
            nv[i] = cscale(acc, p.s0);
          }
          break;
        case OP_CONV_SC_CONS:
          nv[0] = cscale(times_i(dsum, h[0]), p.s0);
          break;
        case OP_GRAD_NORM:
#pragma unroll
          for (int c = 0; c < MAXC; ++c) {
            if (c >= g.C) break;
            nv[c] = (p.zmf && dc) ? make_float2(0.f, 0.f) : cscale(h[(c) * hs], p.s0);
          }
          break;
        case OP_GENERAL: {
          const float2 sq = h[0];
          const float2 gn = (p.zmf && dc) ? make_float2(0.f, 0.f) : h[hs];
          nv[0] = cadd(cadd(cscale(sq, p.s0), cscale(times_i(dsum, sq), p.s1)), cscale(gn, p.s2));
        } break;
        case OP_CAHN_HILLIARD:
          nv[0] = cscale(h[0], p.s0 * lap);
          break;
        case OP_PROJ3D: {
          // Leray: n + (i d) q, q = -inv_lap (i d . n), inv_lap = 1/lap (0 at k = 0), lap = -|d|^2
          float2 n0 = h[0], n1 = h[hs], n2 = h[2 * hs];
          if (lap != 0.f) {
            const float il = 1.f / lap;
            const float2 sd = make_float2(d[0] * n0.x + d[1] * n1.x + d[2] * n2.x, d[0] * n0.y + d[1] * n1.y + d[2] * n2.y);
            const float2 dv = make_float2(-sd.y, sd.x);
            const float2 q = make_float2(-il * dv.x, -il * dv.y);
            n0 = cadd(n0, make_float2(-d[0] * q.y, d[0] * q.x));
            n1 = cadd(n1, make_float2(-d[1] * q.y, d[1] * q.x));
            n2 = cadd(n2, make_float2(-d[2] * q.y, d[2] * q.x));
          }
          nv[0] = n0;
          nv[1] = n1;
          nv[2] = n2;
        } break;
        default:  // -b F[.] (non-conservative convection, vorticity) or F[.] (polynomial, Gray-Scott): scale s0
#pragma unroll
          for (int c = 0; c < MAXC; ++c) {
            if (c >= g.C) break;
            nv[c] = cscale(h[(c) * hs], p.s0);
          }
          break;
      }
    }
  if (p.op == OP_VORT && k[0] == 0 && k[1] == P.inj_mode) nv[0].x += P.inj_value;
  if (p.op == OP_PROJ3D && P.inj_mode >= 0 && k[0] == 0 && k[1] == P.inj_mode && k[2] == 0) nv[0].x += P.inj_value;
}

}  // namespace ndg
}  // namespace exgb
