// exgb_ndgen.cu -- staged ETDRK path for the nonlinearities that have no
// fused kernel: the four convection variants, gradient norm, polynomial and
// general nonlinearities in 2D and 3D, and the Cahn-Hilliard, Gray-Scott and
// Belousov-Zhabotinsky reaction terms in 1D, 2D and 3D.
//
// Reference: nonlin_fun/_convection.py:104-231, _gradient_norm.py:68-101,
// _polynomial.py:56-76, _general_nonlinear.py:99-119,
// stepper/reaction/_cahn_hilliard.py:12-45 (CahnHilliardNonlinearFun),
// stepper/reaction/_gray_scott.py:9-46 (GrayScottNonlinearFun),
// stepper/reaction/_belousov_zhabotinsky.py:14-51 (BelousovZhabotinskyNonlinearFun),
// nonlin_fun/_base.py:73-137 (pre-mask before every inverse transform,
// post-mask after every forward transform), etdrk/_etdrk_1..4.py (stages).
//
// One ETDRK stage over a chunk of samples is five steps:
//   derive    : masked state and its spectral derivatives -> NI spectra
//   irfftn    : NI inverse transforms per sample
//   pointwise : the products of the nonlinearity at every grid point, in
//               place over the physical fields -> NF real fields
//   rfftn     : NF forward transforms per sample
//   combine   : post-mask, derivative multipliers and scales -> N^ per
//               channel, then the ETDRK stage update of every channel of the
//               mode in the same thread
// Stage buffers live in a grow-only workspace; the coefficient tables are in
// the plan's natural layout [lin_ch][N..., N/2+1].
#include <cuda_runtime.h>

#include <algorithm>

#include "exgb_internal.h"
#include "exgb_stage.cuh"

namespace exgb {

void* workspace(size_t bytes, int slot_offset);
int rfftn_impl(cudaStream_t st, int D, int N, int64_t count, const float* in, float2* out);
int irfftn_impl(cudaStream_t st, int D, int N, int64_t count, const float2* in, float* out);

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

// W[b][f] = the NI spectra whose inverse transforms the pointwise step needs
__global__ void derive_kernel(Geo g, Prog p, int64_t cb, const float2* __restrict__ X, float2* __restrict__ W) {
  const int64_t total = cb * g.per;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = t / g.per, r = t - b * g.per;
    int k[3];
    mode_of(g, r, k);
    const bool m = kept(g, k);
    float d[3];
    for (int a = 0; a < 3; ++a) d[a] = g.ks * (float)k[a];
    const float2* x = X + b * g.C * g.per + r;
    float2* w = W + b * p.NI * g.per + r;
    const float2 z = make_float2(0.f, 0.f);
    switch (p.op) {
      case OP_CONV_MC_NONCONS:
        for (int c = 0; c < g.C; ++c) {
          const float2 u = m ? x[c * g.per] : z;
          w[c * g.per] = u;
          for (int j = 0; j < g.D; ++j) w[(g.C + c * g.D + j) * g.per] = times_i(d[j], u);
        }
        break;
      case OP_CONV_SC_NONCONS: {
        const float2 u = m ? x[0] : z;
        w[0] = u;
        float s = 0.f;
        for (int j = 0; j < g.D; ++j) s += d[j];
        w[g.per] = times_i(s, u);
      } break;
      case OP_GRAD_NORM:
        for (int c = 0; c < g.C; ++c) {
          const float2 u = m ? x[c * g.per] : z;
          for (int j = 0; j < g.D; ++j) w[(c * g.D + j) * g.per] = times_i(d[j], u);
        }
        break;
      case OP_GENERAL: {
        const float2 u = m ? x[0] : z;
        w[0] = u;
        for (int j = 0; j < g.D; ++j) w[(1 + j) * g.per] = times_i(d[j], u);
      } break;
      case OP_VORT: {
        // stream function psi = w / Lap with 1/Lap = 1 at k = 0; u = i k_y psi, v = -i k_x psi,
        // w_x = i k_x w, w_y = i k_y w (k_x the leading axis, k_y the rfft axis)
        const float2 wv = m ? x[0] : z;
        const float lap = -(d[0] * d[0] + d[1] * d[1]);
        const float il = lap != 0.f ? 1.f / lap : 1.f;
        const float2 psi = cscale(wv, il);
        w[0] = times_i(d[1], psi);
        w[g.per] = times_i(-d[0], psi);
        w[2 * g.per] = times_i(d[0], wv);
        w[3 * g.per] = times_i(d[1], wv);
      } break;
      default:  // the masked state itself, one spectrum per channel
        for (int c = 0; c < g.C; ++c) w[c * g.per] = m ? x[c * g.per] : z;
        break;
    }
  }
}

// Physical fields Ph[b][0..NI) -> products Q[b][0..NF) at every grid point.
__global__ void pointwise_kernel(Geo g, Prog p, int64_t cb, const float* __restrict__ Ph, float* __restrict__ Q) {
  const int64_t total = cb * g.npts;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = t / g.npts, q = t - b * g.npts;
    const float* src = Ph + b * p.NI * g.npts + q;
    float* f = Q + b * p.NF * g.npts + q;
    float in[MAXC + MAXC * 3];
    for (int i = 0; i < p.NI; ++i) in[i] = src[i * g.npts];
    switch (p.op) {
      case OP_CONV_MC_CONS: {
        int o = 0;
        for (int i = 0; i < g.C; ++i)
          for (int j = i; j < g.C; ++j) f[(o++) * g.npts] = in[i] * in[j];
      } break;
      case OP_CONV_MC_NONCONS:
        for (int i = 0; i < g.C; ++i) {
          float s = 0.f;
          for (int j = 0; j < g.D; ++j) s += in[j] * in[g.C + i * g.D + j];
          f[i * g.npts] = s;
        }
        break;
      case OP_CONV_SC_CONS:
        f[0] = in[0] * in[0];
        break;
      case OP_CONV_SC_NONCONS:
        f[0] = in[0] * in[1];
        break;
      case OP_GRAD_NORM:
        for (int c = 0; c < g.C; ++c) {
          float s = 0.f;
          for (int j = 0; j < g.D; ++j) s += in[c * g.D + j] * in[c * g.D + j];
          f[c * g.npts] = s;
        }
        break;
      case OP_POLY:
        for (int c = 0; c < g.C; ++c) {
          // sum_k c_k u^k with the powers accumulated as the reference does
          const float u = in[c];
          float pw = 1.f, acc = 0.f;
          for (int i = 0; i < p.npoly; ++i) {
            acc += p.poly[i] * pw;
            pw *= u;
          }
          f[c * g.npts] = acc;
        }
        break;
      case OP_GENERAL: {
        float s = 0.f;
        for (int j = 0; j < g.D; ++j) s += in[1 + j] * in[1 + j];
        f[0] = in[0] * in[0];
        f[g.npts] = s;
      } break;
      case OP_CAHN_HILLIARD:
        f[0] = in[0] * in[0] * in[0];
        break;
      case OP_GRAY_SCOTT: {
        const float u0 = in[0], u1 = in[1];
        const float uvv = u0 * (u1 * u1);
        f[0] = p.feed * (1.f - u0) - uvv;
        f[g.npts] = -(p.feed + p.kill) * u1 + uvv;
      } break;
      case OP_VORT:
        f[0] = fmaf(in[0], in[2], in[1] * in[3]);
        break;
      case OP_BZ: {
        const float u0 = in[0], u1 = in[1], u2 = in[2];
        const float u01 = u0 * u1;
        f[0] = u0 + u1 - u01 - u0 * u0;
        f[g.npts] = u2 - u1 - u01;
        f[2 * g.npts] = u0 - u2;
      } break;
    }
  }
}

// index of the product u_i u_j (i <= j) among the C(C+1)/2 symmetric products
__device__ __forceinline__ int sym_index(int i, int j, int C) {
  if (i > j) {
    const int t = i;
    i = j;
    j = t;
  }
  return i * C - (i * (i - 1)) / 2 + (j - i);
}

// Post-mask and multipliers of the NF forward spectra -> N^ of every channel;
// then the ETDRK stage update (stage >= 0) or N^ written out (stage < 0).
__global__ void combine_kernel(PlanDev P, Geo g, Prog p, int64_t cb, const float2* __restrict__ H, StageBufs sb,
                               int stage, float2* __restrict__ nout) {
  const int64_t total = cb * g.per;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = t / g.per, r = t - b * g.per;
    int k[3];
    mode_of(g, r, k);
    const bool m = kept(g, k);
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
    const float2* h = H + b * p.NF * g.per + r;
    float2 nv[MAXC];
    for (int c = 0; c < MAXC; ++c) nv[c] = make_float2(0.f, 0.f);
    if (m) {
      switch (p.op) {
        case OP_CONV_MC_CONS:
          for (int i = 0; i < g.C; ++i) {
            float2 acc = make_float2(0.f, 0.f);
            for (int j = 0; j < g.D; ++j) acc = cadd(acc, times_i(d[j], h[sym_index(i, j, g.C) * g.per]));
            nv[i] = cscale(acc, p.s0);
          }
          break;
        case OP_CONV_SC_CONS:
          nv[0] = cscale(times_i(dsum, h[0]), p.s0);
          break;
        case OP_GRAD_NORM:
          for (int c = 0; c < g.C; ++c) nv[c] = (p.zmf && dc) ? make_float2(0.f, 0.f) : cscale(h[c * g.per], p.s0);
          break;
        case OP_GENERAL: {
          const float2 sq = h[0];
          const float2 gn = (p.zmf && dc) ? make_float2(0.f, 0.f) : h[g.per];
          nv[0] = cadd(cadd(cscale(sq, p.s0), cscale(times_i(dsum, sq), p.s1)), cscale(gn, p.s2));
        } break;
        case OP_CAHN_HILLIARD:
          nv[0] = cscale(h[0], p.s0 * lap);
          break;
        default:  // -b F[.] (non-conservative convection, vorticity) or F[.] (polynomial, Gray-Scott): scale s0
          for (int c = 0; c < g.C; ++c) nv[c] = cscale(h[c * g.per], p.s0);
          break;
      }
    }
    if (p.op == OP_VORT && k[0] == 0 && k[1] == P.inj_mode) nv[0].x += P.inj_value;
    const int64_t base = b * g.C * g.per + r;
    if (stage < 0) {
      for (int c = 0; c < g.C; ++c) nout[base + c * g.per] = nv[c];
      continue;
    }
    for (int c = 0; c < g.C; ++c) {
      const int64_t ci = (P.lin_ch == 1 ? 0 : (int64_t)c * g.per) + r;
      stage_upd_at(P, sb, base + c * g.per, ci, stage, nv[c]);
    }
  }
}

// c2r projection of a physical round trip on the last-axis columns k = 0 and
// k = N/2: v(k_lead) <- (v(k_lead) + conj(v(-k_lead))) / 2 (1D: Re v).
__global__ void project_kernel(Geo g, int64_t nfields, float2* __restrict__ X) {
  const int ncols = (g.N % 2 == 0) ? 2 : 1;
  int64_t lead = 1;
  for (int a = 0; a < g.D - 1; ++a) lead *= g.N;
  const int64_t total = nfields * ncols * lead;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t f = t / (ncols * lead);
    const int64_t rr = t - f * ncols * lead;
    const int col = (int)(rr / lead);
    const int64_t li = rr - (int64_t)col * lead;
    // index of -k_lead
    int64_t lj = 0, rest = li, mul = 1;
    for (int a = 0; a < g.D - 1; ++a) {
      const int i = (int)(rest % g.N);
      rest /= g.N;
      lj += (int64_t)((g.N - i) % g.N) * mul;
      mul *= g.N;
    }
    if (lj < li) continue;  // the pair is handled by its smaller index
    const int kc = col == 0 ? 0 : g.N / 2;
    float2* base = X + f * g.per + kc;
    const float2 a = base[li * g.M], c = base[lj * g.M];
    const float2 pv = make_float2(0.5f * (a.x + c.x), 0.5f * (a.y - c.y));
    base[li * g.M] = pv;
    base[lj * g.M] = cconj(pv);
  }
}

static unsigned grid_for(int64_t n, int sm) {
  const int64_t b = (n + 255) / 256;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)sm * 32));
}

}  // namespace ndg

using namespace ndg;

// Does the staged path step this plan?  (The fused kernels cover the 1D
// single-channel nonlinearities, 2D vorticity and 3D projected convection.)
// Can the staged path step this plan?  Besides the plans it always takes, it steps the 1D
// nonlinearities and 2D vorticity at the sizes the fused kernels do not cover (a prime factor above
// 5, or a grid longer than one CTA's shared memory holds).
bool ndgen_can(const exgb_plan_desc& d) {
  if (d.order < 1 || d.nonlin_kind == EXGB_NL_ZERO) return false;
  switch (d.nonlin_kind) {
    case EXGB_NL_CONVECTION:
    case EXGB_NL_GRADIENT_NORM:
    case EXGB_NL_POLYNOMIAL:
    case EXGB_NL_GENERAL:
    case EXGB_NL_CAHN_HILLIARD:
    case EXGB_NL_GRAY_SCOTT:
    case EXGB_NL_BELOUSOV_ZHABOTINSKY:
      return true;
    case EXGB_NL_VORTICITY_2D:
    case EXGB_NL_VORTICITY_2D_KOLMOGOROV:
      return d.num_spatial_dims == 2;
    default:
      return false;
  }
}

bool ndgen_handles(const exgb_plan_desc& d) {
  if (d.order < 1 || d.nonlin_kind == EXGB_NL_ZERO) return false;
  switch (d.nonlin_kind) {
    case EXGB_NL_CAHN_HILLIARD:
    case EXGB_NL_GRAY_SCOTT:
    case EXGB_NL_BELOUSOV_ZHABOTINSKY:
      return true;
    case EXGB_NL_CONVECTION:
    case EXGB_NL_GRADIENT_NORM:
    case EXGB_NL_POLYNOMIAL:
    case EXGB_NL_GENERAL:
      return d.num_spatial_dims >= 2;
    default:
      return false;
  }
}

// Channel rules of the reference's nonlinear functions, checked at plan creation.
int ndgen_validate(const exgb_plan_desc& d) {
  const int C = d.num_channels, D = d.num_spatial_dims;
  if (d.dealiasing_fraction < 0 && (d.nonlin_kind == EXGB_NL_CAHN_HILLIARD || d.nonlin_kind == EXGB_NL_GRAY_SCOTT ||
                                    d.nonlin_kind == EXGB_NL_BELOUSOV_ZHABOTINSKY))
    return fail(EXGB_EINVAL, "Nonlinear function was set up without dealiasing");
  switch (d.nonlin_kind) {
    case EXGB_NL_CONVECTION:
      if (d.single_channel) {
        if (C != 1) return fail(EXGB_ESHAPE, "single-channel convection has one channel");
      } else if (C != D) {
        return fail(EXGB_ESHAPE, "Number of channels in u_hat should match number of spatial dimensions");
      }
      return EXGB_OK;
    case EXGB_NL_GRADIENT_NORM:
    case EXGB_NL_POLYNOMIAL:
      if (C > MAXC) return fail(EXGB_EUNSUPPORTED, "at most 3 channels on the staged path");
      return EXGB_OK;
    case EXGB_NL_GENERAL:
    case EXGB_NL_CAHN_HILLIARD:
      if (C != 1) return fail(EXGB_ESHAPE, "this nonlinear function has one channel");
      return EXGB_OK;
    case EXGB_NL_GRAY_SCOTT:
      if (C != 2) return fail(EXGB_ESHAPE, "num_channels must be 2");
      return EXGB_OK;
    case EXGB_NL_BELOUSOV_ZHABOTINSKY:
      if (C != 3) return fail(EXGB_ESHAPE, "num_channels must be 3");
      return EXGB_OK;
    case EXGB_NL_VORTICITY_2D:
    case EXGB_NL_VORTICITY_2D_KOLMOGOROV:
      if (D != 2) return fail(EXGB_EUNSUPPORTED, "vorticity convection needs num_spatial_dims == 2");
      if (C != 1) return fail(EXGB_ESHAPE, "vorticity formulation has one channel");
      return EXGB_OK;
    default:
      return fail(EXGB_EUNSUPPORTED, "nonlinear function not handled by the staged path");
  }
}

static Prog make_prog(const exgb_plan_desc& d) {
  const int C = d.num_channels, D = d.num_spatial_dims;
  const float b = (float)d.scale;
  Prog p{};
  p.s0 = 1.f;
  switch (d.nonlin_kind) {
    case EXGB_NL_CONVECTION:
      if (d.single_channel) {
        p.op = d.conservative ? OP_CONV_SC_CONS : OP_CONV_SC_NONCONS;
        p.NI = d.conservative ? 1 : 2;
        p.NF = 1;
      } else {
        p.op = d.conservative ? OP_CONV_MC_CONS : OP_CONV_MC_NONCONS;
        p.NI = d.conservative ? C : C + C * D;
        p.NF = d.conservative ? C * (C + 1) / 2 : C;
      }
      p.s0 = d.conservative ? -0.5f * b : -b;
      break;
    case EXGB_NL_GRADIENT_NORM:
      p.op = OP_GRAD_NORM;
      p.NI = C * D;
      p.NF = C;
      p.s0 = -0.5f * b;
      p.zmf = d.zero_mode_fix;
      break;
    case EXGB_NL_POLYNOMIAL:
      p.op = OP_POLY;
      p.NI = p.NF = C;
      p.npoly = d.num_poly;
      for (int i = 0; i < d.num_poly; ++i) p.poly[i] = (float)d.poly[i];
      break;
    case EXGB_NL_GENERAL:
      p.op = OP_GENERAL;
      p.NI = 1 + D;
      p.NF = 2;
      p.s0 = (float)d.scale_list[0];
      p.s1 = 0.5f * (float)d.scale_list[1];
      p.s2 = 0.5f * (float)d.scale_list[2];
      p.zmf = d.zero_mode_fix;
      break;
    case EXGB_NL_CAHN_HILLIARD:
      p.op = OP_CAHN_HILLIARD;
      p.NI = p.NF = 1;
      p.s0 = b;
      break;
    case EXGB_NL_BELOUSOV_ZHABOTINSKY:
      p.op = OP_BZ;
      p.NI = p.NF = 3;
      break;
    case EXGB_NL_VORTICITY_2D:
    case EXGB_NL_VORTICITY_2D_KOLMOGOROV:
      p.op = OP_VORT;
      p.NI = 4;
      p.NF = 1;
      p.s0 = -b;
      break;
    default:  // Gray-Scott
      p.op = OP_GRAY_SCOTT;
      p.NI = p.NF = 2;
      p.feed = (float)d.reaction[0];
      p.kill = (float)d.reaction[1];
      break;
  }
  return p;
}

// Fourier-space stepping (nsteps steps, c2r projection after each when
// `project`) or, with `nonlinear_only`, N^ of the input written to `out`.
int ndgen_run(const exgb_plan* plan, cudaStream_t st, const float2* in, float2* out, int64_t batch, int nsteps,
              int project, int nonlinear_only) {
  const PlanDev& P = plan->dev;
  const exgb_plan_desc& d = plan->desc;
  Geo g;
  g.D = P.D;
  g.N = P.N;
  g.M = P.M;
  g.C = P.C;
  g.K = std::min(P.kmax, P.N / 2);
  g.per = (int64_t)plan->n_modes;
  g.npts = 1;
  for (int a = 0; a < P.D; ++a) g.npts *= P.N;
  g.ks = P.kscale;
  const Prog p = make_prog(d);
  const int sm = plan->sm_count;
  const int C = P.C;
  if (batch == 0) return EXGB_OK;
  if (!nonlinear_only && nsteps == 0) {
    if (in != out) EXGB_CUDA(cudaMemcpyAsync(out, in, sizeof(float2) * batch * C * g.per, cudaMemcpyDeviceToDevice, st));
    return EXGB_OK;
  }
  const int nb = stage_nbufs(P.order);
  const int SP = std::max(p.NI, p.NF);
  const size_t per_sample =
      sizeof(float2) * (size_t)g.per * (size_t)(nb * C + SP) + sizeof(float) * (size_t)g.npts * (p.NI + p.NF);
  const int64_t cb = std::max<int64_t>(1, std::min<int64_t>(batch, (int64_t)((size_t)(1u << 30) / per_sample)));
  char* ws = (char*)workspace(per_sample * (size_t)cb, 5);
  if (!ws) return fail(EXGB_ENOMEM, "workspace allocation failed");
  const int64_t fsz = (int64_t)C * g.per * cb;
  float2* q = (float2*)ws;
  StageBufs sb{};
  sb.U = q;
  q += fsz;
  if (P.order == 2 || P.order == 3) {
    sb.S = q;
    sb.N0 = q + fsz;
    if (P.order == 3) sb.N1 = q + 2 * fsz;
  } else if (P.order == 4) {
    sb.S1 = q;
    sb.S = q + fsz;
    sb.N0 = q + 2 * fsz;
    sb.N1 = q + 3 * fsz;
    sb.N2 = q + 4 * fsz;
  }
  q = (float2*)ws + (int64_t)nb * fsz;
  float2* WH = q;  // NI spectra before the inverse transforms, NF after the forward ones
  float* Ph = (float*)(WH + (int64_t)SP * g.per * cb);
  float* Qp = Ph + (int64_t)p.NI * g.npts * cb;
  const int nst = nonlinear_only ? 1 : P.order;
  const int Q = nonlinear_only ? 1 : nsteps * P.order;
  for (int64_t b0 = 0; b0 < batch; b0 += cb) {
    const int64_t n = std::min<int64_t>(cb, batch - b0);
    const float2* src = in + b0 * C * g.per;
    float2* dst = out + b0 * C * g.per;
    EXGB_CUDA(cudaMemcpyAsync(sb.U, src, sizeof(float2) * C * g.per * n, cudaMemcpyDeviceToDevice, st));
    for (int qq = 0; qq < Q; ++qq) {
      const int stage = qq % nst;
      const float2* xin = (stage == 0) ? sb.U : (P.order == 4 && stage == 1) ? sb.S1 : sb.S;
      derive_kernel<<<grid_for(n * g.per, sm), 256, 0, st>>>(g, p, n, xin, WH);
      int rc = irfftn_impl(st, g.D, g.N, n * p.NI, WH, Ph);
      if (rc) return rc;
      pointwise_kernel<<<grid_for(n * g.npts, sm), 256, 0, st>>>(g, p, n, Ph, Qp);
      rc = rfftn_impl(st, g.D, g.N, n * p.NF, Qp, WH);
      if (rc) return rc;
      if (nonlinear_only) {
        combine_kernel<<<grid_for(n * g.per, sm), 256, 0, st>>>(P, g, p, n, WH, sb, -1, dst);
      } else {
        combine_kernel<<<grid_for(n * g.per, sm), 256, 0, st>>>(P, g, p, n, WH, sb, stage, nullptr);
        if (stage == nst - 1 && project)
          project_kernel<<<grid_for(n * C * 2 * (g.per / g.M), sm), 256, 0, st>>>(g, n * C, sb.U);
      }
      EXGB_CUDA(cudaGetLastError());
    }
    if (!nonlinear_only)
      EXGB_CUDA(cudaMemcpyAsync(dst, sb.U, sizeof(float2) * C * g.per * n, cudaMemcpyDeviceToDevice, st));
  }
  return EXGB_OK;
}

}  // namespace exgb
