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
#include "exgb_ndops.cuh"
#include "exgb_stage.cuh"

namespace exgb {

void* workspace(size_t bytes, int slot_offset);
int rfftn_impl(cudaStream_t st, int D, int N, int64_t count, const float* in, float2* out);
int irfftn_impl(cudaStream_t st, int D, int N, int64_t count, const float2* in, float* out);

namespace ndg {

// W[b][f] = the NI spectra whose inverse transforms the pointwise step needs
__global__ void derive_kernel(Geo g, Prog p, int64_t cb, const float2* __restrict__ X, float2* __restrict__ W) {
  const int64_t total = cb * g.per;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = t / g.per, r = t - b * g.per;
    int k[3];
    mode_of(g, r, k);
    const bool m = kept(g, k);
    derive_mode(g, p, k, m, X + b * g.C * g.per + r, g.per, W + b * p.NI * g.per + r, g.per);
  }
}

// Physical fields Ph[b][0..NI) -> products Q[b][0..NF) at every grid point.
__global__ void pointwise_kernel(Geo g, Prog p, int64_t cb, const float* __restrict__ Ph, float* __restrict__ Q) {
  const int64_t total = cb * g.npts;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = t / g.npts, q = t - b * g.npts;
    const float* src = Ph + b * p.NI * g.npts + q;
    float* f = Q + b * p.NF * g.npts + q;
    float in[kMaxNI];
    load_point(src, g.npts, p.NI, in);
    pointwise_point_reg(g, p, in, f, g.npts);
  }
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
    float2 nv[MAXC];
    combine_mode(P, g, p, k, m, H + b * p.NF * g.per + r, g.per, nv);
    const int64_t base = b * g.C * g.per + r;
    if (stage < 0) {
#pragma unroll
      for (int c = 0; c < MAXC; ++c)
        if (c < g.C) nout[base + c * g.per] = nv[c];
      continue;
    }
    // every channel's stage loads in flight together (compile-time channel indices keep nv in registers)
    int64_t so[MAXC], co[MAXC];
#pragma unroll
    for (int c = 0; c < MAXC; ++c) {
      const int cc = c < g.C ? c : 0;
      so[c] = base + cc * g.per;
      co[c] = (P.lin_ch == 1 ? 0 : (int64_t)cc * g.per) + r;
    }
    stage_upd_channels<MAXC>(P, sb, g.C, so, co, stage, nv);
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
    case EXGB_NL_PROJECTED_3D:
    case EXGB_NL_PROJECTED_3D_KOLMOGOROV:
      return d.num_spatial_dims == 3;
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
    case EXGB_NL_PROJECTED_3D:
    case EXGB_NL_PROJECTED_3D_KOLMOGOROV:
      if (D != 3) return fail(EXGB_EUNSUPPORTED, "projected convection needs num_spatial_dims == 3");
      if (C != 3) return fail(EXGB_ESHAPE, "Number of channels in u_hat should match number of spatial dimensions");
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
    case EXGB_NL_PROJECTED_3D:
    case EXGB_NL_PROJECTED_3D_KOLMOGOROV:
      p.op = OP_PROJ3D;
      p.NI = 6;
      p.NF = 3;
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

bool pass2d_supported(int D, int N, int NI, int NF);
int pass2d_run(const exgb_plan* plan, const ndg::Geo& g, const ndg::Prog& p, cudaStream_t st, const float2* in,
               float2* out, int64_t batch, int nsteps, int project, int nonlinear_only);

// Does a 2D staged plan of this description run on the three-pass path (exgb_pass2d.cu)?  Its
// coefficient tables are then column-major, as the fused 2D kernels keep them.
bool ndgen_pass2d(const exgb_plan_desc& d) {
  if (d.num_spatial_dims != 2) return false;
  const Prog p = make_prog(d);
  return pass2d_supported(2, d.num_points, p.NI, p.NF);
}

bool pass3d_supported(int D, int N, int NI, int NF);
int pass3d_run(const exgb_plan* plan, const ndg::Geo& g, const ndg::Prog& p, cudaStream_t st, const float2* in,
               float2* out, int64_t batch, int nsteps, int project, int nonlinear_only);

// Does a 3D staged plan of this description run on the three-pass path (exgb_pass3d.cu)?  Its
// coefficient tables are then plane-major ([lin_ch][kz][kx][ky]).
bool ndgen_pass3d(const exgb_plan_desc& d) {
  if (d.num_spatial_dims != 3 || !ndgen_can(d)) return false;
  const Prog p = make_prog(d);
  return pass3d_supported(3, d.num_points, p.NI, p.NF);
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
  if (P.D == 2 && plan->tables_transposed)
    return pass2d_run(plan, g, p, st, in, out, batch, nsteps, project, nonlinear_only);
  if (P.D == 3 && plan->tables_transposed)
    return pass3d_run(plan, g, p, st, in, out, batch, nsteps, project, nonlinear_only);
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
