// exgb_api.cu -- C ABI entry points, plan construction and the FP64
// phi-coefficient kernel of libexgb.so.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "exgb_internal.h"

namespace exgb {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  g_last_error = std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e);
  return EXGB_ECUDA;
}

// Factor n into radices 8, 4, 2, 5, 3 (largest power-of-two radices first).
bool make_fft_plan(int n, FftPlan* p) {
  if (n < 1) return false;
  p->n = n;
  p->npass = 0;
  int m = n;
  while (m % 8 == 0 && m > 4) {
    // keep a radix-4 or radix-2 tail instead of a trailing radix-8 when
    // fewer passes do not result
    p->radix[p->npass++] = 8;
    m /= 8;
    if (p->npass >= kMaxPass) return false;
  }
  while (m % 4 == 0) {
    p->radix[p->npass++] = 4;
    m /= 4;
    if (p->npass >= kMaxPass) return false;
  }
  while (m % 2 == 0) {
    p->radix[p->npass++] = 2;
    m /= 2;
    if (p->npass >= kMaxPass) return false;
  }
  while (m % 5 == 0) {
    p->radix[p->npass++] = 5;
    m /= 5;
    if (p->npass >= kMaxPass) return false;
  }
  while (m % 3 == 0) {
    p->radix[p->npass++] = 3;
    m /= 3;
    if (p->npass >= kMaxPass) return false;
  }
  if (m != 1) return false;
  if (p->npass == 0) {  // n == 1: identity (one trivial radix-... pass is not needed)
    return false;
  }
  fft_plan_finalize(p);
  return true;
}

int build_twiddles(int n, float2** d_tw) {
  std::vector<float2> h(n);
  for (int k = 0; k < n; ++k) {
    // exp(-2 pi i k / n), evaluated in double and rounded once
    const double a = -2.0 * M_PI * (double)k / (double)n;
    h[k] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
  EXGB_CUDA(cudaMalloc(d_tw, sizeof(float2) * n));
  EXGB_CUDA(cudaMemcpy(*d_tw, h.data(), sizeof(float2) * n, cudaMemcpyHostToDevice));
  return EXGB_OK;
}

// ---------------------------------------------------------------- FP64 coefficients
__device__ __forceinline__ double2 zmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 zdiv(double2 a, double2 b) {
  // scaled division to avoid overflow of |b|^2 for stiff modes
  const double s = fmax(fabs(b.x), fabs(b.y));
  if (s == 0.0) {
    const double inf = __longlong_as_double(0x7ff0000000000000ULL);
    return make_double2(a.x * inf, a.y * inf);
  }
  const double bx = b.x / s, by = b.y / s;
  const double d = bx * bx + by * by;
  const double ax = a.x / s, ay = a.y / s;
  return make_double2((ax * bx + ay * by) / d, (ay * bx - ax * by) / d);
}
__device__ __forceinline__ double2 zexp(double2 z) {
  double s, c;
  sincos(z.y, &s, &c);
  const double e = exp(z.x);
  return make_double2(e * c, e * s);
}
__device__ __forceinline__ double2 zadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 zsub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 zs(double s) { return make_double2(s, 0.0); }

// One thread per mode.  Reference: etdrk/_base_etdrk.py:62 (E), the scan
// bodies of etdrk/_etdrk_1.py:69-76, _etdrk_2.py:77-89, _etdrk_3.py:161-189,
// _etdrk_4.py:175-196 (contour means, real part), _etdrk_3/4 :156/:170 (E_half).
// Output index: same as input (1D, or 2D row-major) or ky-major for 2D
// when `transpose_2d` is set.
__global__ void coef_kernel(const double2* __restrict__ L, int64_t total, int N, int M, int layout, double dt,
                            int ncp, double radius, int order, float2* __restrict__ E, float2* __restrict__ Eh,
                            float* __restrict__ c, int64_t nmodes_all) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  int64_t o = i;
  if (layout == 1) {
    const int64_t per = (int64_t)N * M;
    const int64_t ch = i / per;
    const int64_t r = i - ch * per;
    const int64_t kx = r / M, ky = r - kx * M;
    o = ch * per + ky * N + kx;
  } else if (layout == 2) {
    const int64_t pl = (int64_t)N * N, per = pl * M;
    const int64_t ch = i / per;
    const int64_t r = i - ch * per;
    const int64_t q = r / M, kz = r - q * M;  // q = kx N + ky
    o = ch * per + kz * pl + q;
  }
  const double2 Ldt = make_double2(L[i].x * dt, L[i].y * dt);
  const double2 e = zexp(Ldt);
  const double2 eh = zexp(make_double2(0.5 * Ldt.x, 0.5 * Ldt.y));
  E[o] = make_float2((float)e.x, (float)e.y);
  Eh[o] = make_float2((float)eh.x, (float)eh.y);
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (int j = 1; j <= ncp; ++j) {
    double s, co;
    sincospi(2.0 * ((double)j - 0.5) / (double)ncp, &s, &co);
    const double2 lr = make_double2(radius * co + Ldt.x, radius * s + Ldt.y);
    const double2 el = zexp(lr);
    const double2 elh = zexp(make_double2(0.5 * lr.x, 0.5 * lr.y));
    const double2 lr2 = zmul(lr, lr);
    const double2 lr3 = zmul(lr2, lr);
    if (order == 1 || order == 2) {
      acc[0] += zdiv(zsub(el, zs(1.0)), lr).x;
      if (order == 2) acc[1] += zdiv(zsub(zsub(el, zs(1.0)), lr), lr2).x;
    } else if (order == 3 || order == 4) {
      acc[0] += zdiv(zsub(elh, zs(1.0)), lr).x;
      // (-4 - lr + e (4 - 3 lr + lr^2)) / lr^3
      const double2 p4 = zadd(zsub(zs(4.0), make_double2(3.0 * lr.x, 3.0 * lr.y)), lr2);
      const double2 cA = zdiv(zadd(zsub(zs(-4.0), lr), zmul(el, p4)), lr3);
      // (-4 - 3 lr - lr^2 + e (4 - lr)) / lr^3
      const double2 cC = zdiv(zadd(zsub(zsub(zs(-4.0), make_double2(3.0 * lr.x, 3.0 * lr.y)), lr2),
                                   zmul(el, zsub(zs(4.0), lr))),
                              lr3);
      // (2 + lr + e (-2 + lr)) / lr^3
      const double2 cB = zdiv(zadd(zadd(zs(2.0), lr), zmul(el, zadd(zs(-2.0), lr))), lr3);
      if (order == 3) {
        acc[1] += zdiv(zsub(el, zs(1.0)), lr).x;
        acc[2] += cA.x;
        acc[3] += 4.0 * cB.x;
        acc[4] += cC.x;
      } else {
        acc[3] += cA.x;
        acc[4] += cB.x;
        acc[5] += cC.x;
      }
    }
  }
  for (int q = 0; q < 6; ++q) c[q * nmodes_all + o] = (float)(dt * (acc[q] / (double)ncp));
  if (order == 4) {
    const float c1 = (float)(dt * (acc[0] / (double)ncp));
    c[1 * nmodes_all + o] = c1;  // coef_2 = coef_1 (etdrk/_etdrk_4.py:192)
    c[2 * nmodes_all + o] = c1;  // coef_3 = coef_1 (:193)
  }
}

// Largest integer k >= 0 with float(k) <= float(fraction * (N//2) - 1); the
// comparison happens in float32 as in the reference (nonlin_fun/_base.py:59-71
// with _spectral.py:331-337 under JAX's default float32).
static int dealias_kmax(double fraction, int N) {
  if (fraction < 0) return N;  // no mask
  const double cutoff = fraction * (double)(N / 2) - 1.0;
  const float cf = (float)cutoff;
  int k = -1;
  while (k + 1 <= N / 2 && (float)(k + 1) <= cf) ++k;
  return k;
}

static bool factorable(int n) {
  if (n < 2) return false;
  for (int p : {2, 3, 5})
    while (n % p == 0) n /= p;
  return n == 1;
}

}  // namespace exgb

using namespace exgb;

extern "C" {

int exgb_version(void) { return EXGB_VERSION; }

const char* exgb_last_error(void) { return g_last_error.c_str(); }

int exgb_device_info(int* sm_count, int* cc_major, int* cc_minor) {
  int dev = 0;
  EXGB_CUDA(cudaGetDevice(&dev));
  if (sm_count) EXGB_CUDA(cudaDeviceGetAttribute(sm_count, cudaDevAttrMultiProcessorCount, dev));
  if (cc_major) EXGB_CUDA(cudaDeviceGetAttribute(cc_major, cudaDevAttrComputeCapabilityMajor, dev));
  if (cc_minor) EXGB_CUDA(cudaDeviceGetAttribute(cc_minor, cudaDevAttrComputeCapabilityMinor, dev));
  return EXGB_OK;
}

int exgb_plan_destroy(exgb_plan* plan) {
  if (!plan) return EXGB_OK;
  cudaFree(plan->d_dev);
  cudaFree(plan->d_tw);
  cudaFree(plan->d_E);
  cudaFree(plan->d_Eh);
  cudaFree(plan->d_c);
  cudaFree(plan->d_scratch);
  cudaFree(plan->d_scratch_tail);
  cudaFree(plan->d_tc_scratch);
  cudaFree(plan->d_status);
  delete plan;
  return EXGB_OK;
}

int exgb_plan_create(const exgb_plan_desc* desc, exgb_plan** out) {
  if (!desc || !out) return fail(EXGB_EINVAL, "exgb_plan_create: NULL argument");
  *out = nullptr;
  const exgb_plan_desc& d = *desc;
  if (d.num_spatial_dims < 1 || d.num_spatial_dims > 3)
    return fail(EXGB_EUNSUPPORTED, "num_spatial_dims must be 1, 2 or 3");
  if (d.order < 0 || d.order > 4)
    return fail(EXGB_ENOTIMPL, "Order " + std::to_string(d.order) + " not implemented.");
  if (d.num_points < 2) return fail(EXGB_EINVAL, "num_points must be >= 2");
  {
    // every N the transforms take: 2^a 3^b 5^c (any length in 1D), other N through Bluestein
    const int trc = transform_supported(d.num_points);
    if (trc) return trc;
  }
  if (d.num_channels < 1) return fail(EXGB_ESHAPE, "num_channels must be >= 1");
  if (d.linear_operator_channels != 1 && d.linear_operator_channels != d.num_channels)
    return fail(EXGB_ESHAPE, "linear operator must have 1 or num_channels channels");
  if (!d.linear_operator) return fail(EXGB_EINVAL, "linear_operator is NULL");
  if (d.num_circle_points < 1) return fail(EXGB_EINVAL, "num_circle_points must be >= 1");
  if (d.num_poly < 0 || d.num_poly > 8) return fail(EXGB_EINVAL, "at most 8 polynomial coefficients");
  const int D = d.num_spatial_dims, N = d.num_points, M = N / 2 + 1;
  const bool nonlinear = d.order >= 1 && d.nonlin_kind != EXGB_NL_ZERO;

  // supported (D, kind) combinations of this build.  The fused kernels take N = 2^a 3^b 5^c (1D: one
  // instance in one CTA's shared memory; 2D vorticity: N <= 1024); other sizes of the 1D
  // nonlinearities and of 2D vorticity are stepped by the staged path on the general transforms.
  const bool smooth = factorable(d.num_points);
  bool staged = ndgen_handles(d);
  if (!staged && d.order >= 1 && d.nonlin_kind != EXGB_NL_ZERO && ndgen_can(d)) {
    if (d.num_spatial_dims == 1 && d.nonlin_kind <= EXGB_NL_GENERAL)
      staged = !smooth || !etdrk1d_fits(d.num_points, d.order);
    else if (d.num_spatial_dims == 2 &&
             (d.nonlin_kind == EXGB_NL_VORTICITY_2D || d.nonlin_kind == EXGB_NL_VORTICITY_2D_KOLMOGOROV)) {
      // The fused kernels win up to N = 256 (register FFTs at 64 / 128 / 256, the generic cluster
      // kernel in between); from N = 320 on the three-pass path wins (measured at 512^2: 1.06e10
      // against 6.9e9 DOF-steps/s).  EXGB_2D_PATH=fused / staged overrides the choice where the
      // other path can hold the plan (a comparison knob; both compute the same arithmetic).
      const int N = d.num_points;
      const char* path = getenv("EXGB_2D_PATH");
      const std::string pick = path ? std::string(path) : std::string();
      const bool reg = (N == 64 || N == 128 || N == 256);
      bool want_staged = !reg && N >= 320;
      if (pick == "fused") want_staged = false;
      if (pick == "staged") want_staged = true;
      staged = !smooth || N > 1024 || (want_staged && ndgen_pass2d(d));
    } else if (d.num_spatial_dims == 3 &&
               (d.nonlin_kind == EXGB_NL_PROJECTED_3D || d.nonlin_kind == EXGB_NL_PROJECTED_3D_KOLMOGOROV)) {
      // 3D projected convection runs on the three-pass path where it holds the plan (N = 32, 64),
      // on the five-kernel path of exgb_3d.cu otherwise; EXGB_3D_PATH=generic forces the latter
      const char* path = getenv("EXGB_3D_PATH");
      staged = !(path && std::string(path) == "generic") && ndgen_pass3d(d);
    }
  }
  if (d.order >= 1 && d.nonlin_kind != EXGB_NL_ZERO) {
    if (d.nonlin_kind < EXGB_NL_ZERO || d.nonlin_kind > EXGB_NL_BELOUSOV_ZHABOTINSKY)
      return fail(EXGB_EINVAL, "unknown nonlinear function");
    if (staged) {
      const int rc = ndgen_validate(d);
      if (rc) return rc;
    } else if (D == 1) {
      if (d.nonlin_kind > EXGB_NL_GENERAL)
        return fail(EXGB_EUNSUPPORTED, "this nonlinear function needs num_spatial_dims == 2 or 3");
      if (d.num_channels != 1) return fail(EXGB_ESHAPE, "Number of channels in u_hat should match number of spatial dimensions");
    } else if (d.nonlin_kind == EXGB_NL_VORTICITY_2D || d.nonlin_kind == EXGB_NL_VORTICITY_2D_KOLMOGOROV) {
      if (D != 2) return fail(EXGB_EUNSUPPORTED, "vorticity convection needs num_spatial_dims == 2");
      if (d.num_channels != 1) return fail(EXGB_ESHAPE, "vorticity formulation has one channel");
    } else {
      if (D != 3) return fail(EXGB_EUNSUPPORTED, "projected convection needs num_spatial_dims == 3");
      if (d.num_channels != 3)
        return fail(EXGB_ESHAPE, "Number of channels in u_hat should match number of spatial dimensions");
    }
  }

  exgb_plan* p = new exgb_plan();
  p->desc = d;
  p->staged = staged ? 1 : 0;
  p->desc.linear_operator = nullptr;  // host pointer not retained
  PlanDev& v = p->dev;
  std::memset(&v, 0, sizeof(v));
  v.D = D;
  v.N = N;
  v.M = M;
  v.rN = (float)(1.0 / (double)N);
  v.C = d.num_channels;
  v.order = d.order;
  v.kind = nonlinear ? d.nonlin_kind : EXGB_NL_ZERO;
  v.lin_ch = d.linear_operator_channels;
  v.kmax = (d.nonlin_kind == EXGB_NL_ZERO) ? N : dealias_kmax(d.dealiasing_fraction, N);
  v.kscale = (float)(2.0 * M_PI / d.domain_extent);
  v.inj_mode = -1;
  {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&p->sm_count, cudaDevAttrMultiProcessorCount, dev);
  }

  // length-N plan and twiddles of the fused kernels (N = 2^a 3^b 5^c); the staged, 3D and
  // linear paths go through the general transforms instead
  int rc = EXGB_OK;
  if (smooth) {
    if (!make_fft_plan(N, &v.fft)) {
      exgb_plan_destroy(p);
      return fail(EXGB_ENOTFACTORABLE, "cannot build an FFT plan for N=" + std::to_string(N));
    }
    rc = build_twiddles(N, &p->d_tw);
    if (rc) {
      exgb_plan_destroy(p);
      return rc;
    }
    v.tw = p->d_tw;
  }

  // nonlinear parameters
  const float b = (float)d.scale;
  switch (v.kind) {
    case EXGB_NL_CONVECTION:
      if (d.conservative) v.alpha = -0.5f * b;
      else v.beta = -b;
      break;
    case EXGB_NL_GRADIENT_NORM:
      v.gamma = -0.5f * b;
      v.zero_mode_fix = d.zero_mode_fix;
      break;
    case EXGB_NL_POLYNOMIAL:
      v.npoly = d.num_poly;
      for (int i = 0; i < d.num_poly; ++i) v.poly[i] = (float)d.poly[i];
      break;
    case EXGB_NL_GENERAL:
      v.npoly = 3;
      v.poly[2] = (float)d.scale_list[0];
      v.alpha = 0.5f * (float)d.scale_list[1];
      v.gamma = 0.5f * (float)d.scale_list[2];
      v.zero_mode_fix = d.zero_mode_fix;
      break;
    case EXGB_NL_VORTICITY_2D_KOLMOGOROV: {
      const int k = d.injection_mode;
      if (k < 0 || k > v.kmax) {
        exgb_plan_destroy(p);
        return fail(EXGB_EUNSUPPORTED, "injection_mode must lie inside the dealiasing mask");
      }
      // coef_extraction scaling at (kx=0, ky=k): N * (N or N/2) (_spectral.py:403-457)
      const double right = (k == 0 || (N % 2 == 0 && k == N / 2)) ? (double)N : (double)N / 2.0;
      v.inj_mode = k;
      v.inj_value = (float)(-(double)k * d.injection_scale * ((double)N * right));
    }
      // fall through
    case EXGB_NL_VORTICITY_2D:
      v.conv_scale = b;
      break;
    case EXGB_NL_PROJECTED_3D_KOLMOGOROV: {
      const int k = d.injection_mode;
      if (k < 0 || k > N / 2) {
        exgb_plan_destroy(p);
        return fail(EXGB_EUNSUPPORTED, "injection_mode out of range");
      }
      // coef_extraction scaling at (0, k, 0): N * (N/2 or N) * N, first channel only, no -k factor
      // (nonlin_fun/_projected_convection.py:202-220)
      const double mid = (k == 0 || (N % 2 == 0 && k == N / 2)) ? (double)N : (double)N / 2.0;
      v.inj_mode = k;
      v.inj_value = (float)(d.injection_scale * ((double)N * mid * (double)N));
    } break;
    default:
      break;
  }
  v.needs_ux = (v.beta != 0.f || v.gamma != 0.f);
  v.needs_q = (v.beta != 0.f || v.gamma != 0.f || v.npoly > 0);

  // coefficient tables
  size_t per = (size_t)M;
  for (int i = 0; i < D - 1; ++i) per *= (size_t)N;
  p->n_modes = per;
  const size_t nall = per * (size_t)v.lin_ch;
  // layout of the coefficient tables: 1 = [lin_ch][ky][kx] (2D fused and three-pass paths),
  // 2 = [lin_ch][kz][kx][ky] (3D three-pass path), 0 = natural
  const char* path3 = getenv("EXGB_3D_PATH");
  const bool generic3 = path3 && std::string(path3) == "generic";
  const int transpose = (D == 2 && d.order >= 1 && (!staged || ndgen_pass2d(d)))                  ? 1
                        : (D == 3 && d.order >= 1 && staged && !generic3 && ndgen_pass3d(d)) ? 2
                                                                                              : 0;
  p->tables_transposed = transpose;
  double2* d_L = nullptr;
  cudaError_t e;
  if ((e = cudaMalloc(&d_L, sizeof(double2) * nall)) != cudaSuccess ||
      (e = cudaMalloc(&p->d_E, sizeof(float2) * nall)) != cudaSuccess ||
      (e = cudaMalloc(&p->d_Eh, sizeof(float2) * nall)) != cudaSuccess ||
      (e = cudaMalloc(&p->d_c, sizeof(float) * nall * 6)) != cudaSuccess) {
    cudaFree(d_L);
    exgb_plan_destroy(p);
    return fail(EXGB_ENOMEM, std::string("plan allocation failed: ") + cudaGetErrorString(e));
  }
  if ((e = cudaMemcpy(d_L, d.linear_operator, sizeof(double2) * nall, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemset(p->d_c, 0, sizeof(float) * nall * 6)) != cudaSuccess) {
    cudaFree(d_L);
    exgb_plan_destroy(p);
    return cuda_fail(e, "plan upload");
  }
  {
    const int th = 128;
    const int64_t blocks = ((int64_t)nall + th - 1) / th;
    coef_kernel<<<(unsigned)blocks, th>>>(d_L, (int64_t)nall, N, M, transpose, d.dt, d.num_circle_points,
                                          d.circle_radius, d.order, p->d_E, p->d_Eh, p->d_c, (int64_t)nall);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
  }
  cudaFree(d_L);
  if (e != cudaSuccess) {
    exgb_plan_destroy(p);
    return cuda_fail(e, "coef_kernel");
  }
  v.E = p->d_E;
  v.Eh = p->d_Eh;
  for (int q = 0; q < 6; ++q) v.c[q] = p->d_c + (size_t)q * nall;

  if (D == 2 && v.kind != EXGB_NL_ZERO && !staged) {
    rc = etdrk2d_configure(p);
    if (rc) {
      exgb_plan_destroy(p);
      return rc;
    }
  }
  if ((e = cudaMalloc(&p->d_dev, sizeof(PlanDev))) != cudaSuccess ||
      (e = cudaMemcpy(p->d_dev, &p->dev, sizeof(PlanDev), cudaMemcpyHostToDevice)) != cudaSuccess) {
    exgb_plan_destroy(p);
    return cuda_fail(e, "plan device copy");
  }
  *out = p;
  return EXGB_OK;
}

int exgb_plan_kmax(const exgb_plan* plan) {
  if (!plan) return fail(EXGB_EINVAL, "NULL plan");
  return plan->dev.kmax >= plan->dev.N ? -1 : plan->dev.kmax;
}

int exgb_plan_get_table(const exgb_plan* plan, int which, void* host_out, size_t bytes) {
  if (!plan || !host_out) return fail(EXGB_EINVAL, "NULL argument");
  const size_t nall = plan->n_modes * (size_t)plan->dev.lin_ch;
  const bool cplx = which <= 1;
  const size_t need = nall * (cplx ? sizeof(float2) : sizeof(float));
  if (which < 0 || which > 7) return fail(EXGB_EINVAL, "table index must be 0..7");
  if (bytes != need) return fail(EXGB_ESHAPE, "host buffer has the wrong size");
  const void* src = which == 0 ? (const void*)plan->d_E
                    : which == 1 ? (const void*)plan->d_Eh
                                 : (const void*)(plan->d_c + (size_t)(which - 2) * nall);
  std::vector<char> tmp(need);
  EXGB_CUDA(cudaMemcpy(tmp.data(), src, need, cudaMemcpyDeviceToHost));
  if (plan->tables_transposed == 0) {
    std::memcpy(host_out, tmp.data(), need);
    return EXGB_OK;
  }
  const int N = plan->dev.N, M = plan->dev.M;
  const size_t es = cplx ? sizeof(float2) : sizeof(float);
  char* dst = (char*)host_out;
  if (plan->tables_transposed == 2) {
    const size_t pl = (size_t)N * N, per = pl * M;
    for (int ch = 0; ch < plan->dev.lin_ch; ++ch)
      for (size_t q = 0; q < pl; ++q)
        for (int kz = 0; kz < M; ++kz)
          std::memcpy(dst + (ch * per + q * M + kz) * es, tmp.data() + (ch * per + kz * pl + q) * es, es);
    return EXGB_OK;
  }
  for (int ch = 0; ch < plan->dev.lin_ch; ++ch)
    for (int kx = 0; kx < N; ++kx)
      for (int ky = 0; ky < M; ++ky) {
        const size_t o = (size_t)ch * N * M + (size_t)kx * M + ky;
        const size_t s = (size_t)ch * N * M + (size_t)ky * N + kx;
        std::memcpy(dst + o * es, tmp.data() + s * es, es);
      }
  return EXGB_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- autotuner knobs
extern "C" int exgb_plan_tune(exgb_plan* plan, int kind, const int* values, int n) {
  if (!plan || (n > 0 && !values)) return fail(EXGB_EINVAL, "NULL argument");
  if (kind == EXGB_TUNE_RADICES) {
    if (n < 1 || n > kMaxPass) return fail(EXGB_EINVAL, "bad number of radix passes");
    long prod = 1;
    for (int i = 0; i < n; ++i) {
      const int r = values[i];
      if (r != 2 && r != 3 && r != 4 && r != 5 && r != 8) return fail(EXGB_EINVAL, "radices must be 2, 3, 4, 5 or 8");
      prod *= r;
    }
    if (prod != plan->dev.N) return fail(EXGB_EINVAL, "radices must multiply to N");
    plan->dev.fft.npass = n;
    for (int i = 0; i < n; ++i) plan->dev.fft.radix[i] = values[i];
    fft_plan_finalize(&plan->dev.fft);
    EXGB_CUDA(cudaMemcpy(plan->d_dev, &plan->dev, sizeof(PlanDev), cudaMemcpyHostToDevice));
    return EXGB_OK;
  }
  if (kind == EXGB_TUNE_CLUSTER) {
    if (plan->dev.D != 2 || plan->dev.kind == EXGB_NL_ZERO || plan->dev.order == 0 || plan->staged)
      return fail(EXGB_EUNSUPPORTED, "cluster size applies to 2D vorticity plans");
    const int G = n > 0 ? values[0] : 0;
    if (G < 0 || G > 8) return fail(EXGB_EINVAL, "cluster size must be 1..8 (0 = automatic)");
    EXGB_CUDA(cudaDeviceSynchronize());
    cudaFree(plan->d_scratch);
    plan->d_scratch = nullptr;
    const int old = plan->tune_cluster;
    plan->tune_cluster = G;
    int rc = etdrk2d_configure(plan);
    if (rc || (G && plan->cfg2d.G != G)) {
      cudaFree(plan->d_scratch);
      plan->d_scratch = nullptr;
      plan->tune_cluster = old;
      const int rc2 = etdrk2d_configure(plan);
      if (rc2) return rc2;
      return fail(EXGB_EUNSUPPORTED, "this cluster size does not fit the plan");
    }
    return EXGB_OK;
  }
  if (kind == EXGB_TUNE_PRECISION) {
    const int v = n > 0 ? values[0] : EXGB_DFT_FP32;
    if (v == EXGB_DFT_FP32) {
      plan->precision = 0;
      return EXGB_OK;
    }
    if (v != EXGB_DFT_SPLIT_BF16) return fail(EXGB_EINVAL, "precision must be EXGB_DFT_FP32 or EXGB_DFT_SPLIT_BF16");
    const int rc = tcdft2d_configure(plan);
    if (rc) return rc;
    plan->precision = 1;
    return EXGB_OK;
  }
  if (kind == EXGB_TUNE_WAIT_BUDGET) {
    const long long v = n > 0 ? values[0] : 0;
    if (v < 0) return fail(EXGB_EINVAL, "wait budget must be >= 0 (0 = the normal budget)");
    plan->tc_first_wait_budget = v;
    return EXGB_OK;
  }
  if (kind == EXGB_TUNE_ITEMS_PER_CTA) {
    if (plan->dev.D != 1 || plan->staged)
      return fail(EXGB_EUNSUPPORTED, "items per CTA applies to 1D single-channel plans");
    plan->tune_items_per_cta = n > 0 ? std::max(0, std::min(64, values[0])) : 0;
    return EXGB_OK;
  }
  if (kind == EXGB_TUNE_THREADS) {
    if (plan->dev.D != 1 || plan->staged)
      return fail(EXGB_EUNSUPPORTED, "threads per CTA applies to 1D single-channel plans");
    const int t = n > 0 ? values[0] : 0;
    if (t != 0 && t != 64 && t != 128 && t != 256) return fail(EXGB_EINVAL, "threads per CTA must be 64, 128 or 256 (0 = auto)");
    plan->tune_threads_1d = t;
    return EXGB_OK;
  }
  return fail(EXGB_EINVAL, "unknown tuning kind");
}

extern "C" int exgb_plan_status(const exgb_plan* plan) {
  if (!plan) return fail(EXGB_EINVAL, "NULL plan");
  if (!plan->d_status) return EXGB_OK;
  int h = 0;
  EXGB_CUDA(cudaMemcpy(&h, plan->d_status, sizeof(int), cudaMemcpyDeviceToHost));
  if (h) {
    // read and clear: a later call reports only the waits that gave up after this one
    EXGB_CUDA(cudaMemset(plan->d_status, 0, sizeof(int)));
    return fail(h, "a bounded device wait of the tensor-core kernel gave up");
  }
  return EXGB_OK;
}

extern "C" int exgb_plan_fused_launches(const exgb_plan* plan, int64_t batch, int* launches) {
  if (!plan || !launches) return fail(EXGB_EINVAL, "null plan or output");
  if (batch < 0) return fail(EXGB_EINVAL, "negative batch");
  const PlanDev& P = plan->dev;
  int n = 0;
  if (batch > 0 && P.D == 2 && P.kind != EXGB_NL_ZERO && P.order > 0 && !plan->staged) {
    if (plan->precision == 1 || plan->cfg2d.variant != 1) n = 1;
    else n = vort2d_launches(plan, batch);
  }
  *launches = n;
  return EXGB_OK;
}

extern "C" int exgb_plan_get_tuning(const exgb_plan* plan, int* out, int n) {
  // out[0] = npass, out[1..npass] = radices, then cluster size, items per CTA
  if (!plan || !out || n < 2 + kMaxPass + 1) return fail(EXGB_EINVAL, "bad output buffer");
  out[0] = plan->dev.fft.npass;
  for (int i = 0; i < kMaxPass; ++i) out[1 + i] = i < plan->dev.fft.npass ? plan->dev.fft.radix[i] : 0;
  out[1 + kMaxPass] = plan->cfg2d.G;
  out[2 + kMaxPass] = plan->tune_items_per_cta;
  if (n >= 4 + kMaxPass) out[3 + kMaxPass] = plan->precision;
  if (n >= 5 + kMaxPass) out[4 + kMaxPass] = plan->tune_threads_1d;
  return EXGB_OK;
}
