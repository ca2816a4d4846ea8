// exgb_step.cu -- stepping entry points of the C ABI: dispatch between the
// fused 1D kernel, the 2D cluster kernel, the 3D path, the staged N-D path
// and the linear (ETDRK0) kernel, and
// the physical-space wrappers (rfftn -> Fourier steps -> irfftn).
#include <cuda_runtime.h>

#include <algorithm>

#include "exgb_internal.h"

namespace exgb {

void* workspace(size_t bytes, int slot_offset);
int rfftn_impl(cudaStream_t st, int D, int N, int64_t count, const float* in, float2* out);
int irfftn_impl(cudaStream_t st, int D, int N, int64_t count, const float2* in, float* out);

// ETDRK0 (etdrk/_etdrk_0.py:30-34) for 2D fields: u^ <- E u^, nsteps times,
// with the c2r projection on ky = 0 and ky = N/2 after every step when
// `project` is set.  One thread per {kx, N-kx} pair of one column.
__global__ void etdrk0_2d_kernel(const float2* __restrict__ E, int transposed, int N, int lin_ch, int C,
                                 int64_t batch, const float2* in, float2* out, int nsteps, int project) {
  const int M = N / 2 + 1, half = N / 2 + 1;
  const int64_t per_field = (int64_t)M * half;
  const int64_t total = per_field * C * batch;
  const bool even = (N & 1) == 0;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t field = t / per_field;  // b * C + ch
    const int64_t r = t - field * per_field;
    const int ky = (int)(r / half), kx = (int)(r - (int64_t)ky * half);
    const int ch = (int)(field % C);
    const int kx2 = (kx == 0) ? 0 : N - kx;
    if (kx2 < kx) continue;  // pair handled by the smaller index (N odd: kx2 > kx always)
    const int lc = lin_ch == 1 ? 0 : ch;
    const int64_t tb = (int64_t)lc * N * M;
    const int64_t e1 = transposed ? tb + (int64_t)ky * N + kx : tb + (int64_t)kx * M + ky;
    const int64_t e2 = transposed ? tb + (int64_t)ky * N + kx2 : tb + (int64_t)kx2 * M + ky;
    const float2 E1 = E[e1], E2 = E[e2];
    const float2* src = in + field * (int64_t)N * M;
    float2* dst = out + field * (int64_t)N * M;
    float2 v1 = src[(int64_t)kx * M + ky];
    float2 v2 = src[(int64_t)kx2 * M + ky];
    const bool proj = project && (ky == 0 || (even && ky == N / 2));
    for (int s = 0; s < nsteps; ++s) {
      v1 = cmul(E1, v1);
      v2 = cmul(E2, v2);
      if (proj) {
        const float2 p = make_float2(0.5f * (v1.x + v2.x), 0.5f * (v1.y - v2.y));
        v1 = p;
        v2 = cconj(p);
      }
    }
    dst[(int64_t)kx * M + ky] = v1;
    if (kx2 != kx) dst[(int64_t)kx2 * M + ky] = v2;
  }
}

// ETDRK0 for 1D fields of N/2+1 modes: u^ <- E u^, nsteps times; the c2r projection keeps the real
// part of the k = 0 and (N even) k = N/2 modes.  One thread per mode.
__global__ void etdrk0_1d_kernel(const float2* __restrict__ E, int N, int lin_ch, int C, int64_t batch,
                                 const float2* in, float2* out, int nsteps, int project) {
  const int M = N / 2 + 1;
  const int64_t total = (int64_t)M * C * batch;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t field = t / M;
    const int k = (int)(t - field * M);
    const int lc = lin_ch == 1 ? 0 : (int)(field % C);
    const float2 e = E[(int64_t)lc * M + k];
    const bool proj = project && (k == 0 || ((N & 1) == 0 && k == N / 2));
    float2 v = in[t];
    for (int s = 0; s < nsteps; ++s) {
      v = cmul(e, v);
      if (proj) v.y = 0.f;
    }
    out[t] = v;
  }
}

int etdrk0_apply(const exgb_plan* plan, cudaStream_t st, const float2* in, float2* out, int64_t batch, int nsteps,
                 int project) {
  const PlanDev& P = plan->dev;
  if (P.D == 1) {
    const int64_t total = (int64_t)P.M * P.C * batch;
    const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, (int64_t)plan->sm_count * 16));
    etdrk0_1d_kernel<<<blocks, 256, 0, st>>>(P.E, P.N, P.lin_ch, P.C, batch, in, out, nsteps, project);
    EXGB_CUDA(cudaGetLastError());
    return EXGB_OK;
  }
  const int transposed = (P.D == 2 && P.order >= 1) ? 1 : 0;
  const int64_t total = (int64_t)(P.N / 2 + 1) * (P.N / 2 + 1) * P.C * batch;
  if (total <= 0) return EXGB_OK;
  const int th = 256;
  const unsigned blocks = (unsigned)std::min<int64_t>((total + th - 1) / th, (int64_t)plan->sm_count * 16);
  etdrk0_2d_kernel<<<blocks, th, 0, st>>>(P.E, transposed, P.N, P.lin_ch, P.C, batch, in, out, nsteps, project);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

static bool linear_only(const PlanDev& P) { return P.order == 0 || P.kind == EXGB_NL_ZERO; }

// 1D plans stepped by the fused 1D kernel: N = 2^a 3^b 5^c and one instance fits in a CTA's shared
// memory (the other 1D plans run on the staged path or, when linear, on etdrk0_1d_kernel)
static bool fused1d(const exgb_plan* plan) {
  const PlanDev& P = plan->dev;
  return P.D == 1 && !plan->staged && P.fft.n > 0 && etdrk1d_fits(P.N, P.order);
}

int steps3d_run(const exgb_plan* plan, cudaStream_t st, const float2* in, float2* out, int64_t batch, int nsteps,
                int project, int nonlinear_only);

// Fourier-space multi-step for the plans without a fused 1D kernel: staged
// N-D plans, 2D and 3D.
static int fourier_steps_2d(const exgb_plan* plan, cudaStream_t st, const float2* in, float2* out, int64_t batch,
                            int nsteps, int project) {
  if (plan->staged) return ndgen_run(plan, st, in, out, batch, nsteps, project, 0);
  if (plan->dev.D == 3) return steps3d_run(plan, st, in, out, batch, nsteps, project, 0);
  if (linear_only(plan->dev)) return etdrk0_apply(plan, st, in, out, batch, nsteps, project);
  return etdrk2d_run(plan, st, in, out, batch, nsteps, project, 0);
}

static size_t hat_elems(const PlanDev& P, int64_t batch) {
  size_t e = (size_t)batch * P.C * (P.N / 2 + 1);
  for (int i = 0; i < P.D - 1; ++i) e *= (size_t)P.N;
  return e;
}
static size_t phys_elems(const PlanDev& P, int64_t batch) {
  size_t e = (size_t)batch * P.C;
  for (int i = 0; i < P.D; ++i) e *= (size_t)P.N;
  return e;
}

}  // namespace exgb

using namespace exgb;

extern "C" {

int exgb_step_fourier(const exgb_plan* plan, void* stream, const void* u_hat_in, void* u_hat_out, int64_t batch) {
  return exgb_repeat_fourier(plan, stream, u_hat_in, u_hat_out, batch, 1);
}

int exgb_repeat_fourier(const exgb_plan* plan, void* stream, const void* u_hat0, void* u_hat_out, int64_t batch,
                        int32_t nsteps) {
  if (!plan) return fail(EXGB_EINVAL, "NULL argument");
  if (batch < 0 || nsteps < 0) return fail(EXGB_EINVAL, "negative batch or nsteps");
  if (batch == 0) return EXGB_OK;  // an empty batch touches no memory (its pointers may be NULL)
  if (!u_hat0 || !u_hat_out) return fail(EXGB_EINVAL, "NULL argument");
  cudaStream_t st = (cudaStream_t)stream;
  if (nsteps == 0) {  // zero steps return the state itself, bit for bit
    if (u_hat_out != u_hat0)
      EXGB_CUDA(cudaMemcpyAsync(u_hat_out, u_hat0, sizeof(float2) * hat_elems(plan->dev, batch),
                                cudaMemcpyDeviceToDevice, st));
    return EXGB_OK;
  }
  if (fused1d(plan))
    return etdrk1d_run(plan, st, nullptr, (const float2*)u_hat0, nullptr, (float2*)u_hat_out, batch, nsteps, 0, 0, 0,
                       0);
  return fourier_steps_2d(plan, st, (const float2*)u_hat0, (float2*)u_hat_out, batch, nsteps, 0);
}

int exgb_nonlinear(const exgb_plan* plan, void* stream, const void* u_hat_in, void* n_hat_out, int64_t batch) {
  if (!plan) return fail(EXGB_EINVAL, "NULL argument");
  if (batch < 0) return fail(EXGB_EINVAL, "negative batch");
  if (batch == 0) return EXGB_OK;
  if (!u_hat_in || !n_hat_out) return fail(EXGB_EINVAL, "NULL argument");
  cudaStream_t st = (cudaStream_t)stream;
  const PlanDev& P = plan->dev;
  if (P.kind == EXGB_NL_ZERO || P.order == 0) {
    EXGB_CUDA(cudaMemsetAsync(n_hat_out, 0, sizeof(float2) * hat_elems(P, batch), st));
    return EXGB_OK;
  }
  if (plan->staged) return ndgen_run(plan, st, (const float2*)u_hat_in, (float2*)n_hat_out, batch, 0, 0, 1);
  if (P.D == 3) return steps3d_run(plan, st, (const float2*)u_hat_in, (float2*)n_hat_out, batch, 0, 0, 1);
  if (fused1d(plan))
    return etdrk1d_run(plan, st, nullptr, (const float2*)u_hat_in, nullptr, (float2*)n_hat_out, batch, 0, 0, 0, 0,
                       1);
  return etdrk2d_run(plan, st, (const float2*)u_hat_in, (float2*)n_hat_out, batch, 0, 0, 1);
}

int exgb_repeat(const exgb_plan* plan, void* stream, const float* u0, float* u_out, int64_t batch, int32_t nsteps) {
  if (!plan) return fail(EXGB_EINVAL, "NULL argument");
  if (batch < 0 || nsteps < 0) return fail(EXGB_EINVAL, "negative batch or nsteps");
  if (batch == 0) return EXGB_OK;
  if (!u0 || !u_out) return fail(EXGB_EINVAL, "NULL argument");
  cudaStream_t st = (cudaStream_t)stream;
  const PlanDev& P = plan->dev;
  if (nsteps == 0) {  // zero steps return the state itself, bit for bit
    if (u_out != u0)
      EXGB_CUDA(cudaMemcpyAsync(u_out, u0, sizeof(float) * phys_elems(P, batch), cudaMemcpyDeviceToDevice, st));
    return EXGB_OK;
  }
  if (fused1d(plan)) return etdrk1d_run(plan, st, u0, nullptr, u_out, nullptr, batch, nsteps, 1, 0, 0, 0);
  float2* hat = (float2*)workspace(sizeof(float2) * hat_elems(P, batch), 2);
  if (!hat) return fail(EXGB_ENOMEM, "workspace allocation failed");
  int rc = rfftn_impl(st, P.D, P.N, batch * P.C, u0, hat);
  if (rc) return rc;
  rc = fourier_steps_2d(plan, st, hat, hat, batch, nsteps, 1);
  if (rc) return rc;
  return irfftn_impl(st, P.D, P.N, batch * P.C, hat, u_out);
}

int exgb_step(const exgb_plan* plan, void* stream, const float* u_in, float* u_out, int64_t batch) {
  return exgb_repeat(plan, stream, u_in, u_out, batch, 1);
}

int exgb_rollout(const exgb_plan* plan, void* stream, const float* u0, float* traj, int64_t batch, int32_t nsteps,
                 int32_t include_init) {
  if (!plan) return fail(EXGB_EINVAL, "NULL argument");
  if (batch < 0 || nsteps < 0) return fail(EXGB_EINVAL, "negative batch or nsteps");
  if (batch == 0) return EXGB_OK;
  if (!u0 || !traj) return fail(EXGB_EINVAL, "NULL argument");
  cudaStream_t st = (cudaStream_t)stream;
  const PlanDev& P = plan->dev;
  if (fused1d(plan))
    return etdrk1d_run(plan, st, u0, nullptr, traj, nullptr, batch, nsteps, 1, 1, include_init ? 1 : 0, 0);
  const int T = nsteps + (include_init ? 1 : 0);
  const size_t frame = phys_elems(P, 1);  // floats per sample
  const size_t pitch = sizeof(float) * frame * T;
  if (include_init)
    EXGB_CUDA(cudaMemcpy2DAsync(traj, pitch, u0, sizeof(float) * frame, sizeof(float) * frame, (size_t)batch,
                                cudaMemcpyDeviceToDevice, st));
  if (nsteps == 0) return EXGB_OK;
  float2* hat = (float2*)workspace(sizeof(float2) * hat_elems(P, batch), 2);
  float* tmp = (float*)workspace(sizeof(float) * phys_elems(P, batch), 3);
  if (!hat || !tmp) return fail(EXGB_ENOMEM, "workspace allocation failed");
  int rc = rfftn_impl(st, P.D, P.N, batch * P.C, u0, hat);
  if (rc) return rc;
  for (int t = 0; t < nsteps; ++t) {
    rc = fourier_steps_2d(plan, st, hat, hat, batch, 1, 1);
    if (rc) return rc;
    rc = irfftn_impl(st, P.D, P.N, batch * P.C, hat, tmp);
    if (rc) return rc;
    float* dst = traj + (size_t)(t + (include_init ? 1 : 0)) * frame;
    EXGB_CUDA(cudaMemcpy2DAsync(dst, pitch, tmp, sizeof(float) * frame, sizeof(float) * frame, (size_t)batch,
                                cudaMemcpyDeviceToDevice, st));
  }
  return EXGB_OK;
}

}  // extern "C"
