// exgb_internal.h -- plan object and helpers shared by the .cu files of
// libexgb.so.  Not part of the public ABI (include/exgb.h is).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/exgb.h"
#include "exgb_fft.cuh"

namespace exgb {

// Device-visible, trivially copyable description of a plan.  Kernels get it
// by value (2D) or from a device array (1D work queue).
struct PlanDev {
  int D, N, M, C, order, kind;
  int kmax;        // largest |k| kept by the dealiasing mask on every axis
  int lin_ch;      // 1 or C coefficient sets
  float rN;        // 1/N in FP32 (the c2r scaling of the 1D kernel's packed inverse transforms)
  FftPlan fft;     // length-N complex FFT
  const float2* tw;  // N twiddles exp(-2 pi i k / N)
  // Coefficient tables.  1D: [lin_ch][M].  2D: [lin_ch][ky][kx] (ky-major).
  const float2* E;
  const float2* Eh;
  const float* c[6];
  float kscale;      // 2 pi / L (float32, as the reference's scaled wavenumbers)
  // 1D pseudo-spectral form of every 1D nonlinearity:
  //   N^ = mask . ( alpha ik F[u^2] + F[ beta u u_x + gamma (u_x^2 - zmf*mean) + sum_k poly_k u^k ] )
  float alpha, beta, gamma;
  int zero_mode_fix;
  int npoly;
  float poly[8];
  int needs_ux;      // beta != 0 || gamma != 0
  int needs_q;       // beta, gamma or poly present
  // 2D vorticity
  float conv_scale;  // b (the kernel applies -b)
  float inj_value;   // -k gamma * coef_extraction scaling at (0, k)
  int inj_mode;      // -1: none
};

struct Plan2DConfig {
  int G;        // CTAs per sample (cluster size)
  int threads;  // threads per CTA
  int cols_per_cta;   // masked columns owned by one CTA (max)
  int rows_per_cta;   // physical rows owned by one CTA
  int CB;       // columns per column-phase batch
  int RB;       // rows per row-phase batch (even)
  int mixed_in_smem;
  int variant;   // 0: generic Stockham kernel, 1: register-FFT kernel (compile-time N)
  size_t smem_bytes;
  int clusters;       // persistent clusters launched
  size_t scratch_per_cluster;  // float2 elements of global scratch per cluster
};

}  // namespace exgb

struct exgb_plan {
  exgb_plan_desc desc;
  exgb::PlanDev dev;
  exgb::PlanDev* d_dev = nullptr;  // device copy (for the work queue)
  // owned device allocations
  float2* d_tw = nullptr;
  float2* d_E = nullptr;
  float2* d_Eh = nullptr;
  float* d_c = nullptr;  // 6 contiguous tables
  size_t n_modes = 0;    // modes per coefficient set
  // 2D
  exgb::Plan2DConfig cfg2d{};
  void* d_scratch = nullptr;
  size_t scratch_bytes = 0;
  // 2D register-FFT kernel, automatic cluster choice only: a second configuration with larger
  // clusters (fewer rows per CTA, so a shorter wave) for the samples of a partial last wave;
  // G = 0 when unused
  exgb::Plan2DConfig cfg2d_tail{};
  void* d_scratch_tail = nullptr;
  int sm_count = 0;
  // autotuner overrides (0 = automatic choice)
  int tune_cluster = 0;          // 2D: CTAs per cluster
  int tune_items_per_cta = 0;    // 1D: instances per work item
  int tune_threads_1d = 0;       // 1D: threads per CTA (0 = 256)
  // 2D vorticity transforms: 0 = FP32 register FFTs, 1 = split-BF16 tensor-core DFT
  int precision = 0;
  void* d_tc_scratch = nullptr;
  size_t tc_scratch_per_cta = 0;
  size_t tc_const_offset = 0;    // byte offset of the constant DFT tiles inside d_tc_scratch
  int* d_status = nullptr;       // device wait status of the tensor-core kernel (0 = ok)
  // clock cycles of the tensor-core kernel's first MMA-completion wait per launch (0 = the normal
  // budget); set only by tests, through EXGB_TUNE_WAIT_BUDGET, to make that wait run out
  long long tc_first_wait_budget = 0;
  // stepped by the staged N-D path (exgb_ndgen.cu) instead of a fused kernel
  int staged = 0;
  // coefficient table layout: 0 natural, 1 = 2D [lin_ch][ky][kx] (the fused 2D kernels' and the 2D
  // three-pass layout), 2 = 3D [lin_ch][kz][kx][ky] (the 3D three-pass layout)
  int tables_transposed = 0;
};

namespace exgb {

// thread-local last error
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

#define EXGB_CUDA(call)                                   \
  do {                                                    \
    cudaError_t _e = (call);                              \
    if (_e != cudaSuccess) return exgb::cuda_fail(_e, #call); \
  } while (0)

bool make_fft_plan(int n, FftPlan* p);
int build_twiddles(int n, float2** d_tw);

// launchers (defined in the kernel .cu files)
int launch_rfft1d(cudaStream_t st, const exgb::FftPlan& fp, const float2* tw, int64_t rows, const float* in,
                  float2* out);
int launch_irfft1d(cudaStream_t st, const exgb::FftPlan& fp, const float2* tw, int64_t rows, const float2* in,
                   float* out, float scale);
int launch_cfft_axis(cudaStream_t st, const exgb::FftPlan& fp, const float2* tw, bool inverse, int64_t outer,
                     int64_t outer_stride, int64_t inner, int64_t elem_stride, const float2* in, float2* out,
                     float scale);

int etdrk1d_run(const exgb_plan* plan, cudaStream_t st, const float* u0_phys, const float2* u0_hat,
                float* out_phys, float2* out_hat, int64_t batch, int nsteps, int project, int emit_traj,
                int include_init, int nonlinear_only);
int etdrk2d_run(const exgb_plan* plan, cudaStream_t st, const float2* u_hat_in, float2* u_hat_out, int64_t batch,
                int nsteps, int project, int nonlinear_only);
int etdrk2d_configure(exgb_plan* plan);
int vort2d_configure(exgb_plan* plan);
int vort2d_launches(const exgb_plan* plan, int64_t batch);
int vort2d_run(const exgb_plan* plan, cudaStream_t st, const float2* in, float2* out, int64_t batch, int nsteps,
               int project, int nonlinear_only);
bool tcdft2d_supported(const exgb_plan* plan);
int tcdft2d_configure(exgb_plan* plan);
int tcdft2d_run(const exgb_plan* plan, cudaStream_t st, const float2* in, float2* out, int64_t batch, int nsteps,
                int project, int nonlinear_only);
bool ndgen_handles(const exgb_plan_desc& d);
bool ndgen_can(const exgb_plan_desc& d);
bool ndgen_pass2d(const exgb_plan_desc& d);
bool ndgen_pass3d(const exgb_plan_desc& d);
// 0 when rfftn / irfftn take transforms of length n on this device (any n with a prime factor
// above 5 up to the Bluestein limit, 2^a 3^b 5^c of any length in 1D), else an EXGB_E* code
int transform_supported(int n);
// does the fused 1D kernel hold one instance of N points at this ETDRK order in shared memory?
bool etdrk1d_fits(int N, int order);
int ndgen_validate(const exgb_plan_desc& d);
int ndgen_run(const exgb_plan* plan, cudaStream_t st, const float2* in, float2* out, int64_t batch, int nsteps,
              int project, int nonlinear_only);
int etdrk0_apply(const exgb_plan* plan, cudaStream_t st, const float2* in, float2* out, int64_t batch, int nsteps,
                 int project);

// FP32 sum with Kahan compensation per thread (the thread's running sum carries its rounding error);
// device reductions combine the per-thread results by a pairwise warp/block tree.  About 1e-7 relative
// for the metric and normalisation sums, as the reference's FP32 reductions; the GPU keeps FP64 for
// the phi-coefficient contour integrals only.
struct KahanSum {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    const float y = x - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
};

}  // namespace exgb
