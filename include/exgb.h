/*
 * exgb.h -- C ABI of libexgb.so, the GB300 (sm_103a) ETDRK pseudo-spectral
 * stepping library.
 *
 * Plain C types only: device pointers are `void*`/`float*` to CUDA global
 * memory, streams are `cudaStream_t` passed as `void*` (NULL = legacy default
 * stream).  Every call returns 0 on success or a negative EXGB_E* code; the
 * message of the last failure on the calling thread is exgb_last_error().
 * No C++ exception crosses this boundary.
 *
 * Data layout (C-contiguous, batch first, as jax.vmap over the reference
 * functions produces):
 *   physical field   float32   (B, C, N, ..., N)
 *   Fourier field    complex64 (B, C, N, ..., N/2+1), interleaved re/im
 *   trajectory       float32   (B, T, C, N, ..., N)
 * `in` and `out` may alias for the step functions.
 *
 * Each entry point names the exponax 0.2.0 function it replaces
 * (paths inside the exponax project).
 */
#ifndef EXGB_H
#define EXGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EXGB_VERSION 1

/* status codes */
#define EXGB_OK 0
#define EXGB_EINVAL (-1)          /* bad argument (NULL pointer, bad enum) */
#define EXGB_ESHAPE (-2)          /* shape / channel / dimension mismatch */
#define EXGB_ENOTFACTORABLE (-3)  /* N has a prime factor above 5 and is too long for the Bluestein transform */
#define EXGB_ECUDA (-4)           /* a CUDA runtime call failed */
#define EXGB_ETIMEOUT (-5)        /* a bounded device wait gave up */
#define EXGB_EGUARD (-6)          /* spectral-energy / non-finite guard tripped */
#define EXGB_ENOMEM (-7)          /* device allocation failed */
#define EXGB_EUNSUPPORTED (-8)    /* valid for the reference, not built here */
#define EXGB_ENOTIMPL (-9)        /* ETDRK order outside 0..4 */

/* nonlinear function kinds (exponax/nonlin_fun/) */
#define EXGB_NL_ZERO 0               /* ZeroNonlinearFun            _zero.py:7-38 */
#define EXGB_NL_CONVECTION 1         /* ConvectionNonlinearFun      _convection.py:7-245 */
#define EXGB_NL_GRADIENT_NORM 2      /* GradientNormNonlinearFun    _gradient_norm.py:8-101 */
#define EXGB_NL_POLYNOMIAL 3         /* PolynomialNonlinearFun      _polynomial.py:6-76 */
#define EXGB_NL_GENERAL 4            /* GeneralNonlinearFun         _general_nonlinear.py:9-119 */
#define EXGB_NL_VORTICITY_2D 5       /* VorticityConvection2d       _vorticity_convection.py:8-99 */
#define EXGB_NL_VORTICITY_2D_KOLMOGOROV 6 /* VorticityConvection2dKolmogorov :102-182 */
#define EXGB_NL_PROJECTED_3D 7       /* ProjectedConvection3d       _projected_convection.py:19-136 */
#define EXGB_NL_PROJECTED_3D_KOLMOGOROV 8 /* ProjectedConvection3dKolmogorov :139-226 */
#define EXGB_NL_CAHN_HILLIARD 9      /* CahnHilliardNonlinearFun    stepper/reaction/_cahn_hilliard.py:12-45 */
#define EXGB_NL_GRAY_SCOTT 10        /* GrayScottNonlinearFun       stepper/reaction/_gray_scott.py:9-46 */
#define EXGB_NL_BELOUSOV_ZHABOTINSKY 11 /* BelousovZhabotinskyNonlinearFun stepper/reaction/_belousov_zhabotinsky.py:14-51 */

typedef struct exgb_plan exgb_plan;

/* Everything BaseStepper.__init__ (_base_stepper.py:27-157) decides:
 * the linear operator L (already assembled by the stepper class on the host,
 * complex128), the ETDRK order and contour parameters, and the nonlinear
 * function with its scalar parameters. */
typedef struct {
  int32_t num_spatial_dims;        /* D: 1, 2 or 3 */
  int32_t num_points;              /* N >= 2 (prime factors above 5 through Bluestein) */
  int32_t num_channels;            /* C */
  int32_t order;                   /* ETDRK order 0..4 */
  double domain_extent;            /* L */
  double dt;
  const double* linear_operator;   /* host, complex128 interleaved, (lin_ch, N..., N/2+1) */
  int32_t linear_operator_channels;/* 1 (broadcast) or C */
  int32_t num_circle_points;       /* contour points, reference default 16 */
  double circle_radius;            /* reference default 1.0 */
  int32_t nonlin_kind;             /* EXGB_NL_* */
  double dealiasing_fraction;      /* < 0: no dealiasing mask */
  double scale;                    /* b of convection / gradient norm / vorticity */
  int32_t single_channel;          /* ConvectionNonlinearFun.single_channel */
  int32_t conservative;            /* ConvectionNonlinearFun.conservative */
  int32_t zero_mode_fix;           /* GradientNorm / General */
  double scale_list[3];            /* GeneralNonlinearFun.scale_list */
  int32_t num_poly;                /* PolynomialNonlinearFun: number of coefficients (<= 8) */
  double poly[8];
  int32_t injection_mode;          /* Kolmogorov forcing mode k */
  double injection_scale;          /* Kolmogorov forcing amplitude */
  double reaction[2];              /* Gray-Scott feed_rate, kill_rate */
} exgb_plan_desc;

/* One instance of an uneven batch (exgb_queue_rollout). */
typedef struct {
  const exgb_plan* plan;   /* 1D plan of this instance */
  const float* u0;         /* device, (C, N) */
  float* traj;             /* device, (T, C, N), T = nsteps + include_init */
} exgb_work_item;

/* ---- library ---- */
int exgb_version(void);
const char* exgb_last_error(void);
/* Number of SMs / compute capability of the current device (for tests). */
int exgb_device_info(int* sm_count, int* cc_major, int* cc_minor);

/* ---- plans ----
 * exgb_plan_create replaces BaseStepper.__init__ (_base_stepper.py:27-157)
 * together with the coefficient set-up of ETDRK0..4
 * (etdrk/_base_etdrk.py:19-62, _etdrk_1.py:63-76, _etdrk_2.py:71-89,
 * _etdrk_3.py:154-189, _etdrk_4.py:168-196): E = exp(dt L) and the
 * phi-function contour means are evaluated in FP64 on the GPU and stored
 * as FP32, real part only, as the reference does. */
int exgb_plan_create(const exgb_plan_desc* desc, exgb_plan** out);
int exgb_plan_destroy(exgb_plan* plan);
/* Copy the coefficient tables to host (for parity tests).  which: 0 = E,
 * 1 = E_half (complex64, 2 floats per mode); 2..7 = coef_1..coef_6 (float32).
 * Layout (lin_ch, N..., N/2+1), row-major like the reference arrays. */
int exgb_plan_get_table(const exgb_plan* plan, int which, void* host_out, size_t bytes);
/* Largest dealiasing-mask wavenumber kept per axis (-1: no mask). */
int exgb_plan_kmax(const exgb_plan* plan);

/* Autotuner knobs (no reference counterpart; used by exponax_gb300.autotune,
 * which times candidates on the device and caches the winner):
 *   EXGB_TUNE_RADICES       values = radix order of the length-N Stockham FFT
 *                           (1D kernel, transforms, generic 2D kernel)
 *   EXGB_TUNE_CLUSTER       values[0] = CTAs per cluster of the 2D vorticity kernels
 *                           (register-FFT and generic), 1..8 (0 = auto)
 *   EXGB_TUNE_ITEMS_PER_CTA values[0] = 1D instances per work item (0 = auto)
 *   EXGB_TUNE_THREADS       values[0] = threads per CTA of the 1D kernel: 64, 128, 256
 *                           (0 = default, 256)
 * exgb_plan_get_tuning writes npass, the kMaxPass (12) radix slots, the
 * cluster size and the items per CTA (n >= 15), the precision (n >= 16) and
 * the 1D threads per CTA (n >= 17). */
#define EXGB_TUNE_RADICES 0
#define EXGB_TUNE_CLUSTER 1
#define EXGB_TUNE_ITEMS_PER_CTA 2
/* EXGB_TUNE_PRECISION values[0] = arithmetic of the 2D vorticity transforms:
 *   EXGB_DFT_FP32        FP32 register/Stockham FFTs (default)
 *   EXGB_DFT_SPLIT_BF16  dense DFT contractions on the tcgen05 tensor cores in
 *                        split-BF16 form (hi.hi + hi.lo + lo.hi, FP32
 *                        accumulation); N = 128, dealiasing cutoff <= 47.
 * exgb_plan_get_tuning reports it after the items per CTA. */
#define EXGB_TUNE_PRECISION 3
#define EXGB_DFT_FP32 0
#define EXGB_DFT_SPLIT_BF16 1
#define EXGB_TUNE_THREADS 4
/* EXGB_TUNE_WAIT_BUDGET values[0] = clock cycles allowed to the first
 * MMA-completion wait of each launch of the split-BF16 tensor-core kernel
 * (0 = the normal budget of about 2 s).  For tests of the timeout path only:
 * a budget of a few cycles makes that wait give up while its MMAs are still
 * in flight; the kernel then waits for them with the normal budget, releases
 * its tensor memory and reports EXGB_ETIMEOUT through exgb_plan_status. */
#define EXGB_TUNE_WAIT_BUDGET 5
int exgb_plan_tune(exgb_plan* plan, int kind, const int* values, int n);
int exgb_plan_get_tuning(const exgb_plan* plan, int* out, int n);
/* Kernel launches of the fused 2D stepping kernel that one exgb_repeat_fourier
 * (or exgb_step_fourier) call makes for `batch` samples, written to *launches:
 * 1, or 2 when the register-FFT kernel runs the samples of a partial last wave
 * on its tail configuration (larger clusters); 0 for plans without a fused 2D
 * kernel.  No reference counterpart (launch accounting for benchmarks). */
int exgb_plan_fused_launches(const exgb_plan* plan, int64_t batch, int* launches);
/* Synchronises the device and returns EXGB_ETIMEOUT if a bounded wait inside
 * the tensor-core kernel of this plan gave up since the last call (the
 * outputs of that launch are then invalid); the status is cleared on read. */
int exgb_plan_status(const exgb_plan* plan);

/* ---- spectral transforms ----
 * exgb_rfftn replaces spectral.fft  (_spectral.py:614-656): rfftn over the
 *   last D axes, norm="backward".
 * exgb_irfftn replaces spectral.ifft (_spectral.py:659-721): irfftn with
 *   s=(N,)*D; imaginary parts of the c2r axis' DC/Nyquist bins are ignored
 *   as numpy/pocketfft do.  `count` = B*C fields. */
int exgb_rfftn(void* stream, int num_spatial_dims, int num_points, int64_t count,
               const float* in, void* out);
int exgb_irfftn(void* stream, int num_spatial_dims, int num_points, int64_t count,
                const void* in, float* out);

/* ---- stepping ----
 * exgb_step_fourier replaces BaseStepper.step_fourier (_base_stepper.py:222-239)
 *   = ETDRKn.step_fourier, vmapped over the batch.
 * exgb_step replaces BaseStepper.__call__/step (_base_stepper.py:201-271).
 * exgb_nonlinear replaces BaseNonlinearFun.__call__ of the plan's
 *   nonlinear function (nonlin_fun/), vmapped. */
int exgb_step_fourier(const exgb_plan* plan, void* stream, const void* u_hat_in, void* u_hat_out,
                      int64_t batch);
int exgb_step(const exgb_plan* plan, void* stream, const float* u_in, float* u_out, int64_t batch);
int exgb_nonlinear(const exgb_plan* plan, void* stream, const void* u_hat_in, void* n_hat_out,
                   int64_t batch);

/* exgb_repeat replaces _utils.repeat(stepper, n) (_utils.py:189-254): n
 *   steps, each through physical space (the c2r projection is applied after
 *   every step), final state only.
 * exgb_repeat_fourier replaces RepeatedStepper.step_fourier
 *   (_repeated_stepper.py:85-102): n steps kept in Fourier space.
 * exgb_rollout replaces _utils.rollout(stepper, n, include_init)
 *   (_utils.py:92-186): trajectory (B, n + include_init, C, N...). */
int exgb_repeat(const exgb_plan* plan, void* stream, const float* u0, float* u_out, int64_t batch,
                int32_t nsteps);
int exgb_repeat_fourier(const exgb_plan* plan, void* stream, const void* u_hat0, void* u_hat_out,
                        int64_t batch, int32_t nsteps);
int exgb_rollout(const exgb_plan* plan, void* stream, const float* u0, float* traj, int64_t batch,
                 int32_t nsteps, int32_t include_init);

/* Same result as exgb_repeat_fourier for 2D vorticity plans (N in {64, 128,
 * 256}, ETDRK order >= 1, FP32 transforms), for callers that cannot allocate
 * device memory where they step (e.g. inside a framework's custom call that
 * may only use the buffers it is given).  No counterpart in the reference.
 * Calls no cudaMalloc/cudaFree: the stage buffers live in an 8 MiB
 * file-scope device array that every GPU loading the library keeps until
 * exit; plans needing more than 8 MiB per cluster, and plans switched to
 * EXGB_DFT_SPLIT_BF16, are rejected with EXGB_EUNSUPPORTED.  Every call
 * looks up the array's address on the current device; the first call on a
 * device also loads the module there (make it before any stream capture).
 * All calls share the array: calls that overlap on the GPU race and must be
 * serialised by the caller. */
int exgb_repeat_fourier_noalloc(const exgb_plan* plan, void* stream, const void* u_hat0, void* u_hat_out,
                                int64_t batch, int32_t nsteps);

/* Uneven batch in one persistent launch: instances of different 1D plans
 * (PDE, N, dt) share a device work queue.  No reference counterpart: the
 * reference runs one jax.vmap(rollout) per (PDE, N) group in sequence
 * (_utils.py:92-186 under jax.vmap).  Items are scheduled longest-first. */
int exgb_queue_rollout(const exgb_work_item* items, int64_t n_items, int32_t nsteps,
                       int32_t include_init, void* stream);

/* The same launch split in two so that it can be captured in a CUDA graph:
 * exgb_queue_prepare uploads the (sorted) item list once into a queue object
 * (allocates); exgb_queue_launch resets the queue head and launches the
 * persistent kernel (two stream operations, no allocation, no host
 * synchronisation: capturable by cudaStreamBeginCapture / torch.cuda.graph).
 * A prepared queue may be launched any number of times, not concurrently. */
typedef struct exgb_queue exgb_queue;
int exgb_queue_prepare(const exgb_work_item* items, int64_t n_items, int32_t nsteps, int32_t include_init,
                       exgb_queue** out);
int exgb_queue_launch(exgb_queue* queue, void* stream);
int exgb_queue_destroy(exgb_queue* queue);

/* Leray projection (nonlin_fun/_leray.py:114-136, order 2): for `count`
 * vector fields of D = 2 or 3 channels in Fourier space (count, D, N..., N/2+1),
 * v^ <- v^ + ik p^, p^ = -(ik . v^) / Lap with 1/Lap = 0 at k = 0. */
int exgb_leray(void* stream, int num_spatial_dims, int num_points, double domain_extent, int64_t count,
               const void* in, void* out);

/* map_between_resolutions (_interpolation.py:195-285) for D = 1, 2, 3:
 * spectral re-sampling of count = B*C fields from N_old to N_new points. */
int exgb_map_between_resolutions(void* stream, int num_spatial_dims, int n_old, int n_new,
                                 int64_t count, const float* in, float* out, int oddball_zero);
/* exgb_fourier_interp replaces FourierInterpolator.__call__ (_interpolation.py:22-112) at
 * num_queries points x (num_queries, D) float32: out (num_queries, C) = Re sum over the rfftn modes
 * of coef[c][mode] exp(i k . x), k the scaled wavenumbers 2 pi n / domain_extent; coef (C, N...,
 * N/2+1) complex64 is the rfftn of the state divided by the "reconstruction" scaling array. */
int exgb_fourier_interp(void* stream, int num_spatial_dims, int num_points, int num_channels, const void* coef,
                        float domain_extent, int64_t num_queries, const float* x, float* out);

/* ---- evaluation ----
 * exgb_spectrum replaces get_spectrum (_spectral.py:866-1030) on count = B*C
 * Fourier fields (count, N..., N/2+1) of D = 1..3 axes: out (count, N/2+1)
 * float32, power (power != 0) or amplitude spectrum, radial bins summed
 * (average = 0) or averaged (average != 0; empty bins NaN).  D = 1: no binning.
 * exgb_field_sums: for count fields of n floats, out[4 f + 0..3] = sum (a-b)^2,
 * sum b^2, sum a b, sum a^2 (FP64) -- the sums behind nRMSE
 * (metrics/_spatial.py:537-586) and correlation (metrics/_correlation.py:33-60). */
int exgb_spectrum(void* stream, int num_spatial_dims, int num_points, int64_t count, const void* u_hat,
                  float* out, int power, int average);
int exgb_field_sums(void* stream, int64_t count, int64_t n, const float* a, const float* b, double* out);
/* The metric families of metrics/_spatial.py, _fourier.py and _derivative.py reduce to these sums
 * (FP64), combined on the host:
 * exgb_field_pnorms: count fields of n floats; out[3 f + 0..2] = sum |a - b|^p, sum |a|^p,
 *   sum |b|^p (b may be NULL: the difference is a, the last sum 0) -- spatial_aggregator (:8-83).
 * exgb_fourier_pnorms: count rfftn fields (N..., N/2+1) of D = 1..3 axes; the sums of
 *   fourier_aggregator (_fourier.py:15-140): |c| < 1e-5 dropped, band low <= max_d |k_d| <= high,
 *   |c|^p over the "reconstruction" scaling array; derivative_order < 0: one sum per field,
 *   else D sums per field weighted by |2 pi k_d / domain_extent|^(derivative_order p). */
int exgb_field_pnorms(void* stream, int64_t count, int64_t n, const float* a, const float* b, float p,
                      double* out);
int exgb_fourier_pnorms(void* stream, int num_spatial_dims, int num_points, int64_t count, const void* u_hat,
                        float p, float derivative_order, int low, int high, float domain_extent, double* out);

/* ---- helpers of the Python surface ----
 * exgb_axpy: out = x + alpha y over n floats (ForcedStepper, _forced_stepper.py:64-65, :86-87;
 *   complex fields pass 2n floats).
 * exgb_scatter_modes: zero count Fourier fields of field_elems complex64 each, then write
 *   vals[f * nmodes + m] at element idx[m] of field f (random-series initial conditions).
 * exgb_normalize_fields: per field of n floats subtract the mean (zero_mean), then divide by
 *   the population standard deviation (std_one) or by max |u - mean| (max_one) -- normalize_ic
 *   (ic/_base_ic.py:18-32); std_one without zero_mean divides by the standard deviation without
 *   centring (SineWaves1d, ic/_sine_waves_1d.py:72-77); std_one with max_one is EXGB_EINVAL. */
int exgb_axpy(void* stream, int64_t n, float alpha, const float* x, const float* y, float* out);
int exgb_scatter_modes(void* stream, int64_t count, int64_t field_elems, int nmodes, const int64_t* idx,
                       const void* vals, void* hat);
int exgb_normalize_fields(void* stream, int64_t count, int64_t n, float* u, int zero_mean, int std_one,
                          int max_one);
/* exgb_mode_scale replaces Poisson.step_fourier (_poisson.py:67-82): out[f][r] = table[r] * in[f][r]
 * for count Fourier fields of per complex64 modes; table is a device array of per complex64
 * values (the Poisson solver passes -1/Lap^(order/2), 0 where the operator vanishes).  in and
 * out may alias. */
int exgb_mode_scale(void* stream, int64_t count, int64_t per, const void* table, const void* in, void* out);
/* exgb_mode_mix2 replaces Wave.step_fourier (stepper/_wave.py:143-224) applied nsteps times: for
 * count samples of two Fourier fields (h, v) of per complex64 modes each, (h, v) <- M (h, v) per
 * mode, M a real 2x2 matrix given as mat[4][per] float32 on the device (m00, m01, m10, m11).  The
 * Wave stepper passes its exact one-step map (the diagonalising transform, the ETDRK0 factors and
 * the inverse transform composed; the mean mode's h += dt v folded in).  in and out may alias. */
int exgb_mode_mix2(void* stream, int64_t count, int64_t per, const float* mat, const void* in, void* out,
                   int nsteps);
/* exgb_spectral_derivative replaces the Fourier-space part of spectral.derivative
 * (_spectral.py:724-791): out (count, D, N..., N/2+1) = (i 2 pi k_d / domain_extent)^order times
 * in (count, N..., N/2+1), complex64.
 * exgb_make_incompressible replaces that of spectral.make_incompressible (_spectral.py:794-863):
 * for count samples of D velocity spectra (count, D, N..., N/2+1), u_d - i k_d Lap^-1 (sum_j i k_j u_j)
 * with 1/Lap taken as 1 at k = 0.  in and out may alias for the projection, not for the derivative. */
int exgb_spectral_derivative(void* stream, int num_spatial_dims, int num_points, int64_t count, int order,
                             float domain_extent, const void* in, void* out);
int exgb_make_incompressible(void* stream, int num_spatial_dims, int num_points, int64_t count, const void* in,
                             void* out);

/* Self-check of the tcgen05 tensor-core layer (no reference counterpart):
 * d (128 x n, FP32) = a (128 x k) . b (n x k)^T, device pointers, row-major.
 * split = 0: inputs rounded to bf16, one product; split = 1: split-BF16
 * three-product form.  16 <= n <= 256, 16 <= k <= 128, multiples of 16.
 * Synchronous. */
int exgb_tc_gemm_check(void* stream, int n, int k, const float* a, const float* b, float* d, int split);

#ifdef __cplusplus
}
#endif

#endif /* EXGB_H */
