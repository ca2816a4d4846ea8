// exgb_noalloc.cu -- Fourier-space stepping that allocates no memory.
//
// Some callers cannot call cudaMalloc from the place where they step a
// batch: code running under an allocator they do not own (an XLA custom call
// that may only use the buffers XLA hands it, a caching allocator that must
// see every device allocation), or code that must not trigger the implicit
// device synchronisation cudaMalloc/cudaFree can cause.  For them,
// exgb_repeat_fourier_noalloc runs the fused 2D vorticity kernel with its
// stage buffers in a file-scope device array instead of the plan's
// allocation.  The plan itself is still created (and allocates) beforehand.
//
// The array holds kStaticScratchBytes (8 MiB) on every GPU where the library
// is loaded, for the life of the process.  Every call shares it and it keeps
// the last call's contents; the kernel writes every stage buffer entry
// before reading it, so nothing needs clearing between calls.  Calls whose
// kernels overlap on the GPU (different streams, or graphs replayed
// concurrently) race on the array and must be serialised by the caller.
#include <cuda_runtime.h>

#include "exgb_internal.h"

namespace exgb {

int vort2d_run_scratch(const exgb_plan* plan, cudaStream_t st, const float2* in, float2* out, int64_t batch,
                       int nsteps, int project, float2* scratch, size_t scratch_elems);

constexpr size_t kStaticScratchBytes = 8u << 20;
constexpr size_t kStaticScratchElems = kStaticScratchBytes / sizeof(float2);

static __device__ __align__(256) float2 g_static_scratch[kStaticScratchElems];

// Device address of g_static_scratch on the current device.  In host code the
// array's name is only a host-side stand-in, so the address is looked up with
// that device current.  It is looked up on every call (a cheap runtime query),
// so a context torn down and re-created (cudaDeviceReset) never leaves a stale
// address behind; the first call on a device also loads the module there,
// which is why that first call should come before any stream capture.
static int static_scratch(float2** out) {
  float2* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress((void**)&p, g_static_scratch);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_static_scratch)");
  *out = p;
  return EXGB_OK;
}

}  // namespace exgb

using namespace exgb;

extern "C" int exgb_repeat_fourier_noalloc(const exgb_plan* plan, void* stream, const void* u_hat0,
                                           void* u_hat_out, int64_t batch, int32_t nsteps) {
  if (!plan) return fail(EXGB_EINVAL, "NULL argument");
  if (batch < 0 || nsteps < 0) return fail(EXGB_EINVAL, "negative batch or nsteps");
  if (plan->dev.D != 2 || plan->dev.kind == EXGB_NL_ZERO || plan->dev.order == 0 || plan->cfg2d.variant != 1)
    return fail(EXGB_EUNSUPPORTED,
                "exgb_repeat_fourier_noalloc runs 2D vorticity plans with N in {64, 128, 256} and ETDRK order >= 1");
  // The split-BF16 tensor-core kernel keeps its operands in plan-owned scratch; this entry point
  // runs only the FP32 register-FFT kernel, so a plan switched to split-BF16 is refused rather than
  // silently stepped with other arithmetic than exgb_repeat_fourier would use.
  if (plan->precision != EXGB_DFT_FP32)
    return fail(EXGB_EUNSUPPORTED,
                "exgb_repeat_fourier_noalloc runs FP32 transforms only; this plan is set to split-BF16");
  const size_t need = plan->cfg2d.scratch_per_cluster * sizeof(float2);
  if (need > kStaticScratchBytes)
    return fail(EXGB_EUNSUPPORTED, "this plan needs " + std::to_string(need) +
                                       " bytes of stage buffers per cluster, more than the 8 MiB static scratch");
  if (batch == 0) return EXGB_OK;  // an empty batch touches no memory (its pointers may be NULL)
  if (!u_hat0 || !u_hat_out) return fail(EXGB_EINVAL, "NULL argument");
  float2* scratch = nullptr;
  const int rc = static_scratch(&scratch);
  if (rc) return rc;
  return vort2d_run_scratch(plan, (cudaStream_t)stream, (const float2*)u_hat0, (float2*)u_hat_out, batch, nsteps, 0,
                            scratch, kStaticScratchElems);
}
