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

#include <mutex>

#include "exgb_internal.h"

namespace exgb {

int vort2d_run_scratch(const exgb_plan* plan, cudaStream_t st, const float2* in, float2* out, int64_t batch,
                       int nsteps, int project, float2* scratch, size_t scratch_elems);

constexpr size_t kStaticScratchBytes = 8u << 20;
constexpr size_t kStaticScratchElems = kStaticScratchBytes / sizeof(float2);

static __device__ __align__(256) float2 g_static_scratch[kStaticScratchElems];

// Device address of g_static_scratch, looked up once per device (with that
// device current) on the first call made on it.
static std::mutex g_static_mu;
static float2* g_static_ptr[64] = {nullptr};

static int static_scratch(float2** out) {
  int dev = 0;
  EXGB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(EXGB_EUNSUPPORTED, "device index out of range for the static scratch table");
  std::lock_guard<std::mutex> lk(g_static_mu);
  if (!g_static_ptr[dev]) {
    float2* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress((void**)&p, g_static_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_static_scratch)");
    g_static_ptr[dev] = p;
  }
  *out = g_static_ptr[dev];
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
