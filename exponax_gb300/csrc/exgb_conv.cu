// exgb_conv.cu -- kernels of the learned coarse-step corrector: a periodic
// 3x3 convolutional residual network on H x 64 grids, BF16 weights and
// activations, FP32 accumulation, trained with Adam.
//
// No counterpart in the reference (the nearest precedent is the 1D
// SimplePeriodicConvNet of the reference's learning_burgers notebook).
//
// Layouts: activations NHWC, C = 48 channels (bf16); the single-channel
// input/output fields are float32 (B, H, 64).  Weights W[tap][co][ci],
// tap = (dy+1)*3 + (dx+1), periodic wrap in both directions.
//
// * conv48_tc_kernel: 48 -> 48 channels as an implicit GEMM on the tcgen05
//   tensor cores (kind::f16, bf16 x bf16 -> FP32 in tensor memory): a tile
//   is 2 rows x 64 columns, the three horizontal taps of a row offset
//   stacked along N (N = 144), inputs by TMA; the epilogue adds the
//   neighbours' partial sums, the bias and applies GELU (forward) or
//   multiplies by GELU'(pre) of the layer below (backward-data, with
//   flipped weights).
// * conv_in1 / conv_out1: the 1 -> 48 and 48 -> 1 layers (SIMT, weights
//   in the constant bank).
// * weight gradients: per-CTA partial sums over pixel chunks, then a
//   deterministic reduction.
// * adam_kernel: FP32 master weights, bf16 working copies (and the flipped
//   copy used by backward-data).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <mutex>

#include "exgb_internal.h"
#include "exgb_tc.cuh"

namespace exgb {

constexpr int kC = 48;     // hidden channels
constexpr int kW = 64;     // grid width (columns)

// GELU in its tanh form (Hendrycks & Gimpel, "Gaussian Error Linear Units", 2016):
//   gelu(x) = x / 2 (1 + tanh(u)),  u = sqrt(2 / pi) (x + 0.044715 x^3),
// with the hardware tanh (tanh.approx.f32, relative error about 2^-11, below the bf16 rounding of
// the activations); gelu'(x) = (1 + t) / 2 + x / 2 (1 - t^2) sqrt(2 / pi) (1 + 3 0.044715 x^2).
__device__ __forceinline__ float tanh_hw(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
constexpr float kGeluA = 0.79788456080286536f;            // sqrt(2 / pi)
constexpr float kGeluB = 0.79788456080286536f * 0.044715f;
__device__ __forceinline__ float gelu_f(float x) {
  const float t = tanh_hw(x * fmaf(kGeluB, x * x, kGeluA));
  const float h = 0.5f * x;
  return fmaf(h, t, h);
}
__device__ __forceinline__ float gelu_d(float x) {
  const float x2 = x * x;
  const float t = tanh_hw(x * fmaf(kGeluB, x2, kGeluA));
  const float du = fmaf(3.f * kGeluB, x2, kGeluA);
  return fmaf(0.5f * x * du, fmaf(-t, t, 1.f), fmaf(0.5f, t, 0.5f));
}

// Packed FP32 helpers (add/mul/fma .f32x2: two lanes of a channel pair per instruction, each rounded like
// the scalar operation it replaces).
__device__ __forceinline__ float2 bc2(float s) { return make_float2(s, s); }
__device__ __forceinline__ float2 gelu_f2(float2 x) {
  const float2 u = __fmul2_rn(x, __ffma2_rn(__fmul2_rn(x, x), bc2(kGeluB), bc2(kGeluA)));
  const float2 t = make_float2(tanh_hw(u.x), tanh_hw(u.y));
  const float2 h = __fmul2_rn(x, bc2(0.5f));
  return __ffma2_rn(h, t, h);
}
__device__ __forceinline__ float2 bf2_to_f2(uint32_t u) {
  return __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&u));
}
__device__ __forceinline__ uint32_t f2_to_bf2(float2 v) {  // round to nearest, v.x in the low half
  uint32_t r;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(v.y), "f"(v.x));
  return r;
}

// 48 -> 48 channels as an implicit GEMM on the tcgen05 tensor cores.  A tile is 2 output rows x 64
// columns = 128 pixels (M = 128).  A tcgen05.mma of K = 16 costs its issuing thread ~143 cycles for
// any N up to 256, so the three horizontal taps of a row offset dy are stacked along N: operand B of
// row offset dy is W[(dy, dx)][co][ci] for dx = -1, 0, +1 one after the other (N = 144 rows n =
// 48 (dx + 1) + co, K-major), and
//   D[p][n] = sum_dy sum_ci x[y_p + dy][x_p][ci] W[(dy, dx)][co][ci]
// holds, for pixel p = (y_p, x_p), input column x_p's contribution to output column x_p - dx: 9 MMAs
// of N = 144 per tile.  The epilogue adds out[y][x] = D[(y, x - 1)][dx = -1] + D[(y, x)][0] +
// D[(y, x + 1)][+1] (periodic in x) through a padded FP32 exchange buffer in shared memory.
//
// Operand A of row offset dy is read straight from a stage holding the tile's 4 input rows, unshifted
// and periodic in y: pixel slot q = 64 r + c holds x[y0 - 1 + r][c], K-major without swizzle as
// 8-channel chunks ((q, channel) at chunk * 4096 + q * 16 + (channel % 8) * 2), so the 128 pixels of
// output rows (y0, y0 + 1) under row offset dy are the 128 consecutive slots from q = 64 (1 + dy)
// (stride byte offset 128, leading byte offset 4096): one descriptor.  The stage is exactly the
// layout a TMA box of 8 channels x 64 columns x 4 rows lands in.
//
// Warp roles, handing tiles over through mbarriers (every wait clock-bounded; a wait that gives up
// raises a CTA-wide abort flag and the status word read by exgb_conv_status):
//   warp 13     (one thread) loads a tile's 4 input rows by TMA (cp.async.bulk.tensor, one box per
//               8-channel chunk, or per row where the rows wrap in y) into one of kStages stages once
//               empty[s] says it is free; the bytes complete full[s]
//   warp 12     waits full[s] and accumulator a free, issues the 9 MMAs, commits to empty[s] and
//               accfull[a]
//   warps 0-11  wait accfull[a], read the accumulator (warp w: TMEM lanes 32 (w % 4).. = pixels, 16
//               channels of each dx block), free it, publish the dx = -1 / +1 partial sums, add the
//               neighbours' ones, apply bias and GELU (or GELU' for the backward pass) and store
//               their pixel's channels (32-byte sectors)
namespace ctc {
constexpr int kEpilogueWarps = 12;
constexpr int kMmaWarp = kEpilogueWarps;                       // 12
constexpr int kTmaWarp = kMmaWarp + 1;                         // 13
constexpr int kThreads = 32 * (kTmaWarp + 1);                  // 448
constexpr int kEpilogueThreads = 32 * kEpilogueWarps;
constexpr int kStages = 4;                                     // input stages in flight
constexpr int kHaloRows = 4;                                   // 2 output rows + 1 above + 1 below
constexpr int kN = 3 * kC;                                     // 144: the three dx taps stacked along N
constexpr int kCe = kC / 3;                                    // 16 channels per epilogue thread
constexpr uint32_t kSlots = kHaloRows * kW;                    // 256 pixel slots
constexpr uint32_t kChunkStride = kSlots * 16;                 // 4096 B between 8-channel chunks
constexpr uint32_t kStageBytes = (kC / 8) * kChunkStride;      // 24576 B per stage
constexpr uint32_t kDyBytes = kN * kC * 2;                     // 13824 B of weights per row offset dy
constexpr uint32_t kWBytes = 3 * kDyBytes;
constexpr int kXPix = kC + 4;                                  // floats per pixel in the exchange buffer
constexpr uint32_t kXBytes = 2u * 128u * kXPix * 4u;           // [dx = -1 | +1][pixel][kXPix] floats
constexpr uint32_t kOffW = kStages * kStageBytes;
constexpr uint32_t kOffX = kOffW + kWBytes;                    // dx = -1 / +1 partial sums of a tile
constexpr uint32_t kOffBar = kOffX + kXBytes;                  // 2 kStages + 5 mbarriers
constexpr uint32_t kSmemBytes = kOffBar + (2 * kStages + 5) * 8;
constexpr uint32_t kAccCols = 256;                             // accumulator a at TMEM column 256 a (144 used)
constexpr long long kWaitBudget = 4000000000LL;                // clock cycles (~2 s)
static_assert(kSmemBytes + 1024 <= 227 * 1024, "conv tile does not fit in shared memory");
static_assert(kStageBytes % 1024 == 0 && kWBytes % 16 == 0 && kXBytes % 16 == 0,
              "aligned regions");
static_assert(kN % 16 == 0 && kN <= 256, "M = 128 needs N a multiple of 16, at most 256");
static_assert(kC % 3 == 0 && kCe % 4 == 0, "epilogue channel groups of whole 16-byte pieces");
}  // namespace ctc

// cuTensorMapEncodeTiled, reached through the runtime's driver entry point (no link against libcuda)
typedef CUresult (*PFN_encode)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                               const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                               CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

__device__ int g_conv_status;  // EXGB_ETIMEOUT after a bounded wait of the conv kernel gave up

// TMA: the tile's 4 input rows (y0 - 1 .. y0 + 2, periodic inside the image) into a stage, chunk by
// chunk (box: 8 channels x 64 columns x 4 rows, or 1 row each where the rows wrap), completing on
// mbarrier `bar` by transaction bytes (kStageBytes in either case)
__device__ __forceinline__ void tma_load3(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
      ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* mbar, uint32_t bytes) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}\n" ::"r"(
                   tc::smem_u32(mbar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void conv_tma_tile(const CUtensorMap* map4, const CUtensorMap* map1, int H, int tile,
                                              uint32_t stage_saddr, uint64_t* bar) {
  const int tiles_per_img = H / 2;
  const int b = tile / tiles_per_img, y0 = (tile - b * tiles_per_img) * 2;
  mbar_arrive_expect_tx(bar, ctc::kStageBytes);
  const uint32_t mb = tc::smem_u32(bar);
  if (y0 >= 1 && y0 + 2 <= H - 1) {
#pragma unroll
    for (int ch = 0; ch < kC / 8; ++ch)
      tma_load3(stage_saddr + (uint32_t)ch * ctc::kChunkStride, map4, ch * 8, 0, b * H + y0 - 1, mb);
  } else {
#pragma unroll
    for (int r = 0; r < ctc::kHaloRows; ++r) {
      int gy = y0 + r - 1;
      gy = gy < 0 ? gy + H : (gy >= H ? gy - H : gy);
#pragma unroll
      for (int ch = 0; ch < kC / 8; ++ch)
        tma_load3(stage_saddr + (uint32_t)ch * ctc::kChunkStride + (uint32_t)(r * kW) * 16u, map1, ch * 8, 0,
                  b * H + gy, mb);
    }
  }
}

__device__ __forceinline__ void mbar_arrive(uint64_t* mbar) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}\n" ::"r"(tc::smem_u32(mbar))
               : "memory");
}
// named barrier `id` over the `n` threads of the epilogue warps of one output row
__device__ __forceinline__ void row_sync(uint32_t id, uint32_t n) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}
// the same barrier, returning whether any of its threads passed `c` true: the warps of a row leave
// their tile loop together (a warp leaving alone would strand the others at the next barrier)
__device__ __forceinline__ bool row_any(uint32_t id, uint32_t n, bool c) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred pc, pr;\n\t"
      "setp.ne.u32 pc, %1, 0;\n\t"
      "bar.red.or.pred pr, %2, %3, pc;\n\t"
      "selp.u32 %0, 1, 0, pr;\n\t}\n"
      : "=r"(r)
      : "r"((uint32_t)c), "r"(id), "r"(n)
      : "memory");
  return r != 0;
}

// bulk copy of `bytes` (multiple of 16) from shared to global memory, tracked by the bulk-group counter
__device__ __forceinline__ void bulk_store(void* gdst, uint32_t ssrc, uint32_t bytes) {
  asm volatile(
      "{\n\t.reg .u64 g;\n\tcvta.to.global.u64 g, %0;\n\t"
      "cp.async.bulk.global.shared::cta.bulk_group [g], [%1], %2;\n\t}\n" ::"l"(gdst),
      "r"(ssrc), "r"(bytes)
      : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// the sources of every committed bulk copy have been read (their shared memory may be rewritten)
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// every committed bulk copy has completed
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

__device__ __forceinline__ void conv_issue(uint32_t stage_saddr, uint32_t w_saddr, uint32_t d_tmem) {
  const uint32_t idesc = tc::idesc_bf16(128, ctc::kN);
#pragma unroll
  for (int dy = 0; dy < 3; ++dy) {
    const uint32_t a0 = stage_saddr + (uint32_t)(dy * kW) * 16u;  // halo rows dy, dy + 1
#pragma unroll
    for (int s = 0; s < kC / 16; ++s) {
      const uint64_t ad = tc::smem_desc(a0 + (uint32_t)s * 2u * ctc::kChunkStride, ctc::kChunkStride, 128u);
      const uint64_t bd = tc::kmaj_desc(w_saddr + (uint32_t)dy * ctc::kDyBytes, kC, s);
      tc::mma_bf16(d_tmem, ad, bd, idesc, (dy | s) != 0 ? 1u : 0u);
    }
  }
}

// mode 0: forward  out_post = gelu(conv(x) + bias), and out_pre = conv(x) + bias unless out_pre is NULL
// mode 1: backward data  out_pre (= dPre of the layer below) = conv_flipped(x = dPre) * gelu'(aux = pre below)
__global__ void __launch_bounds__(ctc::kThreads, 1) conv48_tc_kernel(const __grid_constant__ CUtensorMap map4,
                                                                  const __grid_constant__ CUtensorMap map1, int B, int H,
                                                                  const __nv_bfloat16* __restrict__ w,
                                                                  const float* __restrict__ bias, int mode,
                                                                  const __nv_bfloat16* __restrict__ aux,
                                                                  __nv_bfloat16* __restrict__ out_pre,
                                                                  __nv_bfloat16* __restrict__ out_post) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint32_t s_tmem;
  __shared__ int s_abort;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + ctc::kOffBar);
  uint64_t* full = bars;                         // [kStages] the TMA bytes of stage s have landed
  uint64_t* empty = bars + ctc::kStages;         // [kStages] the MMAs that read stage s have completed
  uint64_t* accfull = bars + 2 * ctc::kStages;   // [2] accumulator a holds a finished tile
  uint64_t* accempty = accfull + 2;              // [2] the epilogue has read accumulator a
  uint64_t* drain = accfull + 4;                 // every MMA of this CTA has completed (before the TMEM is released)
  float* xbuf = reinterpret_cast<float*>(smem + ctc::kOffX);  // [2][128 pixels][kXPix]
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ntiles = B * (H / 2);
  const uint32_t sbase = tc::smem_u32(smem);
  const uint32_t wsaddr = sbase + ctc::kOffW;
  // outputs of the forward pass go to out_post (and out_pre), of the backward pass to out_pre
  __nv_bfloat16* out_a = mode == 0 ? out_post : out_pre;
  __nv_bfloat16* out_b = mode == 0 ? out_pre : nullptr;

  // weights -> one K-major tile of N = 144 rows per row offset dy: row n = 48 (dx + 1) + co holds
  // W[tap = 3 (dy + 1) + (dx + 1)][co][ci] (consecutive threads: consecutive rows)
  for (int t = tid; t < 3 * ctc::kN * (kC / 8); t += ctc::kThreads) {
    const int n = t % ctc::kN, rest = t / ctc::kN;  // rest = dy * 6 + chunk
    const int ch = rest % (kC / 8), dy = rest / (kC / 8);
    const int tap = 3 * dy + n / kC, co = n % kC;
    *reinterpret_cast<uint4*>(smem + ctc::kOffW + dy * ctc::kDyBytes + tc::kmaj_chunk(n, ch, kC)) =
        *reinterpret_cast<const uint4*>(w + ((size_t)tap * kC + co) * kC + ch * 8);
  }
  if (warp == ctc::kMmaWarp) {
    tc::tmem_alloc(&s_tmem, 2 * ctc::kAccCols);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    s_abort = 0;
    for (int i = 0; i < ctc::kStages; ++i) {
      tc::mbar_init(full + i, 1);
      tc::mbar_init(empty + i, 1);
    }
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(accfull + i, 1);
      tc::mbar_init(accempty + i, ctc::kEpilogueThreads);
    }
    tc::mbar_init(drain, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc::fence_proxy_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = s_tmem;
  // a wait that gives up: raise the abort flag (every role then leaves its loop at its next check)
  auto give_up = [&]() {
    atomicExch(&s_abort, 1);
    atomicExch(&g_conv_status, EXGB_ETIMEOUT);
  };
  auto aborted = [&]() { return *reinterpret_cast<volatile int*>(&s_abort) != 0; };

  if (warp == ctc::kTmaWarp) {
    // ---------------- TMA (lane 0): tile i of this CTA goes to stage i % kStages once the stage is free
    if (lane == 0) {
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&map4)) : "memory");
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&map1)) : "memory");
      int i = 0;
      for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++i) {
        const int s = i % ctc::kStages;
        const uint32_t par = ((uint32_t)(i / ctc::kStages) & 1u) ^ 1u;  // the first use of a stage passes at once
        if (!tc::mbar_wait(empty + s, par, ctc::kWaitBudget)) { give_up(); break; }
        if (aborted()) break;
        conv_tma_tile(&map4, &map1, H, tile, sbase + (uint32_t)s * ctc::kStageBytes, full + s);
      }
      // no TMA copy may still be writing shared memory when the CTA ends (after an abort the MMA
      // thread may not have waited for the last ones): wait for the last issued tiles' bytes
      for (int j = i - ctc::kStages < 0 ? 0 : i - ctc::kStages; j < i; ++j)
        if (!tc::mbar_wait(full + (j % ctc::kStages), (uint32_t)(j / ctc::kStages) & 1u, ctc::kWaitBudget)) give_up();
    }
    __syncwarp();
  } else if (warp == ctc::kMmaWarp) {
    // ---------------- MMA issuer (lane 0)
    if (lane == 0) {
      int i = 0;
      for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++i) {
        const int s = i % ctc::kStages, a = i & 1;
        const uint32_t spar = (uint32_t)(i / ctc::kStages) & 1u, apar = (uint32_t)(i >> 1) & 1u;
        if (!tc::mbar_wait(full + s, spar, ctc::kWaitBudget)) { give_up(); break; }
        if (!tc::mbar_wait(accempty + a, apar ^ 1u, ctc::kWaitBudget)) { give_up(); break; }
        if (aborted()) break;
        tc::fence_after_sync();
        conv_issue(sbase + (uint32_t)s * ctc::kStageBytes, wsaddr, tmem + (uint32_t)a * ctc::kAccCols);
        tc::mma_commit(empty + s);
        tc::mma_commit(accfull + a);
      }
      // one more commit tracks every MMA issued above: after it arrives none is in flight
      tc::mma_commit(drain);
      if (!tc::mbar_wait(drain, 0u, ctc::kWaitBudget)) give_up();
    }
    __syncwarp();
  } else {
    // ---------------- epilogue: warp w reads TMEM lanes 32 (w % 4) + lane = pixel m, channels
    // 16 (w / 4) .. + 15 of each dx block.  The 6 warps of an output row (quadrants 2 r, 2 r + 1) sync
    // among themselves only: the horizontal neighbours are in the same row.  Each thread stores its
    // pixel's 16 channels (one whole 32-byte sector) straight to global memory.
    constexpr int kCe = ctc::kCe;
    constexpr uint32_t kRowThreads = ctc::kEpilogueThreads / 2;
    const int m = 32 * (warp & 3) + lane;
    const int c0 = kCe * (warp >> 2);
    const int orow = (warp & 3) >> 1;
    const uint32_t rbar = 1u + (uint32_t)orow;
    const int row = m / kW, xx = m % kW;
    const int ml = row * kW + ((xx - 1) & (kW - 1)), mr = row * kW + ((xx + 1) & (kW - 1));
    float bv[kCe];
#pragma unroll
    for (int j = 0; j < kCe; ++j) bv[j] = mode == 0 ? bias[c0 + j] : 0.f;
    const int xm = m * ctc::kXPix + c0;              // this pixel's dx = -1 partials (+ kXHalf / 2: dx = +1)
    const int xl = ml * ctc::kXPix + c0;             // left neighbour's dx = -1 partials
    const int xr = (128 + mr) * ctc::kXPix + c0;     // right neighbour's dx = +1 partials
    int i = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++i) {
      const int a = i & 1;
      const uint32_t par = (uint32_t)(i >> 1) & 1u;
      const bool ok = tc::mbar_wait(accfull + a, par, ctc::kWaitBudget);
      if (!ok) give_up();
      tc::fence_after_sync();
      const uint32_t ta = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)a * ctc::kAccCols + (uint32_t)c0;
      // d[b][j]: accumulator column 48 b + c0 + j, block b = dx + 1 (not read if the wait gave up)
      float d[3][kCe];
      if (ok) {
        tc::tmem_ld16(ta, d[0]);
        tc::tmem_ld16(ta + (uint32_t)kC, d[1]);
        tc::tmem_ld16(ta + 2u * kC, d[2]);
      } else {
#pragma unroll
        for (int b = 0; b < 3; ++b)
#pragma unroll
          for (int j = 0; j < kCe; ++j) d[b][j] = 0.f;
      }
      tc::fence_before_sync();
      mbar_arrive(accempty + a);  // accumulator a may be overwritten by the MMAs of tile i + 2
      // publish the dx = -1 / +1 partial sums (the row's readers of the previous tile passed its final
      // barrier; a second buffer for alternate tiles would cost an input stage, measured slower)
      float* xh = xbuf;
#pragma unroll
      for (int q = 0; q < kCe / 4; ++q) {
        *reinterpret_cast<float4*>(xh + xm + 4 * q) =
            make_float4(d[0][4 * q], d[0][4 * q + 1], d[0][4 * q + 2], d[0][4 * q + 3]);
        *reinterpret_cast<float4*>(xh + 128 * ctc::kXPix + xm + 4 * q) =
            make_float4(d[2][4 * q], d[2][4 * q + 1], d[2][4 * q + 2], d[2][4 * q + 3]);
      }
      // one barrier of the row: partial sums published, and its warps agree whether to stop
      if (row_any(rbar, kRowThreads, !ok || aborted())) break;
      // out[x] = D[x - 1][dx = -1] + D[x][dx = 0] + D[x + 1][dx = +1] (periodic in x within the row)
      float v[kCe];  // channel pairs on the packed FP32 pipe
#pragma unroll
      for (int q = 0; q < kCe / 4; ++q) {
        const float4 l4 = *reinterpret_cast<const float4*>(xh + xl + 4 * q);
        const float4 r4 = *reinterpret_cast<const float4*>(xh + xr + 4 * q);
        const float2 s0 = __fadd2_rn(__fadd2_rn(make_float2(d[1][4 * q], d[1][4 * q + 1]), make_float2(l4.x, l4.y)),
                                     make_float2(r4.x, r4.y));
        const float2 s1 = __fadd2_rn(
            __fadd2_rn(make_float2(d[1][4 * q + 2], d[1][4 * q + 3]), make_float2(l4.z, l4.w)), make_float2(r4.z, r4.w));
        v[4 * q] = s0.x;
        v[4 * q + 1] = s0.y;
        v[4 * q + 2] = s1.x;
        v[4 * q + 3] = s1.y;
      }
      uint32_t ra[kCe / 2], rb[kCe / 2];
      if (mode == 0) {
#pragma unroll
        for (int j = 0; j < kCe / 2; ++j) {
          const float2 v01 = __fadd2_rn(make_float2(v[2 * j], v[2 * j + 1]), make_float2(bv[2 * j], bv[2 * j + 1]));
          rb[j] = f2_to_bf2(v01);
          ra[j] = f2_to_bf2(gelu_f2(v01));
        }
      } else {
        // pixel m of this tile: 128 * tile + m in the batch (tiles are consecutive row pairs)
        const size_t o = ((size_t)tile * 128 + m) * kC + c0;
#pragma unroll
        for (int q = 0; q < kCe / 8; ++q) {
          const uint4 pr = *reinterpret_cast<const uint4*>(aux + o + 8 * q);
          const uint32_t prw[4] = {pr.x, pr.y, pr.z, pr.w};
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const __nv_bfloat162 pp = *reinterpret_cast<const __nv_bfloat162*>(&prw[j]);
            const float v0 = v[8 * q + 2 * j] * gelu_d(__bfloat162float(pp.x));
            const float v1 = v[8 * q + 2 * j + 1] * gelu_d(__bfloat162float(pp.y));
            const __nv_bfloat162 r = __floats2bfloat162_rn(v0, v1);
            ra[4 * q + j] = *reinterpret_cast<const uint32_t*>(&r);
          }
        }
      }
      // this thread's 16 channels of pixel m: one whole 32-byte sector of the output
      const size_t o = ((size_t)tile * 128 + m) * kC + c0;
      *reinterpret_cast<uint4*>(out_a + o) = make_uint4(ra[0], ra[1], ra[2], ra[3]);
      *reinterpret_cast<uint4*>(out_a + o + 8) = make_uint4(ra[4], ra[5], ra[6], ra[7]);
      if (out_b) {
        *reinterpret_cast<uint4*>(out_b + o) = make_uint4(rb[0], rb[1], rb[2], rb[3]);
        *reinterpret_cast<uint4*>(out_b + o + 8) = make_uint4(rb[4], rb[5], rb[6], rb[7]);
      }
      row_sync(rbar, kRowThreads);  // the row's threads have read this tile's neighbour partials
    }
  }

  // every MMA this CTA issued has completed (drain barrier above) before the tensor memory is released
  tc::fence_before_sync();
  __syncthreads();
  if (warp == ctc::kMmaWarp) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, 2 * ctc::kAccCols);
  }
}


// Weights of the thin layers live in the constant bank.  Every thread of a warp reads the same weight
// at once, and an FMA takes a constant-bank operand with no load instruction and no traffic through
// L1 (read from shared memory as broadcast 16-byte loads, the 432 weights per pixel kept the L1 data
// return 88 % busy in the 1 -> 48 layer).  Each launch first copies its layer's weights in on its own
// stream (exgb_conv_in1 / exgb_conv_out1 order the users of a bank across streams).
__constant__ __align__(16) float c_in1[9 * kC + kC];  // [tap][co], then the bias [co]
__constant__ __align__(16) float c_out1[9 * kC + 4];  // [tap][ci], then the bias
__device__ __forceinline__ float2 cpair(const float* c, int i) { return *reinterpret_cast<const float2*>(c + i); }

// 1 -> 48 forward: pre = conv(x) + b, post = gelu(pre).  One thread per pixel of sample blockIdx.y; the
// multiply-adds and the GELU's arithmetic run on the packed FP32 pipe over output channel pairs (each
// input held as a broadcast pair, the weights constant-bank operands).  A block stages its 256 pixels'
// 96-byte outputs in shared memory (112-byte rows: conflict-free 16-byte accesses) and stores them as
// consecutive 16-byte pieces.  `pre` (training only) is written straight from the threads; NULL at
// inference.
constexpr int kIn1Pix = 56;  // bf16 per staged output pixel (48 used)
__global__ void __launch_bounds__(256) conv_in1_kernel(const float* __restrict__ x, int H,
                                                       __nv_bfloat16* __restrict__ pre,
                                                       __nv_bfloat16* __restrict__ post) {
  __shared__ __align__(16) __nv_bfloat16 stage[256 * kIn1Pix];
  const int npix = H * kW;
  const int p0 = blockIdx.x * 256;
  const int p = p0 + threadIdx.x;
  const bool live = p < npix;
  const float* xb = x + (int64_t)blockIdx.y * npix;
  const int64_t ob = (int64_t)blockIdx.y * npix;
  float2 vb[9];
  {
    const int pp = live ? p : 0;
    const int y = pp / kW, xx = pp % kW;
#pragma unroll
    for (int tap = 0; tap < 9; ++tap) {
      int gy = y + tap / 3 - 1;
      gy = gy < 0 ? gy + H : (gy >= H ? gy - H : gy);
      const int gx = (xx + tap % 3 - 1) & (kW - 1);
      vb[tap] = bc2(__ldg(xb + gy * kW + gx));
    }
  }
#pragma unroll
  for (int q = 0; q < kC / 8; ++q) {
    float2 acc[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[j] = cpair(c_in1, 9 * kC + q * 8 + 2 * j);
#pragma unroll
    for (int tap = 0; tap < 9; ++tap)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[j] = __ffma2_rn(cpair(c_in1, tap * kC + q * 8 + 2 * j), vb[tap], acc[j]);
    uint32_t hp[4], hq[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      hp[j] = f2_to_bf2(acc[j]);
      hq[j] = f2_to_bf2(gelu_f2(acc[j]));
    }
    *reinterpret_cast<uint4*>(stage + threadIdx.x * kIn1Pix + q * 8) = make_uint4(hq[0], hq[1], hq[2], hq[3]);
    if (pre && live) *reinterpret_cast<uint4*>(pre + (ob + p) * kC + q * 8) = make_uint4(hp[0], hp[1], hp[2], hp[3]);
  }
  __syncthreads();
  const int np = min(256, npix - p0);
  for (int e = threadIdx.x; e < np * (kC / 8); e += blockDim.x) {
    const int pl = e / (kC / 8), q = e - pl * (kC / 8);
    *reinterpret_cast<uint4*>(post + (ob + p0 + pl) * kC + q * 8) =
        *reinterpret_cast<const uint4*>(stage + pl * kIn1Pix + q * 8);
  }
}

// 48 -> 1 forward: out = base + scale * (conv(h) + b), as tap sums.  A block owns kOut1Rows output rows
// of sample blockIdx.y.  Each thread first takes kOut1Px pixels of the kOut1Rows + 2 input rows (the
// halo included), reads each pixel's 48 channels once and forms its nine tap sums
// P[tap][p] = sum_ci w[tap][ci] h[p][ci] on the packed FP32 pipe (channel pairs, the weights
// constant-bank operands) into shared memory; then each output pixel adds the sums of its neighbours,
// out[y][x] = b + sum_tap P[tap][y + dy][x + dx].  (A thread per output pixel reading its 9 x 48 inputs
// from rows staged in shared memory took 68 us at batch 256 of 64^2 grids, bound by those reads.)
constexpr int kOut1Rows = 8;                          // output rows per block
constexpr int kOut1In = kOut1Rows + 2;                // input rows per block
constexpr int kOut1Px = 2;                            // input pixels per thread in the tap-sum phase
constexpr int kOut1Threads = kOut1In * kW / kOut1Px;  // 320
__global__ void __launch_bounds__(kOut1Threads, 3) conv_out1_kernel(const __nv_bfloat16* __restrict__ h, int H,
                                                                 const float* __restrict__ base, float scale,
                                                                 float* __restrict__ out) {
  __shared__ float part[9][kOut1In * kW];  // [tap][input pixel of the block]
  const int y0 = blockIdx.x * kOut1Rows;
  const __nv_bfloat16* hb = h + (int64_t)blockIdx.y * H * kW * kC;
  const uint4* src[kOut1Px];
#pragma unroll
  for (int i = 0; i < kOut1Px; ++i) {
    const int pl = threadIdx.x + i * kOut1Threads;  // 0 .. kOut1In * kW - 1
    int gy = (y0 - 1 + pl / kW) % H;
    if (gy < 0) gy += H;
    src[i] = reinterpret_cast<const uint4*>(hb + ((int64_t)gy * kW + pl % kW) * kC);
  }
  float2 acc[kOut1Px][9];
#pragma unroll
  for (int i = 0; i < kOut1Px; ++i)
#pragma unroll
    for (int tap = 0; tap < 9; ++tap) acc[i][tap] = make_float2(0.f, 0.f);
#pragma unroll
  for (int q = 0; q < kC / 8; ++q) {
    float2 a[kOut1Px][4];
#pragma unroll
    for (int i = 0; i < kOut1Px; ++i) {
      const uint4 u = __ldg(src[i] + q);
      a[i][0] = bf2_to_f2(u.x);
      a[i][1] = bf2_to_f2(u.y);
      a[i][2] = bf2_to_f2(u.z);
      a[i][3] = bf2_to_f2(u.w);
    }
#pragma unroll
    for (int tap = 0; tap < 9; ++tap)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float2 wp = cpair(c_out1, tap * kC + q * 8 + 2 * j);
#pragma unroll
        for (int i = 0; i < kOut1Px; ++i) acc[i][tap] = __ffma2_rn(a[i][j], wp, acc[i][tap]);
      }
  }
#pragma unroll
  for (int i = 0; i < kOut1Px; ++i)
#pragma unroll
    for (int tap = 0; tap < 9; ++tap) part[tap][threadIdx.x + i * kOut1Threads] = acc[i][tap].x + acc[i][tap].y;
  __syncthreads();
  const float b0 = c_out1[9 * kC];
  for (int o = threadIdx.x; o < kOut1Rows * kW; o += kOut1Threads) {
    const int oy = o / kW, ox = o % kW;
    if (y0 + oy >= H) break;
    float s = b0;
#pragma unroll
    for (int tap = 0; tap < 9; ++tap) s += part[tap][(oy + tap / 3) * kW + ((ox + tap % 3 - 1) & (kW - 1))];
    const int64_t pi = ((int64_t)blockIdx.y * H + y0 + oy) * kW + ox;
    out[pi] = (base ? base[pi] : 0.f) + scale * s;
  }
}

// backward of the 48 -> 1 layer w.r.t. its input, times GELU'(pre):
// dpre[p][ci] = gelu'(pre[p][ci]) * sum_tap w[tap][ci] * dout[p - shift(tap)].  One thread per
// (pixel, 8-channel chunk), coalesced 16-byte loads and stores.
__global__ void conv_out1_bwd_data_kernel(const float* __restrict__ dout, int H, const float* __restrict__ w,
                                          const __nv_bfloat16* __restrict__ pre, __nv_bfloat16* __restrict__ dpre) {
  __shared__ float wsm[9 * kC];
  for (int t = threadIdx.x; t < 9 * kC; t += blockDim.x) wsm[t] = w[t];
  __syncthreads();
  const int n = H * kW * (kC / 8);  // per sample (blockIdx.y)
  const float* db = dout + (int64_t)blockIdx.y * H * kW;
  const int64_t ob = (int64_t)blockIdx.y * n;
  for (int tl = blockIdx.x * blockDim.x + threadIdx.x; tl < n; tl += gridDim.x * blockDim.x) {
    const int p = tl / (kC / 8);
    const int cg = tl - p * (kC / 8);
    const int y = p / kW, xx = p % kW;
    const int64_t t = ob + tl;
    float g[9];
#pragma unroll
    for (int tap = 0; tap < 9; ++tap) {
      int gy = y - (tap / 3 - 1);
      gy = gy < 0 ? gy + H : (gy >= H ? gy - H : gy);
      const int gx = (xx - (tap % 3 - 1)) & (kW - 1);
      g[tap] = __ldg(db + gy * kW + gx);
    }
    const uint4 pr = *reinterpret_cast<const uint4*>(pre + t * 8);
    const uint32_t prw[4] = {pr.x, pr.y, pr.z, pr.w};
    uint32_t res[4];
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) {
      const int ci = cg * 8 + 2 * jj;
      float s0 = 0.f, s1 = 0.f;
#pragma unroll
      for (int tap = 0; tap < 9; ++tap) {
        s0 = fmaf(wsm[tap * kC + ci], g[tap], s0);
        s1 = fmaf(wsm[tap * kC + ci + 1], g[tap], s1);
      }
      const float2 pf = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&prw[jj]));
      const __nv_bfloat162 rr = __floats2bfloat162_rn(s0 * gelu_d(pf.x), s1 * gelu_d(pf.y));
      res[jj] = *reinterpret_cast<const uint32_t*>(&rr);
    }
    *reinterpret_cast<uint4*>(dpre + t * 8) = make_uint4(res[0], res[1], res[2], res[3]);
  }
}

// Weight-gradient partial sums of a 48 -> 48 layer over one pixel chunk:
// part[chunk][tap][co][ci] = sum_{p in chunk} dpre[p][co] * x[p + shift(tap)][ci]
// (+ bias partials part_b[chunk][co] from tap 4).  One CTA per (chunk, tap).
constexpr int kChunk = 512;
__global__ void __launch_bounds__(256) wgrad48_kernel(const __nv_bfloat16* __restrict__ dpre,
                                                      const __nv_bfloat16* __restrict__ x, int B, int H,
                                                      float* __restrict__ part, float* __restrict__ part_b) {
  __shared__ float dsm[64][kC + 1];
  __shared__ float xsm[64][kC + 1];
  const int chunk = blockIdx.x, tap = blockIdx.y;
  const int dy = tap / 3 - 1, dx = tap % 3 - 1;
  const int64_t n = (int64_t)B * H * kW;
  const int64_t p0 = (int64_t)chunk * kChunk;
  const int tid = threadIdx.x;
  // thread -> 9 (co, ci) outputs: co = tid % 48 ... use a 48 x 48 grid over 256 threads
  float acc[9];
  int oc[9], oi[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    const int e = tid + 256 * q;  // 0 .. 2303
    oc[q] = e / kC;
    oi[q] = e % kC;
    acc[q] = 0.f;
  }
  float bacc = 0.f;
  for (int s = 0; s < kChunk; s += 64) {
    __syncthreads();
    for (int t = tid; t < 64 * kC; t += 256) {
      const int pp = t / kC, c = t % kC;
      const int64_t p = p0 + s + pp;
      float dv = 0.f, xv = 0.f;
      if (p < n) {
        const int64_t b = p / (H * kW);
        const int r = (int)(p % (H * kW));
        const int y = r / kW, xx = r % kW;
        const int gy = (y + dy + H) % H, gx = (xx + dx + kW) % kW;
        dv = __bfloat162float(dpre[p * kC + c]);
        xv = __bfloat162float(x[((b * H + gy) * kW + gx) * kC + c]);
      }
      dsm[pp][c] = dv;
      xsm[pp][c] = xv;
    }
    __syncthreads();
#pragma unroll 4
    for (int pp = 0; pp < 64; ++pp) {
#pragma unroll
      for (int q = 0; q < 9; ++q) acc[q] = fmaf(dsm[pp][oc[q]], xsm[pp][oi[q]], acc[q]);
    }
    if (tap == 4 && tid < kC)
      for (int pp = 0; pp < 64; ++pp) bacc += dsm[pp][tid];
  }
#pragma unroll
  for (int q = 0; q < 9; ++q) part[((size_t)chunk * 9 + tap) * kC * kC + oc[q] * kC + oi[q]] = acc[q];
  if (tap == 4 && tid < kC) part_b[(size_t)chunk * kC + tid] = bacc;
}

// Weight/bias partials of the thin layers over one pixel chunk.
// mode 0 (1 -> 48): part[chunk][tap][co] = sum_p dpre[p][co] x[p + shift]; bias from tap 4
// mode 1 (48 -> 1): part[chunk][tap][ci] = sum_p dout[p] h[p + shift][ci]; bias = sum dout
__global__ void wgrad_thin_kernel(int mode, const float* __restrict__ f32, const __nv_bfloat16* __restrict__ b16,
                                  int B, int H, float* __restrict__ part, float* __restrict__ part_b) {
  const int chunk = blockIdx.x;
  const int64_t n = (int64_t)B * H * kW;
  const int64_t p0 = (int64_t)chunk * kChunk;
  const int tid = threadIdx.x;  // 9 * 48 = 432 outputs over 512 threads
  const int tap = tid / kC, c = tid % kC;
  float acc = 0.f, bacc = 0.f;
  if (tid < 9 * kC) {
    const int dy = tap / 3 - 1, dx = tap % 3 - 1;
    for (int s = 0; s < kChunk; ++s) {
      const int64_t p = p0 + s;
      if (p >= n) break;
      const int64_t b = p / (H * kW);
      const int r = (int)(p % (H * kW));
      const int y = r / kW, xx = r % kW;
      const int64_t q = (b * H + (y + dy + H) % H) * kW + (xx + dx + kW) % kW;
      if (mode == 0) {
        const float d = __bfloat162float(b16[p * kC + c]);
        acc = fmaf(d, f32[q], acc);
        if (tap == 4) bacc += d;
      } else {
        const float d = f32[p];
        acc = fmaf(d, __bfloat162float(b16[q * kC + c]), acc);
        if (tap == 4 && c == 0) bacc += d;
      }
    }
    part[(size_t)chunk * 9 * kC + tid] = acc;
    if (tap == 4 && mode == 0) part_b[(size_t)chunk * kC + c] = bacc;
    if (tap == 4 && mode == 1 && c == 0) part_b[chunk] = bacc;
  }
}

// sum over chunks: out[i] = sum_c part[c][i]
__global__ void reduce_parts_kernel(const float* __restrict__ part, int nchunk, int64_t len, float* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int c = 0; c < nchunk; ++c) s += part[(size_t)c * len + i];
    out[i] = s;
  }
}

// Adam (Kingma & Ba) with bias correction on FP32 master weights; writes
// the bf16 working copy and, for 48 -> 48 layers (is48), the flipped,
// channel-transposed copy used by backward-data: wf[8 - tap][ci][co] = w[tap][co][ci].
__global__ void adam_kernel(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                            const float* __restrict__ g, int64_t n, float lr, float b1, float b2, float eps, float bc1,
                            float bc2, __nv_bfloat16* __restrict__ w16, __nv_bfloat16* __restrict__ wflip, int is48) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float upd = lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    const float wi = w[i] - upd;
    w[i] = wi;
    if (w16) w16[i] = __float2bfloat16_rn(wi);
    if (is48 && wflip) {
      const int tap = (int)(i / (kC * kC));
      const int r = (int)(i % (kC * kC));
      const int co = r / kC, ci = r % kC;
      wflip[(size_t)(8 - tap) * kC * kC + ci * kC + co] = __float2bfloat16_rn(wi);
    }
  }
}

// Copy FP32 weights to the bf16 working copy (+ flipped copy), no update.
__global__ void cast_weights_kernel(const float* __restrict__ w, int64_t n, __nv_bfloat16* __restrict__ w16,
                                    __nv_bfloat16* __restrict__ wflip, int is48) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float wi = w[i];
    if (w16) w16[i] = __float2bfloat16_rn(wi);
    if (is48 && wflip) {
      const int tap = (int)(i / (kC * kC));
      const int r = (int)(i % (kC * kC));
      const int co = r / kC, ci = r % kC;
      wflip[(size_t)(8 - tap) * kC * kC + ci * kC + co] = __float2bfloat16_rn(wi);
    }
  }
}

// loss = sum (pred - target)^2 / n per block partials; grad = 2 (pred - target) / n * scale
__global__ void mse_kernel(const float* __restrict__ pred, const float* __restrict__ target, int64_t n, float scale,
                           float* __restrict__ grad, float* __restrict__ loss_part) {
  __shared__ float red[256];
  float s = 0.f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float d = pred[i] - target[i];
    s += d * d;
    grad[i] = 2.f * d / (float)n * scale;
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) loss_part[blockIdx.x] = red[0];
}

// Spectral-energy guard: per sample, the fraction of the correction's
// energy above |k| > kg relative to the plain state's total energy (both
// from rfft2 half-spectra, (B, H, 33)); samples over `thresh` or with a
// non-finite correction keep the plain coarse state.
__global__ void guard_kernel(const float2* __restrict__ corr_hat, const float2* __restrict__ plain_hat, int B, int H,
                             int kg, float thresh, const float* __restrict__ plain, float* __restrict__ state,
                             int* __restrict__ tripped) {
  const int M = kW / 2 + 1;
  __shared__ float s_hi[256], s_all[256];
  __shared__ int s_bad;
  const int b = blockIdx.x;
  float hi = 0.f, all = 0.f;
  int bad = 0;
  for (int t = threadIdx.x; t < H * M; t += blockDim.x) {
    const int kx = t / M, ky = t % M;
    const int sx = kx <= (H - 1) / 2 ? kx : kx - H;
    const float w = (ky == 0 || ky == kW / 2) ? 1.f : 2.f;  // Hermitian weight of the half spectrum
    const float2 c = corr_hat[(size_t)b * H * M + t];
    const float2 p = plain_hat[(size_t)b * H * M + t];
    const float ce = c.x * c.x + c.y * c.y;
    if (!isfinite(ce)) bad = 1;
    if (sx * sx + ky * ky > kg * kg) hi += w * ce;
    all += w * (p.x * p.x + p.y * p.y);
  }
  s_hi[threadIdx.x] = hi;
  s_all[threadIdx.x] = all;
  if (threadIdx.x == 0) s_bad = 0;
  __syncthreads();
  if (bad) atomicOr(&s_bad, 1);
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      s_hi[threadIdx.x] += s_hi[threadIdx.x + o];
      s_all[threadIdx.x] += s_all[threadIdx.x + o];
    }
    __syncthreads();
  }
  const bool trip = s_bad || !(s_hi[0] <= thresh * s_all[0]);
  if (trip) {
    for (int t = threadIdx.x; t < H * kW; t += blockDim.x) state[(size_t)b * H * kW + t] = plain[(size_t)b * H * kW + t];
  }
  if (threadIdx.x == 0) tripped[b] = trip ? 1 : 0;
}

static unsigned blocks_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (unsigned)(b < 1 ? 1 : (b > 65535 * 4 ? 65535 * 4 : b));
}

// The users of one constant bank of thin-layer weights on one device, in launch order: a launch waits
// (on its stream) for the previous user's kernel before its copy overwrites the bank.  Inside a stream
// capture the graph's own order applies.
struct ConstBank {
  std::mutex mu;
  cudaEvent_t done = nullptr;
};
constexpr int kMaxDevices = 64;
static ConstBank g_bank_in1[kMaxDevices], g_bank_out1[kMaxDevices];
static int bank_device(int* dev) {
  EXGB_CUDA(cudaGetDevice(dev));
  if (*dev < 0 || *dev >= kMaxDevices) return fail(EXGB_EUNSUPPORTED, "device index out of range");
  return EXGB_OK;
}

// Copy nw weights and nb bias values (one copy where the bias follows the weights, as in the
// corrector's parameter vector) into the constant bank `sym` on `st`, then run `launch` on `st`.
template <class F>
static int with_const_weights(ConstBank& bk, const void* sym, const float* w, int nw, const float* b, int nb,
                              cudaStream_t st, F&& launch) {
  std::lock_guard<std::mutex> lock(bk.mu);
  if (!bk.done) EXGB_CUDA(cudaEventCreateWithFlags(&bk.done, cudaEventDisableTiming));
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  EXGB_CUDA(cudaStreamIsCapturing(st, &cs));
  const bool captured = cs != cudaStreamCaptureStatusNone;
  if (!captured) {
    cudaError_t e = cudaStreamWaitEvent(st, bk.done, 0);
    if (e == cudaErrorInvalidResourceHandle) {
      // the event went with a context torn down since (cudaDeviceReset): start a new one
      cudaGetLastError();
      EXGB_CUDA(cudaEventCreateWithFlags(&bk.done, cudaEventDisableTiming));
      e = cudaStreamWaitEvent(st, bk.done, 0);
    }
    EXGB_CUDA(e);
  }
  if (b == w + nw) {
    EXGB_CUDA(cudaMemcpyToSymbolAsync(sym, w, sizeof(float) * (size_t)(nw + nb), 0, cudaMemcpyDeviceToDevice, st));
  } else {
    EXGB_CUDA(cudaMemcpyToSymbolAsync(sym, w, sizeof(float) * (size_t)nw, 0, cudaMemcpyDeviceToDevice, st));
    EXGB_CUDA(cudaMemcpyToSymbolAsync(sym, b, sizeof(float) * (size_t)nb, sizeof(float) * (size_t)nw,
                                      cudaMemcpyDeviceToDevice, st));
  }
  launch();
  EXGB_CUDA(cudaGetLastError());
  if (!captured) EXGB_CUDA(cudaEventRecord(bk.done, st));
  return EXGB_OK;
}

}  // namespace exgb

using namespace exgb;

extern "C" {

int exgb_conv48(void* stream, const void* x, int B, int H, const void* w, const float* bias, int mode,
                const void* aux, void* out_pre, void* out_post) {
  if (!x || !w || B < 0 || H < 2 || H % 2 || (mode == 0 && (!bias || !out_post)) ||
      (mode == 1 && (!aux || !out_pre)) || (mode != 0 && mode != 1))
    return fail(EXGB_EINVAL, "exgb_conv48: bad arguments (H must be even)");
  if (B == 0) return EXGB_OK;
  static int sm_count[64] = {0};
  int dev = 0;
  EXGB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(EXGB_EUNSUPPORTED, "device index out of range");
  if (!sm_count[dev]) EXGB_CUDA(cudaDeviceGetAttribute(&sm_count[dev], cudaDevAttrMultiProcessorCount, dev));
  // set on every call: a context re-created after cudaDeviceReset starts without it
  EXGB_CUDA(cudaFuncSetAttribute(conv48_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ctc::kSmemBytes));
  const int64_t ntiles = (int64_t)B * (H / 2);
  if (ntiles > 2147483647LL) return fail(EXGB_EINVAL, "exgb_conv48: too many tiles");
  if (((uintptr_t)x & 15) != 0) return fail(EXGB_EINVAL, "exgb_conv48: input not 16-byte aligned");
  // tensor maps of the input (bf16, dims innermost first: 48 channels, 64 columns, B H rows), boxes of
  // 8 channels x 64 columns x 4 rows and x 1 row
  CUtensorMap map4, map1;
  {
    static PFN_encode encode = nullptr;
    if (!encode) {
      void* fn = nullptr;
      cudaDriverEntryPointQueryResult q;
      EXGB_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
      if (q != cudaDriverEntryPointSuccess || !fn) return fail(EXGB_ECUDA, "cuTensorMapEncodeTiled not available");
      encode = (PFN_encode)fn;
    }
    const cuuint64_t dims[3] = {(cuuint64_t)kC, (cuuint64_t)kW, (cuuint64_t)B * H};
    const cuuint64_t strides[2] = {(cuuint64_t)kC * 2, (cuuint64_t)kW * kC * 2};
    const cuuint32_t estr[3] = {1, 1, 1};
    const cuuint32_t box4[3] = {8, (cuuint32_t)kW, (cuuint32_t)ctc::kHaloRows}, box1[3] = {8, (cuuint32_t)kW, 1};
    CUresult r = encode(&map4, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(x), dims, strides, box4, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r == CUDA_SUCCESS)
      r = encode(&map1, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(x), dims, strides, box1, estr,
                 CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(EXGB_ECUDA, "exgb_conv48: tensor map encoding failed");
  }
  const unsigned grid = (unsigned)std::min<int64_t>(ntiles, sm_count[dev]);
  conv48_tc_kernel<<<grid, ctc::kThreads, ctc::kSmemBytes, (cudaStream_t)stream>>>(
      map4, map1, B, H, (const __nv_bfloat16*)w, bias, mode, (const __nv_bfloat16*)aux, (__nv_bfloat16*)out_pre,
      (__nv_bfloat16*)out_post);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

// Synchronises the device; EXGB_ETIMEOUT if a bounded wait of the tensor-core conv kernel gave up
// since the last call (its outputs are then invalid).  The status is cleared on read.
int exgb_conv_status(void) {
  int h = 0;
  EXGB_CUDA(cudaMemcpyFromSymbol(&h, g_conv_status, sizeof(int)));
  if (h) {
    const int zero = 0;
    EXGB_CUDA(cudaMemcpyToSymbol(g_conv_status, &zero, sizeof(int)));
    return fail(h, "a bounded device wait of the tensor-core conv kernel gave up");
  }
  return EXGB_OK;
}

int exgb_conv_in1(void* stream, const float* x, int B, int H, const float* w, const float* bias, void* pre,
                  void* post) {
  if (!x || !w || !bias || !post || B < 0 || H < 1) return fail(EXGB_EINVAL, "NULL argument or bad shape");
  if ((int64_t)B * H == 0) return EXGB_OK;
  if ((int64_t)B * H > 2147483647LL) return fail(EXGB_EINVAL, "too many rows");
  if (B > 65535) return fail(EXGB_EINVAL, "batch above 65535");
  int dev = 0;
  if (const int rc = bank_device(&dev)) return rc;
  return with_const_weights(g_bank_in1[dev], (const void*)c_in1, w, 9 * kC, bias, kC, (cudaStream_t)stream, [&]() {
    conv_in1_kernel<<<dim3((H * kW + 255) / 256, B), 256, 0, (cudaStream_t)stream>>>(x, H, (__nv_bfloat16*)pre,
                                                                                     (__nv_bfloat16*)post);
  });
}

int exgb_conv_out1(void* stream, const void* h, int B, int H, const float* w, const float* bias, const float* base,
                   float scale, float* out) {
  if (!h || !w || !bias || !out || B < 0 || H < 1) return fail(EXGB_EINVAL, "NULL argument or bad shape");
  if ((int64_t)B * H == 0) return EXGB_OK;
  if ((int64_t)B * H > 2147483647LL) return fail(EXGB_EINVAL, "too many rows");
  if (B > 65535) return fail(EXGB_EINVAL, "batch above 65535");
  int dev = 0;
  if (const int rc = bank_device(&dev)) return rc;
  return with_const_weights(g_bank_out1[dev], (const void*)c_out1, w, 9 * kC, bias, 1, (cudaStream_t)stream, [&]() {
    conv_out1_kernel<<<dim3((H + kOut1Rows - 1) / kOut1Rows, B), kOut1Threads, 0, (cudaStream_t)stream>>>(
        (const __nv_bfloat16*)h, H, base, scale, out);
  });
}

int exgb_conv_out1_bwd_data(void* stream, const float* dout, int B, int H, const float* w, const void* pre,
                            void* dpre) {
  if (!dout || !w || !pre || !dpre || B < 0 || H < 1) return fail(EXGB_EINVAL, "NULL argument or bad shape");
  if (B == 0) return EXGB_OK;
  if (B > 65535) return fail(EXGB_EINVAL, "batch above 65535");
  conv_out1_bwd_data_kernel<<<dim3((H * kW * (kC / 8) + 255) / 256, B), 256, 0, (cudaStream_t)stream>>>(
      dout, H, w, (const __nv_bfloat16*)pre, (__nv_bfloat16*)dpre);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

// part must hold nchunk * 9*48*48 floats (48->48) or nchunk * 9*48 (thin); part_b nchunk * 48.
int exgb_wgrad(void* stream, int kind, const void* a, const void* bsrc, int B, int H, float* part, float* part_b,
               float* dw, float* db) {
  if (!a || !bsrc || !part || !part_b || !dw || !db || B < 0 || H < 1 || kind < 0 || kind > 2)
    return fail(EXGB_EINVAL, "exgb_wgrad: NULL argument, bad shape or kind");
  if (B == 0) return EXGB_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t n = (int64_t)B * H * kW;
  if ((n + kChunk - 1) / kChunk > 2147483647LL) return fail(EXGB_EINVAL, "exgb_wgrad: too many pixels");
  const int nchunk = (int)((n + kChunk - 1) / kChunk);
  if (kind == 0) {  // 48 -> 48: a = dpre (bf16), bsrc = layer input (bf16)
    wgrad48_kernel<<<dim3(nchunk, 9), 256, 0, st>>>((const __nv_bfloat16*)a, (const __nv_bfloat16*)bsrc, B, H, part,
                                                    part_b);
    reduce_parts_kernel<<<blocks_for(9 * kC * kC), 256, 0, st>>>(part, nchunk, 9 * kC * kC, dw);
    reduce_parts_kernel<<<1, 64, 0, st>>>(part_b, nchunk, kC, db);
  } else if (kind == 1) {  // 1 -> 48: a = dpre (bf16), bsrc = input field (f32)
    wgrad_thin_kernel<<<nchunk, 512, 0, st>>>(0, (const float*)bsrc, (const __nv_bfloat16*)a, B, H, part, part_b);
    reduce_parts_kernel<<<blocks_for(9 * kC), 256, 0, st>>>(part, nchunk, 9 * kC, dw);
    reduce_parts_kernel<<<1, 64, 0, st>>>(part_b, nchunk, kC, db);
  } else {  // 48 -> 1: a = dout (f32), bsrc = layer input (bf16)
    wgrad_thin_kernel<<<nchunk, 512, 0, st>>>(1, (const float*)a, (const __nv_bfloat16*)bsrc, B, H, part, part_b);
    reduce_parts_kernel<<<blocks_for(9 * kC), 256, 0, st>>>(part, nchunk, 9 * kC, dw);
    reduce_parts_kernel<<<1, 64, 0, st>>>(part_b, nchunk, 1, db);
  }
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

int exgb_adam(void* stream, float* w, float* m, float* v, const float* g, int64_t n, float lr, float b1, float b2,
              float eps, int64_t t, void* w16, void* wflip, int is48) {
  if (!w || !m || !v || !g || n < 0 || t < 1 || (is48 && wflip && n != 9 * kC * kC))
    return fail(EXGB_EINVAL, "exgb_adam: NULL argument, n < 0, t < 1, or a flipped copy of other than 9*48*48 weights");
  if (n == 0) return EXGB_OK;
  const float bc1 = 1.f - powf(b1, (float)t), bc2 = 1.f - powf(b2, (float)t);
  adam_kernel<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>(w, m, v, g, n, lr, b1, b2, eps, bc1, bc2,
                                                               (__nv_bfloat16*)w16, (__nv_bfloat16*)wflip, is48);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

int exgb_cast_weights(void* stream, const float* w, int64_t n, void* w16, void* wflip, int is48) {
  if (!w || n < 0 || (is48 && wflip && n != 9 * kC * kC))
    return fail(EXGB_EINVAL, "exgb_cast_weights: NULL argument, n < 0, or a flipped copy of other than 9*48*48 weights");
  if (n == 0) return EXGB_OK;
  cast_weights_kernel<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>(w, n, (__nv_bfloat16*)w16,
                                                                       (__nv_bfloat16*)wflip, is48);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

int exgb_mse(void* stream, const float* pred, const float* target, int64_t n, float scale, float* grad,
             float* loss_part, int nblocks) {
  if (!pred || !target || !grad || !loss_part || n < 0 || nblocks < 1 || nblocks > 65535)
    return fail(EXGB_EINVAL, "exgb_mse: NULL argument, n < 0 or nblocks outside 1..65535");
  mse_kernel<<<nblocks, 256, 0, (cudaStream_t)stream>>>(pred, target, n, scale, grad, loss_part);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

int exgb_guard(void* stream, const void* corr_hat, const void* plain_hat, int B, int H, int kg, float thresh,
               const float* plain, float* state, int* tripped) {
  if (!corr_hat || !plain_hat || !plain || !state || !tripped || B < 0 || H < 1 || kg < 0)
    return fail(EXGB_EINVAL, "exgb_guard: NULL argument or bad shape");
  if (B == 0) return EXGB_OK;
  guard_kernel<<<B, 256, 0, (cudaStream_t)stream>>>((const float2*)corr_hat, (const float2*)plain_hat, B, H, kg,
                                                    thresh, plain, state, tripped);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

}  // extern "C"
