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
// * conv48_mma_kernel: 48 -> 48 channels as an implicit GEMM on the tensor
//   cores (mma.sync m16n8k16, bf16 x bf16 -> f32): a CTA computes 4 rows x
//   64 columns x 48 output channels from a shared-memory halo tile; the
//   epilogue adds the bias and applies GELU (forward) or multiplies by
//   GELU'(pre) of the layer below (backward-data, with flipped weights).
// * conv_in1 / conv_out1: the 1 -> 48 and 48 -> 1 layers (SIMT).
// * weight gradients: per-CTA partial sums over pixel chunks, then a
//   deterministic reduction.
// * adam_kernel: FP32 master weights, bf16 working copies (and the flipped
//   copy used by backward-data).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "exgb_internal.h"

namespace exgb {

constexpr int kC = 48;     // hidden channels
constexpr int kW = 64;     // grid width (columns)
constexpr int kCP = 56;    // padded channel stride in shared memory (bank-conflict free)
constexpr int kTR = 4;     // output rows per CTA

__device__ __forceinline__ float gelu_f(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_d(float x) {
  const float cdf = 0.5f * (1.f + erff(x * 0.70710678118654752f));
  const float pdf = 0.39894228040143268f * __expf(-0.5f * x * x);
  return cdf + x * pdf;
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// mode 0: forward  out_pre = conv(x) + bias, out_post = gelu(out_pre)
// mode 1: backward data  out_pre (= dPre of the layer below) = conv_flipped(x = dPre) * gelu'(aux = pre below)
__global__ void __launch_bounds__(256, 2) conv48_mma_kernel(const __nv_bfloat16* __restrict__ x, int H,
                                                           const __nv_bfloat16* __restrict__ w,
                                                           const float* __restrict__ bias, int mode,
                                                           const __nv_bfloat16* __restrict__ aux,
                                                           __nv_bfloat16* __restrict__ out_pre,
                                                           __nv_bfloat16* __restrict__ out_post) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __nv_bfloat16* xs = reinterpret_cast<__nv_bfloat16*>(smem_raw);           // (kTR+2) x (kW+2) x kCP
  __nv_bfloat16* ws = xs + (kTR + 2) * (kW + 2) * kCP;                        // 9 x kC x kCP
  const int tiles_per_img = H / kTR;
  const int b = blockIdx.x / tiles_per_img;
  const int y0 = (blockIdx.x % tiles_per_img) * kTR;
  const int tid = threadIdx.x;

  // weights -> smem (9 * 48 rows of 48 ci, 16-byte chunks)
  for (int t = tid; t < 9 * kC * (kC / 8); t += 256) {
    const int row = t / (kC / 8), ch = t % (kC / 8);
    *reinterpret_cast<uint4*>(ws + row * kCP + ch * 8) = *reinterpret_cast<const uint4*>(w + row * kC + ch * 8);
  }
  // halo tile -> smem, periodic wrap
  const __nv_bfloat16* xb = x + (size_t)b * H * kW * kC;
  for (int t = tid; t < (kTR + 2) * (kW + 2) * (kC / 8); t += 256) {
    const int ch = t % (kC / 8);
    const int pix = t / (kC / 8);
    const int r = pix / (kW + 2), c = pix % (kW + 2);
    const int gy = (y0 + r - 1 + H) % H, gx = (c - 1 + kW) % kW;
    *reinterpret_cast<uint4*>(xs + pix * kCP + ch * 8) =
        *reinterpret_cast<const uint4*>(xb + ((size_t)gy * kW + gx) * kC + ch * 8);
  }
  __syncthreads();

  const int warp = tid >> 5, lane = tid & 31;
  const int g = lane >> 2, tig = lane & 3;
  float acc[2][6][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 6; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.f;

  // this warp: pixels [warp*32, warp*32+32) of the 4 x 64 tile
  int prow[2][2], pcol[2][2];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int p = warp * 32 + i * 16 + g + 8 * h;
      prow[i][h] = p / kW;
      pcol[i][h] = p % kW;
    }

#pragma unroll 1
  for (int tap = 0; tap < 9; ++tap) {
    const int dy = tap / 3 - 1, dx = tap % 3 - 1;
#pragma unroll
    for (int kc = 0; kc < kC / 16; ++kc) {
      uint32_t a[2][4];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int sp = (prow[i][h] + 1 + dy) * (kW + 2) + (pcol[i][h] + 1 + dx);
          const __nv_bfloat16* src = xs + sp * kCP + kc * 16 + tig * 2;
          a[i][h] = *reinterpret_cast<const uint32_t*>(src);
          a[i][2 + h] = *reinterpret_cast<const uint32_t*>(src + 8);
        }
      }
      // register order of the A fragment: {row g, k 0-7}, {row g+8, k 0-7}, {row g, k 8-15}, {row g+8, k 8-15}
#pragma unroll
      for (int j = 0; j < 6; ++j) {
        const __nv_bfloat16* wsrc = ws + (tap * kC + j * 8 + g) * kCP + kc * 16 + tig * 2;
        const uint32_t b0 = *reinterpret_cast<const uint32_t*>(wsrc);
        const uint32_t b1 = *reinterpret_cast<const uint32_t*>(wsrc + 8);
#pragma unroll
        for (int i = 0; i < 2; ++i) mma_bf16(acc[i][j], a[i][0], a[i][1], a[i][2], a[i][3], b0, b1);
      }
    }
  }

  // epilogue: C fragment {row g, cols 2tig, 2tig+1}, {row g+8, same cols}
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int p = warp * 32 + i * 16 + g + 8 * h;
      const size_t o = (((size_t)b * H + y0 + p / kW) * kW + (p % kW)) * kC;
#pragma unroll
      for (int j = 0; j < 6; ++j) {
        const int co = j * 8 + tig * 2;
        float v0 = acc[i][j][2 * h], v1 = acc[i][j][2 * h + 1];
        if (mode == 0) {
          v0 += bias[co];
          v1 += bias[co + 1];
          *reinterpret_cast<__nv_bfloat162*>(out_pre + o + co) = __floats2bfloat162_rn(v0, v1);
          *reinterpret_cast<__nv_bfloat162*>(out_post + o + co) = __floats2bfloat162_rn(gelu_f(v0), gelu_f(v1));
        } else {
          const __nv_bfloat162 pr = *reinterpret_cast<const __nv_bfloat162*>(aux + o + co);
          v0 *= gelu_d(__bfloat162float(pr.x));
          v1 *= gelu_d(__bfloat162float(pr.y));
          *reinterpret_cast<__nv_bfloat162*>(out_pre + o + co) = __floats2bfloat162_rn(v0, v1);
        }
      }
    }
}

// 1 -> 48 forward: pre = conv(x) + b, post = gelu(pre).  One thread per pixel.
__global__ void conv_in1_kernel(const float* __restrict__ x, int B, int H, const float* __restrict__ w,
                                const float* __restrict__ bias, __nv_bfloat16* __restrict__ pre,
                                __nv_bfloat16* __restrict__ post) {
  __shared__ float wsm[9 * kC + kC];
  for (int t = threadIdx.x; t < 9 * kC; t += blockDim.x) wsm[t] = w[t];  // [tap][co]
  for (int t = threadIdx.x; t < kC; t += blockDim.x) wsm[9 * kC + t] = bias[t];
  __syncthreads();
  const int64_t n = (int64_t)B * H * kW;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = p / (H * kW);
    const int r = (int)(p % (H * kW));
    const int y = r / kW, xx = r % kW;
    float v[9];
#pragma unroll
    for (int tap = 0; tap < 9; ++tap) {
      const int gy = (y + tap / 3 - 1 + H) % H, gx = (xx + tap % 3 - 1 + kW) % kW;
      v[tap] = x[(b * H + gy) * kW + gx];
    }
    for (int co = 0; co < kC; co += 2) {
      float s0 = wsm[9 * kC + co], s1 = wsm[9 * kC + co + 1];
#pragma unroll
      for (int tap = 0; tap < 9; ++tap) {
        s0 = fmaf(wsm[tap * kC + co], v[tap], s0);
        s1 = fmaf(wsm[tap * kC + co + 1], v[tap], s1);
      }
      *reinterpret_cast<__nv_bfloat162*>(pre + p * kC + co) = __floats2bfloat162_rn(s0, s1);
      *reinterpret_cast<__nv_bfloat162*>(post + p * kC + co) = __floats2bfloat162_rn(gelu_f(s0), gelu_f(s1));
    }
  }
}

// 48 -> 1 forward: out = base + scale * (conv(h) + b).  One thread per pixel.
__global__ void conv_out1_kernel(const __nv_bfloat16* __restrict__ h, int B, int H, const float* __restrict__ w,
                                 const float* __restrict__ bias, const float* __restrict__ base, float scale,
                                 float* __restrict__ out) {
  __shared__ float wsm[9 * kC];
  for (int t = threadIdx.x; t < 9 * kC; t += blockDim.x) wsm[t] = w[t];  // [tap][ci]
  __syncthreads();
  const int64_t n = (int64_t)B * H * kW;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = p / (H * kW);
    const int r = (int)(p % (H * kW));
    const int y = r / kW, xx = r % kW;
    float s = bias[0];
#pragma unroll 1
    for (int tap = 0; tap < 9; ++tap) {
      const int gy = (y + tap / 3 - 1 + H) % H, gx = (xx + tap % 3 - 1 + kW) % kW;
      const __nv_bfloat16* src = h + ((b * H + gy) * kW + gx) * kC;
      for (int ci = 0; ci < kC; ci += 2) {
        const float2 f = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(src + ci));
        s = fmaf(wsm[tap * kC + ci], f.x, s);
        s = fmaf(wsm[tap * kC + ci + 1], f.y, s);
      }
    }
    out[p] = (base ? base[p] : 0.f) + scale * s;
  }
}

// backward of the 48 -> 1 layer w.r.t. its input, times GELU'(pre):
// dpre[p][ci] = gelu'(pre[p][ci]) * sum_tap w[tap][ci] * dout[p - shift(tap)]
__global__ void conv_out1_bwd_data_kernel(const float* __restrict__ dout, int B, int H, const float* __restrict__ w,
                                          const __nv_bfloat16* __restrict__ pre, __nv_bfloat16* __restrict__ dpre) {
  __shared__ float wsm[9 * kC];
  for (int t = threadIdx.x; t < 9 * kC; t += blockDim.x) wsm[t] = w[t];
  __syncthreads();
  const int64_t n = (int64_t)B * H * kW;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = p / (H * kW);
    const int r = (int)(p % (H * kW));
    const int y = r / kW, xx = r % kW;
    float g[9];
#pragma unroll
    for (int tap = 0; tap < 9; ++tap) {
      const int gy = (y - (tap / 3 - 1) + H) % H, gx = (xx - (tap % 3 - 1) + kW) % kW;
      g[tap] = dout[(b * H + gy) * kW + gx];
    }
    for (int ci = 0; ci < kC; ci += 2) {
      float s0 = 0.f, s1 = 0.f;
#pragma unroll
      for (int tap = 0; tap < 9; ++tap) {
        s0 = fmaf(wsm[tap * kC + ci], g[tap], s0);
        s1 = fmaf(wsm[tap * kC + ci + 1], g[tap], s1);
      }
      const float2 pr = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(pre + p * kC + ci));
      *reinterpret_cast<__nv_bfloat162*>(dpre + p * kC + ci) =
          __floats2bfloat162_rn(s0 * gelu_d(pr.x), s1 * gelu_d(pr.y));
    }
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

}  // namespace exgb

using namespace exgb;

extern "C" {

int exgb_conv48(void* stream, const void* x, int B, int H, const void* w, const float* bias, int mode,
                const void* aux, void* out_pre, void* out_post) {
  if (!x || !w || !out_pre || H % kTR || (mode == 0 && (!bias || !out_post)) || (mode == 1 && !aux))
    return fail(EXGB_EINVAL, "exgb_conv48: bad arguments (H must be a multiple of 4)");
  const size_t smem = sizeof(__nv_bfloat16) * ((size_t)(kTR + 2) * (kW + 2) * kCP + (size_t)9 * kC * kCP);
  EXGB_CUDA(cudaFuncSetAttribute(conv48_mma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const unsigned grid = (unsigned)B * (H / kTR);
  conv48_mma_kernel<<<grid, 256, smem, (cudaStream_t)stream>>>(
      (const __nv_bfloat16*)x, H, (const __nv_bfloat16*)w, bias, mode, (const __nv_bfloat16*)aux,
      (__nv_bfloat16*)out_pre, (__nv_bfloat16*)out_post);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

int exgb_conv_in1(void* stream, const float* x, int B, int H, const float* w, const float* bias, void* pre,
                  void* post) {
  if (!x || !w || !bias || !pre || !post) return fail(EXGB_EINVAL, "NULL argument");
  const int64_t n = (int64_t)B * H * kW;
  conv_in1_kernel<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>(x, B, H, w, bias, (__nv_bfloat16*)pre,
                                                                   (__nv_bfloat16*)post);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

int exgb_conv_out1(void* stream, const void* h, int B, int H, const float* w, const float* bias, const float* base,
                   float scale, float* out) {
  if (!h || !w || !bias || !out) return fail(EXGB_EINVAL, "NULL argument");
  const int64_t n = (int64_t)B * H * kW;
  conv_out1_kernel<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16*)h, B, H, w, bias, base,
                                                                    scale, out);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

int exgb_conv_out1_bwd_data(void* stream, const float* dout, int B, int H, const float* w, const void* pre,
                            void* dpre) {
  const int64_t n = (int64_t)B * H * kW;
  conv_out1_bwd_data_kernel<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>(dout, B, H, w, (const __nv_bfloat16*)pre,
                                                                             (__nv_bfloat16*)dpre);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

// part must hold nchunk * 9*48*48 floats (48->48) or nchunk * 9*48 (thin); part_b nchunk * 48.
int exgb_wgrad(void* stream, int kind, const void* a, const void* bsrc, int B, int H, float* part, float* part_b,
               float* dw, float* db) {
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t n = (int64_t)B * H * kW;
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
  const float bc1 = 1.f - powf(b1, (float)t), bc2 = 1.f - powf(b2, (float)t);
  adam_kernel<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>(w, m, v, g, n, lr, b1, b2, eps, bc1, bc2,
                                                               (__nv_bfloat16*)w16, (__nv_bfloat16*)wflip, is48);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

int exgb_cast_weights(void* stream, const float* w, int64_t n, void* w16, void* wflip, int is48) {
  cast_weights_kernel<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>(w, n, (__nv_bfloat16*)w16,
                                                                       (__nv_bfloat16*)wflip, is48);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

int exgb_mse(void* stream, const float* pred, const float* target, int64_t n, float scale, float* grad,
             float* loss_part, int nblocks) {
  mse_kernel<<<nblocks, 256, 0, (cudaStream_t)stream>>>(pred, target, n, scale, grad, loss_part);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

int exgb_guard(void* stream, const void* corr_hat, const void* plain_hat, int B, int H, int kg, float thresh,
               const float* plain, float* state, int* tripped) {
  guard_kernel<<<B, 256, 0, (cudaStream_t)stream>>>((const float2*)corr_hat, (const float2*)plain_hat, B, H, kg,
                                                    thresh, plain, state, tripped);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}

}  // extern "C"
