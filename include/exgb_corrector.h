/*
 * exgb_corrector.h -- C ABI of libexgb.so for the learned coarse-step
 * corrector: a periodic 3x3 convolutional residual network on H x 64 grids
 * (1 -> 48 -> 48 x 4 -> 1 channels, GELU in its tanh form, BF16 weights and
 * activations, FP32 accumulation) with its backward pass, Adam and the
 * spectral-energy guard.  The reference has no counterpart (its nearest
 * precedent is the 1D SimplePeriodicConvNet of
 * docs/examples/learning_burgers_autoregressive_neural_operator.ipynb).
 *
 * Conventions are those of exgb.h: device pointers to CUDA global memory,
 * the stream as `void*` (NULL = legacy default stream), 0 or a negative
 * EXGB_E* code, exgb_last_error() for the message.
 *
 * Layouts (C-contiguous):
 *   single-channel field   float32  (B, H, 64)
 *   hidden activations     bf16     (B, H, 64, 48)   (NHWC)
 *   48 -> 48 weights       bf16     (9, 48, 48)      W[tap][co][ci]
 *   thin-layer weights     float32  (9, 48)          W[tap][co] (1 -> 48) or W[tap][ci] (48 -> 1)
 * with tap = 3 (dy + 1) + (dx + 1); every convolution wraps periodically in
 * both directions.
 */
#ifndef EXGB_CORRECTOR_H
#define EXGB_CORRECTOR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 48 -> 48 layer on the tcgen05 tensor cores.  mode 0 (forward): out_post =
 * gelu(conv(x) + bias), and out_pre = conv(x) + bias unless out_pre is NULL.
 * mode 1 (backward data): out_pre = conv(x, w) * gelu'(aux), with w the
 * flipped, channel-transposed weights (exgb_adam / exgb_cast_weights write
 * them) and aux the pre-activations of the layer below.  H must be even and
 * x 16-byte aligned.  Bounded device waits: see exgb_conv_status. */
int exgb_conv48(void* stream, const void* x, int B, int H, const void* w, const float* bias, int mode,
                const void* aux, void* out_pre, void* out_post);

/* Synchronises the device; EXGB_ETIMEOUT if a bounded wait of exgb_conv48
 * gave up since the last call (its outputs are then invalid).  Cleared on
 * read. */
int exgb_conv_status(void);

/* 1 -> 48 forward: pre = conv(x) + bias (NULL: not written), post =
 * gelu(pre).  x float32 (B, H, 64); w (9, 48) and bias (48,) float32. */
int exgb_conv_in1(void* stream, const float* x, int B, int H, const float* w, const float* bias, void* pre,
                  void* post);

/* 48 -> 1 forward: out = base + scale * (conv(h) + bias[0]); base may be
 * NULL (0).  w (9, 48) float32. */
int exgb_conv_out1(void* stream, const void* h, int B, int H, const float* w, const float* bias, const float* base,
                   float scale, float* out);

/* Backward of the 48 -> 1 layer w.r.t. its input, times gelu'(pre):
 * dpre[p][ci] = gelu'(pre[p][ci]) sum_tap w[tap][ci] dout[p - shift(tap)]. */
int exgb_conv_out1_bwd_data(void* stream, const float* dout, int B, int H, const float* w, const void* pre,
                            void* dpre);

/* Weight and bias gradients, as per-chunk partial sums (chunks of 512
 * pixels) and a deterministic reduction into dw, db (float32).
 *   kind 0 (48 -> 48): a = dpre (bf16), bsrc = layer input (bf16);
 *                      part holds nchunk * 9*48*48 floats, part_b nchunk * 48
 *   kind 1 (1 -> 48):  a = dpre (bf16), bsrc = input field (float32);
 *                      part nchunk * 9*48, part_b nchunk * 48
 *   kind 2 (48 -> 1):  a = dout (float32), bsrc = layer input (bf16);
 *                      part nchunk * 9*48, part_b nchunk
 * with nchunk = ceil(B * H * 64 / 512). */
int exgb_wgrad(void* stream, int kind, const void* a, const void* bsrc, int B, int H, float* part, float* part_b,
               float* dw, float* db);

/* One Adam step (bias-corrected, step count t >= 1) on n FP32 master weights
 * w with moments m, v and gradient g; writes the bf16 working copy w16
 * unless it is NULL and, for a 48 -> 48 layer (is48, n = 9*48*48), the
 * flipped copy wflip unless it is NULL. */
int exgb_adam(void* stream, float* w, float* m, float* v, const float* g, int64_t n, float lr, float b1, float b2,
              float eps, int64_t t, void* w16, void* wflip, int is48);

/* The bf16 working copy (and flipped copy, is48) of n FP32 weights; either
 * output may be NULL. */
int exgb_cast_weights(void* stream, const float* w, int64_t n, void* w16, void* wflip, int is48);

/* Mean squared error: loss_part[b] = per-block sums of (pred - target)^2 over
 * nblocks blocks (1..65535), grad = 2 (pred - target) / n * scale. */
int exgb_mse(void* stream, const float* pred, const float* target, int64_t n, float scale, float* grad,
             float* loss_part, int nblocks);

/* Spectral-energy guard: per sample of corr_hat / plain_hat (complex64,
 * (B, H, 33) half spectra), trips when the correction's energy above
 * |k| > kg exceeds thresh times the plain state's energy, or is not finite;
 * a tripped sample's state (B, H, 64) is overwritten by plain.  tripped[b]
 * = 1 / 0. */
int exgb_guard(void* stream, const void* corr_hat, const void* plain_hat, int B, int H, int kg, float thresh,
               const float* plain, float* state, int* tripped);

#ifdef __cplusplus
}
#endif

#endif /* EXGB_CORRECTOR_H */
