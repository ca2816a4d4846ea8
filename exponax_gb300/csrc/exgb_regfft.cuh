// exgb_regfft.cuh -- register-resident FFTs with compile-time sizes.
//
// A length-N sequence (N = E * T) is held by a group of T consecutive lanes
// of one warp; lane l owns the E points x[l + T j], j = 0..E-1.  The FFT is
// the two-level Cooley-Tukey split N = E x T:
//   1. length-E DFT over j inside the lane (registers),
//   2. twiddle by w_N^(l k1) (table in shared memory),
//   3. transpose through a per-group shared-memory tile (E x (T+1), padded
//      against bank conflicts; __syncwarp only, no block barrier),
//   4. length-T DFTs over l, lane l taking rows k1 = l + T q.
// The output lands in the same "lane l owns X[l + T j]" distribution, so
// chains of transforms and pointwise products need no data movement.
// Small DFTs (2, 4, 8, 16, 32) are straight-line code with constant
// twiddles exp(-+2 pi i m / 32) written from their exact values.
#pragma once

#include "exgb_fft.cuh"

namespace exgb {

// cos(2 pi q / 32), q = 0..8
__host__ __device__ constexpr float kCos32(int q) {
  return q == 0   ? 1.0f
         : q == 1 ? 0.98078528040323044913f
         : q == 2 ? 0.92387953251128675613f
         : q == 3 ? 0.83146961230254523708f
         : q == 4 ? 0.70710678118654752440f
         : q == 5 ? 0.55557023301960222474f
         : q == 6 ? 0.38268343236508977173f
         : q == 7 ? 0.19509032201612826785f
                  : 0.0f;
}

// exp(-2 pi i m / 32) (forward) as (cos, -sin)
__host__ __device__ constexpr float tw32_re(int m) {
  return (m & 31) / 8 == 0   ? kCos32((m & 31) % 8)
         : (m & 31) / 8 == 1 ? -kCos32(8 - (m & 31) % 8)
         : (m & 31) / 8 == 2 ? -kCos32((m & 31) % 8)
                             : kCos32(8 - (m & 31) % 8);
}
__host__ __device__ constexpr float tw32_sin(int m) {
  return (m & 31) / 8 == 0   ? kCos32(8 - (m & 31) % 8)
         : (m & 31) / 8 == 1 ? kCos32((m & 31) % 8)
         : (m & 31) / 8 == 2 ? -kCos32(8 - (m & 31) % 8)
                             : -kCos32((m & 31) % 8);
}

// v * exp(-+ 2 pi i m / 32), with the trivial angles special-cased
template <int M, bool INV>
__device__ __forceinline__ float2 cmul_c32(float2 v) {
  constexpr int m = M & 31;
  if constexpr (m == 0) return v;
  else if constexpr (m == 8) return mul_mi<INV>(v);                                   // -+ i
  else if constexpr (m == 16) return make_float2(-v.x, -v.y);                         // -1
  else if constexpr (m == 24) return mul_mi<!INV>(v);                                  // +- i
  else {
    constexpr float c = tw32_re(m);
    constexpr float s = INV ? tw32_sin(m) : -tw32_sin(m);  // imaginary part of the twiddle
    return make_float2(fmaf(v.x, c, -v.y * s), fmaf(v.x, s, v.y * c));
  }
}

template <int R, bool INV>
struct SmallDft;

template <bool INV>
struct SmallDft<2, INV> {
  __device__ __forceinline__ static void run(float2* v) { dft2<INV>(v[0], v[1]); }
};
template <bool INV>
struct SmallDft<4, INV> {
  __device__ __forceinline__ static void run(float2* v) { dft4<INV>(v); }
};
template <bool INV>
struct SmallDft<8, INV> {
  __device__ __forceinline__ static void run(float2* v) { dft8<INV>(v); }
};

// R = A * B: n = B n1 + n2, X[k1 + A k2] = DFT_B_n2( w_R^(n2 k1) DFT_A_n1(x[B n1 + n2]) )
template <int A, int B, bool INV>
struct CompositeDft {
  static constexpr int R = A * B;
  __device__ __forceinline__ static void run(float2* v) {
    float2 y[B][A];
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) {
      float2 t[A];
#pragma unroll
      for (int n1 = 0; n1 < A; ++n1) t[n1] = v[B * n1 + n2];
      SmallDft<A, INV>::run(t);
#pragma unroll
      for (int k1 = 0; k1 < A; ++k1) y[n2][k1] = t[k1];
    }
    twiddle<1, 1>(y);
#pragma unroll
    for (int k1 = 0; k1 < A; ++k1) {
      float2 t[B];
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) t[n2] = y[n2][k1];
      SmallDft<B, INV>::run(t);
#pragma unroll
      for (int k2 = 0; k2 < B; ++k2) v[k1 + A * k2] = t[k2];
    }
  }
  // y[n2][k1] *= w_R^(n2 k1) for all n2, k1 (compile-time recursion over indices)
  template <int N2, int K1>
  __device__ __forceinline__ static void twiddle(float2 (&y)[B][A]) {
    if constexpr (N2 < B) {
      if constexpr (K1 < A) {
        y[N2][K1] = cmul_c32<N2 * K1 * (32 / R), INV>(y[N2][K1]);
        twiddle<N2, K1 + 1>(y);
      } else {
        twiddle<N2 + 1, 1>(y);
      }
    }
  }
};

template <bool INV>
struct SmallDft<16, INV> {
  __device__ __forceinline__ static void run(float2* v) { CompositeDft<4, 4, INV>::run(v); }
};
template <bool INV>
struct SmallDft<32, INV> {
  __device__ __forceinline__ static void run(float2* v) { CompositeDft<4, 8, INV>::run(v); }
};

// Group FFT: T lanes (a power of two <= 32, aligned inside the warp), E
// points per lane, N = E * T.  `tile` is this group's scratch of
// E * (T + 1) float2; `twl` the table w_N^(l k1) laid out [k1][l] (forward
// sign).  `mask` is the warp mask of this group's lanes.
template <int E, int T, bool INV>
__device__ __forceinline__ void group_fft(float2 (&v)[E], int l, float2* tile, const float2* __restrict__ twl,
                                          unsigned mask) {
  static_assert(E % T == 0, "E must be a multiple of T");
  SmallDft<E, INV>::run(v);
#pragma unroll
  for (int k1 = 1; k1 < E; ++k1) {
    float2 w = twl[k1 * T + l];
    if (INV) w.y = -w.y;
    v[k1] = cmul(v[k1], w);
  }
#pragma unroll
  for (int k1 = 0; k1 < E; ++k1) tile[k1 * (T + 1) + l] = v[k1];
  __syncwarp(mask);
#pragma unroll
  for (int q = 0; q < E / T; ++q) {
    float2 u[T];
    const int k1 = l + T * q;
#pragma unroll
    for (int m = 0; m < T; ++m) u[m] = tile[k1 * (T + 1) + m];
    SmallDft<T, INV>::run(u);
    // output X[k1 + E k2] -> j = q + (E / T) k2
#pragma unroll
    for (int k2 = 0; k2 < T; ++k2) v[q + (E / T) * k2] = u[k2];
  }
  __syncwarp(mask);
}

// Two independent group FFTs of the same size and direction, interleaved
// for instruction-level parallelism: shared twiddle loads, the transposes
// one after the other through the same tile.
template <int E, int T, bool INV>
__device__ __forceinline__ void group_fft_x2(float2 (&v)[E], float2 (&w)[E], int l, float2* tile,
                                             const float2* __restrict__ twl, unsigned mask) {
  static_assert(E % T == 0, "E must be a multiple of T");
  SmallDft<E, INV>::run(v);
  SmallDft<E, INV>::run(w);
#pragma unroll
  for (int k1 = 1; k1 < E; ++k1) {
    float2 t = twl[k1 * T + l];
    if (INV) t.y = -t.y;
    v[k1] = cmul(v[k1], t);
    w[k1] = cmul(w[k1], t);
  }
#pragma unroll
  for (int k1 = 0; k1 < E; ++k1) tile[k1 * (T + 1) + l] = v[k1];
  __syncwarp(mask);
  float2 u[E / T][T];
#pragma unroll
  for (int q = 0; q < E / T; ++q)
#pragma unroll
    for (int m = 0; m < T; ++m) u[q][m] = tile[(l + T * q) * (T + 1) + m];
  __syncwarp(mask);
#pragma unroll
  for (int k1 = 0; k1 < E; ++k1) tile[k1 * (T + 1) + l] = w[k1];
  __syncwarp(mask);
#pragma unroll
  for (int q = 0; q < E / T; ++q) {
    float2 z[T];
#pragma unroll
    for (int m = 0; m < T; ++m) z[m] = tile[(l + T * q) * (T + 1) + m];
    SmallDft<T, INV>::run(u[q]);
    SmallDft<T, INV>::run(z);
#pragma unroll
    for (int k2 = 0; k2 < T; ++k2) {
      v[q + (E / T) * k2] = u[q][k2];
      w[q + (E / T) * k2] = z[k2];
    }
  }
  __syncwarp(mask);
}

template <int N>
struct RegCfg;
template <>
struct RegCfg<32> {
  static constexpr int E = 8, T = 4;
};
template <>
struct RegCfg<64> {
  static constexpr int E = 8, T = 8;
};
template <>
struct RegCfg<128> {
  static constexpr int E = 16, T = 8;
};
template <>
struct RegCfg<256> {
  static constexpr int E = 16, T = 16;
};
template <>
struct RegCfg<512> {
  static constexpr int E = 32, T = 16;
};

// floats between consecutive groups' tiles: E*(T+1) complex, padded so that
// two groups sharing a 16-lane shared-memory phase use different banks
template <int E, int T>
__host__ __device__ constexpr int tile_stride() {
  return (T >= 16) ? E * (T + 1) : ((E * (T + 1) * 2) % 32 == 16 ? E * (T + 1) : E * (T + 1) + 8);
}

}  // namespace exgb
