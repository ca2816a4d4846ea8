// exgb_fft.cuh -- shared-memory Stockham FFT building blocks for sm_103a.
//
// A length-n complex FFT (n = 2^a 3^b 5^c) runs as a sequence of radix-R
// passes (R in {2,3,4,5,8}).  Pass p reads R elements at stride n/R,
// twiddles them with exp(-+2 pi i r k / (Ns R)) (k = j mod Ns, Ns = product
// of the earlier radices), does a radix-R DFT in registers and writes them
// to (j - k) R + k + r Ns, which leaves the result in natural order after the
// last pass (Stockham autosort, no bit reversal).  Twiddles come from a
// table tw[k] = exp(-2 pi i k / n) computed in FP64 on the host.
//
// All threads of a block (or of a named-barrier group) cooperate on `count`
// independent sequences; one barrier separates passes.  Sequences live in
// shared memory; source/destination addressing is supplied by small
// functors so that the first pass can gather and the last pass can scatter
// into whatever layout the caller needs.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace exgb {

constexpr int kMaxPass = 12;

struct FftPlan {
  int n;
  int npass;
  int radix[kMaxPass];
  // per pass, set by fft_plan_finalize: butterflies per sequence (n / R), product of the earlier
  // radices (Ns), twiddle-table step ((n / R) / Ns), and FP32 reciprocals of the first two for the
  // quotient estimate of fdiv
  int nb[kMaxPass];
  int ns[kMaxPass];
  int step[kMaxPass];
  float rnb[kMaxPass];
  float rns[kMaxPass];
};

// Host: fill the per-pass constants of a plan whose n, npass and radix[] are set.
inline void fft_plan_finalize(FftPlan* p) {
  int Ns = 1;
  for (int i = 0; i < p->npass; ++i) {
    const int R = p->radix[i];
    p->nb[i] = p->n / R;
    p->ns[i] = Ns;
    p->step[i] = (p->n / R) / Ns;
    p->rnb[i] = (float)(1.0 / (double)p->nb[i]);
    p->rns[i] = (float)(1.0 / (double)Ns);
    Ns *= R;
  }
}

// t / d for 0 <= t < 2^24 and d >= 1, with rd = (float)(1 / d): the FP32 product is within 1 of the
// quotient there, so one correction step makes it exact (a dependent chain of a few instructions
// instead of the ~20 of an integer division by a runtime divisor)
__device__ __forceinline__ int fdiv(int t, int d, float rd) {
  int q = __float2int_rz(__int2float_rn(t) * rd);
  const int r = t - q * d;
  q += (r >= d) - (r < 0);
  return q;
}

// ---------------------------------------------------------------- complex helpers
// Additions, subtractions and real scalings of complex values run on the packed FP32 pipe (one
// add/fma/mul .f32x2 for both components, each rounded like the scalar operation; a - b is the exact
// product -1 * b added to a in one rounding).  Measured against the scalar forms on the register-FFT
// kernels: 2.9 % faster at 256^2, 6 % at 512^2, 2.4 % on the 3D three-pass path.
#if !defined(EXGB_SCALAR_COMPLEX)
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return __fmul2_rn(a, make_float2(s, s)); }
#else  // the scalar forms, for a translation unit where they measured faster
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
#endif
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
// multiply by -i (forward) or +i (inverse)
template <bool INV>
__device__ __forceinline__ float2 mul_mi(float2 a) {
  return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// ---------------------------------------------------------------- small DFTs
template <bool INV>
__device__ __forceinline__ void dft2(float2& a, float2& b) {
  float2 t = a;
  a = cadd(t, b);
  b = csub(t, b);
}

template <bool INV>
__device__ __forceinline__ void dft4(float2* v) {
  float2 t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
  float2 t2 = cadd(v[1], v[3]), t3 = mul_mi<INV>(csub(v[1], v[3]));
  v[0] = cadd(t0, t2);
  v[2] = csub(t0, t2);
  v[1] = cadd(t1, t3);
  v[3] = csub(t1, t3);
}

template <bool INV>
__device__ __forceinline__ void dft8(float2* v) {
  const float c = 0.70710678118654752440f;  // sqrt(1/2)
  float2 e[4] = {v[0], v[2], v[4], v[6]};
  float2 o[4] = {v[1], v[3], v[5], v[7]};
  dft4<INV>(e);
  dft4<INV>(o);
  // w8^k = exp(-+ i pi k / 4)
  float2 o1 = INV ? make_float2(c * (o[1].x - o[1].y), c * (o[1].x + o[1].y))
                  : make_float2(c * (o[1].x + o[1].y), c * (o[1].y - o[1].x));
  float2 o2 = mul_mi<INV>(o[2]);
  float2 o3 = INV ? make_float2(-c * (o[3].x + o[3].y), c * (o[3].x - o[3].y))
                  : make_float2(c * (o[3].y - o[3].x), -c * (o[3].x + o[3].y));
  v[0] = cadd(e[0], o[0]);
  v[4] = csub(e[0], o[0]);
  v[1] = cadd(e[1], o1);
  v[5] = csub(e[1], o1);
  v[2] = cadd(e[2], o2);
  v[6] = csub(e[2], o2);
  v[3] = cadd(e[3], o3);
  v[7] = csub(e[3], o3);
}

template <bool INV>
__device__ __forceinline__ void dft3(float2* v) {
  const float s = 0.86602540378443864676f;  // sin(2 pi / 3)
  float2 t = cadd(v[1], v[2]);
  float2 m = make_float2(v[0].x - 0.5f * t.x, v[0].y - 0.5f * t.y);
  float2 d = cscale(csub(v[1], v[2]), s);
  v[0] = cadd(v[0], t);
  float2 id = mul_mi<INV>(d);  // -+ i d
  v[1] = cadd(m, id);
  v[2] = csub(m, id);
}

template <bool INV>
__device__ __forceinline__ void dft5(float2* v) {
  const float c1 = 0.30901699437494742410f;   // cos(2 pi / 5)
  const float c2 = -0.80901699437494742410f;  // cos(4 pi / 5)
  const float s1 = 0.95105651629515357212f;   // sin(2 pi / 5)
  const float s2 = 0.58778525229247312917f;   // sin(4 pi / 5)
  float2 t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
  float2 t3 = csub(v[1], v[4]), t4 = csub(v[2], v[3]);
  float2 a0 = v[0];
  float2 m1 = make_float2(a0.x + c1 * t1.x + c2 * t2.x, a0.y + c1 * t1.y + c2 * t2.y);
  float2 m2 = make_float2(a0.x + c2 * t1.x + c1 * t2.x, a0.y + c2 * t1.y + c1 * t2.y);
  float2 n1 = make_float2(s1 * t3.x + s2 * t4.x, s1 * t3.y + s2 * t4.y);
  float2 n2 = make_float2(s2 * t3.x - s1 * t4.x, s2 * t3.y - s1 * t4.y);
  v[0] = cadd(a0, cadd(t1, t2));
  float2 in1 = mul_mi<INV>(n1), in2 = mul_mi<INV>(n2);
  v[1] = cadd(m1, in1);
  v[4] = csub(m1, in1);
  v[2] = cadd(m2, in2);
  v[3] = csub(m2, in2);
}

template <int R, bool INV>
__device__ __forceinline__ void dftR(float2* v) {
  if constexpr (R == 2) dft2<INV>(v[0], v[1]);
  else if constexpr (R == 3) dft3<INV>(v);
  else if constexpr (R == 4) dft4<INV>(v);
  else if constexpr (R == 5) dft5<INV>(v);
  else if constexpr (R == 8) dft8<INV>(v);
}

// ---------------------------------------------------------------- address maps
// Contiguous sequences: element k of sequence s at p[s * sstride + k].
struct LinMap {
  float2* p;
  int sstride;
  __device__ __forceinline__ float2& operator()(int s, int k) const { return p[s * sstride + k]; }
};

// ---------------------------------------------------------------- one pass
template <int R, bool INV, class Src, class Dst>
__device__ __forceinline__ void stockham_bfly(const Src& src, const Dst& dst, int s, int j, int k, int stride,
                                              int Ns, int step, const float2* __restrict__ tw) {
  float2 v[R];
#pragma unroll
  for (int r = 0; r < R; ++r) v[r] = src(s, j + r * stride);
  if (Ns > 1) {
#pragma unroll
    for (int r = 1; r < R; ++r) {
      float2 w = tw[r * k * step];
      if (INV) w.y = -w.y;
      v[r] = cmul(v[r], w);
    }
  }
  dftR<R, INV>(v);
  const int base = (j - k) * R + k;
#pragma unroll
  for (int r = 0; r < R; ++r) dst(s, base + r * Ns) = v[r];
}

// One radix-R pass over `count` sequences: nb = n / R butterflies per sequence, Ns the product of
// the earlier radices, step = nb / Ns, rnb / rns the FP32 reciprocals of nb / Ns (FftPlan).
template <bool INV, class Src, class Dst>
__device__ __forceinline__ void stockham_pass(int R, const Src& src, const Dst& dst, int count, int nb, int Ns,
                                              int step, float rnb, float rns, const float2* __restrict__ tw,
                                              int tid, int nthr) {
  const int total = nb * count;
  const bool fast = total < (1 << 24);  // fdiv's exact range (uniform across the block)
  switch (R) {
#define EXGB_PASS_CASE(RR)                                                      \
  case RR:                                                                      \
    for (int t = tid; t < total; t += nthr) {                                   \
      const int s = fast ? fdiv(t, nb, rnb) : t / nb;                           \
      const int j = t - s * nb;                                                 \
      const int k = j - (fast ? fdiv(j, Ns, rns) : j / Ns) * Ns;                \
      stockham_bfly<RR, INV>(src, dst, s, j, k, nb, Ns, step, tw);              \
    }                                                                           \
    break;
    EXGB_PASS_CASE(2)
    EXGB_PASS_CASE(3)
    EXGB_PASS_CASE(4)
    EXGB_PASS_CASE(5)
    EXGB_PASS_CASE(8)
#undef EXGB_PASS_CASE
    default:
      break;
  }
}

// Group barrier: whole block (id 0) or a named barrier over `nthr` threads.
struct BlockSync {
  __device__ __forceinline__ void operator()() const { __syncthreads(); }
};
struct NamedSync {
  int id, nthr;
  __device__ __forceinline__ void operator()() const {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthr) : "memory");
  }
};

// Full FFT of `count` sequences.  Input in buf0 (contiguous, stride n);
// passes ping-pong buf0 <-> buf1; the last pass writes through `out`.
// `out` must not alias the source of the last pass (buf0 if npass is odd,
// buf1 if even).  A barrier follows every pass (including the last).
template <bool INV, class Out, class Sync>
__device__ void block_fft(const FftPlan& p, float2* buf0, float2* buf1, const Out& out, int count,
                          const float2* __restrict__ tw, int tid, int nthr, const Sync& sync) {
  const int n = p.n;
  int Ns = 1;
  float2* src = buf0;
  float2* dst = buf1;
  for (int pass = 0; pass < p.npass; ++pass) {
    const int R = p.radix[pass];
    if (pass == p.npass - 1) {
      stockham_pass<INV>(R, LinMap{src, n}, out, count, p.nb[pass], Ns, p.step[pass], p.rnb[pass], p.rns[pass], tw,
                         tid, nthr);
    } else {
      stockham_pass<INV>(R, LinMap{src, n}, LinMap{dst, n}, count, p.nb[pass], Ns, p.step[pass], p.rnb[pass],
                         p.rns[pass], tw, tid, nthr);
    }
    sync();
    Ns *= R;
    float2* t = src;
    src = dst;
    dst = t;
  }
}

// Full FFT of `count` sequences whose first pass reads through the functor `in` (operator()(s, k)
// returning element k of sequence s) and whose last pass writes through `out`, so that an
// elementwise step before and after the transform costs no pass of its own.  Intermediate passes
// ping-pong b0 <-> b1 (pass p writes b0 for even p, b1 for odd p); `out` must not alias the source
// of the last pass (b0 if npass is even, b1 if npass > 1 is odd; `in` if npass == 1).  A barrier
// follows every pass.
template <bool INV, class In, class Out, class Sync>
__device__ void block_fft_io(const FftPlan& p, const In& in, float2* b0, float2* b1, const Out& out, int count,
                             const float2* __restrict__ tw, int tid, int nthr, const Sync& sync) {
  const int n = p.n;
  int Ns = 1;
  for (int pass = 0; pass < p.npass; ++pass) {
    const int R = p.radix[pass];
    const bool last = pass == p.npass - 1;
    float2* dst = (pass & 1) ? b1 : b0;
    if (pass == 0) {
      if (last)
        stockham_pass<INV>(R, in, out, count, p.nb[0], Ns, p.step[0], p.rnb[0], p.rns[0], tw, tid, nthr);
      else
        stockham_pass<INV>(R, in, LinMap{dst, n}, count, p.nb[0], Ns, p.step[0], p.rnb[0], p.rns[0], tw, tid,
                           nthr);
    } else {
      float2* src = (pass & 1) ? b0 : b1;
      if (last)
        stockham_pass<INV>(R, LinMap{src, n}, out, count, p.nb[pass], Ns, p.step[pass], p.rnb[pass], p.rns[pass],
                           tw, tid, nthr);
      else
        stockham_pass<INV>(R, LinMap{src, n}, LinMap{dst, n}, count, p.nb[pass], Ns, p.step[pass], p.rnb[pass],
                           p.rns[pass], tw, tid, nthr);
    }
    sync();
    Ns *= R;
  }
}

// Where block_fft_io's last pass writes when `out` is a LinMap over one of b0 / b1.
__host__ __device__ __forceinline__ float2* io_result_buf(const FftPlan& p, float2* b0, float2* b1) {
  return ((p.npass - 1) & 1) ? b1 : b0;
}

// Buffer that holds the result when the input starts in buf0 and the last
// pass writes through a LinMap over the returned buffer.
__host__ __device__ __forceinline__ float2* result_buf(const FftPlan& p, float2* buf0, float2* buf1) {
  return (p.npass & 1) ? buf1 : buf0;
}

// ---------------------------------------------------------------- real <-> complex packing
// Two Hermitian half-spectra A, B (length n/2+1) -> full spectrum
// Z[k] = A~[k] + i B~[k] with A~ the Hermitian extension of A whose DC and
// Nyquist bins are taken real (what a c2r transform does).  The inverse
// complex FFT of Z is then a + i b, a = irfft(A)*n, b = irfft(B)*n.
__device__ __forceinline__ float2 pack_pair(float2 a, float2 b, bool conj_ext, bool real_only) {
  if (real_only) {
    a.y = 0.f;
    b.y = 0.f;
  } else if (conj_ext) {
    a.y = -a.y;
    b.y = -b.y;
  }
  return make_float2(a.x - b.y, a.y + b.x);
}

// Z = FFT(p + i q) -> half spectra P[k], Q[k] for 0 <= k <= n/2.
__device__ __forceinline__ void unpack_pair(float2 zk, float2 znk, float2& P, float2& Q) {
  // P = (Z[k] + conj(Z[n-k])) / 2 ; Q = (Z[k] - conj(Z[n-k])) / (2i)
  P = make_float2(0.5f * (zk.x + znk.x), 0.5f * (zk.y - znk.y));
  Q = make_float2(0.5f * (zk.y + znk.y), -0.5f * (zk.x - znk.x));
}

}  // namespace exgb
