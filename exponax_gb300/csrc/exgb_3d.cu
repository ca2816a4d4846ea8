// exgb_3d.cu -- 3D velocity-form Navier-Stokes / Kolmogorov flow stepping
// (NavierStokesVelocity, KolmogorovFlowVelocity) and 3D linear ETDRK0.
//
// Reference: nonlin_fun/_projected_convection.py:19-226 (curl, u x curl u,
// post-mask, Leray projection, forcing), nonlin_fun/_leray.py:114-136
// (P(v^) = v^ + ik p^, p^ = -inv_lap (ik . v^), inv_lap(0) = 0),
// etdrk/_etdrk_1..4.py (stage formulas).
//
// Staged design over chunks of samples: per ETDRK stage
//   derive3d  : mask . (ik x u^) and mask . u^        -> 6 spectra
//   irfftn(3D): 6 inverse transforms (rows c2r + two strided column passes)
//   cross3d   : u x (curl u) in physical space       -> 3 real fields
//   rfftn(3D) : 3 forward transforms
//   stage3d   : post-mask, Leray projection, forcing and the ETDRK stage
//               update for all three channels of a mode in one thread
// The stage buffers are plan-owned (allocated on the first call at a given
// chunk size).
#include <cuda_runtime.h>

#include <algorithm>

#include "exgb_internal.h"

namespace exgb {

void* workspace(size_t bytes, int slot_offset);
int rfftn_impl(cudaStream_t st, int D, int N, int64_t count, const float* in, float2* out);
int irfftn_impl(cudaStream_t st, int D, int N, int64_t count, const float2* in, float* out);

struct Geo3 {
  int N, M;
  int64_t per;  // N*N*M modes per field
  int K;        // mask cutoff
  float ks;     // 2 pi / L
};

__device__ __forceinline__ void mode3(const Geo3& g, int64_t r, int& kx, int& ky, int& kz) {
  kz = (int)(r % g.M);
  const int64_t t = r / g.M;
  ky = (int)(t % g.N);
  kx = (int)(t / g.N);
}
__device__ __forceinline__ int sgn3(int i, int N) { return (i <= (N - 1) / 2) ? i : i - N; }

// W[b][0..2] = mask (ik x X[b]); W[b][3..5] = mask X[b]
__global__ void derive3d_kernel(Geo3 g, int64_t cb, const float2* __restrict__ X, float2* __restrict__ W) {
  const int64_t total = cb * g.per;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = t / g.per, r = t - b * g.per;
    int kx, ky, kz;
    mode3(g, r, kx, ky, kz);
    const int sx = sgn3(kx, g.N), sy = sgn3(ky, g.N);
    const bool m = (abs(sx) <= g.K) && (abs(sy) <= g.K) && (kz <= g.K);
    const float2* x = X + b * 3 * g.per + r;
    float2* w = W + b * 6 * g.per + r;
    if (!m) {
      for (int f = 0; f < 6; ++f) w[f * g.per] = make_float2(0.f, 0.f);
      continue;
    }
    const float d0 = g.ks * sx, d1 = g.ks * sy, d2 = g.ks * kz;  // d_a = i d_a
    const float2 u0 = x[0], u1 = x[g.per], u2 = x[2 * g.per];
    // (i d) x u: c1 = i(d1 u2 - d2 u1), c2 = i(d2 u0 - d0 u2), c3 = i(d0 u1 - d1 u0)
    const float2 a1 = make_float2(d1 * u2.x - d2 * u1.x, d1 * u2.y - d2 * u1.y);
    const float2 a2 = make_float2(d2 * u0.x - d0 * u2.x, d2 * u0.y - d0 * u2.y);
    const float2 a3 = make_float2(d0 * u1.x - d1 * u0.x, d0 * u1.y - d1 * u0.y);
    w[0] = make_float2(-a1.y, a1.x);
    w[g.per] = make_float2(-a2.y, a2.x);
    w[2 * g.per] = make_float2(-a3.y, a3.x);
    w[3 * g.per] = u0;
    w[4 * g.per] = u1;
    w[5 * g.per] = u2;
  }
}

// C[b][c] = (velocity x curl)_c with velocity = P[b][3..5], curl = P[b][0..2]
__global__ void cross3d_kernel(int64_t n3, int64_t cb, const float* __restrict__ P, float* __restrict__ C) {
  const int64_t total = cb * n3;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = t / n3, r = t - b * n3;
    const float* p = P + b * 6 * n3 + r;
    const float w0 = p[0], w1 = p[n3], w2 = p[2 * n3];
    const float v0 = p[3 * n3], v1 = p[4 * n3], v2 = p[5 * n3];
    float* c = C + b * 3 * n3 + r;
    c[0] = v1 * w2 - v2 * w1;
    c[n3] = v2 * w0 - v0 * w2;
    c[2 * n3] = v0 * w1 - v1 * w0;
  }
}

struct Bufs3 {
  float2 *U, *S1, *S, *N0, *N1, *N2;  // each (cb, 3, per)
};

__device__ __forceinline__ float2 upd3(const PlanDev& P, const Bufs3& b, int64_t o, int64_t c, int stage, float2 nv) {
  switch (P.order) {
    case 1: {
      const float2 r = cadd(cmul(P.E[c], b.U[o]), cscale(nv, P.c[0][c]));
      b.U[o] = r;
      return r;
    }
    case 2:
      if (stage == 0) {
        const float2 s = cadd(cmul(P.E[c], b.U[o]), cscale(nv, P.c[0][c]));
        b.N0[o] = nv;
        b.S[o] = s;
        return s;
      } else {
        const float2 r = cadd(b.S[o], cscale(csub(nv, b.N0[o]), P.c[1][c]));
        b.U[o] = r;
        return r;
      }
    case 3:
      if (stage == 0) {
        const float2 s = cadd(cmul(P.Eh[c], b.U[o]), cscale(nv, P.c[0][c]));
        b.N0[o] = nv;
        b.S[o] = s;
        return s;
      } else if (stage == 1) {
        const float2 s = cadd(cmul(P.E[c], b.U[o]), cscale(csub(cscale(nv, 2.f), b.N0[o]), P.c[1][c]));
        b.N1[o] = nv;
        b.S[o] = s;
        return s;
      } else {
        float2 r = cmul(P.E[c], b.U[o]);
        r = cadd(r, cscale(b.N0[o], P.c[2][c]));
        r = cadd(r, cscale(b.N1[o], P.c[3][c]));
        r = cadd(r, cscale(nv, P.c[4][c]));
        b.U[o] = r;
        return r;
      }
    default:
      if (stage == 0) {
        const float2 s = cadd(cmul(P.Eh[c], b.U[o]), cscale(nv, P.c[0][c]));
        b.N0[o] = nv;
        b.S1[o] = s;
        return s;
      } else if (stage == 1) {
        const float2 s = cadd(cmul(P.Eh[c], b.U[o]), cscale(nv, P.c[0][c]));
        b.N1[o] = nv;
        b.S[o] = s;
        return s;
      } else if (stage == 2) {
        const float2 s = cadd(cmul(P.Eh[c], b.S1[o]), cscale(csub(cscale(nv, 2.f), b.N0[o]), P.c[0][c]));
        b.N2[o] = nv;
        b.S[o] = s;
        return s;
      } else {
        float2 r = cmul(P.E[c], b.U[o]);
        r = cadd(r, cscale(b.N0[o], P.c[3][c]));
        r = cadd(r, cscale(cadd(b.N1[o], b.N2[o]), 2.f * P.c[4][c]));
        r = cadd(r, cscale(nv, P.c[5][c]));
        b.U[o] = r;
        return r;
      }
  }
}

// Post-mask + Leray projection + forcing of the transformed convection H,
// then (stage >= 0) the ETDRK update, or (stage < 0) N^ written to `nout`.
__global__ void stage3d_kernel(PlanDev P, Geo3 g, int64_t cb, const float2* __restrict__ H, Bufs3 b, int stage,
                               float2* __restrict__ nout) {
  const int64_t total = cb * g.per;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t bb = t / g.per, r = t - bb * g.per;
    int kx, ky, kz;
    mode3(g, r, kx, ky, kz);
    const int sx = sgn3(kx, g.N), sy = sgn3(ky, g.N);
    const bool m = (abs(sx) <= g.K) && (abs(sy) <= g.K) && (kz <= g.K);
    const float2* h = H + bb * 3 * g.per + r;
    float2 n0 = make_float2(0.f, 0.f), n1 = n0, n2 = n0;
    if (m) {
      n0 = h[0];
      n1 = h[g.per];
      n2 = h[2 * g.per];
      // Leray: v + (i d) p, p = -inv_lap (i d . v), inv_lap = 1/lap (0 at k = 0), lap = -|d|^2
      const float d0 = g.ks * sx, d1 = g.ks * sy, d2 = g.ks * kz;
      const float lap = -(d0 * d0 + d1 * d1 + d2 * d2);
      if (lap != 0.f) {
        const float il = 1.f / lap;
        // div = i (d0 n0 + d1 n1 + d2 n2)
        const float2 s = make_float2(d0 * n0.x + d1 * n1.x + d2 * n2.x, d0 * n0.y + d1 * n1.y + d2 * n2.y);
        const float2 div = make_float2(-s.y, s.x);
        const float2 p = make_float2(-il * div.x, -il * div.y);
        // (i d_a) p
        n0 = cadd(n0, make_float2(-d0 * p.y, d0 * p.x));
        n1 = cadd(n1, make_float2(-d1 * p.y, d1 * p.x));
        n2 = cadd(n2, make_float2(-d2 * p.y, d2 * p.x));
      }
    }
    if (P.inj_mode >= 0 && kx == 0 && sy == P.inj_mode && kz == 0) n0.x += P.inj_value;
    const int64_t base = bb * 3 * g.per + r;
    if (stage < 0) {
      nout[base] = n0;
      nout[base + g.per] = n1;
      nout[base + 2 * g.per] = n2;
      continue;
    }
    const int64_t cidx = r;  // one coefficient set shared by the three channels
    upd3(P, b, base, cidx, stage, n0);
    upd3(P, b, base + g.per, cidx, stage, n1);
    upd3(P, b, base + 2 * g.per, cidx, stage, n2);
  }
}

// c2r projection of a physical round trip on the kz = 0 and kz = N/2 planes:
// v(kx,ky) <- (v(kx,ky) + conj(v(-kx,-ky))) / 2, one thread per pair.
__global__ void proj3d_kernel(Geo3 g, int64_t nfields, float2* __restrict__ X) {
  const int nplanes = (g.N % 2 == 0) ? 2 : 1;
  const int64_t per_plane = (int64_t)g.N * g.N;
  const int64_t total = nfields * nplanes * per_plane;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t f = t / (nplanes * per_plane);
    const int64_t rr = t - f * nplanes * per_plane;
    const int pl = (int)(rr / per_plane);
    const int64_t q = rr - (int64_t)pl * per_plane;
    const int kx = (int)(q / g.N), ky = (int)(q % g.N);
    const int kx2 = (g.N - kx) % g.N, ky2 = (g.N - ky) % g.N;
    const int64_t i1 = (int64_t)kx * g.N + ky, i2 = (int64_t)kx2 * g.N + ky2;
    if (i2 < i1) continue;  // the pair is handled by its smaller index
    const int kz = pl == 0 ? 0 : g.N / 2;
    float2* base = X + f * g.per + kz;
    const float2 a = base[i1 * g.M], c = base[i2 * g.M];
    const float2 p = make_float2(0.5f * (a.x + c.x), 0.5f * (a.y - c.y));
    base[i1 * g.M] = p;
    base[i2 * g.M] = cconj(p);
  }
}

// ETDRK0 in 3D (any channel count): u^ <- E u^ with the optional projection.
__global__ void scale3d_kernel(const float2* __restrict__ E, int lin_ch, int C, Geo3 g, int64_t nfields,
                               const float2* in, float2* out) {
  const int64_t total = nfields * g.per;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t f = t / g.per, r = t - f * g.per;
    const int ch = (int)(f % C);
    out[t] = cmul(E[(lin_ch == 1 ? 0 : (int64_t)ch * g.per) + r], in[t]);
  }
}

static unsigned grid_for(int64_t n, int sm) {
  const int64_t b = (n + 255) / 256;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)sm * 32));
}

// Multi-step in Fourier space for 3D plans; `project` applies the c2r
// projection after every step (repeat / rollout semantics).
int steps3d_run(const exgb_plan* plan, cudaStream_t st, const float2* in, float2* out, int64_t batch, int nsteps,
                int project, int nonlinear_only) {
  const PlanDev& P = plan->dev;
  Geo3 g;
  g.N = P.N;
  g.M = P.M;
  g.per = (int64_t)P.N * P.N * P.M;
  g.K = std::min(P.kmax, P.N / 2);
  g.ks = P.kscale;
  const int sm = plan->sm_count;
  const int64_t n3 = (int64_t)P.N * P.N * P.N;
  const int C = P.C;
  const bool linear = (P.order == 0 || P.kind == EXGB_NL_ZERO);
  if (linear) {
    if (nonlinear_only) {
      EXGB_CUDA(cudaMemsetAsync(out, 0, sizeof(float2) * (size_t)batch * C * g.per, st));
      return EXGB_OK;
    }
    const int64_t nf = batch * C;
    if (nsteps == 0 && in != out)
      EXGB_CUDA(cudaMemcpyAsync(out, in, sizeof(float2) * nf * g.per, cudaMemcpyDeviceToDevice, st));
    const float2* src = in;
    for (int s = 0; s < nsteps; ++s) {
      scale3d_kernel<<<grid_for(nf * g.per, sm), 256, 0, st>>>(P.E, P.lin_ch, C, g, nf, src, out);
      if (project) proj3d_kernel<<<grid_for(nf * g.N * g.N * 2, sm), 256, 0, st>>>(g, nf, out);
      src = out;
    }
    EXGB_CUDA(cudaGetLastError());
    return EXGB_OK;
  }
  if (C != 3) return fail(EXGB_ESHAPE, "3D projected convection needs 3 channels");
  // chunk of samples whose buffers fit in ~1 GiB
  const int nb = P.order <= 1 ? 1 : P.order == 2 ? 3 : P.order == 3 ? 4 : 6;
  const size_t per_sample = sizeof(float2) * (size_t)g.per * (3 * nb + 6 + 3) + sizeof(float) * (size_t)n3 * 9;
  int64_t cb = std::max<int64_t>(1, std::min<int64_t>(batch, (int64_t)((size_t)(1u << 30) / per_sample)));
  char* ws = (char*)workspace(per_sample * (size_t)cb, 4);
  if (!ws) return fail(EXGB_ENOMEM, "workspace allocation failed");
  float2* q = (float2*)ws;
  const int64_t fsz = 3 * g.per * cb;
  Bufs3 b{};
  b.U = q;
  q += fsz;
  if (P.order >= 2) {
    b.S = q;
    q += fsz;
    b.N0 = q;
    q += fsz;
  }
  if (P.order >= 3) {
    b.N1 = q;
    q += fsz;
  }
  if (P.order == 4) {
    b.S1 = q;
    q += fsz;
    b.N2 = q;
    q += fsz;
  }
  float2* W = q;
  q += 2 * fsz;
  float2* H = q;
  q += fsz;
  float* Pp = (float*)q;
  float* Cp = Pp + 6 * n3 * cb;
  const int nst = nonlinear_only ? 1 : P.order;
  for (int64_t b0 = 0; b0 < batch; b0 += cb) {
    const int64_t nb_ = std::min<int64_t>(cb, batch - b0);
    const float2* src = in + b0 * 3 * g.per;
    float2* dst = out + b0 * 3 * g.per;
    EXGB_CUDA(cudaMemcpyAsync(b.U, src, sizeof(float2) * 3 * g.per * nb_, cudaMemcpyDeviceToDevice, st));
    const int Q = nonlinear_only ? 1 : nsteps * P.order;
    for (int qq = 0; qq < Q; ++qq) {
      const int stage = qq % nst;
      const float2* xin = (stage == 0) ? b.U : (P.order == 4 && stage == 1) ? b.S1 : b.S;
      derive3d_kernel<<<grid_for(nb_ * g.per, sm), 256, 0, st>>>(g, nb_, xin, W);
      int rc = irfftn_impl(st, 3, g.N, nb_ * 6, W, Pp);
      if (rc) return rc;
      cross3d_kernel<<<grid_for(nb_ * n3, sm), 256, 0, st>>>(n3, nb_, Pp, Cp);
      rc = rfftn_impl(st, 3, g.N, nb_ * 3, Cp, H);
      if (rc) return rc;
      if (nonlinear_only) {
        stage3d_kernel<<<grid_for(nb_ * g.per, sm), 256, 0, st>>>(P, g, nb_, H, b, -1, dst);
      } else {
        stage3d_kernel<<<grid_for(nb_ * g.per, sm), 256, 0, st>>>(P, g, nb_, H, b, stage, nullptr);
        if (stage == nst - 1 && project)
          proj3d_kernel<<<grid_for(nb_ * 3 * g.N * g.N * 2, sm), 256, 0, st>>>(g, nb_ * 3, b.U);
      }
      EXGB_CUDA(cudaGetLastError());
    }
    if (!nonlinear_only)
      EXGB_CUDA(cudaMemcpyAsync(dst, b.U, sizeof(float2) * 3 * g.per * nb_, cudaMemcpyDeviceToDevice, st));
  }
  return EXGB_OK;
}

}  // namespace exgb

namespace exgb {

// Standalone Leray projection of `count` D-channel fields (D = 2 or 3).
__global__ void leray_kernel(int D, int N, float ks, int64_t count, const float2* in, float2* out) {
  const int M = N / 2 + 1;
  const int64_t per = (D == 2) ? (int64_t)N * M : (int64_t)N * N * M;
  const int64_t total = count * per;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t f = t / per, r = t - f * per;
    int k[3] = {0, 0, 0};
    k[D - 1] = (int)(r % M);
    int64_t rest = r / M;
    for (int a = D - 2; a >= 0; --a) {
      const int i = (int)(rest % N);
      rest /= N;
      k[a] = (i <= (N - 1) / 2) ? i : i - N;
    }
    float d[3];
    float lap = 0.f;
    for (int a = 0; a < D; ++a) {
      d[a] = ks * (float)k[a];
      lap -= d[a] * d[a];
    }
    const float2* v = in + f * D * per + r;
    float2* o = out + f * D * per + r;
    float2 vv[3];
    float2 s = make_float2(0.f, 0.f);
    for (int a = 0; a < D; ++a) {
      vv[a] = v[a * per];
      s.x += d[a] * vv[a].x;
      s.y += d[a] * vv[a].y;
    }
    if (lap != 0.f) {
      const float il = 1.f / lap;
      const float2 div = make_float2(-s.y, s.x);
      const float2 p = make_float2(-il * div.x, -il * div.y);
      for (int a = 0; a < D; ++a) vv[a] = cadd(vv[a], make_float2(-d[a] * p.y, d[a] * p.x));
    }
    for (int a = 0; a < D; ++a) o[a * per] = vv[a];
  }
}

}  // namespace exgb

extern "C" int exgb_leray(void* stream, int num_spatial_dims, int num_points, double domain_extent, int64_t count,
                          const void* in, void* out) {
  using namespace exgb;
  if (!in || !out) return fail(EXGB_EINVAL, "NULL pointer");
  if (num_spatial_dims < 2 || num_spatial_dims > 3) return fail(EXGB_EUNSUPPORTED, "Leray projection needs D = 2 or 3");
  if (num_points < 2 || count < 0) return fail(EXGB_EINVAL, "bad size");
  const int64_t per = (num_spatial_dims == 2) ? (int64_t)num_points * (num_points / 2 + 1)
                                              : (int64_t)num_points * num_points * (num_points / 2 + 1);
  const int64_t total = count * per;
  if (total == 0) return EXGB_OK;
  const unsigned blocks = (unsigned)std::min<int64_t>((total + 255) / 256, 65535);
  leray_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(num_spatial_dims, num_points,
                                                         (float)(2.0 * M_PI / domain_extent), count,
                                                         (const float2*)in, (float2*)out);
  EXGB_CUDA(cudaGetLastError());
  return EXGB_OK;
}
