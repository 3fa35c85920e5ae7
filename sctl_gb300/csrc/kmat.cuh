// Dense kernel-matrix emission for GenericKernel::KernelMatrix
// (generic-kernel.txx:213-329): M[(s*K0+k0)][(t*K1+k1)] = scale * K_{k0,k1}(x_t - y_s, n_s),
// row-major, source-major.  Write-bandwidth bound for large blocks: each CTA
// row covers KM_SROWS sources, threads run along targets so every store of a
// warp is one contiguous segment of a matrix row.
#pragma once

#include "direct.cuh"

namespace sctlgpu {

constexpr int KM_THREADS = 128;
constexpr int KM_SROWS = 4;

// Plain (FP64 / FP32) entries.
template <int KER, class Real, int NEWTON>
__device__ __forceinline__ void kmat_entries_plain(const Real (&d)[3], const Real (&n)[3], Real (&u)[3][3]) {
  const Real r2 = fma(d[2], d[2], fma(d[1], d[1], d[0] * d[0]));
  Real y = rsqrt_seed(r2);
  y = newton_rsqrt<NEWTON>(y, Real(0.5) * r2);
  y = r2 > Real(0) ? y : Real(0);
  if constexpr (KER == KER_LFXU) {
    u[0][0] = y;
  } else if constexpr (KER == KER_LDXU) {
    u[0][0] = fma(d[2], n[2], fma(d[1], n[1], d[0] * n[0])) * (y * y * y);
  } else if constexpr (KER == KER_SFXU) {
    const Real y3 = y * y * y;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) u[i][j] = (i == j ? y : Real(0)) + d[i] * d[j] * y3;
  } else {
    const Real y2 = y * y;
    const Real c = fma(d[2], n[2], fma(d[1], n[1], d[0] * n[0])) * (y2 * y2 * y);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) u[i][j] = d[i] * d[j] * c;
  }
}

// Double-float entries from a normalised difference dh + dl (the MXDF prologue of direct.cuh).
template <int KER>
__device__ __forceinline__ void kmat_entries_df(const float (&dh)[3], const float (&dl)[3], const float (&nh)[3],
                                                const float (&nl)[3], double (&u)[3][3]) {
  const f2 p0 = two_prod(dh[0], dh[0]), p1 = two_prod(dh[1], dh[1]), p2 = two_prod(dh[2], dh[2]);
  const f2 s1 = two_sum(p0.h, p1.h);
  const f2 s2 = two_sum(s1.h, p2.h);
  const float R = s2.h;
  float Rl = fmaf(dh[2], dl[2], fmaf(dh[1], dl[1], dh[0] * dl[0]));
  Rl = fmaf(2.f, Rl, (p0.l + p1.l) + (p2.l + s1.l) + s2.l);
  float y0 = rsqrt_seed(R);
  y0 = R > 0.f ? y0 : 0.f;
  const f2 q = two_prod(y0, y0);
  float rho = fmaf(-q.h, R, 1.f);
  rho = fmaf(-q.l, R, rho);
  rho = fmaf(-q.h, Rl, rho);
  const f2 y = {y0, (0.5f * y0) * rho};
  auto D = [](f2 v) { return (double)v.h + (double)v.l; };
  if constexpr (KER == KER_LFXU) {
    u[0][0] = D(y);
  } else {
    f2 y3 = df_mulf(q, y0);
    y3.l = fmaf(y3.h, 1.5f * rho, y3.l);
    if constexpr (KER == KER_LDXU) {
      u[0][0] = D(df_mul(df_dot3(dh, dl, nh[0], nh[1], nh[2], nl[0], nl[1], nl[2]), y3));
    } else if constexpr (KER == KER_SFXU) {
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          f2 v = df_mul(df_mul(f2{dh[i], dl[i]}, f2{dh[j], dl[j]}), y3);
          if (i == j) v = df_add(v, y);
          u[i][j] = D(v);
        }
    } else {
      const f2 q2 = df_mul(q, q);
      f2 y5 = df_mulf(q2, y0);
      y5.l = fmaf(y5.h, 2.5f * rho, y5.l);
      const f2 c = df_mul(df_dot3(dh, dl, nh[0], nh[1], nh[2], nl[0], nl[1], nl[2]), y5);
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) u[i][j] = D(df_mul(df_mul(f2{dh[i], dl[i]}, f2{dh[j], dl[j]}), c));
    }
  }
}

// grid.x over target blocks of KM_THREADS; grid.y strides over source groups of KM_SROWS.
template <int KER, int MODE, int NEWTON, class Real>
__global__ void __launch_bounds__(KM_THREADS)
    kernel_matrix_kernel(int64_t nt, const Real* __restrict__ r_trg, int64_t ns, const Real* __restrict__ r_src,
                         const Real* __restrict__ n_src, Real* __restrict__ M, double scale, const BBox* bb) {
  constexpr int K0 = KDims<KER>::K0, K1 = KDims<KER>::K1, ND = KDims<KER>::ND;
  const int64_t t = (int64_t)blockIdx.x * KM_THREADS + threadIdx.x;
  if (t >= nt) return;
  const int64_t ld = nt * K1;
  if constexpr (MODE == MODE_MXDF) {
    const MixedFrame fr = frame_from_bbox(bb);
    float th[3], tl[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) split_coord(fr, k, (double)r_trg[t * 3 + k], th[k], tl[k]);
    for (int64_t s0 = (int64_t)blockIdx.y * KM_SROWS; s0 < ns; s0 += (int64_t)gridDim.y * KM_SROWS)
    for (int si = 0; si < KM_SROWS; ++si) {
      const int64_t s = s0 + si;
      if (s >= ns) break;
      float sh[3], sl[3], nh[3] = {0, 0, 0}, nl[3] = {0, 0, 0};
#pragma unroll
      for (int k = 0; k < 3; ++k) split_coord(fr, k, (double)r_src[s * 3 + k], sh[k], sl[k]);
      if (ND)
#pragma unroll
        for (int k = 0; k < 3; ++k) split_val((double)n_src[s * 3 + k], nh[k], nl[k]);
      float dh[3], dl[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const f2 v = fast_two_sum(th[k] - sh[k], tl[k] - sl[k]);
        dh[k] = v.h;
        dl[k] = v.l;
      }
      double u[3][3];
      kmat_entries_df<KER>(dh, dl, nh, nl, u);
#pragma unroll
      for (int k0 = 0; k0 < K0; ++k0)
#pragma unroll
        for (int k1 = 0; k1 < K1; ++k1) M[(s * K0 + k0) * ld + t * K1 + k1] = (Real)(u[k0][k1] * scale);
    }
  } else {
    const Real x0 = r_trg[t * 3], x1 = r_trg[t * 3 + 1], x2 = r_trg[t * 3 + 2];
    for (int64_t s0 = (int64_t)blockIdx.y * KM_SROWS; s0 < ns; s0 += (int64_t)gridDim.y * KM_SROWS)
    for (int si = 0; si < KM_SROWS; ++si) {
      const int64_t s = s0 + si;
      if (s >= ns) break;
      const Real d[3] = {x0 - r_src[s * 3], x1 - r_src[s * 3 + 1], x2 - r_src[s * 3 + 2]};
      Real n[3] = {0, 0, 0};
      if (ND) {
        n[0] = n_src[s * 3];
        n[1] = n_src[s * 3 + 1];
        n[2] = n_src[s * 3 + 2];
      }
      Real u[3][3];
      kmat_entries_plain<KER, Real, NEWTON>(d, n, u);
#pragma unroll
      for (int k0 = 0; k0 < K0; ++k0)
#pragma unroll
        for (int k1 = 0; k1 < K1; ++k1) M[(s * K0 + k0) * ld + t * K1 + k1] = u[k0][k1] * (Real)scale;
    }
  }
}

}  // namespace sctlgpu
