// Dense kernel-matrix emission for GenericKernel::KernelMatrix
// (generic-kernel.txx:213-329): M[(s*K0+k0)][(t*K1+k1)] = scale * K_{k0,k1}(x_t - y_s, n_s),
// row-major, source-major.  Threads run along targets, so a warp's stores to a
// matrix row are one contiguous segment; grid.y strides over groups of sources.
// FP64 and FP32 entries come from the plain formula (write-bandwidth bound in
// FP32, FP64-pipe bound in FP64); the mixed mode evaluates double-float entries
// and rounds them to FP64 without FP64 instructions (df_convert.h).
#pragma once

#include "df_convert.h"
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

// grid.x over target blocks of KM_THREADS; grid.y strides over source groups of KM_SROWS.
template <int KER, int MODE, int NEWTON, class Real>
__global__ void __launch_bounds__(KM_THREADS)
    kernel_matrix_kernel(int64_t nt, const Real* __restrict__ r_trg, int64_t ns, const Real* __restrict__ r_src,
                         const Real* __restrict__ n_src, Real* __restrict__ M, double scale, const BBox* bb) {
  constexpr int K0 = KDims<KER>::K0, K1 = KDims<KER>::K1, ND = KDims<KER>::ND;
  const int64_t t = (int64_t)blockIdx.x * KM_THREADS + threadIdx.x;
  if (t >= nt) return;
  const int64_t ld = nt * K1;
  {
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

// ---- mixed precision: double-float entries, written as rounded doubles ----
// One launch, no scratch: every point is split once into hi + lo floats (the
// target by its thread, a CTA's group of sources by the CTA into shared
// memory); a coordinate difference is formed by TwoSum of the hi parts plus
// the difference of the lo parts (accurate to ~2^-48 of the coordinates).
// Per entry the kernel is evaluated in double-float and stored through
// df_to_double, so the FP64 pipe is not on the per-entry path.  The scale
// factor is folded in as a double-float constant.
constexpr int KMD_SROWS = 8;     // sources staged per group
constexpr int KMD_GROUPS = 8;    // groups per CTA before the grid strides (amortises the target split)

template <int ND>
struct KmSrc {
  float xh, yh, zh, xl, yl, zl;
};
template <>
struct KmSrc<3> {
  float xh, yh, zh, xl, yl, zl, nh0, nh1, nh2, nl0, nl1, nl2;
};

// Double-float entries of one (target, source) pair, rounded to FP64: w[k0][k1].
template <int KER, class SrcT>
__device__ __forceinline__ void kmat_df_pair(const float (&th)[3], const float (&tl)[3], const SrcT& r, f2 S,
                                             double (&w)[3][3]) {
  constexpr int ND = KDims<KER>::ND;
  const float sh[3] = {r.xh, r.yh, r.zh}, sl[3] = {r.xl, r.yl, r.zl};
  float dh[3], dl[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const f2 a = two_sum(th[k], -sh[k]);
    const f2 v = two_sum(a.h, a.l + (tl[k] - sl[k]));  // |a.h| may be as small as the lo terms
    dh[k] = v.h;
    dl[k] = v.l;
  }
  const f2 p0 = two_prod(dh[0], dh[0]), p1 = two_prod(dh[1], dh[1]), p2 = two_prod(dh[2], dh[2]);
  const f2 s1 = two_sum(p0.h, p1.h);
  const f2 s2 = two_sum(s1.h, p2.h);
  const float R = s2.h;
  float Rl = fmaf(dh[2], dl[2], fmaf(dh[1], dl[1], dh[0] * dl[0]));
  Rl = fmaf(2.f, Rl, (p0.l + p1.l) + (p2.l + s1.l) + s2.l);
  float y0 = rsqrt_seed(R);
  y0 = R > 0.f ? y0 : 0.f;  // r = 0: every entry 0
  const f2 q = two_prod(y0, y0);
  float rho = fmaf(-q.h, R, 1.f);
  rho = fmaf(-q.l, R, rho);
  rho = fmaf(-q.h, Rl, rho);
  float nh[3] = {0.f, 0.f, 0.f}, nl[3] = {0.f, 0.f, 0.f};
  if constexpr (ND == 3) {
    nh[0] = r.nh0, nh[1] = r.nh1, nh[2] = r.nh2;
    nl[0] = r.nl0, nl[1] = r.nl1, nl[2] = r.nl2;
  }
  if constexpr (KER == KER_LFXU) {
    const f2 y = {y0, (0.5f * y0) * rho};
    const f2 u = df_mul(y, S);
    w[0][0] = df_to_double(u.h, u.l);
  } else {
    f2 y3 = df_mulf(q, y0);  // y0^3 (1 + 3 rho / 2)
    y3.l = fmaf(y3.h, 1.5f * rho, y3.l);
    if constexpr (KER == KER_LDXU) {
      const f2 u = df_mul(df_mul(df_dot3(dh, dl, nh[0], nh[1], nh[2], nl[0], nl[1], nl[2]), y3), S);
      w[0][0] = df_to_double(u.h, u.l);
    } else {
      const f2 d[3] = {{dh[0], dl[0]}, {dh[1], dl[1]}, {dh[2], dl[2]}};
      f2 c, diag = {0.f, 0.f};
      if constexpr (KER == KER_SFXU) {  // u_ij = S (delta_ij y + d_i d_j y^3)
        const f2 y = {y0, (0.5f * y0) * rho};
        diag = df_mul(y, S);
        c = df_mul(y3, S);
      } else {  // u_ij = S d_i d_j (d . n) y^5
        const f2 q2 = df_mul(q, q);
        f2 y5 = df_mulf(q2, y0);  // y0^5 (1 + 5 rho / 2)
        y5.l = fmaf(y5.h, 2.5f * rho, y5.l);
        c = df_mul(df_mul(df_dot3(dh, dl, nh[0], nh[1], nh[2], nl[0], nl[1], nl[2]), y5), S);
      }
      f2 e[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) e[i] = df_mul(d[i], c);
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = i; j < 3; ++j) {
          f2 v = df_mul(e[i], d[j]);
          if (KER == KER_SFXU && i == j) v = df_add(v, diag);
          w[i][j] = w[j][i] = df_to_double(v.h, v.l);
        }
    }
  }
}

// grid.x over target blocks of KM_THREADS; grid.y strides over source blocks of
// KMD_GROUPS x KMD_SROWS.  One-component kernels store straight from registers
// (a warp's entries of a row are 32 consecutive doubles); three-component
// kernels stage each warp's three row segments (96 doubles each) in shared
// memory and write them as 16-byte vectors when the rows are 16-byte aligned
// (`vec`).
template <int KER>
__global__ void __launch_bounds__(KM_THREADS)
    kernel_matrix_df_kernel(int64_t nt, const double* __restrict__ r_trg, int64_t ns,
                            const double* __restrict__ r_src, const double* __restrict__ n_src,
                            double* __restrict__ M, float scale_h, float scale_l, int vec) {
  constexpr int K0 = KDims<KER>::K0, K1 = KDims<KER>::K1, ND = KDims<KER>::ND;
  constexpr int WARPS = KM_THREADS / 32;
  __shared__ KmSrc<ND> srec[KMD_SROWS];
  __shared__ __align__(16) double stage[K1 > 1 ? WARPS : 1][K1 > 1 ? K0 * 32 * K1 : 2];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t t0 = (int64_t)blockIdx.x * KM_THREADS + warp * 32;  // this warp's first target
  const int64_t t = t0 + lane;
  const bool live = t < nt;
  const int nvalid = (int)(nt - t0 < 32 ? (nt - t0 > 0 ? nt - t0 : 0) : 32);
  const int64_t ld = nt * K1;
  float th[3] = {0.f, 0.f, 0.f}, tl[3] = {0.f, 0.f, 0.f};
  if (live)
#pragma unroll
    for (int k = 0; k < 3; ++k) split_val(r_trg[t * 3 + k], th[k], tl[k]);
  const f2 S = {scale_h, scale_l};
  constexpr int BLOCK = KMD_GROUPS * KMD_SROWS;
  for (int64_t b0 = (int64_t)blockIdx.y * BLOCK; b0 < ns; b0 += (int64_t)gridDim.y * BLOCK) {
    for (int64_t s0 = b0; s0 < b0 + BLOCK && s0 < ns; s0 += KMD_SROWS) {
      const int nrow = (int)(ns - s0 < KMD_SROWS ? ns - s0 : KMD_SROWS);
      __syncthreads();  // the previous group's records are no longer read
      if (threadIdx.x < nrow) {
        const int64_t s = s0 + threadIdx.x;
        KmSrc<ND> r;
        split_val(r_src[s * 3 + 0], r.xh, r.xl);
        split_val(r_src[s * 3 + 1], r.yh, r.yl);
        split_val(r_src[s * 3 + 2], r.zh, r.zl);
        if constexpr (ND == 3) {
          split_val(n_src[s * 3 + 0], r.nh0, r.nl0);
          split_val(n_src[s * 3 + 1], r.nh1, r.nl1);
          split_val(n_src[s * 3 + 2], r.nh2, r.nl2);
        }
        srec[threadIdx.x] = r;
      }
      __syncthreads();
#pragma unroll 1
      for (int si = 0; si < nrow; ++si) {
        const int64_t s = s0 + si;
        double w[3][3];
        kmat_df_pair<KER>(th, tl, srec[si], S, w);
        if constexpr (K1 == 1) {
          if (live) M[s * ld + t] = w[0][0];
        } else {
          double* st = stage[warp];
#pragma unroll
          for (int k0 = 0; k0 < K0; ++k0)
#pragma unroll
            for (int k1 = 0; k1 < K1; ++k1) st[k0 * 32 * K1 + lane * K1 + k1] = w[k0][k1];
          __syncwarp();
          const int len = nvalid * K1;  // doubles of each row segment
          for (int k0 = 0; k0 < K0; ++k0) {
            double* row = M + (s * K0 + k0) * ld + t0 * K1;
            const double* sr = st + k0 * 32 * K1;
            if (vec) {
              for (int i = 2 * lane; i + 1 < len; i += 64)
                *reinterpret_cast<double2*>(row + i) = *reinterpret_cast<const double2*>(sr + i);
              if ((len & 1) && lane == 0) row[len - 1] = sr[len - 1];
            } else {
              for (int i = lane; i < len; i += 32) row[i] = sr[i];
            }
          }
          __syncwarp();
        }
      }
    }
  }
}

}  // namespace sctlgpu
