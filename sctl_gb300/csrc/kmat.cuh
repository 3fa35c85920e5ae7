// Dense kernel-matrix emission for GenericKernel::KernelMatrix
// (generic-kernel.txx:213-329): M[(s*K0+k0)][(t*K1+k1)] = scale * K_{k0,k1}(x_t - y_s, n_s),
// row-major, source-major.  Write-bandwidth bound for large blocks: each CTA
// row covers KM_SROWS sources, threads run along targets so every store of a
// warp is one contiguous segment of a matrix row.
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
// Targets and sources are split once on the call's common grid (exact hi/lo
// differences, as in the mixed direct sum); per entry the kernel is evaluated
// in double-float and stored through df_to_double, so the FP64 pipe is not on
// the per-entry path.  The scale factor is folded in as a double-float constant.
constexpr int KMD_SROWS = 8;

struct KmTrg {
  float xh, yh, zh, xl, yl, zl;
};
template <int ND>
struct KmSrc {
  float xh, yh, zh, pad0, xl, yl, zl, pad1;
};
template <>
struct KmSrc<3> {
  float xh, yh, zh, nh0, xl, yl, zl, nl0, nh1, nh2, nl1, nl2;
};

__global__ void kmat_pack_trg_kernel(int64_t n, const double* __restrict__ x, KmTrg* __restrict__ out,
                                     const BBox* bb) {
  const MixedFrame fr = frame_from_bbox(bb);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    KmTrg r;
    split_coord(fr, 0, x[i * 3 + 0], r.xh, r.xl);
    split_coord(fr, 1, x[i * 3 + 1], r.yh, r.yl);
    split_coord(fr, 2, x[i * 3 + 2], r.zh, r.zl);
    out[i] = r;
  }
}

template <int ND>
__global__ void kmat_pack_src_kernel(int64_t n, const double* __restrict__ x, const double* __restrict__ nrm,
                                     KmSrc<ND>* __restrict__ out, const BBox* bb) {
  const MixedFrame fr = frame_from_bbox(bb);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    KmSrc<ND> r;
    memset(&r, 0, sizeof(r));
    split_coord(fr, 0, x[i * 3 + 0], r.xh, r.xl);
    split_coord(fr, 1, x[i * 3 + 1], r.yh, r.yl);
    split_coord(fr, 2, x[i * 3 + 2], r.zh, r.zl);
    if constexpr (ND == 3) {
      split_val(nrm[i * 3 + 0], r.nh0, r.nl0);
      split_val(nrm[i * 3 + 1], r.nh1, r.nl1);
      split_val(nrm[i * 3 + 2], r.nh2, r.nl2);
    }
    out[i] = r;
  }
}

// grid.x over target blocks of KM_THREADS; grid.y strides over source groups of KMD_SROWS.
template <int KER>
__global__ void __launch_bounds__(KM_THREADS)
    kernel_matrix_df_kernel(int64_t nt, const KmTrg* __restrict__ trg, int64_t ns,
                            const KmSrc<KDims<KER>::ND>* __restrict__ src, double* __restrict__ M, float scale_h,
                            float scale_l) {
  constexpr int K0 = KDims<KER>::K0, K1 = KDims<KER>::K1, ND = KDims<KER>::ND;
  const int64_t t = (int64_t)blockIdx.x * KM_THREADS + threadIdx.x;
  if (t >= nt) return;
  const int64_t ld = nt * K1;
  const KmTrg tg = trg[t];
  const float th[3] = {tg.xh, tg.yh, tg.zh}, tl[3] = {tg.xl, tg.yl, tg.zl};
  const f2 S = {scale_h, scale_l};
  for (int64_t s0 = (int64_t)blockIdx.y * KMD_SROWS; s0 < ns; s0 += (int64_t)gridDim.y * KMD_SROWS) {
#pragma unroll 1
    for (int si = 0; si < KMD_SROWS; ++si) {
      const int64_t s = s0 + si;
      if (s >= ns) break;
      const KmSrc<ND> r = src[s];  // the same record for the whole warp: one broadcast load
      const float sh[3] = {r.xh, r.yh, r.zh}, sl[3] = {r.xl, r.yl, r.zl};
      float dh[3], dl[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const f2 v = fast_two_sum(th[k] - sh[k], tl[k] - sl[k]);
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
      double* row = M + (s * K0) * ld + t * K1;
      if constexpr (KER == KER_LFXU) {
        const f2 y = {y0, (0.5f * y0) * rho};
        const f2 u = df_mul(y, S);
        row[0] = df_to_double(u.h, u.l);
      } else {
        f2 y3 = df_mulf(q, y0);  // y0^3 (1 + 3 rho / 2)
        y3.l = fmaf(y3.h, 1.5f * rho, y3.l);
        if constexpr (KER == KER_LDXU) {
          float nh[3], nl[3];
          if constexpr (ND == 3) {
            nh[0] = r.nh0, nh[1] = r.nh1, nh[2] = r.nh2;
            nl[0] = r.nl0, nl[1] = r.nl1, nl[2] = r.nl2;
          }
          const f2 u = df_mul(df_mul(df_dot3(dh, dl, nh[0], nh[1], nh[2], nl[0], nl[1], nl[2]), y3), S);
          row[0] = df_to_double(u.h, u.l);
        } else {
          const f2 d[3] = {{dh[0], dl[0]}, {dh[1], dl[1]}, {dh[2], dl[2]}};
          f2 c, diag = {0.f, 0.f};
          if constexpr (KER == KER_SFXU) {  // u_ij = S (delta_ij y + d_i d_j y^3)
            const f2 y = {y0, (0.5f * y0) * rho};
            diag = df_mul(y, S);
            c = df_mul(y3, S);
          } else {  // u_ij = S d_i d_j (d . n) y^5
            float nh[3] = {0.f, 0.f, 0.f}, nl[3] = {0.f, 0.f, 0.f};
            if constexpr (ND == 3) {
              nh[0] = r.nh0, nh[1] = r.nh1, nh[2] = r.nh2;
              nl[0] = r.nl0, nl[1] = r.nl1, nl[2] = r.nl2;
            }
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
              const double w = df_to_double(v.h, v.l);
              row[i * ld + j] = w;
              if (j != i) row[j * ld + i] = w;
            }
        }
      }
    }
  }
}

}  // namespace sctlgpu
