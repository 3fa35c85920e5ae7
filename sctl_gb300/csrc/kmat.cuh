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

}  // namespace sctlgpu
