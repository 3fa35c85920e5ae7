// The other micro-kernels of kernel_functions.hpp -- Laplace gradient and
// Hessian, BiotSavart, Helmholtz (complex values as real/imaginary pairs),
// Stokes traction, source/sink and pressure -- through one templated tiled
// direct sum and one kernel-matrix kernel, in FP64 or FP32.
//
// Each kernel is written once, as its KDIM0 x KDIM1 matrix u(r, n) (the
// reference's uKerMatrix); Eval applies it to the density (v_k1 += sum_k0
// u[k0][k1] f_k0, the reference's generic path for kernels without a fused
// apply and the same values as its fused applies) and KernelMatrix writes it.
// 1/r comes from the hardware estimate plus the reference's Newton schedule
// for `digits`; r^2 == 0 gives u == 0.  Sources are packed into records of
// 16-byte multiples (x y z, normal, density) and staged one tile at a time by
// the bulk-copy engine, double-buffered, as in direct.cuh; each CTA writes
// FP64 partials per source slice, reduced in a fixed order (deterministic).
#pragma once

#include "launch_direct.cuh"

namespace sctlgpu {

template <int K>
struct XK;
#define SCTLGPU_XK(K, nd, k0, k1, num, den)                                      \
  template <>                                                                    \
  struct XK<K> {                                                                 \
    static constexpr int ND = nd, K0 = k0, K1 = k1;                              \
    static constexpr double scale() {                                            \
      return (double)(num) / ((double)(den) * 3.14159265358979323846264338327950288); \
    }                                                                            \
  };
// id, NormalDim, SrcDim, TrgDim, uKerScaleFactor = num / (den * pi)
SCTLGPU_XK(4, 0, 1, 3, -1, 4)   // Laplace3D_FxdU        kernel_functions.hpp:88-90
SCTLGPU_XK(5, 0, 1, 9, 1, 4)    // Laplace3D_Fxd2U       :374-376
SCTLGPU_XK(6, 3, 1, 3, 1, 4)    // Laplace3D_DxdU        :400-402
SCTLGPU_XK(7, 0, 3, 3, 1, 4)    // BiotSavart3D_FxU      :424-426
SCTLGPU_XK(8, 0, 3, 9, -1, 4)   // BiotSavart3D_FxdU     :459-461
SCTLGPU_XK(9, 0, 2, 2, 1, 4)    // Helmholtz3D_FxU       :499-501
SCTLGPU_XK(10, 3, 2, 2, -1, 4)  // Helmholtz3D_DxU       :537-539
SCTLGPU_XK(11, 0, 2, 6, 1, 4)   // Helmholtz3D_FxdU      :581-583
SCTLGPU_XK(12, 0, 2, 6, 1, 4)   // HelmholtzDiff3D_FxdU  :635-637
SCTLGPU_XK(13, 0, 3, 9, -3, 4)  // Stokes3D_FxT          :228-230
SCTLGPU_XK(14, 0, 4, 3, 1, 8)   // Stokes3D_FSxU         :272-274
SCTLGPU_XK(15, 0, 3, 4, 1, 8)   // Stokes3D_FxUP         :333-335
#undef SCTLGPU_XK

__device__ __forceinline__ void sin_cos(double x, double* s, double* c) { sincos(x, s, c); }
__device__ __forceinline__ void sin_cos(float x, float* s, float* c) { sincosf(x, s, c); }

// u(r, n) of kernel K (the reference's uKerMatrix formulas).
template <int K, int NEWTON, class R>
__device__ __forceinline__ void xumat(R (&u)[XK<K>::K0][XK<K>::K1], const R (&r)[3], const R* n, R mu) {
  const R r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
  const bool live = r2 > R(0);
  const R x = live ? r2 : R(1);
  R rinv = newton_rsqrt<NEWTON>(rsqrt_seed(x), R(0.5) * x);
  rinv = live ? rinv : R(0);
  const R rinv2 = rinv * rinv, rinv3 = rinv2 * rinv;
  if constexpr (K == 4) {  // grad of 1/r (times -1 in the scale): r / r^3
#pragma unroll
    for (int i = 0; i < 3; ++i) u[0][i] = r[i] * rinv3;
  } else if constexpr (K == 5) {  // Hessian: 3 r r^T / r^5 - I / r^3
    const R t5 = R(3) * rinv3 * rinv2;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) u[0][i * 3 + j] = t5 * r[i] * r[j] - (i == j ? rinv3 : R(0));
  } else if constexpr (K == 6) {  // grad of the double layer: n / r^3 - 3 (r.n) r / r^5
    const R rdotn = r[0] * n[0] + r[1] * n[1] + r[2] * n[2];
    const R t5 = R(3) * rdotn * rinv3 * rinv2;
#pragma unroll
    for (int i = 0; i < 3; ++i) u[0][i] = n[i] * rinv3 - r[i] * t5;
  } else if constexpr (K == 7) {  // f x r / r^3
    u[0][0] = R(0);
    u[0][1] = -r[2] * rinv3;
    u[0][2] = r[1] * rinv3;
    u[1][0] = r[2] * rinv3;
    u[1][1] = R(0);
    u[1][2] = -r[0] * rinv3;
    u[2][0] = -r[1] * rinv3;
    u[2][1] = r[0] * rinv3;
    u[2][2] = R(0);
  } else if constexpr (K == 8) {  // gradient of BiotSavart: the 3 x 9 table of :466-478
    const R t5 = R(3) * rinv3 * rinv2;
    const R a = t5 * r[0], b = t5 * r[1], c = t5 * r[2];
    u[0][0] = R(0);
    u[0][1] = R(0);
    u[0][2] = R(0);
    u[1][0] = c * r[0];
    u[1][1] = c * r[1];
    u[1][2] = -rinv3 + c * r[2];
    u[2][0] = -b * r[0];
    u[2][1] = rinv3 - b * r[1];
    u[2][2] = -b * r[2];
    u[0][3] = -c * r[0];
    u[0][4] = -c * r[1];
    u[0][5] = rinv3 - c * r[2];
    u[1][3] = R(0);
    u[1][4] = R(0);
    u[1][5] = R(0);
    u[2][3] = -rinv3 + a * r[0];
    u[2][4] = a * r[1];
    u[2][5] = a * r[2];
    u[0][6] = b * r[0];
    u[0][7] = -rinv3 + b * r[1];
    u[0][8] = b * r[2];
    u[1][6] = rinv3 - a * r[0];
    u[1][7] = -a * r[1];
    u[1][8] = -a * r[2];
    u[2][6] = R(0);
    u[2][7] = R(0);
    u[2][8] = R(0);
  } else if constexpr (K >= 9 && K <= 12) {  // Helmholtz: e^{i mu r} / r and derivatives
    R s, c;
    R cm1;  // cos(mu r) - 1 (HelmholtzDiff only)
    if constexpr (K == 12) {  // half-angle form, accurate as mu r -> 0 (:647-651)
      R sh, ch;
      sin_cos(r2 * rinv * mu * R(0.5), &sh, &ch);
      s = R(2) * sh * ch;
      cm1 = -R(2) * sh * sh;
      c = R(1) + cm1;
    } else {
      sin_cos(r2 * rinv * mu, &s, &c);
      cm1 = c;
    }
    if constexpr (K == 9) {
      u[0][0] = c * rinv;
      u[0][1] = s * rinv;
      u[1][0] = -u[0][1];
      u[1][1] = u[0][0];
    } else if constexpr (K == 10) {
      const R ndotr = n[0] * r[0] + n[1] * r[1] + n[2] * r[2];
      u[0][0] = (-mu * s - c * rinv) * rinv2 * ndotr;
      u[0][1] = (mu * c - s * rinv) * rinv2 * ndotr;
      u[1][0] = -u[0][1];
      u[1][1] = u[0][0];
    } else {
      const R G0 = (-mu * s - cm1 * rinv) * rinv2;
      const R G1 = (mu * c - s * rinv) * rinv2;
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        u[0][i * 2 + 0] = G0 * r[i];
        u[0][i * 2 + 1] = G1 * r[i];
        u[1][i * 2 + 0] = -u[0][i * 2 + 1];
        u[1][i * 2 + 1] = u[0][i * 2 + 0];
      }
    }
  } else if constexpr (K == 13) {  // traction: r_i r_j r_k / r^5
    const R rinv5 = rinv2 * rinv2 * rinv;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int k = 0; k < 3; ++k) u[i][j * 3 + k] = r[i] * r[j] * r[k] * rinv5;
  } else if constexpr (K == 14 || K == 15) {  // Stokeslet plus source/sink row, or plus pressure column
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) u[i][j] = (i == j ? rinv : R(0)) + r[i] * r[j] * rinv3;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      if constexpr (K == 14)
        u[3][j] = r[j] * rinv3;
      else
        u[j][3] = r[j] * rinv3;
    }
  }
}

// Packed source record: x y z, normal (ND), density (K0), zero padding to 16 bytes.
template <int K, class R>
struct XRec {
  static constexpr int N = 3 + XK<K>::ND + XK<K>::K0;
  static constexpr int W = ((N * (int)sizeof(R) + 15) / 16) * 16 / (int)sizeof(R);
  R v[W];
};

template <int K, class R>
__global__ void xpack_kernel(int64_t ns, const R* __restrict__ xs, const R* __restrict__ nrm,
                             const R* __restrict__ f, XRec<K, R>* __restrict__ recs) {
  constexpr int ND = XK<K>::ND, K0 = XK<K>::K0, W = XRec<K, R>::W;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += (int64_t)gridDim.x * blockDim.x) {
    XRec<K, R> r;
#pragma unroll
    for (int i = 0; i < W; ++i) r.v[i] = R(0);
#pragma unroll
    for (int i = 0; i < 3; ++i) r.v[i] = xs[s * 3 + i];
#pragma unroll
    for (int i = 0; i < ND; ++i) r.v[3 + i] = nrm[s * 3 + i];
#pragma unroll
    for (int i = 0; i < K0; ++i) r.v[3 + ND + i] = f[s * K0 + i];
    recs[s] = r;
  }
}

constexpr int XT_THREADS = 128, XT_T = 2, XT_S = 256;

struct XParams {
  int64_t nt, ns, chunk;
  const void* r_trg;
  const void* recs;
  double* partial;
  unsigned* status;
  double mu;
};

template <int K, class R, int NEWTON>
__global__ void __launch_bounds__(XT_THREADS) xdirect_kernel(XParams p) {
  using Rec = XRec<K, R>;
  constexpr int ND = XK<K>::ND, K0 = XK<K>::K0, K1 = XK<K>::K1;
  extern __shared__ __align__(128) unsigned char xsm[];
  Rec* tiles = reinterpret_cast<Rec*>(xsm);
  uint64_t* bars = reinterpret_cast<uint64_t*>(xsm + 2 * XT_S * sizeof(Rec));

  const int64_t t0 = (int64_t)blockIdx.x * XT_THREADS * XT_T;
  const int64_t s_begin = (int64_t)blockIdx.y * p.chunk;
  const int64_t s_end = imin64(p.ns, s_begin + p.chunk);
  const int64_t n_src = s_end - s_begin;
  const int ntiles = (int)((n_src + XT_S - 1) / XT_S);
  const Rec* src = reinterpret_cast<const Rec*>(p.recs) + s_begin;

  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int b = 0; b < 2 && b < ntiles; ++b) {
      const uint32_t cnt = (uint32_t)imin64((int64_t)XT_S, n_src - (int64_t)b * XT_S);
      mbar_arrive_expect_tx(&bars[b], cnt * (uint32_t)sizeof(Rec));
      bulk_g2s(tiles + b * XT_S, src + (int64_t)b * XT_S, cnt * (uint32_t)sizeof(Rec), &bars[b]);
    }
  }

  const R* rt = reinterpret_cast<const R*>(p.r_trg);
  const R mu = (R)p.mu;
  R xt[XT_T][3], acc[XT_T][K1];
  double tot[XT_T][K1];
#pragma unroll
  for (int j = 0; j < XT_T; ++j) {
    int64_t i = t0 + threadIdx.x + (int64_t)j * XT_THREADS;
    i = i < p.nt ? i : p.nt - 1;
#pragma unroll
    for (int k = 0; k < 3; ++k) xt[j][k] = rt[i * 3 + k];
#pragma unroll
    for (int k = 0; k < K1; ++k) tot[j][k] = 0.0;
  }

  bool timed_out = false;
  for (int kt = 0; kt < ntiles; ++kt) {
    const int buf = kt & 1;
    if (!mbar_wait_bounded(&bars[buf], (uint32_t)((kt >> 1) & 1), p.status)) timed_out = true;
    const Rec* tile = tiles + buf * XT_S;
    const int cnt = (int)imin64((int64_t)XT_S, n_src - (int64_t)kt * XT_S);
#pragma unroll
    for (int j = 0; j < XT_T; ++j)
#pragma unroll
      for (int k = 0; k < K1; ++k) acc[j][k] = R(0);
    for (int s = 0; s < cnt; ++s) {
      const Rec rec = tile[s];
#pragma unroll
      for (int j = 0; j < XT_T; ++j) {
        const R r[3] = {xt[j][0] - rec.v[0], xt[j][1] - rec.v[1], xt[j][2] - rec.v[2]};
        R u[K0][K1];
        xumat<K, NEWTON, R>(u, r, rec.v + 3, mu);
#pragma unroll
        for (int k1 = 0; k1 < K1; ++k1) {
          R v = acc[j][k1];
#pragma unroll
          for (int k0 = 0; k0 < K0; ++k0) v = fma(u[k0][k1], rec.v[3 + ND + k0], v);
          acc[j][k1] = v;
        }
      }
    }
#pragma unroll
    for (int j = 0; j < XT_T; ++j)
#pragma unroll
      for (int k = 0; k < K1; ++k) tot[j][k] += (double)acc[j][k];
    __syncthreads();  // every thread is done with this buffer
    if (threadIdx.x == 0 && kt + 2 < ntiles) {
      fence_proxy_async_smem();
      const uint32_t c2 = (uint32_t)imin64((int64_t)XT_S, n_src - (int64_t)(kt + 2) * XT_S);
      mbar_arrive_expect_tx(&bars[buf], c2 * (uint32_t)sizeof(Rec));
      bulk_g2s(tiles + buf * XT_S, src + (int64_t)(kt + 2) * XT_S, c2 * (uint32_t)sizeof(Rec), &bars[buf]);
    }
  }
  if (timed_out && threadIdx.x == 0) {
    for (int b = 0; b < 2; ++b) {
      const int k_last = (ntiles - 1) - (((ntiles - 1) - b) & 1);
      if (k_last >= 0) mbar_wait_bounded(&bars[b], (uint32_t)((k_last >> 1) & 1), nullptr);
    }
  }
#pragma unroll
  for (int j = 0; j < XT_T; ++j) {
    const int64_t i = t0 + threadIdx.x + (int64_t)j * XT_THREADS;
    if (i < p.nt) {
#pragma unroll
      for (int k = 0; k < K1; ++k) p.partial[((int64_t)blockIdx.y * p.nt + i) * K1 + k] = tot[j][k];
    }
  }
}

// M[(s*K0 + k0) * (nt*K1) + t*K1 + k1] = scale * u[k0][k1](x_t - y_s, n_s): one thread per target,
// grid.y striding over sources.
template <int K, class R, int NEWTON>
__global__ void __launch_bounds__(128) xkmat_kernel(int64_t nt, const R* __restrict__ r_trg, int64_t ns,
                                                    const R* __restrict__ r_src, const R* __restrict__ n_src,
                                                    R* __restrict__ M, double scale, double mu_d) {
  constexpr int ND = XK<K>::ND, K0 = XK<K>::K0, K1 = XK<K>::K1;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  const R mu = (R)mu_d;
  const int64_t ld = nt * K1;
  const R x0 = r_trg[t * 3], x1 = r_trg[t * 3 + 1], x2 = r_trg[t * 3 + 2];
  for (int64_t s = blockIdx.y; s < ns; s += gridDim.y) {
    const R r[3] = {x0 - r_src[s * 3], x1 - r_src[s * 3 + 1], x2 - r_src[s * 3 + 2]};
    R nn[3] = {R(0), R(0), R(0)};
    if (ND)
#pragma unroll
      for (int k = 0; k < 3; ++k) nn[k] = n_src[s * 3 + k];
    R u[K0][K1];
    xumat<K, NEWTON, R>(u, r, nn, mu);
#pragma unroll
    for (int k0 = 0; k0 < K0; ++k0)
#pragma unroll
      for (int k1 = 0; k1 < K1; ++k1) M[(s * K0 + k0) * ld + t * K1 + k1] = (R)((double)u[k0][k1] * scale);
  }
}

template <int K, class R, int NEWTON>
cudaError_t run_xdirect(const EvalCall& c) {
  using Rec = XRec<K, R>;
  constexpr int K1 = XK<K>::K1;
  cudaStream_t st = c.stream;
  const size_t smem = 2 * XT_S * sizeof(Rec) + 2 * sizeof(uint64_t);
  static int occ = [&] {
    int o = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, xdirect_kernel<K, R, NEWTON>, XT_THREADS, smem);
    return o > 0 ? o : 1;
  }();
  const int64_t per_cta = (int64_t)XT_THREADS * XT_T;
  const int64_t tblocks = (c.nt + per_cta - 1) / per_cta;
  const int nsplit0 = choose_nsplit(tblocks, c.ns, XT_S, c.sms * occ);
  int64_t chunk = (c.ns + nsplit0 - 1) / nsplit0;
  chunk = ((chunk + XT_S - 1) / XT_S) * XT_S;
  const int nsplit = (int)((c.ns + chunk - 1) / chunk);

  const size_t rec_bytes = (size_t)c.ns * sizeof(Rec);
  const size_t part_off = (rec_bytes + 255) / 256 * 256;
  const size_t part_bytes = (size_t)nsplit * (size_t)c.nt * K1 * sizeof(double);
  char* scratch = nullptr;
  SCTLGPU_TRY(cudaMallocAsync((void**)&scratch, part_off + part_bytes, st));
  Rec* recs = reinterpret_cast<Rec*>(scratch);
  double* partial = reinterpret_cast<double*>(scratch + part_off);
  cudaError_t err = cudaSuccess;
  do {
    xpack_kernel<K, R><<<grid_for(c.ns, 256, c.sms), 256, 0, st>>>(c.ns, (const R*)c.r_src, (const R*)c.n_src,
                                                                   (const R*)c.v_src, recs);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    XParams p;
    p.nt = c.nt;
    p.ns = c.ns;
    p.chunk = chunk;
    p.r_trg = c.r_trg;
    p.recs = recs;
    p.partial = partial;
    p.status = c.status;
    p.mu = c.ctx;
    dim3 grid((unsigned)tblocks, (unsigned)nsplit);
    if (c.timing && c.timing->enabled) cudaEventRecord(c.timing->start, st);
    xdirect_kernel<K, R, NEWTON><<<grid, XT_THREADS, smem, st>>>(p);
    if (c.timing && c.timing->enabled) {
      cudaEventRecord(c.timing->stop, st);
      c.timing->recorded = true;
    }
    g_launches.fetch_add(1, std::memory_order_relaxed);
    const int64_t nout = c.nt * K1;
    reduce_partials_kernel<R><<<grid_for(nout, 256, c.sms), 256, 0, st>>>(nout, nsplit, partial, XK<K>::scale(),
                                                                          c.accumulate ? 1 : 0, (R*)c.v_trg);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    err = cudaGetLastError();
  } while (0);
  cudaError_t e2 = cudaFreeAsync(scratch, st);
  return err != cudaSuccess ? err : e2;
}

template <int K, class R, int NEWTON>
cudaError_t run_xkmat(const KmatCall& c) {
  const unsigned gx = (unsigned)((c.nt + 127) / 128);
  const int64_t want = (int64_t)c.sms * 16 / std::max<int64_t>(1, gx) + 1;
  const unsigned gy = (unsigned)std::max<int64_t>(1, std::min<int64_t>({c.ns, want, 65535}));
  xkmat_kernel<K, R, NEWTON><<<dim3(gx, gy), 128, 0, c.stream>>>(c.nt, (const R*)c.r_trg, c.ns, (const R*)c.r_src,
                                                                 (const R*)c.n_src, (R*)c.M, XK<K>::scale(), c.ctx);
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return cudaGetLastError();
}

// Dispatch over kernel ids 4..15 and Newton counts 0..NMAX for one real type.
template <class R, int NMAX>
struct XDispatch {
  template <int K, int N>
  static cudaError_t eval_n(const EvalCall& c, int n) {
    if constexpr (N < NMAX) {
      if (n <= N) return run_xdirect<K, R, N>(c);
      return eval_n<K, N + 1>(c, n);
    } else {
      return run_xdirect<K, R, N>(c);
    }
  }
  template <int K, int N>
  static cudaError_t kmat_n(const KmatCall& c, int n) {
    if constexpr (N < NMAX) {
      if (n <= N) return run_xkmat<K, R, N>(c);
      return kmat_n<K, N + 1>(c, n);
    } else {
      return run_xkmat<K, R, N>(c);
    }
  }
  template <int K>
  static cudaError_t eval_k(const EvalCall& c, int n) {
    if constexpr (K > 15) {
      return cudaErrorInvalidValue;
    } else {
      if (c.kernel == K) return eval_n<K, 0>(c, n);
      return eval_k<K + 1>(c, n);
    }
  }
  template <int K>
  static cudaError_t kmat_k(const KmatCall& c, int n) {
    if constexpr (K > 15) {
      return cudaErrorInvalidValue;
    } else {
      if (c.kernel == K) return kmat_n<K, 0>(c, n);
      return kmat_k<K + 1>(c, n);
    }
  }
};

}  // namespace sctlgpu
