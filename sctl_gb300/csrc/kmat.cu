// Kernel-matrix launches (GenericKernel::KernelMatrix, generic-kernel.txx:213-329).
#include "kmat.cuh"
#include "launch_direct.cuh"

namespace sctlgpu {

template <int KER, int MODE, int NEWTON, class Real>
static cudaError_t run_kmat(const KmatCall& c, BBox* bb) {
  const int64_t tb = (c.nt + KM_THREADS - 1) / KM_THREADS;
  const int64_t sg = (c.ns + KM_SROWS - 1) / KM_SROWS;
  dim3 grid((unsigned)tb, (unsigned)std::min<int64_t>(sg, 65535));
  if (c.timing && c.timing->enabled) cudaEventRecord(c.timing->start, c.stream);
  kernel_matrix_kernel<KER, MODE, NEWTON, Real><<<grid, KM_THREADS, 0, c.stream>>>(
      c.nt, (const Real*)c.r_trg, c.ns, (const Real*)c.r_src, (const Real*)c.n_src, (Real*)c.M, scale_of<KER>(), bb);
  if (c.timing && c.timing->enabled) {
    cudaEventRecord(c.timing->stop, c.stream);
    c.timing->recorded = true;
  }
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return cudaGetLastError();
}

template <int MODE, class Real, int NEWTON>
static cudaError_t kmat_dispatch(const KmatCall& c, BBox* bb) {
  switch (c.kernel) {
    case KER_LFXU: return run_kmat<KER_LFXU, MODE, NEWTON, Real>(c, bb);
    case KER_LDXU: return run_kmat<KER_LDXU, MODE, NEWTON, Real>(c, bb);
    case KER_SFXU: return run_kmat<KER_SFXU, MODE, NEWTON, Real>(c, bb);
    default: return run_kmat<KER_SDXU, MODE, NEWTON, Real>(c, bb);
  }
}

cudaError_t kmat_f64(const KmatCall& c, int newton) {
  switch (newton) {
    case 0: return kmat_dispatch<MODE_F64, double, 0>(c, nullptr);
    case 1: return kmat_dispatch<MODE_F64, double, 1>(c, nullptr);
    case 2: return kmat_dispatch<MODE_F64, double, 2>(c, nullptr);
    default: return kmat_dispatch<MODE_F64, double, 3>(c, nullptr);
  }
}

cudaError_t kmat_f32(const KmatCall& c, int newton) {
  switch (newton) {
    case 0: return kmat_dispatch<MODE_F32, float, 0>(c, nullptr);
    case 1: return kmat_dispatch<MODE_F32, float, 1>(c, nullptr);
    default: return kmat_dispatch<MODE_F32, float, 2>(c, nullptr);
  }
}

// Mixed precision: one launch (points split in the kernel), no scratch.
template <int KER>
static cudaError_t run_kmat_df(const KmatCall& c) {
  const double scale = scale_of<KER>();
  const float sh = (float)scale, sl = (float)(scale - (double)sh);
  const int64_t tb = (c.nt + KM_THREADS - 1) / KM_THREADS;
  const int64_t sb = (c.ns + KMD_GROUPS * KMD_SROWS - 1) / (KMD_GROUPS * KMD_SROWS);
  dim3 grid((unsigned)tb, (unsigned)std::min<int64_t>(sb, 65535));
  // 16-byte row segments: M 16-byte aligned and an even row length (every row then starts aligned;
  // each warp's segment starts 768 bytes after the previous one's)
  const int vec = (((uintptr_t)c.M & 15) == 0 && ((c.nt * KDims<KER>::K1) & 1) == 0) ? 1 : 0;
  if (c.timing && c.timing->enabled) cudaEventRecord(c.timing->start, c.stream);
  kernel_matrix_df_kernel<KER><<<grid, KM_THREADS, 0, c.stream>>>(
      c.nt, (const double*)c.r_trg, c.ns, (const double*)c.r_src, (const double*)c.n_src, (double*)c.M, sh, sl, vec);
  if (c.timing && c.timing->enabled) {
    cudaEventRecord(c.timing->stop, c.stream);
    c.timing->recorded = true;
  }
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return cudaGetLastError();
}

cudaError_t kmat_mixed_df(const KmatCall& c) {
  if (c.nt <= 0 || c.ns <= 0) return cudaSuccess;
  switch (c.kernel) {
    case KER_LFXU: return run_kmat_df<KER_LFXU>(c);
    case KER_LDXU: return run_kmat_df<KER_LDXU>(c);
    case KER_SFXU: return run_kmat_df<KER_SFXU>(c);
    default: return run_kmat_df<KER_SDXU>(c);
  }
}

}  // namespace sctlgpu
