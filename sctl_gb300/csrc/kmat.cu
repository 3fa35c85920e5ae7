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


}  // namespace sctlgpu
