// Mixed-precision direct sums (SCTLGPU_MIXED): FP32 arithmetic on split
// coordinates for digits <= 7, double-float arithmetic on the packed FP32 pipe
// (direct_pk.cuh) for digits 8..11.
#include "launch_direct.cuh"

namespace sctlgpu {

__global__ void bbox_init_kernel(BBox* bb) {
  if (threadIdx.x < 3) {
    bb->lo[threadIdx.x] = ~0ull;
    bb->hi[threadIdx.x] = 0ull;
  }
}

cudaError_t compute_bbox(cudaStream_t s, int64_t nt, const double* r_trg, int64_t ns, const double* r_src, BBox* bb) {
  int dev = 0, sms = 0;
  SCTLGPU_TRY(cudaGetDevice(&dev));
  SCTLGPU_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  bbox_init_kernel<<<1, 32, 0, s>>>(bb);
  g_launches.fetch_add(1, std::memory_order_relaxed);
  if (nt > 0) {
    bbox_kernel<double><<<grid_for(nt, 256, sms), 256, 0, s>>>(nt, r_trg, bb);
    g_launches.fetch_add(1, std::memory_order_relaxed);
  }
  if (ns > 0) {
    bbox_kernel<double><<<grid_for(ns, 256, sms), 256, 0, s>>>(ns, r_src, bb);
    g_launches.fetch_add(1, std::memory_order_relaxed);
  }
  return cudaGetLastError();
}

template <int KER>
static cudaError_t eval_lo_k(const EvalCall& c, int newton) {
  return newton <= 0 ? run_direct<KER, MODE_MXLO, 0>(c) : run_direct<KER, MODE_MXLO, 1>(c);
}

cudaError_t eval_mixed_lo(const EvalCall& c, int newton) {
  switch (c.kernel) {
    case KER_LFXU: return eval_lo_k<KER_LFXU>(c, newton);
    case KER_LDXU: return eval_lo_k<KER_LDXU>(c, newton);
    case KER_SFXU: return eval_lo_k<KER_SFXU>(c, newton);
    default: return eval_lo_k<KER_SDXU>(c, newton);
  }
}

cudaError_t eval_mixed_df(const EvalCall& c) {
  switch (c.kernel) {
    case KER_LFXU: return run_direct_pk<KER_LFXU>(c);
    case KER_LDXU: return run_direct_pk<KER_LDXU>(c);
    case KER_SFXU: return run_direct_pk<KER_SFXU>(c);
    default: return run_direct_pk<KER_SDXU>(c);
  }
}

}  // namespace sctlgpu
