// Builds the NearOps table entry of one (kernel, arithmetic, Newton) variant.
#pragma once

#include "launch_direct.cuh"
#include "near.cuh"
#include "near_pk.cuh"

namespace sctlgpu {

template <int KER, int MODE, int NEWTON>
NearOps make_near_ops() {
  using RecT = Rec<KER, MODE>;
  using Cfg = NearCfg<KER, MODE>;
  using Real = typename std::conditional<MODE == MODE_F32, float, double>::type;
  NearOps o;
  o.rec_bytes = sizeof(RecT);
  o.T = Cfg::T;
  o.smem = 2 * Cfg::S * sizeof(RecT) + (size_t)NEAR_THREADS * Cfg::T * KDims<KER>::K1 * sizeof(double) +
           2 * sizeof(uint64_t);
  static int occ = [&] {
    int v = 0;
    if (o.smem > 48 * 1024)
      cudaFuncSetAttribute(near_batch_kernel<KER, MODE, NEWTON>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)o.smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, near_batch_kernel<KER, MODE, NEWTON>, NEAR_THREADS, o.smem);
    return v > 0 ? v : 1;
  }();
  o.occ = occ;
  o.pack = [](cudaStream_t st, int64_t ns, const void* xs, const void* nrm, const void* f, const void* w, void* recs,
              const BBox* bb, int sms) -> cudaError_t {
    if (ns <= 0) return cudaSuccess;
    pack_sources_kernel<KER, MODE, Real><<<grid_for(ns, 256, sms), 256, 0, st>>>(
        ns, (const Real*)xs, (const Real*)nrm, (const Real*)f, (RecT*)recs, bb, (const Real*)w);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
  };
  o.launch = [](cudaStream_t st, unsigned ctas, const NearParams& p) -> cudaError_t {
    const size_t smem = 2 * Cfg::S * sizeof(RecT) + (size_t)NEAR_THREADS * Cfg::T * KDims<KER>::K1 * sizeof(double) +
                        2 * sizeof(uint64_t);
    near_batch_kernel<KER, MODE, NEWTON><<<ctas, NEAR_THREADS, smem, st>>>(p);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
  };
  return o;
}

// The packed double-float variant (mixed, 8..11 digits).
template <int KER>
NearOps make_near_ops_pk() {
  using RecT = RecPk<KER>;
  using Cfg = NearCfgPk<KER>;
  NearOps o;
  o.rec_bytes = sizeof(RecT);
  o.T = Cfg::T;
  o.paired = true;
  o.smem = 2 * Cfg::S * sizeof(RecT) + (size_t)NEAR_THREADS * Cfg::T * KDims<KER>::K1 * sizeof(double) +
           2 * sizeof(uint64_t);
  static int occ = [&] {
    int v = 0;
    if (o.smem > 48 * 1024)
      cudaFuncSetAttribute(near_batch_pk_kernel<KER>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)o.smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, near_batch_pk_kernel<KER>, NEAR_THREADS, o.smem);
    return v > 0 ? v : 1;
  }();
  o.occ = occ;
  o.pack = [](cudaStream_t st, int64_t ns, const void* xs, const void* nrm, const void* f, const void* w, void* recs,
              const BBox* bb, int sms) -> cudaError_t {
    if (ns <= 0) return cudaSuccess;
    const int64_t np = (ns + 1) / 2;
    pack_pairs_kernel<KER><<<grid_for(np, 256, sms), 256, 0, st>>>(ns, (const double*)xs, (const double*)nrm,
                                                                  (const double*)f, (RecT*)recs, bb, (const double*)w);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
  };
  o.pack_blocks = [](cudaStream_t st, int64_t nblk, const NearBlock* pblk, const NearBlock* sblk, int64_t n_pairs,
                     const void* xs, const void* nrm, const void* f, const void* w, void* recs, const BBox* bb,
                     int sms) -> cudaError_t {
    if (n_pairs <= 0 || nblk <= 0) return cudaSuccess;
    pack_block_pairs_kernel<KER><<<grid_for(n_pairs, 256, sms), 256, 0, st>>>(
        nblk, pblk, sblk, n_pairs, (const double*)xs, (const double*)nrm, (const double*)f, (const double*)w,
        (RecT*)recs, bb);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
  };
  o.launch = [](cudaStream_t st, unsigned ctas, const NearParams& p) -> cudaError_t {
    const size_t smem = 2 * Cfg::S * sizeof(RecT) + (size_t)NEAR_THREADS * Cfg::T * KDims<KER>::K1 * sizeof(double) +
                        2 * sizeof(uint64_t);
    near_batch_pk_kernel<KER><<<ctas, NEAR_THREADS, smem, st>>>(p);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
  };
  return o;
}

inline NearOps near_ops_pk(int kernel) {
  switch (kernel) {
    case KER_LFXU: return make_near_ops_pk<KER_LFXU>();
    case KER_LDXU: return make_near_ops_pk<KER_LDXU>();
    case KER_SFXU: return make_near_ops_pk<KER_SFXU>();
    case KER_SDXU_SYM: return make_near_ops_pk<KER_SDXU_SYM>();
    default: return make_near_ops_pk<KER_SDXU>();
  }
}

template <int MODE, int NEWTON>
NearOps near_ops_for(int kernel) {
  switch (kernel) {
    case KER_LFXU: return make_near_ops<KER_LFXU, MODE, NEWTON>();
    case KER_LDXU: return make_near_ops<KER_LDXU, MODE, NEWTON>();
    case KER_SFXU: return make_near_ops<KER_SFXU, MODE, NEWTON>();
    case KER_SDXU_SYM:  // FP64 and mixed plans only (plans with FP32 results refuse it)
      if constexpr (MODE != MODE_F32) return make_near_ops<KER_SDXU_SYM, MODE, NEWTON>();
      return make_near_ops<KER_SDXU, MODE, NEWTON>();
    default: return make_near_ops<KER_SDXU, MODE, NEWTON>();
  }
}

}  // namespace sctlgpu
