// Application of precomputed near-interaction matrices: the GPU form of
// BoundaryIntegralOp::ComputeNearInterac (boundary_integral.txx:1311-1381).
//
// The reference stores one matrix block per (element, near target) pair --
// KDIM1 rows x (element nodes * KDIM0) columns, target-major inside an
// element (K_near, built by SetupNear/KNearSubtract) -- applies every block to
// the element's density (per-block GEMV), scatters the per-pair results to
// target order (ScatterForward) and sums each target's pairs into U.
//
// Here the three steps are one pass: one warp per target walks the target's
// pairs in the caller's target-major order (the reference's near_trg_dsp /
// scatter order), the lanes stream the pair's matrix rows (coalesced, 8-byte
// loads) against the element's density (L2-resident), and the warp reduces in
// a fixed order before one add into U -- deterministic, no atomics.  The
// kernel reads each matrix entry once: it is HBM-bound (8 bytes per
// multiply-add), so the roofline is the copy bandwidth.
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/sctlgpu.h"
#include "launch.h"

namespace sctlgpu {
namespace {

constexpr int NA_WARPS = 8;

struct NearApplyParams {
  int k0, k1;
  int64_t n_trg, n_near, n_pairs, n_elem, n_k, n_f;
  const int64_t* trg_dsp;       // [n_trg + 1]
  const int64_t* trg_pair;      // [n_near] or null (identity)
  const int64_t* pair_elem;     // [n_pairs]
  const int64_t* pair_kdsp;     // [n_pairs] first entry of the pair's block in K
  const int64_t* elem_nds_dsp;  // [n_elem]
  const int64_t* elem_nds_cnt;  // [n_elem]
  const double* K;
  const double* F;
  double* U;
  unsigned* status;
};

// Entries of a pair's block handled per lane per step: 4 loads of each row in
// flight per lane before the multiply-adds that use them.
constexpr int NA_U = 4;

template <int K1>
__device__ __forceinline__ void apply_pair(const double* __restrict__ Kp, const double* __restrict__ Fp, int64_t n,
                                           int lane, double (&acc)[K1]) {
  for (int64_t i0 = 0; i0 < n; i0 += 32 * NA_U) {
    double f[NA_U], k[K1][NA_U];
#pragma unroll
    for (int u = 0; u < NA_U; ++u) {
      const int64_t i = i0 + u * 32 + lane;
      const bool in = i < n;
      f[u] = in ? __ldg(Fp + i) : 0.0;
#pragma unroll
      for (int c = 0; c < K1; ++c) k[c][u] = in ? __ldcs(Kp + c * n + i) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < NA_U; ++u)
#pragma unroll
      for (int c = 0; c < K1; ++c) acc[c] = fma(k[c][u], f[u], acc[c]);
  }
}

template <int K1>
__global__ void __launch_bounds__(32 * NA_WARPS) near_apply_kernel(NearApplyParams p) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * NA_WARPS;
  for (int64_t t = (int64_t)blockIdx.x * NA_WARPS + (threadIdx.x >> 5); t < p.n_trg; t += nwarps) {
    double acc[K1];
#pragma unroll
    for (int c = 0; c < K1; ++c) acc[c] = 0.0;
    int64_t j0 = p.trg_dsp[t], j1 = p.trg_dsp[t + 1];
    bool bad = false;
    if (j0 < 0 || j1 > p.n_near || j1 < j0) {
      bad = true;
      j1 = j0;
    }
    // The target's pairs in chunks of 32: every lane resolves one pair's indices (one round of
    // dependent loads per chunk), then the warp streams the chunk's blocks in order.
    for (int64_t jb = j0; jb < j1; jb += 32) {
      const int64_t j = jb + lane;
      int64_t n = -1, fofs = 0, kofs = 0;
      if (j < j1) {
        const int64_t pr = p.trg_pair ? p.trg_pair[j] : j;
        if (pr >= 0 && pr < p.n_pairs) {
          const int64_t e = p.pair_elem[pr];
          if (e >= 0 && e < p.n_elem) {
            n = p.elem_nds_cnt[e] * p.k0;
            fofs = p.elem_nds_dsp[e] * p.k0;
            kofs = p.pair_kdsp[pr];
            if (n < 0 || fofs < 0 || fofs + n > p.n_f || kofs < 0 || kofs + n * K1 > p.n_k) n = -1;
          }
        }
        if (n < 0) bad = true;
      }
      const int m = (int)(j1 - jb < 32 ? j1 - jb : 32);
      for (int q = 0; q < m; ++q) {
        const int64_t nq = __shfl_sync(0xffffffffu, n, q);
        const int64_t fq = __shfl_sync(0xffffffffu, fofs, q);
        const int64_t kq = __shfl_sync(0xffffffffu, kofs, q);
        if (nq > 0) apply_pair<K1>(p.K + kq, p.F + fq, nq, lane, acc);
      }
    }
#pragma unroll
    for (int c = 0; c < K1; ++c)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
    bad = __any_sync(0xffffffffu, bad);
    if (lane == 0) {
      if (bad && p.status) atomicOr(p.status, 4u);  // an index out of range: that pair skipped
      if (j1 > j0)
#pragma unroll
        for (int c = 0; c < K1; ++c) p.U[t * K1 + c] += acc[c];
    }
  }
}

template <int K1>
void launch_k1(const NearApplyParams& p, unsigned grid, cudaStream_t st) {
  near_apply_kernel<K1><<<grid, 32 * NA_WARPS, 0, st>>>(p);
}

}  // namespace
}  // namespace sctlgpu

using namespace sctlgpu;

extern "C" int sctlgpu_near_matrix_apply(int k0, int k1, int64_t n_trg, const int64_t* trg_dsp, int64_t n_near,
                                         const int64_t* trg_pair, int64_t n_pairs, const int64_t* pair_elem,
                                         const int64_t* pair_kdsp, int64_t n_elem, const int64_t* elem_nds_dsp,
                                         const int64_t* elem_nds_cnt, int64_t n_k, const double* K, int64_t n_f,
                                         const double* F, double* U, void* stream) {
  if (k0 < 1 || !(k1 == 1 || k1 == 2 || k1 == 3 || k1 == 4 || k1 == 9) || n_trg < 0 || n_near < 0 ||
      n_pairs < 0 || n_elem < 0 || n_k < 0 || n_f < 0 || (!trg_pair && n_near > n_pairs))
    return SCTLGPU_ERR_INVALID_SIZE;
  if (n_trg == 0) return SCTLGPU_OK;
  if (!trg_dsp || !U || (n_pairs && (!pair_elem || !pair_kdsp || !K)) ||
      (n_elem && (!elem_nds_dsp || !elem_nds_cnt || !F)))
    return SCTLGPU_ERR_NULL_POINTER;
  int dev;
  unsigned* status;
  int sms;
  int rc = runtime_device(&dev, &status, &sms);
  if (rc) return rc;
  NearApplyParams p{};
  p.k0 = k0;
  p.k1 = k1;
  p.n_trg = n_trg;
  p.n_near = n_near;
  p.n_pairs = n_pairs;
  p.n_elem = n_elem;
  p.n_k = n_k;
  p.n_f = n_f;
  p.trg_dsp = trg_dsp;
  p.trg_pair = trg_pair;
  p.pair_elem = pair_elem;
  p.pair_kdsp = pair_kdsp;
  p.elem_nds_dsp = elem_nds_dsp;
  p.elem_nds_cnt = elem_nds_cnt;
  p.K = K;
  p.F = F;
  p.U = U;
  p.status = status;
  const int64_t ctas = (n_trg + NA_WARPS - 1) / NA_WARPS;
  const int64_t cap = (int64_t)sms * 8;  // 8 CTAs of 8 warps per SM: full occupancy
  const unsigned grid = (unsigned)(ctas < cap ? ctas : cap);
  cudaStream_t st = (cudaStream_t)stream;
  switch (k1) {
    case 1: launch_k1<1>(p, grid, st); break;
    case 2: launch_k1<2>(p, grid, st); break;
    case 3: launch_k1<3>(p, grid, st); break;
    case 4: launch_k1<4>(p, grid, st); break;
    case 9: launch_k1<9>(p, grid, st); break;
    default: return SCTLGPU_ERR_INVALID_SIZE;
  }
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return runtime_record(cudaGetLastError());
}
