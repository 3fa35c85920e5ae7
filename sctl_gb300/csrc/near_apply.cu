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
// kernel reads each matrix entry once, 8 bytes per multiply-add, so its
// roofline is the copy bandwidth.
//
// GB300's FP64 pipe cannot issue one FP64 multiply-add per 8 bytes at HBM
// speed, so a second form takes the blocks stored as float pairs (hi, lo of
// each FP64 weight: the same 8 bytes, converted once by
// sctlgpu_to_float_pairs) and accumulates in double-float on the FP32 pipe.
#include <cstdint>
#include <cuda_runtime.h>

#include <type_traits>

#include "../../include/sctlgpu.h"
#include "common.cuh"
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
  const int64_t* resolved;      // [2 * n_near] or null: per target-major entry its K offset and (F offset, length)
  const double* K;    // FP64 blocks, or
  const float2* K2;   // the same as float pairs
  const double* F;
  const float2* F2;   // F as float pairs (with K2)
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

// acc += k * f in double-float (float pairs); accumulator left unnormalised.
__device__ __forceinline__ void df_fma_acc(f2& acc, float2 k, float2 f) {
  const float p = __fmul_rn(k.x, f.x);
  float e = fmaf(k.x, f.x, -p);
  e = fmaf(k.x, f.y, e);
  e = fmaf(k.y, f.x, e);
  const f2 s = two_sum(acc.h, p);
  acc.h = s.h;
  acc.l += s.l + e;
}

template <int K1>
__device__ __forceinline__ void apply_pair(const float2* __restrict__ Kp, const float2* __restrict__ Fp, int64_t n,
                                           int lane, f2 (&acc)[K1]) {
  for (int64_t i0 = 0; i0 < n; i0 += 32 * NA_U) {
    float2 f[NA_U], k[K1][NA_U];
#pragma unroll
    for (int u = 0; u < NA_U; ++u) {
      const int64_t i = i0 + u * 32 + lane;
      const bool in = i < n;
      f[u] = in ? __ldg(Fp + i) : make_float2(0.f, 0.f);
#pragma unroll
      for (int c = 0; c < K1; ++c) k[c][u] = in ? __ldcs(Kp + c * n + i) : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int u = 0; u < NA_U; ++u)
#pragma unroll
      for (int c = 0; c < K1; ++c) df_fma_acc(acc[c], k[c][u], f[u]);
  }
}

// Two blocks of at most 32 * NA_U entries each: every load of both issued before the
// multiply-adds.
template <int K1>
__device__ __forceinline__ void apply_two_pairs(const float2* __restrict__ Ka, const float2* __restrict__ Fa,
                                                int64_t na, const float2* __restrict__ Kb,
                                                const float2* __restrict__ Fb, int64_t nb, int lane,
                                                f2 (&acc)[K1]) {
  float2 fa[NA_U], fb[NA_U], ka[K1][NA_U], kb[K1][NA_U];
#pragma unroll
  for (int u = 0; u < NA_U; ++u) {
    const int64_t i = u * 32 + lane;
    const bool ia = i < na, ib = i < nb;
    fa[u] = ia ? __ldg(Fa + i) : make_float2(0.f, 0.f);
    fb[u] = ib ? __ldg(Fb + i) : make_float2(0.f, 0.f);
#pragma unroll
    for (int c = 0; c < K1; ++c) {
      ka[c][u] = ia ? __ldcs(Ka + c * na + i) : make_float2(0.f, 0.f);
      kb[c][u] = ib ? __ldcs(Kb + c * nb + i) : make_float2(0.f, 0.f);
    }
  }
#pragma unroll
  for (int u = 0; u < NA_U; ++u)
#pragma unroll
    for (int c = 0; c < K1; ++c) {
      df_fma_acc(acc[c], ka[c][u], fa[u]);
      df_fma_acc(acc[c], kb[c][u], fb[u]);
    }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_sum(f2 v) {  // fixed butterfly order, double-float
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, v.h, o), ol = __shfl_xor_sync(0xffffffffu, v.l, o);
    const f2 s = two_sum(v.h, oh);
    v = {s.h, s.l + (v.l + ol)};
  }
  return (double)v.h + (double)v.l;
}

// x -> interleaved (hi, lo) floats with hi + lo = x to ~2^-48 (in place allowed).
__global__ void to_float_pairs_kernel(int64_t n, const double* x, float2* out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double v = x[i];
    const float h = (float)v;
    out[i] = make_float2(h, (float)(v - (double)h));
  }
}

// Entry j of the resolved table: resolved[2j] = K offset, resolved[2j + 1] = (F offset << 20) | length,
// or -1 for an entry whose indices were out of range.
constexpr int NA_LEN_BITS = 20;

template <int K1, bool PAIRS, bool RESOLVED>
__global__ void __launch_bounds__(32 * NA_WARPS) near_apply_kernel(NearApplyParams p) {
  using Acc = typename std::conditional<PAIRS, f2, double>::type;
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * NA_WARPS;
  int64_t t = (int64_t)blockIdx.x * NA_WARPS + (threadIdx.x >> 5);
  // the next target's pair range is loaded one target ahead
  int64_t nj0 = t < p.n_trg ? p.trg_dsp[t] : 0, nj1 = t < p.n_trg ? p.trg_dsp[t + 1] : 0;
  for (; t < p.n_trg; t += nwarps) {
    Acc acc[K1];
#pragma unroll
    for (int c = 0; c < K1; ++c) acc[c] = Acc{};
    int64_t j0 = nj0, j1 = nj1;
    if (t + nwarps < p.n_trg) {
      nj0 = p.trg_dsp[t + nwarps];
      nj1 = p.trg_dsp[t + nwarps + 1];
    }
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
        if constexpr (RESOLVED) {  // one coalesced 16-byte load per entry
          const int64_t r1 = p.resolved[2 * j + 1];
          kofs = p.resolved[2 * j];
          if (r1 >= 0) {
            n = r1 & ((INT64_C(1) << NA_LEN_BITS) - 1);
            fofs = r1 >> NA_LEN_BITS;
            if (fofs + n > p.n_f || kofs < 0 || kofs + n * K1 > p.n_k) n = -1;
          }
        } else {
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
        }
        if (n < 0) bad = true;
      }
      const int m = (int)(j1 - jb < 32 ? j1 - jb : 32);
      for (int q = 0; q < m;) {
        const int64_t nq = __shfl_sync(0xffffffffu, n, q);
        const int64_t fq = __shfl_sync(0xffffffffu, fofs, q);
        const int64_t kq = __shfl_sync(0xffffffffu, kofs, q);
        if constexpr (PAIRS) {
          // two small blocks at once: twice the bytes in flight per warp
          if (q + 1 < m) {
            const int64_t nq2 = __shfl_sync(0xffffffffu, n, q + 1);
            const int64_t fq2 = __shfl_sync(0xffffffffu, fofs, q + 1);
            const int64_t kq2 = __shfl_sync(0xffffffffu, kofs, q + 1);
            if (nq > 0 && nq <= 32 * NA_U && nq2 > 0 && nq2 <= 32 * NA_U) {
              apply_two_pairs<K1>(p.K2 + kq, p.F2 + fq, nq, p.K2 + kq2, p.F2 + fq2, nq2, lane, acc);
              q += 2;
              continue;
            }
          }
          if (nq > 0) apply_pair<K1>(p.K2 + kq, p.F2 + fq, nq, lane, acc);
        } else {
          if (nq > 0) apply_pair<K1>(p.K + kq, p.F + fq, nq, lane, acc);
        }
        ++q;
      }
    }
    double tot[K1];
#pragma unroll
    for (int c = 0; c < K1; ++c) tot[c] = warp_sum(acc[c]);
    bad = __any_sync(0xffffffffu, bad);
    if (lane == 0) {
      if (bad && p.status) atomicOr(p.status, 4u);  // an index out of range: that pair skipped
      if (j1 > j0)
#pragma unroll
        for (int c = 0; c < K1; ++c) p.U[t * K1 + c] += tot[c];
    }
  }
}

template <int K1>
void launch_k1(const NearApplyParams& p, unsigned grid, cudaStream_t st) {
  if (p.resolved) {
    if (p.K2)
      near_apply_kernel<K1, true, true><<<grid, 32 * NA_WARPS, 0, st>>>(p);
    else
      near_apply_kernel<K1, false, true><<<grid, 32 * NA_WARPS, 0, st>>>(p);
  } else {
    if (p.K2)
      near_apply_kernel<K1, true, false><<<grid, 32 * NA_WARPS, 0, st>>>(p);
    else
      near_apply_kernel<K1, false, false><<<grid, 32 * NA_WARPS, 0, st>>>(p);
  }
}

// The index chain of one target-major entry resolved once (the storage SetupNear keeps).
__global__ void near_resolve_kernel(NearApplyParams p, int64_t* out) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < p.n_near;
       j += (int64_t)gridDim.x * blockDim.x) {
    int64_t n = -1, fofs = 0, kofs = 0;
    const int64_t pr = p.trg_pair ? p.trg_pair[j] : j;
    if (pr >= 0 && pr < p.n_pairs) {
      const int64_t e = p.pair_elem[pr];
      if (e >= 0 && e < p.n_elem) {
        n = p.elem_nds_cnt[e] * p.k0;
        fofs = p.elem_nds_dsp[e] * p.k0;
        kofs = p.pair_kdsp[pr];
        if (n < 0 || n >= (INT64_C(1) << NA_LEN_BITS) || fofs < 0 || fofs + n > p.n_f || kofs < 0 ||
            kofs + n * p.k1 > p.n_k)
          n = -1;
      }
    }
    out[2 * j] = n < 0 ? 0 : kofs;
    out[2 * j + 1] = n < 0 ? -1 : (fofs << NA_LEN_BITS) | n;
  }
}

}  // namespace
}  // namespace sctlgpu

using namespace sctlgpu;

static int near_apply(int k0, int k1, int64_t n_trg, const int64_t* trg_dsp, int64_t n_near, const int64_t* trg_pair,
                      int64_t n_pairs, const int64_t* pair_elem, const int64_t* pair_kdsp, int64_t n_elem,
                      const int64_t* elem_nds_dsp, const int64_t* elem_nds_cnt, int64_t n_k, const double* K,
                      const float* K2, int64_t n_f, const double* F, double* U, void* stream,
                      const int64_t* resolved = nullptr) {
  if (k0 < 1 || !(k1 == 1 || k1 == 2 || k1 == 3 || k1 == 4 || k1 == 9) || n_trg < 0 || n_near < 0 ||
      n_pairs < 0 || n_elem < 0 || n_k < 0 || n_f < 0 || (!trg_pair && !resolved && n_near > n_pairs))
    return SCTLGPU_ERR_INVALID_SIZE;
  if (n_trg == 0) return SCTLGPU_OK;
  if (!trg_dsp || !U || ((resolved ? n_near : n_pairs) && !K && !K2) ||
      (!resolved && ((n_pairs && (!pair_elem || !pair_kdsp)) || (n_elem && (!elem_nds_dsp || !elem_nds_cnt)))) ||
      (resolved == nullptr ? (n_elem && !F) : (n_f && !F)) || (resolved && n_near && !resolved))
    return SCTLGPU_ERR_NULL_POINTER;
  if (K2 && ((uintptr_t)K2 & 7)) return SCTLGPU_ERR_INVALID_SIZE;  // float pairs: 8-byte aligned
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
  p.resolved = resolved;
  p.K = K;
  p.K2 = reinterpret_cast<const float2*>(K2);
  p.F = F;
  p.U = U;
  p.status = status;
  const int64_t ctas = (n_trg + NA_WARPS - 1) / NA_WARPS;
  const int64_t cap = (int64_t)sms * 8;  // 8 CTAs of 8 warps per SM: full occupancy
  const unsigned grid = (unsigned)(ctas < cap ? ctas : cap);
  cudaStream_t st = (cudaStream_t)stream;
  float2* F2 = nullptr;
  if (K2 && n_f > 0) {  // densities as float pairs, once per call (small: nodes x k0)
    const cudaError_t e = cudaMallocAsync((void**)&F2, (size_t)n_f * sizeof(float2), st);
    if (e != cudaSuccess) return runtime_record(e);
    const int64_t b = (n_f + 255) / 256;
    to_float_pairs_kernel<<<(unsigned)(b < (int64_t)sms * 8 ? b : (int64_t)sms * 8), 256, 0, st>>>(n_f, F, F2);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    p.F2 = F2;
  }
  switch (k1) {
    case 1: launch_k1<1>(p, grid, st); break;
    case 2: launch_k1<2>(p, grid, st); break;
    case 3: launch_k1<3>(p, grid, st); break;
    case 4: launch_k1<4>(p, grid, st); break;
    default: launch_k1<9>(p, grid, st); break;  // k1 checked above
  }
  g_launches.fetch_add(1, std::memory_order_relaxed);
  cudaError_t e = cudaGetLastError();
  if (F2) {
    const cudaError_t e2 = cudaFreeAsync(F2, st);
    if (e == cudaSuccess) e = e2;
  }
  return runtime_record(e);
}

extern "C" int sctlgpu_near_matrix_apply(int k0, int k1, int64_t n_trg, const int64_t* trg_dsp, int64_t n_near,
                                         const int64_t* trg_pair, int64_t n_pairs, const int64_t* pair_elem,
                                         const int64_t* pair_kdsp, int64_t n_elem, const int64_t* elem_nds_dsp,
                                         const int64_t* elem_nds_cnt, int64_t n_k, const double* K, int64_t n_f,
                                         const double* F, double* U, void* stream) {
  return near_apply(k0, k1, n_trg, trg_dsp, n_near, trg_pair, n_pairs, pair_elem, pair_kdsp, n_elem, elem_nds_dsp,
                    elem_nds_cnt, n_k, K, nullptr, n_f, F, U, stream);
}

extern "C" int sctlgpu_near_matrix_apply_pairs(int k0, int k1, int64_t n_trg, const int64_t* trg_dsp,
                                               int64_t n_near, const int64_t* trg_pair, int64_t n_pairs,
                                               const int64_t* pair_elem, const int64_t* pair_kdsp, int64_t n_elem,
                                               const int64_t* elem_nds_dsp, const int64_t* elem_nds_cnt,
                                               int64_t n_k, const float* K2, int64_t n_f, const double* F,
                                               double* U, void* stream) {
  return near_apply(k0, k1, n_trg, trg_dsp, n_near, trg_pair, n_pairs, pair_elem, pair_kdsp, n_elem, elem_nds_dsp,
                    elem_nds_cnt, n_k, nullptr, K2, n_f, F, U, stream);
}

extern "C" int sctlgpu_near_matrix_resolve(int k0, int k1, int64_t n_near, const int64_t* trg_pair, int64_t n_pairs,
                                           const int64_t* pair_elem, const int64_t* pair_kdsp, int64_t n_elem,
                                           const int64_t* elem_nds_dsp, const int64_t* elem_nds_cnt, int64_t n_k,
                                           int64_t n_f, int64_t* resolved, void* stream) {
  if (k0 < 1 || !(k1 == 1 || k1 == 2 || k1 == 3 || k1 == 4 || k1 == 9) || n_near < 0 || n_pairs < 0 || n_elem < 0 ||
      n_k < 0 || n_f < 0 || (!trg_pair && n_near > n_pairs))
    return SCTLGPU_ERR_INVALID_SIZE;
  if (n_near == 0) return SCTLGPU_OK;
  if (!resolved || (n_pairs && (!pair_elem || !pair_kdsp)) || (n_elem && (!elem_nds_dsp || !elem_nds_cnt)))
    return SCTLGPU_ERR_NULL_POINTER;
  int dev;
  unsigned* status;
  int sms;
  int rc = runtime_device(&dev, &status, &sms);
  if (rc) return rc;
  NearApplyParams p{};
  p.k0 = k0;
  p.k1 = k1;
  p.n_near = n_near;
  p.n_pairs = n_pairs;
  p.n_elem = n_elem;
  p.n_k = n_k;
  p.n_f = n_f;
  p.trg_pair = trg_pair;
  p.pair_elem = pair_elem;
  p.pair_kdsp = pair_kdsp;
  p.elem_nds_dsp = elem_nds_dsp;
  p.elem_nds_cnt = elem_nds_cnt;
  const int64_t b = (n_near + 255) / 256;
  near_resolve_kernel<<<(unsigned)(b < (int64_t)sms * 8 ? b : (int64_t)sms * 8), 256, 0, (cudaStream_t)stream>>>(
      p, resolved);
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return runtime_record(cudaGetLastError());
}

extern "C" int sctlgpu_near_matrix_apply_resolved(int k0, int k1, int64_t n_trg, const int64_t* trg_dsp,
                                                  int64_t n_near, const int64_t* resolved, int64_t n_k,
                                                  const double* K, const float* K2, int64_t n_f, const double* F,
                                                  double* U, void* stream) {
  if ((K == nullptr) == (K2 == nullptr)) return SCTLGPU_ERR_INVALID_ARGUMENT;  // exactly one form of the blocks
  return near_apply(k0, k1, n_trg, trg_dsp, n_near, nullptr, 0, nullptr, nullptr, 0, nullptr, nullptr, n_k, K, K2,
                    n_f, F, U, stream, resolved);
}

extern "C" int sctlgpu_to_float_pairs(int64_t n, const double* x, float* out, void* stream) {
  if (n < 0) return SCTLGPU_ERR_INVALID_SIZE;
  if (n == 0) return SCTLGPU_OK;
  if (!x || !out) return SCTLGPU_ERR_NULL_POINTER;
  if (((uintptr_t)out & 7) || ((uintptr_t)x & 7)) return SCTLGPU_ERR_INVALID_SIZE;
  int dev, sms;
  unsigned* status;
  int rc = runtime_device(&dev, &status, &sms);
  if (rc) return rc;
  const int64_t b = (n + 255) / 256;
  to_float_pairs_kernel<<<(unsigned)(b < (int64_t)sms * 16 ? b : (int64_t)sms * 16), 256, 0, (cudaStream_t)stream>>>(
      n, x, reinterpret_cast<float2*>(out));
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return runtime_record(cudaGetLastError());
}
