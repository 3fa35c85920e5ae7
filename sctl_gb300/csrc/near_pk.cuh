// The batched near-field kernel (near.cuh) with pair records: double-float
// arithmetic on the packed FP32 pipe (direct_pk.cuh) for the mixed mode at
// 8..11 digits.  Sources are paired within each block -- a record never holds
// sources of two blocks -- so the plan packs per block (pack_block_pairs_kernel)
// and the kernel's block table counts pair records.
#pragma once

#include "direct_pk.cuh"
#include "near.cuh"

namespace sctlgpu {

template <int KER>
struct NearCfgPk {
  static constexpr int T = TileCfgPk<KER>::T;
  static constexpr int S = 128;                 // pair records per tile
  static constexpr int CAP = NEAR_THREADS * T;  // targets of an item at split 1
};

// Pair g of the plan: the block that owns it (pblk: pair offsets and counts,
// sblk: the same blocks' source ranges), sources sblk.s0 + 2j and + 2j + 1.
template <int KER>
__global__ void pack_block_pairs_kernel(int64_t nblk, const NearBlock* __restrict__ pblk,
                                        const NearBlock* __restrict__ sblk, int64_t n_pairs,
                                        const double* __restrict__ xs, const double* __restrict__ nrm,
                                        const double* __restrict__ f, const double* __restrict__ w,
                                        RecPk<KER>* __restrict__ out, const BBox* bb) {
  const MixedFrame fr = frame_from_bbox(bb);
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n_pairs; g += (int64_t)gridDim.x * blockDim.x) {
    // last block whose first pair is <= g (a block without pairs shares its offset with the next one)
    int64_t lo = 0, hi = nblk - 1;
    while (lo < hi) {
      const int64_t mid = (lo + hi + 1) >> 1;
      if (pblk[mid].s0 <= g) lo = mid; else hi = mid - 1;
    }
    const int64_t j = g - pblk[lo].s0;
    const NearBlock sb = sblk[lo];
    out[g] = pair_record<KER>(fr, sb.s0 + 2 * j, 2 * j + 1 < sb.ns, xs, nrm, f, w);
  }
}

template <int KER>
__global__ void __launch_bounds__(NEAR_THREADS) near_batch_pk_kernel(NearParams p) {
  using P = PairPk<KER>;
  using RecT = RecPk<KER>;
  using Cfg = NearCfgPk<KER>;
  constexpr int T = Cfg::T, S = Cfg::S, K1 = KDims<KER>::K1;

  extern __shared__ __align__(128) unsigned char smem_raw[];
  RecT* tiles = reinterpret_cast<RecT*>(smem_raw);
  double* red = reinterpret_cast<double*>(smem_raw + 2 * S * sizeof(RecT));  // [NEAR_THREADS*T][K1]
  uint64_t* bars = reinterpret_cast<uint64_t*>(red + NEAR_THREADS * T * K1);
  __shared__ int64_t s_item;

  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fence_mbar_init();
  }
  const MixedFrame fr = frame_from_bbox(p.bbox);
  const double* rt = reinterpret_cast<const double*>(p.r_trg);
  const RecT* recs = reinterpret_cast<const RecT*>(p.recs);
  uint32_t issued = 0, consumed = 0;  // tiles issued / waited by this CTA (buffer = n & 1, phase = (n >> 1) & 1)
  __syncthreads();

  for (;;) {
    if (threadIdx.x == 0) s_item = (int64_t)atomicAdd(p.counter, 1u);
    __syncthreads();
    const int64_t it = s_item;
    if (it >= p.n_items) break;
    const NearItem item = p.items[it];
    const NearBlock blk = p.blocks[item.block];  // s0, ns in pair records
    const int split = item.split;
    const int gsize = NEAR_THREADS / split;
    const int grp = threadIdx.x / gsize, lane = threadIdx.x % gsize;
    const int64_t tbase = blk.t0 + item.t_off;

    typename P::Trg tg[T];
#pragma unroll
    for (int j = 0; j < T; ++j) {
      const int lt = lane + j * gsize;
      const int64_t k = tbase + (lt < item.nt ? lt : 0);
      P::load_trg(tg[j], rt, p.tidx ? p.tidx[k] : k, fr);
    }

    const RecT* src = recs + blk.s0;
    const int ntiles = (int)((blk.ns + S - 1) / S);
    if (threadIdx.x == 0) {
      for (int b = 0; b < 2 && b < ntiles; ++b) {
        const uint32_t cnt = (uint32_t)imin64((int64_t)S, blk.ns - (int64_t)b * S);
        const int buf = issued & 1;
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&bars[buf], cnt * (uint32_t)sizeof(RecT));
        bulk_g2s(tiles + buf * S, src + (int64_t)b * S, cnt * (uint32_t)sizeof(RecT), &bars[buf]);
        ++issued;
      }
    }
    for (int k = 0; k < ntiles; ++k) {
      const int buf = consumed & 1;
      mbar_wait_bounded(&bars[buf], (consumed >> 1) & 1, p.status);
      ++consumed;
      const RecT* tile = tiles + buf * S;
      const int cnt = (int)imin64((int64_t)S, blk.ns - (int64_t)k * S);
      for (int s = grp; s < cnt; s += split) {
        const RecT rec = tile[s];
#pragma unroll
        for (int j = 0; j < T; ++j) P::apply(tg[j], rec);
      }
#pragma unroll
      for (int j = 0; j < T; ++j) P::flush(tg[j]);
      __syncthreads();  // the buffer is free again
      if (threadIdx.x == 0 && k + 2 < ntiles) {
        const uint32_t c2 = (uint32_t)imin64((int64_t)S, blk.ns - (int64_t)(k + 2) * S);
        const int b2 = issued & 1;
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&bars[b2], c2 * (uint32_t)sizeof(RecT));
        bulk_g2s(tiles + b2 * S, src + (int64_t)(k + 2) * S, c2 * (uint32_t)sizeof(RecT), &bars[b2]);
        ++issued;
      }
    }

    // Combine the split groups' partial sums (group order is fixed: deterministic).
    if (split > 1) {
      for (int g = 1; g < split; ++g) {
        if (grp == g) {
#pragma unroll
          for (int j = 0; j < T; ++j)
#pragma unroll
            for (int c = 0; c < K1; ++c) red[(lane + j * gsize) * K1 + c] = P::result(tg[j], c);
        }
        __syncthreads();
        if (grp == 0) {
#pragma unroll
          for (int j = 0; j < T; ++j)
#pragma unroll
            for (int c = 0; c < K1; ++c) P::add_partial(tg[j], c, red[(lane + j * gsize) * K1 + c]);
        }
        __syncthreads();
      }
    }
    if (grp == 0) {
      const double scale = scale_of<KER>();
#pragma unroll
      for (int j = 0; j < T; ++j) {
        const int lt = lane + j * gsize;
        if (lt >= item.nt) continue;
        const int64_t t = tbase + lt;
#pragma unroll
        for (int c = 0; c < K1; ++c) {
          const double v = P::result(tg[j], c) * scale;
          if (p.map || p.tidx) {
            atomicAdd(&p.out[(p.map ? p.map[t] : p.tidx[t]) * K1 + c], v);
          } else {
            double* o = &p.out[t * K1 + c];
            *o = p.accumulate ? *o + v : v;
          }
        }
      }
    }
    __syncthreads();  // s_item and the reduction buffer are reused by the next item
  }
}

}  // namespace sctlgpu
