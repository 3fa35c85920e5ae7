// Batched near-field direct sums: many independent (source block, target
// block) pairs of uneven sizes in ONE persistent launch.
//
// This is the GPU form of BoundaryIntegralOp's per-block near-field work
// (boundary_integral.txx:1165-1240 KNearSubtract, which calls KernelMatrix per
// near block inside an OpenMP dynamic loop, and :1311-1381 ComputeNearInterac,
// which applies the blocks and scatters into per-target sums): each block b
// adds  scale * sum_{s in block b} K(x_t - y_s, n_s) * w_s * f_s  to each of its
// targets t, either in place (v_out[t]) or scattered through a target map
// (atomic FP64 adds: several blocks may feed one physical target).  With a
// target index list, a block's targets are entries of that list (the
// reference's near lists) and results scatter to the listed targets.
//
// Work decomposition.  The host splits every block into items (block, first
// target, target count, source split) and sorts them by cost, largest first.
// One CTA per (SM x resident slot) pulls items from a device counter
// (atomicAdd).  For an item the CTA's threads form `split` groups; each group
// holds the item's targets in registers (T per thread) and sweeps every
// split-th record of each source tile, tiles staged in shared memory by the
// TMA bulk-copy engine (double-buffered, mbarrier-completed, phases carried
// across items); the groups' partial sums are then combined in shared memory.
// Small blocks (16 targets) use split 8 so all 128 lanes work; the split per
// block size class is chosen by the autotuner (near_plan.cu).
#pragma once

#include "direct.cuh"

namespace sctlgpu {

struct NearBlock {
  int64_t s0, ns;  // sources [s0, s0+ns)
  int64_t t0, nt;  // targets [t0, t0+nt)
};
struct NearItem {
  int32_t block;
  int32_t t_off;  // first target of the item inside its block
  int32_t nt;     // targets of the item
  int32_t split;  // source split (1, 2, 4, 8)
};

struct NearParams {
  const NearItem* items;
  int64_t n_items;
  const NearBlock* blocks;
  const void* r_trg;      // AoS targets (Real), concatenated over blocks, or indexed through tidx
  const int64_t* tidx;    // optional: block target positions -> target indices (near lists)
  const void* recs;       // packed source records, concatenated over blocks
  const int64_t* map;     // optional: output index of every target
  double* out;            // results (double); Real out when !map handled by `out_f`
  float* out_f;           // FP32 output (MODE_F32 only)
  unsigned* counter;      // work-queue head
  unsigned* status;       // device status word
  const BBox* bbox;       // mixed modes
  int accumulate;
};

constexpr int NEAR_THREADS = 128;

template <int KER, int MODE>
struct NearCfg {
  static constexpr int T = (MODE == MODE_MXDF && KER >= KER_SFXU) ? 1 : 2;
  static constexpr int S = 256;
  static constexpr int CAP = NEAR_THREADS * T;  // targets of an item at split 1
};

template <int KER, int MODE, int NEWTON>
__global__ void __launch_bounds__(NEAR_THREADS) near_batch_kernel(NearParams p) {
  using P = Pair<KER, MODE, NEWTON>;
  using RecT = Rec<KER, MODE>;
  using Cfg = NearCfg<KER, MODE>;
  constexpr int T = Cfg::T, S = Cfg::S, K1 = KDims<KER>::K1;
  using TrgReal = typename std::conditional<MODE == MODE_F32, float, double>::type;

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
  MixedFrame fr{};
  if constexpr (MODE == MODE_MXLO || MODE == MODE_MXDF) fr = frame_from_bbox(p.bbox);
  const TrgReal* rt = reinterpret_cast<const TrgReal*>(p.r_trg);
  const RecT* recs = reinterpret_cast<const RecT*>(p.recs);
  uint32_t issued = 0, consumed = 0;  // tiles issued / waited by this CTA (buffer = n & 1, phase = (n >> 1) & 1)
  __syncthreads();

  for (;;) {
    if (threadIdx.x == 0) s_item = (int64_t)atomicAdd(p.counter, 1u);
    __syncthreads();
    const int64_t it = s_item;
    if (it >= p.n_items) break;
    const NearItem item = p.items[it];
    const NearBlock blk = p.blocks[item.block];
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
          } else if (MODE == MODE_F32) {
            float* o = &p.out_f[t * K1 + c];
            *o = p.accumulate ? (float)((double)*o + v) : (float)v;
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
