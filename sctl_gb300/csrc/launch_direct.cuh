// Launch sequence of one direct sum: [bbox] -> pack sources -> tiled sum ->
// ordered reduction of the per-slice partials into v_trg.  Scratch (packed
// records, partials, bbox) comes from the stream-ordered allocator, so the
// sequence is asynchronous and safe to enqueue from several host threads.
#pragma once

#include <algorithm>
#include <mutex>

#include "direct.cuh"
#include "direct_pk.cuh"
#include "launch.h"

namespace sctlgpu {

#define SCTLGPU_TRY(expr)                    \
  do {                                       \
    cudaError_t e_ = (expr);                 \
    if (e_ != cudaSuccess) return e_;        \
  } while (0)

inline int grid_for(int64_t n, int threads, int sms) {
  const int64_t b = (n + threads - 1) / threads;
  return (int)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)sms * 8));
}

// Source split so the grid covers whole waves of resident CTAs (>= 95% of the
// last wave busy when possible), with at least one tile per slice.
inline int choose_nsplit(int64_t tblocks, int64_t ns, int tile, int wave) {
  const int64_t max_split = std::max<int64_t>(1, std::min<int64_t>(1024, (ns + tile - 1) / tile));
  int best = 1;
  double best_eff = 0;
  for (int64_t k = 1; k <= max_split; ++k) {
    const int64_t total = tblocks * k;
    const int64_t waves = (total + wave - 1) / wave;
    const double eff = (double)total / (double)(waves * wave);
    // Prefer few slices: each adds partial traffic and a source re-read.
    if (eff > best_eff + 1e-9) {
      best_eff = eff;
      best = (int)k;
    }
    if (total >= 2 * wave && eff >= 0.95) break;
    if (total >= 64LL * wave) break;
  }
  return best;
}

template <int KER, int MODE, int NEWTON>
cudaError_t run_direct(const EvalCall& c) {
  using RecT = Rec<KER, MODE>;
  using Cfg = TileCfg<KER, MODE>;
  constexpr int K1 = KDims<KER>::K1;
  using Real = typename std::conditional<MODE == MODE_F32, float, double>::type;
  cudaStream_t st = c.stream;

  const size_t smem = 2 * Cfg::S * sizeof(RecT) + 2 * sizeof(uint64_t);
  static int occ = [&] {
    int o = 0;
    if (smem > 48 * 1024)
      cudaFuncSetAttribute(direct_sum_kernel<KER, MODE, NEWTON>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, direct_sum_kernel<KER, MODE, NEWTON>, Cfg::THREADS, smem);
    return o > 0 ? o : 1;
  }();

  const int64_t per_cta = (int64_t)Cfg::THREADS * Cfg::T;
  const int64_t tblocks = (c.nt + per_cta - 1) / per_cta;
  const int nsplit0 = choose_nsplit(tblocks, c.ns, Cfg::S, c.sms * occ);
  int64_t chunk = (c.ns + nsplit0 - 1) / nsplit0;
  chunk = ((chunk + Cfg::S - 1) / Cfg::S) * Cfg::S;
  const int nsplit = (int)((c.ns + chunk - 1) / chunk);

  // Scratch.
  const size_t rec_bytes = (size_t)c.ns * sizeof(RecT);
  const size_t part_bytes = (size_t)nsplit * (size_t)c.nt * K1 * sizeof(double);
  const size_t bbox_bytes = 256;
  char* scratch = nullptr;
  const size_t rec_off = 0;
  const size_t part_off = (rec_bytes + 255) / 256 * 256;
  const size_t bbox_off = part_off + (part_bytes + 255) / 256 * 256;
  SCTLGPU_TRY(cudaMallocAsync((void**)&scratch, bbox_off + bbox_bytes, st));
  RecT* recs = reinterpret_cast<RecT*>(scratch + rec_off);
  double* partial = reinterpret_cast<double*>(scratch + part_off);
  BBox* bb = reinterpret_cast<BBox*>(scratch + bbox_off);

  cudaError_t err = cudaSuccess;
  do {
    if (MODE == MODE_MXLO || MODE == MODE_MXDF) {
      err = compute_bbox(st, c.nt, (const double*)c.r_trg, c.ns, (const double*)c.r_src, bb);
      if (err != cudaSuccess) break;
    }
    pack_sources_kernel<KER, MODE, Real><<<grid_for(c.ns, 256, c.sms), 256, 0, st>>>(
        c.ns, (const Real*)c.r_src, (const Real*)c.n_src, (const Real*)c.v_src, recs, bb);
    g_launches.fetch_add(1, std::memory_order_relaxed);

    DirectParams p;
    p.nt = c.nt;
    p.ns = c.ns;
    p.r_trg = c.r_trg;
    p.recs = recs;
    p.chunk = chunk;
    p.partial = partial;
    p.bbox = bb;
    p.status = c.status;
    dim3 grid((unsigned)tblocks, (unsigned)nsplit);
    if (c.timing && c.timing->enabled) cudaEventRecord(c.timing->start, st);
    direct_sum_kernel<KER, MODE, NEWTON><<<grid, Cfg::THREADS, smem, st>>>(p);
    if (c.timing && c.timing->enabled) {
      cudaEventRecord(c.timing->stop, st);
      c.timing->recorded = true;
    }
    g_launches.fetch_add(1, std::memory_order_relaxed);

    const int64_t nout = c.nt * K1;
    reduce_partials_kernel<Real><<<grid_for(nout, 256, c.sms), 256, 0, st>>>(
        nout, nsplit, partial, scale_of<KER>(), c.accumulate ? 1 : 0, (Real*)c.v_trg);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    err = cudaGetLastError();
  } while (0);
  cudaError_t e2 = cudaFreeAsync(scratch, st);
  return err != cudaSuccess ? err : e2;
}

// Mixed precision, double-float arithmetic on the packed FP32 pipe (direct_pk.cuh):
// the same sequence with pair records.
template <int KER>
cudaError_t run_direct_pk(const EvalCall& c) {
  using RecT = RecPk<KER>;
  using Cfg = TileCfgPk<KER>;
  constexpr int K1 = KDims<KER>::K1;
  cudaStream_t st = c.stream;

  const size_t smem = 2 * Cfg::S * sizeof(RecT) + 2 * sizeof(uint64_t);
  static int occ = [&] {
    int o = 0;
    if (smem > 48 * 1024)
      cudaFuncSetAttribute(direct_sum_pk_kernel<KER>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, direct_sum_pk_kernel<KER>, Cfg::THREADS, smem);
    return o > 0 ? o : 1;
  }();

  const int64_t npairs = (c.ns + 1) / 2;
  const int64_t per_cta = (int64_t)Cfg::THREADS * Cfg::T;
  const int64_t tblocks = (c.nt + per_cta - 1) / per_cta;
  const int nsplit0 = choose_nsplit(tblocks, npairs, Cfg::S, c.sms * occ);
  int64_t chunk = (npairs + nsplit0 - 1) / nsplit0;
  chunk = ((chunk + Cfg::S - 1) / Cfg::S) * Cfg::S;
  const int nsplit = (int)((npairs + chunk - 1) / chunk);

  const size_t rec_bytes = (size_t)npairs * sizeof(RecT);
  const size_t part_bytes = (size_t)nsplit * (size_t)c.nt * K1 * sizeof(double);
  const size_t part_off = (rec_bytes + 255) / 256 * 256;
  const size_t bbox_off = part_off + (part_bytes + 255) / 256 * 256;
  char* scratch = nullptr;
  SCTLGPU_TRY(cudaMallocAsync((void**)&scratch, bbox_off + 256, st));
  RecT* recs = reinterpret_cast<RecT*>(scratch);
  double* partial = reinterpret_cast<double*>(scratch + part_off);
  BBox* bb = reinterpret_cast<BBox*>(scratch + bbox_off);

  cudaError_t err = cudaSuccess;
  do {
    err = compute_bbox(st, c.nt, (const double*)c.r_trg, c.ns, (const double*)c.r_src, bb);
    if (err != cudaSuccess) break;
    pack_pairs_kernel<KER><<<grid_for(npairs, 256, c.sms), 256, 0, st>>>(
        c.ns, (const double*)c.r_src, (const double*)c.n_src, (const double*)c.v_src, recs, bb);
    g_launches.fetch_add(1, std::memory_order_relaxed);

    DirectParams p;
    p.nt = c.nt;
    p.ns = npairs;
    p.r_trg = c.r_trg;
    p.recs = recs;
    p.chunk = chunk;
    p.partial = partial;
    p.bbox = bb;
    p.status = c.status;
    dim3 grid((unsigned)tblocks, (unsigned)nsplit);
    if (c.timing && c.timing->enabled) cudaEventRecord(c.timing->start, st);
    direct_sum_pk_kernel<KER><<<grid, Cfg::THREADS, smem, st>>>(p);
    if (c.timing && c.timing->enabled) {
      cudaEventRecord(c.timing->stop, st);
      c.timing->recorded = true;
    }
    g_launches.fetch_add(1, std::memory_order_relaxed);

    const int64_t nout = c.nt * K1;
    reduce_partials_kernel<double><<<grid_for(nout, 256, c.sms), 256, 0, st>>>(
        nout, nsplit, partial, scale_of<KER>(), c.accumulate ? 1 : 0, (double*)c.v_trg);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    err = cudaGetLastError();
  } while (0);
  cudaError_t e2 = cudaFreeAsync(scratch, st);
  return err != cudaSuccess ? err : e2;
}

}  // namespace sctlgpu
