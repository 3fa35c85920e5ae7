// Batched near-field plans (declared in include/sctlgpu.h): block validation,
// work-item construction with autotuned source splits, LPT ordering, CUDA
// graph capture / replay, and the tile autotuner.
#include <algorithm>
#include <array>
#include <cstdlib>
#include <map>
#include <mutex>
#include <random>
#include <tuple>
#include <vector>

#include "../../include/sctlgpu.h"
#include "launch.h"
#include "near.cuh"

using namespace sctlgpu;

struct sctlgpu_near_plan_s {
  int kernel = 0, mode = 0, digits = -1, imode = 0, newton = 0, K1 = 1, ND = 0;
  NearOps ops;
  int64_t nblk = 0, ns = 0, nt = 0, n_out = 0, n_items = 0, pairs = 0;
  bool has_map = false;
  int device = 0, sms = 1;
  NearItem* d_items = nullptr;
  NearBlock* d_blocks = nullptr;      // the kernel's table (pair records when ops.paired)
  NearBlock* d_src_blocks = nullptr;  // paired plans: every block's source range, for the per-block pack
  int64_t n_pairs = 0;                // paired plans: pair records of all blocks
  bool shared_pairs = false;          // paired plans whose blocks all start and end on pair boundaries
  int64_t* d_map = nullptr;
  int64_t* d_tidx = nullptr;
  int64_t n_index = 0;
  char* d_scratch = nullptr;
  void* d_recs = nullptr;
  BBox* d_bbox = nullptr;
  unsigned* d_counter = nullptr;
  unsigned* d_status = nullptr;
  cudaStream_t cap = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  const void* key[6] = {};
  unsigned key_flags = 0;
  int graph_kernels = 0;
  std::mutex mu;
};

namespace {

int imode_for(int mode, int d, int* newton) {
  *newton = runtime_steps(mode, d);
  if (mode == SCTLGPU_F64) return NEAR_F64;
  if (mode == SCTLGPU_F32) return NEAR_F32;
  if (d <= 7) return NEAR_MXLO;
  if (d <= runtime_mixed_df_max_digits()) return NEAR_MXDF;
  return NEAR_F64;
}

NearOps ops_for(int kernel, int imode, int newton) {
  if (imode == NEAR_F64) return near_ops_f64(kernel, newton);
  if (imode == NEAR_F32) return near_ops_f32(kernel, newton);
  return near_ops_mixed(kernel, imode, newton);
}

int class_of(int64_t nt, int64_t ns) {
  const int a = nt <= 24 ? 0 : nt <= 48 ? 1 : nt <= 96 ? 2 : nt <= 192 ? 3 : 4;
  return a * 2 + (ns <= 512 ? 0 : 1);
}

// Largest split that still keeps every target of the block in one item.
int lane_fill_split(int64_t nt, int T) {
  int s = 1;
  while (s < 8 && (int64_t)(NEAR_THREADS / (2 * s)) * T >= nt) s *= 2;
  return s;
}

void build_items(const std::vector<NearBlock>& blocks, const std::array<int, SCTLGPU_NEAR_CLASSES>& table, int T,
                 std::vector<NearItem>& items) {
  items.clear();
  std::vector<int64_t> cost;
  for (size_t b = 0; b < blocks.size(); ++b) {
    const NearBlock& B = blocks[b];
    if (B.nt <= 0) continue;
    const int split = table[class_of(B.nt, B.ns)];
    const int64_t cap = (int64_t)(NEAR_THREADS / split) * T;
    for (int64_t t = 0; t < B.nt; t += cap) {
      items.push_back({(int32_t)b, (int32_t)t, (int32_t)std::min<int64_t>(cap, B.nt - t), (int32_t)split});
      cost.push_back(std::max<int64_t>(B.ns, 1) * items.back().nt);
    }
  }
  std::vector<size_t> order(items.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return cost[a] > cost[b]; });
  std::vector<NearItem> sorted(items.size());
  for (size_t i = 0; i < order.size(); ++i) sorted[i] = items[order[i]];
  items.swap(sorted);
}

// ------------------------------------------------------------- autotuner
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int, int>, std::array<int, SCTLGPU_NEAR_CLASSES>> g_tune;

cudaError_t time_items(const NearOps& ops, int sms, const std::vector<NearItem>& items, NearItem* d_items,
                       const NearBlock* d_blocks, const void* d_trg, const void* d_recs, double* d_out,
                       unsigned* d_counter, unsigned* d_status, const BBox* d_bbox, cudaStream_t st, float* ms) {
  cudaError_t e = cudaMemcpyAsync(d_items, items.data(), items.size() * sizeof(NearItem), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  NearParams p{};
  p.items = d_items;
  p.n_items = (int64_t)items.size();
  p.blocks = d_blocks;
  p.r_trg = d_trg;
  p.recs = d_recs;
  p.out = d_out;
  p.out_f = (float*)d_out;
  p.counter = d_counter;
  p.status = d_status;
  p.bbox = d_bbox;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  float best = 1e30f;
  for (int rep = 0; rep < 2 && e == cudaSuccess; ++rep) {
    cudaMemsetAsync(d_counter, 0, sizeof(unsigned), st);
    cudaEventRecord(a, st);
    e = ops.launch(st, (unsigned)(sms * ops.occ), p);
    cudaEventRecord(b, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(b);
    float t = 0;
    if (e == cudaSuccess && cudaEventElapsedTime(&t, a, b) == cudaSuccess) best = std::min(best, t);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *ms = best;
  return e;
}

// Times splits 1, 2, 4, 8 for every size class on synthetic blocks (about
// 5e7 interactions per candidate) and keeps the fastest split per class.
int autotune(int kernel, int imode, int newton, const NearOps& ops, int sms, int mode,
             std::array<int, SCTLGPU_NEAR_CLASSES>& table) {
  int dev = 0;
  cudaGetDevice(&dev);
  const auto dkey = std::make_tuple(dev, kernel, imode, newton);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(dkey);
    if (it != g_tune.end()) {
      table = it->second;
      return SCTLGPU_OK;
    }
  }
  for (int c = 0; c < SCTLGPU_NEAR_CLASSES; ++c) {
    static const int64_t rep_nt[5] = {16, 36, 72, 144, 384};
    table[c] = lane_fill_split(rep_nt[c / 2], ops.T);
  }
  const char* env = std::getenv("SCTLGPU_NEAR_AUTOTUNE");
  if (!(env && env[0] == '0')) {
    const size_t real = imode == NEAR_F32 ? sizeof(float) : sizeof(double);
    const int64_t max_ns = 2048, max_nt = 384;
    const int64_t nb_max = std::max<int64_t>(sms, 2LL * sms * ops.occ);
    const int64_t tot_s = nb_max * max_ns, tot_t = nb_max * max_nt;
    // Synthetic points: uniform in a unit cube per block, densities 1, normals +z.
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    std::vector<double> hx(tot_s * 3), hn(tot_s * 3), hf(tot_s * 3, 1.0), ht(tot_t * 3);
    for (auto& v : hx) v = U(rng);
    for (auto& v : ht) v = U(rng) + 0.01;
    for (int64_t i = 0; i < tot_s; ++i) {
      hn[i * 3] = 0;
      hn[i * 3 + 1] = 0;
      hn[i * 3 + 2] = 1;
    }
    std::vector<float> fx, fn, ff, ft;
    const void *px = hx.data(), *pn = hn.data(), *pf = hf.data(), *pt = ht.data();
    if (real == sizeof(float)) {
      fx.assign(hx.begin(), hx.end());
      fn.assign(hn.begin(), hn.end());
      ff.assign(hf.begin(), hf.end());
      ft.assign(ht.begin(), ht.end());
      px = fx.data();
      pn = fn.data();
      pf = ff.data();
      pt = ft.data();
    }
    cudaStream_t st;
    cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    char* buf = nullptr;
    const size_t o_x = 0, o_n = o_x + tot_s * 3 * real, o_f = o_n + tot_s * 3 * real, o_t = o_f + tot_s * 3 * real,
                 o_r = (o_t + tot_t * 3 * real + 255) / 256 * 256, o_o = (o_r + tot_s * ops.rec_bytes + 255) / 256 * 256,
                 o_b = o_o + tot_t * 3 * sizeof(double), o_i = o_b + nb_max * sizeof(NearBlock),
                 o_m = (o_i + nb_max * 64 * sizeof(NearItem) + 255) / 256 * 256, total = o_m + 512;
    cudaError_t e = cudaMalloc(&buf, total);
    if (e == cudaSuccess) {
      cudaMemcpyAsync(buf + o_x, px, tot_s * 3 * real, cudaMemcpyHostToDevice, st);
      cudaMemcpyAsync(buf + o_n, pn, tot_s * 3 * real, cudaMemcpyHostToDevice, st);
      cudaMemcpyAsync(buf + o_f, pf, tot_s * 3 * real, cudaMemcpyHostToDevice, st);
      cudaMemcpyAsync(buf + o_t, pt, tot_t * 3 * real, cudaMemcpyHostToDevice, st);
      BBox* bb = (BBox*)(buf + o_m);
      unsigned* counter = (unsigned*)(buf + o_m + 256);
      unsigned* status = counter + 1;
      cudaMemsetAsync(status, 0, sizeof(unsigned), st);
      if (imode == NEAR_MXLO || imode == NEAR_MXDF)
        e = compute_bbox(st, tot_t, (const double*)(buf + o_t), tot_s, (const double*)(buf + o_x), bb);
      if (e == cudaSuccess)
        e = ops.pack(st, tot_s, buf + o_x, buf + o_n, buf + o_f, nullptr, buf + o_r, bb, sms);
      for (int c = 0; c < SCTLGPU_NEAR_CLASSES && e == cudaSuccess; ++c) {
        static const int64_t rep_nt[5] = {16, 36, 72, 144, 384};
        const int64_t cnt_t = rep_nt[c / 2], cnt_s = (c % 2) ? 2048 : 256;
        const int64_t nb = std::max<int64_t>(sms, std::min<int64_t>(nb_max, (int64_t)5e7 / (cnt_t * cnt_s)));
        std::vector<NearBlock> blocks(nb), kblocks(nb);
        for (int64_t b = 0; b < nb; ++b) {
          blocks[b] = {b * max_ns, cnt_s, b * max_nt, cnt_t};
          // paired records: every block starts at an even source, so pairing the whole list pairs each block
          kblocks[b] = ops.paired ? NearBlock{b * max_ns / 2, cnt_s / 2, b * max_nt, cnt_t} : blocks[b];
        }
        e = cudaMemcpyAsync(buf + o_b, kblocks.data(), nb * sizeof(NearBlock), cudaMemcpyHostToDevice, st);
        float best_ms = 1e30f;
        int best = table[c];
        for (int split = 1; split <= 8 && e == cudaSuccess; split *= 2) {
          std::array<int, SCTLGPU_NEAR_CLASSES> t1;
          t1.fill(split);
          std::vector<NearItem> items;
          build_items(blocks, t1, ops.T, items);
          if ((int64_t)items.size() > nb_max * 64) continue;
          float ms = 0;
          e = time_items(ops, sms, items, (NearItem*)(buf + o_i), (const NearBlock*)(buf + o_b), buf + o_t,
                         buf + o_r, (double*)(buf + o_o), counter, status, bb, st, &ms);
          if (e == cudaSuccess && ms < best_ms) {
            best_ms = ms;
            best = split;
          }
        }
        table[c] = best;
      }
      cudaStreamSynchronize(st);
      cudaFree(buf);
    }
    cudaStreamDestroy(st);
    if (e != cudaSuccess) return runtime_record(e);
  }
  (void)mode;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[dkey] = table;
  return SCTLGPU_OK;
}

cudaError_t enqueue(sctlgpu_near_plan_s* P, const void* const* k, unsigned flags, cudaStream_t s) {
  const void *r_trg = k[0], *r_src = k[1], *n_src = k[2], *v_src = k[3], *w_src = k[4];
  void* v_out = const_cast<void*>(k[5]);
  cudaError_t e = cudaMemsetAsync(P->d_counter, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  if (P->imode == NEAR_MXLO || P->imode == NEAR_MXDF) {
    e = compute_bbox(s, P->nt, (const double*)r_trg, P->ns, (const double*)r_src, P->d_bbox);
    if (e != cudaSuccess) return e;
  }
  if (P->ops.paired && !P->shared_pairs)
    e = P->ops.pack_blocks(s, P->nblk, P->d_blocks, P->d_src_blocks, P->n_pairs, r_src, P->ND ? n_src : nullptr,
                           v_src, w_src, P->d_recs, P->d_bbox, P->sms);
  else
    e = P->ops.pack(s, P->ns, r_src, P->ND ? n_src : nullptr, v_src, w_src, P->d_recs, P->d_bbox, P->sms);
  if (e != cudaSuccess) return e;
  const bool accumulate = flags & SCTLGPU_ACCUMULATE;
  if ((P->has_map || P->d_tidx) && !accumulate) {
    e = cudaMemsetAsync(v_out, 0, (size_t)P->n_out * P->K1 * sizeof(double), s);
    if (e != cudaSuccess) return e;
  }
  NearParams p{};
  p.items = P->d_items;
  p.n_items = P->n_items;
  p.blocks = P->d_blocks;
  p.r_trg = r_trg;
  p.recs = P->d_recs;
  p.map = P->d_map;
  p.tidx = P->d_tidx;
  p.out = (double*)v_out;
  p.out_f = (float*)v_out;
  p.counter = P->d_counter;
  p.status = P->d_status;
  p.bbox = P->d_bbox;
  p.accumulate = accumulate ? 1 : 0;
  if (P->n_items == 0) return cudaSuccess;
  return P->ops.launch(s, (unsigned)(P->sms * P->ops.occ), p);
}

void free_plan(sctlgpu_near_plan_s* P) {
  if (P->exec) cudaGraphExecDestroy(P->exec);
  if (P->graph) cudaGraphDestroy(P->graph);
  if (P->cap) cudaStreamDestroy(P->cap);
  cudaFree(P->d_items);
  cudaFree(P->d_blocks);
  cudaFree(P->d_src_blocks);
  cudaFree(P->d_map);
  cudaFree(P->d_tidx);
  cudaFree(P->d_scratch);
  delete P;
}

// `kernel`: the public id (split-table tuning); `ker`: the kernel evaluated (== kernel, or an
// internal variant); nd, td: normal and target dimensions.
int plan_create(sctlgpu_near_plan* out, int kernel, int ker, int nd, int td, int mode, int digits, int64_t nblk,
                const sctlgpu_block* blocks, int64_t ns, int64_t nt, const int64_t* trg_index, int64_t n_index,
                const int64_t* trg_map, int64_t n_out) {
  if (mode != SCTLGPU_F64 && mode != SCTLGPU_F32 && mode != SCTLGPU_MIXED) return SCTLGPU_ERR_INVALID_MODE;
  if (nblk < 0 || ns < 0 || nt < 0 || nblk > INT32_MAX) return SCTLGPU_ERR_INVALID_SIZE;
  if (nblk > 0 && !blocks) return SCTLGPU_ERR_NULL_POINTER;
  if ((trg_map || trg_index) && mode == SCTLGPU_F32) return SCTLGPU_ERR_INVALID_ARGUMENT;  // scattered outputs are FP64
  if (trg_index && n_index < 0) return SCTLGPU_ERR_INVALID_SIZE;
  const int64_t nlist = trg_index ? n_index : nt;  // block target ranges index this list
  int64_t pairs = 0;
  std::vector<NearBlock> hb((size_t)nblk);
  for (int64_t b = 0; b < nblk; ++b) {
    const sctlgpu_block& B = blocks[b];
    if (B.src_count < 0 || B.trg_count < 0 || B.src_begin < 0 || B.trg_begin < 0 || B.src_begin + B.src_count > ns ||
        B.trg_begin + B.trg_count > nlist || B.trg_count > INT32_MAX)
      return SCTLGPU_ERR_INVALID_SIZE;
    hb[b] = {B.src_begin, B.src_count, B.trg_begin, B.trg_count};
    pairs += B.src_count * B.trg_count;
  }
  if (trg_map) {
    if (n_out < 0) return SCTLGPU_ERR_INVALID_SIZE;
    for (int64_t t = 0; t < nlist; ++t)
      if (trg_map[t] < 0 || trg_map[t] >= n_out) return SCTLGPU_ERR_INVALID_ARGUMENT;
  }
  if (trg_index)
    for (int64_t k = 0; k < n_index; ++k)
      if (trg_index[k] < 0 || trg_index[k] >= nt) return SCTLGPU_ERR_INVALID_ARGUMENT;
  int dev;
  unsigned* status;
  int sms;
  int rc = runtime_device(&dev, &status, &sms);
  if (rc) return rc;

  auto* P = new sctlgpu_near_plan_s();
  P->kernel = kernel;
  P->mode = mode;
  P->digits = digits;
  P->imode = imode_for(mode, runtime_effective_digits(mode, digits), &P->newton);
  P->ops = ops_for(ker, P->imode, P->newton);
  P->K1 = td;
  P->ND = nd;
  P->nblk = nblk;
  P->ns = ns;
  P->nt = nt;
  P->n_out = trg_map ? n_out : nt;  // outputs: mapped, or one per target (direct or through the index list)
  P->has_map = trg_map != nullptr;
  P->device = dev;
  P->sms = sms;
  P->pairs = pairs;

  std::array<int, SCTLGPU_NEAR_CLASSES> table;
  rc = autotune(kernel, P->imode, P->newton, ker == kernel ? P->ops : ops_for(kernel, P->imode, P->newton), sms, mode,
                table);
  if (rc) {
    delete P;
    return rc;
  }
  std::vector<NearItem> items;
  build_items(hb, table, P->ops.T, items);  // size classes and costs by source counts
  P->n_items = (int64_t)items.size();
  std::vector<NearBlock> hk = hb;  // the kernel's table
  if (P->ops.paired) {
    // Blocks that all start on an even source and end on an even one (or at the
    // list's end) share one pairing of the whole list (source 2j with 2j + 1),
    // packed once; otherwise every block's sources are paired on their own.
    bool aligned = true;
    for (const NearBlock& b : hb) aligned = aligned && b.s0 % 2 == 0 && (b.ns % 2 == 0 || b.s0 + b.ns == ns);
    P->shared_pairs = aligned;
    int64_t off = 0;
    for (size_t b = 0; b < hb.size(); ++b) {
      const int64_t np = (hb[b].ns + 1) / 2;
      hk[b] = {aligned ? hb[b].s0 / 2 : off, np, hb[b].t0, hb[b].nt};
      off += np;
    }
    P->n_pairs = aligned ? (ns + 1) / 2 : off;
  }

  cudaError_t e = cudaSuccess;
  const size_t rec_bytes = ((size_t)(P->ops.paired ? P->n_pairs : ns) * P->ops.rec_bytes + 255) / 256 * 256;
  do {
    if ((e = cudaStreamCreateWithFlags(&P->cap, cudaStreamNonBlocking))) break;
    if ((e = cudaMalloc(&P->d_items, std::max<size_t>(1, items.size()) * sizeof(NearItem)))) break;
    if ((e = cudaMalloc(&P->d_blocks, std::max<size_t>(1, hb.size()) * sizeof(NearBlock)))) break;
    if ((e = cudaMalloc(&P->d_scratch, rec_bytes + 512))) break;
    P->d_recs = P->d_scratch;
    P->d_bbox = (BBox*)(P->d_scratch + rec_bytes);
    P->d_counter = (unsigned*)(P->d_scratch + rec_bytes + 256);
    P->d_status = P->d_counter + 1;
    if (!items.empty() &&
        (e = cudaMemcpy(P->d_items, items.data(), items.size() * sizeof(NearItem), cudaMemcpyHostToDevice)))
      break;
    if (!hk.empty() && (e = cudaMemcpy(P->d_blocks, hk.data(), hk.size() * sizeof(NearBlock), cudaMemcpyHostToDevice)))
      break;
    if (P->ops.paired && !P->shared_pairs) {
      if ((e = cudaMalloc(&P->d_src_blocks, std::max<size_t>(1, hb.size()) * sizeof(NearBlock)))) break;
      if (!hb.empty() &&
          (e = cudaMemcpy(P->d_src_blocks, hb.data(), hb.size() * sizeof(NearBlock), cudaMemcpyHostToDevice)))
        break;
    }
    if ((e = cudaMemset(P->d_status, 0, sizeof(unsigned)))) break;
    if (trg_map) {
      if ((e = cudaMalloc(&P->d_map, std::max<int64_t>(1, nlist) * sizeof(int64_t)))) break;
      if (nlist && (e = cudaMemcpy(P->d_map, trg_map, nlist * sizeof(int64_t), cudaMemcpyHostToDevice))) break;
    }
    if (trg_index) {
      if ((e = cudaMalloc(&P->d_tidx, std::max<int64_t>(1, n_index) * sizeof(int64_t)))) break;
      if (n_index && (e = cudaMemcpy(P->d_tidx, trg_index, n_index * sizeof(int64_t), cudaMemcpyHostToDevice))) break;
      P->n_index = n_index;
    }
  } while (0);
  if (e != cudaSuccess) {
    free_plan(P);
    return runtime_record(e);
  }
  *out = P;
  return SCTLGPU_OK;
}

}  // namespace

extern "C" {

int sctlgpu_near_autotune(int kernel, int mode, int digits, int* splits) {
  int nd, sd, td;
  if (kernel < 0 || kernel > SCTLGPU_STOKES3D_DXU) return SCTLGPU_ERR_INVALID_KERNEL;  // the four hot-path kernels
  if (sctlgpu_kernel_dims(kernel, nullptr, &nd, &sd, &td) != SCTLGPU_OK) return SCTLGPU_ERR_INVALID_KERNEL;
  if (mode != SCTLGPU_F64 && mode != SCTLGPU_F32 && mode != SCTLGPU_MIXED) return SCTLGPU_ERR_INVALID_MODE;
  int dev;
  unsigned* status;
  int sms;
  int rc = runtime_device(&dev, &status, &sms);
  if (rc) return rc;
  int newton;
  const int imode = imode_for(mode, runtime_effective_digits(mode, digits), &newton);
  const NearOps ops = ops_for(kernel, imode, newton);
  std::array<int, SCTLGPU_NEAR_CLASSES> table;
  rc = autotune(kernel, imode, newton, ops, sms, mode, table);
  if (rc) return rc;
  if (splits)
    for (int i = 0; i < SCTLGPU_NEAR_CLASSES; ++i) splits[i] = table[i];
  return SCTLGPU_OK;
}

int sctlgpu_near_plan_create(sctlgpu_near_plan* out, int kernel, int mode, int digits, int64_t nblk,
                             const sctlgpu_block* blocks, int64_t ns, int64_t nt, const int64_t* trg_map,
                             int64_t n_out) {
  return sctlgpu_near_plan_create_indexed(out, kernel, mode, digits, nblk, blocks, ns, nt, nullptr, 0, trg_map, n_out);
}

int sctlgpu_near_plan_create_indexed(sctlgpu_near_plan* out, int kernel, int mode, int digits, int64_t nblk,
                                     const sctlgpu_block* blocks, int64_t ns, int64_t nt, const int64_t* trg_index,
                                     int64_t n_index, const int64_t* trg_map, int64_t n_out) {
  if (!out) return SCTLGPU_ERR_NULL_POINTER;
  *out = nullptr;
  int nd, sd, td;
  if (kernel < 0 || kernel > SCTLGPU_STOKES3D_DXU) return SCTLGPU_ERR_INVALID_KERNEL;  // the four hot-path kernels
  if (sctlgpu_kernel_dims(kernel, nullptr, &nd, &sd, &td) != SCTLGPU_OK) return SCTLGPU_ERR_INVALID_KERNEL;
  return plan_create(out, kernel, kernel, nd, td, mode, digits, nblk, blocks, ns, nt, trg_index, n_index, trg_map,
                     n_out);
}

}  // extern "C"

namespace sctlgpu {

int near_plan_create_sym(::sctlgpu_near_plan_s** out, int mode, int digits, int64_t nblk, const void* blocks,
                         int64_t ns, int64_t nt, const int64_t* trg_map, int64_t n_out) {
  if (!out) return SCTLGPU_ERR_NULL_POINTER;
  *out = nullptr;
  if (mode != SCTLGPU_MIXED && mode != SCTLGPU_F64) return SCTLGPU_ERR_INVALID_MODE;
  // split table tuned for the Stokes double layer (the same targets per thread and a similar cost)
  return plan_create(out, SCTLGPU_STOKES3D_DXU, KER_SDXU_SYM, 3, 3, mode, digits, nblk,
                     static_cast<const sctlgpu_block*>(blocks), ns, nt, nullptr, 0, trg_map, n_out);
}

}  // namespace sctlgpu

extern "C" {

int sctlgpu_near_plan_execute(sctlgpu_near_plan P, const void* r_trg, const void* r_src, const void* n_src,
                              const void* v_src, const void* w_src, void* v_out, unsigned flags, void* stream) {
  if (!P) return SCTLGPU_ERR_NULL_POINTER;
  if (flags & ~(unsigned)(SCTLGPU_ACCUMULATE | SCTLGPU_DEVICE_PTRS)) return SCTLGPU_ERR_INVALID_ARGUMENT;
  if ((P->nt > 0 && (!r_trg || !v_out)) || (P->ns > 0 && (!r_src || !v_src || (P->ND && !n_src))))
    return SCTLGPU_ERR_NULL_POINTER;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev != P->device) return SCTLGPU_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(P->mu);
  const void* key[6] = {r_trg, r_src, n_src, v_src, w_src, v_out};
  const unsigned kf = flags & SCTLGPU_ACCUMULATE;
  bool same = P->exec && kf == P->key_flags;
  for (int i = 0; i < 6 && same; ++i) same = key[i] == P->key[i];
  cudaError_t e = cudaSuccess;
  if (!same) {
    const int64_t before = g_launches.load();
    cudaGraph_t g = nullptr;
    e = cudaStreamBeginCapture(P->cap, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return runtime_record(e);
    cudaError_t e1 = enqueue(P, key, kf, P->cap);
    e = cudaStreamEndCapture(P->cap, &g);
    const int captured = (int)(g_launches.load() - before);
    g_launches.fetch_sub(captured);
    if (e1 != cudaSuccess || e != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return runtime_record(e1 != cudaSuccess ? e1 : e);
    }
    bool updated = false;
    if (P->exec) {
      cudaGraphExecUpdateResultInfo info;
      updated = cudaGraphExecUpdate(P->exec, g, &info) == cudaSuccess;
      if (!updated) {
        (void)cudaGetLastError();
        cudaGraphExecDestroy(P->exec);
        P->exec = nullptr;
      }
    }
    if (!updated) {
      e = cudaGraphInstantiate(&P->exec, g, 0);
      if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        P->exec = nullptr;
        return runtime_record(e);
      }
    }
    if (P->graph) cudaGraphDestroy(P->graph);
    P->graph = g;
    for (int i = 0; i < 6; ++i) P->key[i] = key[i];
    P->key_flags = kf;
    P->graph_kernels = captured;
  }
  e = cudaGraphLaunch(P->exec, (cudaStream_t)stream);
  if (e != cudaSuccess) return runtime_record(e);
  g_launches.fetch_add(P->graph_kernels);
  return SCTLGPU_OK;
}

int sctlgpu_near_plan_info(sctlgpu_near_plan P, int64_t* n_items, int64_t* interactions, int* graph_kernels) {
  if (!P) return SCTLGPU_ERR_NULL_POINTER;
  if (n_items) *n_items = P->n_items;
  if (interactions) *interactions = P->pairs;
  if (graph_kernels) *graph_kernels = P->graph_kernels;
  return SCTLGPU_OK;
}

int sctlgpu_near_plan_status(sctlgpu_near_plan P, void* stream) {
  if (!P) return SCTLGPU_ERR_NULL_POINTER;
  unsigned h = 0;
  cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e == cudaSuccess) e = cudaMemcpy(&h, P->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return runtime_record(e);
  if (h) {
    cudaMemset(P->d_status, 0, sizeof(unsigned));
    return SCTLGPU_ERR_DEVICE_TIMEOUT;
  }
  return SCTLGPU_OK;
}

int sctlgpu_near_plan_destroy(sctlgpu_near_plan P) {
  if (!P) return SCTLGPU_OK;
  // The plan's graph may still be running on a caller's stream: wait for the
  // device before its buffers are released.
  cudaDeviceSynchronize();
  free_plan(P);
  return SCTLGPU_OK;
}

}  // extern "C"
