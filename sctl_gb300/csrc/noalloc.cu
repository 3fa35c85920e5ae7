// sctlgpu_eval_mixed_noalloc: the mixed-precision direct sum for callers that
// cannot allocate device memory.
//
// Who needs it: code that runs where cudaMalloc / cudaMallocAsync are not
// allowed or not safe -- a host that has handed the device's memory budget to
// another allocator (a caching pool it must not bypass), a library called
// from inside a region its caller has pinned down (no new allocations after
// start-up), or a hard real-time loop that must not risk an allocation stall
// or an out-of-memory failure mid-run.  Every call of this entry point uses the
// same fixed scratch area instead: a file-scope __device__ array of
// SCTLGPU_NOALLOC_SCRATCH_BYTES that each GPU loading this library holds until
// the process exits.  The caller still provides the device input and output
// arrays.
//
// Consequences for the caller:
//   - the first call on a device resolves the array's device address
//     (cudaGetSymbolAddress) and must therefore run before any stream capture;
//   - all calls share the one array, so calls whose work overlaps on the GPU
//     (different streams, or different host threads without ordering) race on
//     it and produce wrong results; order them on one stream;
//   - problems whose packed sources and partial sums exceed the array are
//     rejected with SCTLGPU_ERR_TOO_LARGE before anything is launched.
#include <atomic>
#include <mutex>

#include "../../include/sctlgpu.h"
#include "launch_direct.cuh"

namespace sctlgpu {
namespace {

constexpr size_t kNoAllocBytes = (size_t)SCTLGPU_NOALLOC_SCRATCH_BYTES;
constexpr size_t kHeaderBytes = 512;  // [0,256): bounding box, [256,260): device status word

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxNoAllocDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kMaxNoAllocDevices] = {};

// Device address of the scratch array on the current device (resolved once per device).
cudaError_t noalloc_scratch(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxNoAllocDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return cudaSuccess;
}

struct NoAllocCall {
  EvalCall c;
  char* scratch;
  int dev = 0;
  bool too_large = false;
};

template <int KER, int MODE, int NEWTON>
cudaError_t run_noalloc(NoAllocCall& a) {
  using RecT = Rec<KER, MODE>;
  using Cfg = TileCfg<KER, MODE>;
  constexpr int K1 = KDims<KER>::K1;
  using Real = double;
  const EvalCall& c = a.c;
  cudaStream_t st = c.stream;

  const size_t smem = 2 * Cfg::S * sizeof(RecT) + 2 * sizeof(uint64_t);
  // Resident CTAs per SM, per device (devices of one process may differ).
  static std::atomic<int> occ_by_dev[kMaxNoAllocDevices] = {};
  int occ = occ_by_dev[a.dev].load(std::memory_order_relaxed);
  if (occ <= 0) {
    if (smem > 48 * 1024)
      SCTLGPU_TRY(cudaFuncSetAttribute(direct_sum_kernel<KER, MODE, NEWTON>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    SCTLGPU_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, direct_sum_kernel<KER, MODE, NEWTON>,
                                                              Cfg::THREADS, smem));
    occ = occ > 0 ? occ : 1;
    occ_by_dev[a.dev].store(occ, std::memory_order_relaxed);
  }

  const int64_t per_cta = (int64_t)Cfg::THREADS * Cfg::T;
  const int64_t tblocks = (c.nt + per_cta - 1) / per_cta;
  const size_t rec_bytes = ((size_t)c.ns * sizeof(RecT) + 255) / 256 * 256;
  auto need = [&](int nsplit) { return kHeaderBytes + rec_bytes + (size_t)nsplit * (size_t)c.nt * K1 * sizeof(double); };
  int nsplit0 = choose_nsplit(tblocks, c.ns, Cfg::S, c.sms * occ);
  while (nsplit0 > 1 && need(nsplit0) > kNoAllocBytes) --nsplit0;
  int64_t chunk = (c.ns + nsplit0 - 1) / nsplit0;
  chunk = ((chunk + Cfg::S - 1) / Cfg::S) * Cfg::S;
  const int nsplit = (int)((c.ns + chunk - 1) / chunk);
  if (need(nsplit) > kNoAllocBytes) {
    a.too_large = true;
    return cudaSuccess;
  }

  BBox* bb = reinterpret_cast<BBox*>(a.scratch);
  unsigned* status = reinterpret_cast<unsigned*>(a.scratch + 256);
  RecT* recs = reinterpret_cast<RecT*>(a.scratch + kHeaderBytes);
  double* partial = reinterpret_cast<double*>(a.scratch + kHeaderBytes + rec_bytes);

  // The array keeps the previous call's contents: the status word must start
  // at zero and the box must start empty; records and partials are fully
  // overwritten below before they are read.
  SCTLGPU_TRY(cudaMemsetAsync(status, 0, sizeof(unsigned), st));
  if (MODE == MODE_MXLO)
    SCTLGPU_TRY(compute_bbox(st, c.nt, (const double*)c.r_trg, c.ns, (const double*)c.r_src, bb));
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
  p.status = status;
  direct_sum_kernel<KER, MODE, NEWTON><<<dim3((unsigned)tblocks, (unsigned)nsplit), Cfg::THREADS, smem, st>>>(p);
  g_launches.fetch_add(1, std::memory_order_relaxed);
  const int64_t nout = c.nt * K1;
  reduce_partials_kernel<Real><<<grid_for(nout, 256, c.sms), 256, 0, st>>>(nout, nsplit, partial, scale_of<KER>(),
                                                                            c.accumulate ? 1 : 0, (Real*)c.v_trg);
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return cudaGetLastError();
}

// The double-float arithmetic of sctlgpu_eval (pair records on the packed FP32
// pipe, direct_pk.cuh) in the same fixed scratch layout.
template <int KER>
cudaError_t run_noalloc_pk(NoAllocCall& a) {
  using RecT = RecPk<KER>;
  using Cfg = TileCfgPk<KER>;
  constexpr int K1 = KDims<KER>::K1;
  const EvalCall& c = a.c;
  cudaStream_t st = c.stream;

  const size_t smem = 2 * Cfg::S * sizeof(RecT) + 2 * sizeof(uint64_t);
  static std::atomic<int> occ_by_dev[kMaxNoAllocDevices] = {};
  int occ = occ_by_dev[a.dev].load(std::memory_order_relaxed);
  if (occ <= 0) {
    if (smem > 48 * 1024)
      SCTLGPU_TRY(cudaFuncSetAttribute(direct_sum_pk_kernel<KER>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
    SCTLGPU_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, direct_sum_pk_kernel<KER>, Cfg::THREADS, smem));
    occ = occ > 0 ? occ : 1;
    occ_by_dev[a.dev].store(occ, std::memory_order_relaxed);
  }

  const int64_t npairs = (c.ns + 1) / 2;
  const int64_t per_cta = (int64_t)Cfg::THREADS * Cfg::T;
  const int64_t tblocks = (c.nt + per_cta - 1) / per_cta;
  const size_t rec_bytes = ((size_t)npairs * sizeof(RecT) + 255) / 256 * 256;
  auto need = [&](int nsplit) { return kHeaderBytes + rec_bytes + (size_t)nsplit * (size_t)c.nt * K1 * sizeof(double); };
  int nsplit0 = choose_nsplit(tblocks, npairs, Cfg::S, c.sms * occ);
  while (nsplit0 > 1 && need(nsplit0) > kNoAllocBytes) --nsplit0;
  int64_t chunk = (npairs + nsplit0 - 1) / nsplit0;
  chunk = ((chunk + Cfg::S - 1) / Cfg::S) * Cfg::S;
  const int nsplit = (int)((npairs + chunk - 1) / chunk);
  if (need(nsplit) > kNoAllocBytes) {
    a.too_large = true;
    return cudaSuccess;
  }

  BBox* bb = reinterpret_cast<BBox*>(a.scratch);
  unsigned* status = reinterpret_cast<unsigned*>(a.scratch + 256);
  RecT* recs = reinterpret_cast<RecT*>(a.scratch + kHeaderBytes);
  double* partial = reinterpret_cast<double*>(a.scratch + kHeaderBytes + rec_bytes);

  // The array keeps the previous call's contents: status word and box are
  // reset; records and partials are fully overwritten before they are read.
  SCTLGPU_TRY(cudaMemsetAsync(status, 0, sizeof(unsigned), st));
  SCTLGPU_TRY(compute_bbox(st, c.nt, (const double*)c.r_trg, c.ns, (const double*)c.r_src, bb));
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
  p.status = status;
  direct_sum_pk_kernel<KER><<<dim3((unsigned)tblocks, (unsigned)nsplit), Cfg::THREADS, smem, st>>>(p);
  g_launches.fetch_add(1, std::memory_order_relaxed);
  const int64_t nout = c.nt * K1;
  reduce_partials_kernel<double><<<grid_for(nout, 256, c.sms), 256, 0, st>>>(nout, nsplit, partial, scale_of<KER>(),
                                                                              c.accumulate ? 1 : 0, (double*)c.v_trg);
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return cudaGetLastError();
}

template <int KER>
cudaError_t noalloc_kernel(NoAllocCall& a, int digits) {
  // The routing of SCTLGPU_MIXED in sctlgpu_eval, from the same rule
  // (runtime_mixed_arith) and the same Newton schedule (runtime_steps): FP32
  // arithmetic on split coordinates, double-float, or FP64.
  const int steps = runtime_steps(SCTLGPU_MIXED, digits);
  switch (runtime_mixed_arith(digits)) {
    case MIXED_ARITH_F32:
      return steps <= 0 ? run_noalloc<KER, MODE_MXLO, 0>(a) : run_noalloc<KER, MODE_MXLO, 1>(a);
    case MIXED_ARITH_DF:
      return run_noalloc_pk<KER>(a);
    default:
      switch (steps) {
        case 0: return run_noalloc<KER, MODE_F64, 0>(a);
        case 1: return run_noalloc<KER, MODE_F64, 1>(a);
        case 2: return run_noalloc<KER, MODE_F64, 2>(a);
        default: return run_noalloc<KER, MODE_F64, 3>(a);
      }
  }
}

}  // namespace
}  // namespace sctlgpu

using namespace sctlgpu;

extern "C" int sctlgpu_eval_mixed_noalloc(int kernel, int digits, int64_t nt, const double* r_trg, int64_t ns,
                                          const double* r_src, const double* n_src, const double* v_src,
                                          double* v_trg, unsigned flags, void* stream) {
  int nd = 0, sd = 0, td = 0;
  if (kernel < 0 || kernel > SCTLGPU_STOKES3D_DXU) return SCTLGPU_ERR_INVALID_KERNEL;  // the four hot-path kernels
  if (sctlgpu_kernel_dims(kernel, nullptr, &nd, &sd, &td) != SCTLGPU_OK) return SCTLGPU_ERR_INVALID_KERNEL;
  if (nt < 0 || ns < 0 || nt > ((int64_t)1 << 40) || ns > ((int64_t)1 << 40)) return SCTLGPU_ERR_INVALID_SIZE;
  if (flags & ~(unsigned)(SCTLGPU_ACCUMULATE | SCTLGPU_DEVICE_PTRS)) return SCTLGPU_ERR_INVALID_ARGUMENT;
  if ((nt > 0 && (!r_trg || !v_trg)) || (ns > 0 && (!r_src || !v_src || (nd && !n_src))))
    return SCTLGPU_ERR_NULL_POINTER;
  const int d = runtime_effective_digits(SCTLGPU_MIXED, digits);
  if (nt == 0) return SCTLGPU_OK;
  cudaStream_t st = (cudaStream_t)stream;
  if (ns == 0) {  // no sources: v_trg = 0 (or unchanged when accumulating); synchronous like every call
    if (flags & SCTLGPU_ACCUMULATE) return SCTLGPU_OK;
    cudaError_t e = cudaMemsetAsync(v_trg, 0, (size_t)nt * td * sizeof(double), st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return runtime_record(e);
  }
  void* scratch = nullptr;
  cudaError_t ce = noalloc_scratch(&scratch);
  if (ce != cudaSuccess) return runtime_record(ce);
  int dev = 0, sms = 0;
  if ((ce = cudaGetDevice(&dev)) != cudaSuccess ||
      (ce = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
    return runtime_record(ce);

  NoAllocCall a;
  a.scratch = (char*)scratch;
  a.dev = dev;
  a.c.kernel = kernel;
  a.c.nt = nt;
  a.c.ns = ns;
  a.c.r_trg = r_trg;
  a.c.r_src = r_src;
  a.c.n_src = nd ? n_src : nullptr;
  a.c.v_src = v_src;
  a.c.v_trg = v_trg;
  a.c.accumulate = (flags & SCTLGPU_ACCUMULATE) != 0;
  a.c.stream = st;
  a.c.status = nullptr;
  a.c.sms = sms > 0 ? sms : 1;
  a.c.timing = nullptr;
  cudaError_t e;
  switch (kernel) {
    case SCTLGPU_LAPLACE3D_FXU: e = noalloc_kernel<KER_LFXU>(a, d); break;
    case SCTLGPU_LAPLACE3D_DXU: e = noalloc_kernel<KER_LDXU>(a, d); break;
    case SCTLGPU_STOKES3D_FXU: e = noalloc_kernel<KER_SFXU>(a, d); break;
    default: e = noalloc_kernel<KER_SDXU>(a, d); break;
  }
  if (a.too_large) return SCTLGPU_ERR_TOO_LARGE;
  if (e != cudaSuccess) return runtime_record(e);
  // Synchronous: wait for the stream, then report a device-side wait timeout
  // recorded in the scratch header (copied into a local, not a new buffer).
  unsigned h = 0;
  if ((e = cudaMemcpyAsync(&h, (char*)scratch + 256, sizeof(unsigned), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return runtime_record(e);
  return h ? SCTLGPU_ERR_DEVICE_TIMEOUT : SCTLGPU_OK;
}
