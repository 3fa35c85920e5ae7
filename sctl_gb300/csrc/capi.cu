// extern "C" boundary of libsctlgpu (declarations and reference citations in
// include/sctlgpu.h): argument checks, digits -> (mode, Newton steps), host
// or device pointers, per-device status word, launch counting and timing.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/sctlgpu.h"
#include "launch.h"

namespace sctlgpu {

std::atomic<int64_t> g_launches{0};

namespace {

constexpr int kMaxDevices = 64;

// Seed accuracy of rsqrt.approx on sm_103a in decimal digits, less log10(5)
// so that r^-5 (Stokes3D_DxU) still meets `digits` after the schedule:
// f32: relative error <= 2^-22.28 -> 6.71 - 0.70; f64 (MUFU.RSQ64H works on
// the high word): <= 2^-20.1 -> 6.05 - 0.70.  Measured on GB300 by
// tests/test_gpu_rsqrt.py.  The reference uses 4.2144 for AVX-512 rsqrt14 and
// 3.4363 for 12-bit rsqrtps / NEON vrsqrte (intrin-wrapper.hpp:1562,1566,3384).
constexpr double kSeedDigitsF32 = 6.01;
constexpr double kSeedDigitsF64 = 5.35;

thread_local std::string tl_cuda_error;
thread_local Timing tl_timing;
thread_local int tl_timing_device = -1;
thread_local cudaStream_t tl_streams[kMaxDevices] = {};
std::atomic<int> g_timing_enabled{0};

std::mutex g_dev_mu;
unsigned* g_status[kMaxDevices] = {};
int g_sms[kMaxDevices] = {};

int record(cudaError_t e) {
  if (e == cudaSuccess) return SCTLGPU_OK;
  tl_cuda_error = cudaGetErrorString(e);
  (void)cudaGetLastError();  // clear a sticky-free error so later calls start clean
  return e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver ? SCTLGPU_ERR_NO_DEVICE : SCTLGPU_ERR_CUDA;
}

// Per-device state: status word, SM count, mem-pool retention.
int device_state(int* dev_out, unsigned** status, int* sms) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return record(e);
  if (dev < 0 || dev >= kMaxDevices) return SCTLGPU_ERR_NO_DEVICE;
  std::lock_guard<std::mutex> lk(g_dev_mu);
  if (!g_status[dev]) {
    unsigned* p = nullptr;
    if ((e = cudaMalloc(&p, 256)) != cudaSuccess) return record(e);
    if ((e = cudaMemset(p, 0, 256)) != cudaSuccess) return record(e);
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t thr = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    g_sms[dev] = n > 0 ? n : 1;
    g_status[dev] = p;
  }
  *dev_out = dev;
  *status = g_status[dev];
  *sms = g_sms[dev];
  return SCTLGPU_OK;
}

int thread_stream(int dev, cudaStream_t* s) {
  if (!tl_streams[dev]) {
    cudaError_t e = cudaStreamCreateWithFlags(&tl_streams[dev], cudaStreamNonBlocking);
    if (e != cudaSuccess) return record(e);
  }
  *s = tl_streams[dev];
  return SCTLGPU_OK;
}

Timing* thread_timing(int dev) {
  if (!g_timing_enabled.load()) {
    tl_timing.enabled = false;
    return &tl_timing;
  }
  if (tl_timing_device != dev) {
    if (tl_timing.start) {
      cudaEventDestroy(tl_timing.start);
      cudaEventDestroy(tl_timing.stop);
    }
    cudaEventCreate(&tl_timing.start);
    cudaEventCreate(&tl_timing.stop);
    tl_timing_device = dev;
  }
  tl_timing.enabled = true;
  tl_timing.recorded = false;
  return &tl_timing;
}

int dims(int kernel, int* nd, int* sd, int* td) {
  switch (kernel) {
    case SCTLGPU_LAPLACE3D_FXU: *nd = 0; *sd = 1; *td = 1; return SCTLGPU_OK;
    case SCTLGPU_LAPLACE3D_DXU: *nd = 3; *sd = 1; *td = 1; return SCTLGPU_OK;
    case SCTLGPU_STOKES3D_FXU: *nd = 0; *sd = 3; *td = 3; return SCTLGPU_OK;
    case SCTLGPU_STOKES3D_DXU: *nd = 3; *sd = 3; *td = 3; return SCTLGPU_OK;
    case SCTLGPU_LAPLACE3D_FXDU: *nd = 0; *sd = 1; *td = 3; return SCTLGPU_OK;
    case SCTLGPU_LAPLACE3D_FXD2U: *nd = 0; *sd = 1; *td = 9; return SCTLGPU_OK;
    case SCTLGPU_LAPLACE3D_DXDU: *nd = 3; *sd = 1; *td = 3; return SCTLGPU_OK;
    case SCTLGPU_BIOTSAVART3D_FXU: *nd = 0; *sd = 3; *td = 3; return SCTLGPU_OK;
    case SCTLGPU_BIOTSAVART3D_FXDU: *nd = 0; *sd = 3; *td = 9; return SCTLGPU_OK;
    case SCTLGPU_HELMHOLTZ3D_FXU: *nd = 0; *sd = 2; *td = 2; return SCTLGPU_OK;
    case SCTLGPU_HELMHOLTZ3D_DXU: *nd = 3; *sd = 2; *td = 2; return SCTLGPU_OK;
    case SCTLGPU_HELMHOLTZ3D_FXDU: *nd = 0; *sd = 2; *td = 6; return SCTLGPU_OK;
    case SCTLGPU_HELMHOLTZDIFF3D_FXDU: *nd = 0; *sd = 2; *td = 6; return SCTLGPU_OK;
    case SCTLGPU_STOKES3D_FXT: *nd = 0; *sd = 3; *td = 9; return SCTLGPU_OK;
    case SCTLGPU_STOKES3D_FSXU: *nd = 0; *sd = 4; *td = 3; return SCTLGPU_OK;
    case SCTLGPU_STOKES3D_FXUP: *nd = 0; *sd = 3; *td = 4; return SCTLGPU_OK;
    default: return SCTLGPU_ERR_INVALID_KERNEL;
  }
}

bool is_helmholtz(int kernel) { return kernel >= SCTLGPU_HELMHOLTZ3D_FXU && kernel <= SCTLGPU_HELMHOLTZDIFF3D_FXDU; }

// The context value a kernel reads (ctx points to a value of the call's real type).
int read_ctx(int kernel, int mode, const void* ctx, double* out) {
  *out = 0.0;
  if (!is_helmholtz(kernel)) return SCTLGPU_OK;
  if (!ctx) return SCTLGPU_ERR_NULL_POINTER;
  *out = mode == SCTLGPU_F32 ? (double)*(const float*)ctx : *(const double*)ctx;
  return SCTLGPU_OK;
}

// digits as the reference reads it: -1 (and >= 16) -> floor(SigBits*log10 2) (vec.txx:376).
int effective_digits(int mode, int digits) {
  const int full = mode == SCTLGPU_F32 ? 6 : 15;
  return (digits < 0 || digits >= 16) ? full : digits;
}

int newton_for(int digits, double seed_digits) {  // mylog2(floor(digits / seed)), intrin-wrapper.hpp:560-562
  long q = (long)std::floor((double)digits / seed_digits);
  int n = 0;
  while (q >= 1) {
    n++;
    q /= 2;
  }
  return n;
}

bool overflows(int64_t n, int64_t per) { return n > (int64_t)(INT64_MAX / 16) / (per > 0 ? per : 1); }

int check_common(int kernel, int mode, int64_t nt, const void* r_trg, int64_t ns, const void* r_src,
                 const void* n_src, int* nd, int* sd, int* td) {
  int rc = dims(kernel, nd, sd, td);
  if (rc) return rc;
  if (mode != SCTLGPU_F64 && mode != SCTLGPU_F32 && mode != SCTLGPU_MIXED) return SCTLGPU_ERR_INVALID_MODE;
  if (nt < 0 || ns < 0 || overflows(nt, 9) || overflows(ns, 9)) return SCTLGPU_ERR_INVALID_SIZE;
  if ((nt > 0 && !r_trg) || (ns > 0 && !r_src) || (ns > 0 && *nd && !n_src)) return SCTLGPU_ERR_NULL_POINTER;
  return SCTLGPU_OK;
}

// Reads and clears the device status word (after the stream has been synchronised).
int take_status(unsigned* status, cudaStream_t s) {
  unsigned h = 0;
  cudaError_t e = cudaMemcpyAsync(&h, status, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return record(e);
  if (h) {
    e = cudaMemsetAsync(status, 0, sizeof(unsigned), s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return record(e);
    return SCTLGPU_ERR_DEVICE_TIMEOUT;
  }
  return SCTLGPU_OK;
}

// Mixed mode: FP32 arithmetic up to 7 digits, double-float 8..kMixedDfMaxDigits,
// FP64 beyond: double-float coordinates carry 47 bits of the bounding box,
// which clustered points at 1e-5 separations turn into ~1e-11 relative error.
constexpr int kMixedDfMaxDigits = 11;

int steps_for(int mode, int d) {
  if (mode == SCTLGPU_F32 || (mode == SCTLGPU_MIXED && d <= 7)) return newton_for(d, kSeedDigitsF32);
  if (mode == SCTLGPU_MIXED && d <= kMixedDfMaxDigits) return 1;  // one double-float step
  return newton_for(d, kSeedDigitsF64);
}

// Arithmetic of SCTLGPU_MIXED at `d` digits (the one routing rule, shared with
// the allocation-free entry).
int mixed_arith(int d) {
  if (d <= 7) return MIXED_ARITH_F32;
  if (d <= kMixedDfMaxDigits) return MIXED_ARITH_DF;
  return MIXED_ARITH_F64;
}

cudaError_t run_eval(EvalCall& c, int mode, int d) {
  if (c.kernel > SCTLGPU_STOKES3D_DXU) {  // FP64 arithmetic also for SCTLGPU_MIXED
    if (mode == SCTLGPU_F32) return eval_ext_f32(c, steps_for(mode, d));
    return eval_ext_f64(c, steps_for(SCTLGPU_F64, d));
  }
  const int n = steps_for(mode, d);
  if (mode == SCTLGPU_F64) return eval_f64(c, n);
  if (mode == SCTLGPU_F32) return eval_f32(c, n);
  switch (mixed_arith(d)) {
    case MIXED_ARITH_F32: return eval_mixed_lo(c, n);
    case MIXED_ARITH_DF: return eval_mixed_df(c);
    default: return eval_f64(c, n);
  }
}

cudaError_t run_kmat(KmatCall& c, int mode, int d) {
  if (c.kernel > SCTLGPU_STOKES3D_DXU) {
    if (mode == SCTLGPU_F32) return kmat_ext_f32(c, steps_for(mode, d));
    return kmat_ext_f64(c, steps_for(SCTLGPU_F64, d));
  }
  // Mixed mode: double-float entries rounded to FP64 by integer operations (no FP64 pipe per
  // entry); beyond the double-float digits, the FP64 formula.
  if (mode == SCTLGPU_F32) return kmat_f32(c, steps_for(mode, d));
  if (mode == SCTLGPU_MIXED && d <= kMixedDfMaxDigits) return kmat_mixed_df(c);
  return kmat_f64(c, steps_for(SCTLGPU_F64, d));
}

}  // namespace

// Shared with the other entry-point files (near_plan.cu).
int runtime_device(int* dev, unsigned** status, int* sms) { return device_state(dev, status, sms); }
int runtime_record(cudaError_t e) { return record(e); }
int runtime_effective_digits(int mode, int digits) { return effective_digits(mode, digits); }
int runtime_steps(int mode, int digits) { return steps_for(mode, digits); }
int runtime_mixed_df_max_digits() { return kMixedDfMaxDigits; }
int runtime_mixed_arith(int digits) { return mixed_arith(digits); }

}  // namespace sctlgpu

using namespace sctlgpu;

extern "C" {

int sctlgpu_kernel_dims(int kernel, int* coord_dim, int* normal_dim, int* src_dim, int* trg_dim) {
  int nd, sd, td;
  const int rc = dims(kernel, &nd, &sd, &td);
  if (rc) return rc;
  if (coord_dim) *coord_dim = 3;
  if (normal_dim) *normal_dim = nd;
  if (src_dim) *src_dim = sd;
  if (trg_dim) *trg_dim = td;
  return SCTLGPU_OK;
}

double sctlgpu_scale_factor(int kernel) {
  const double pi = 3.14159265358979323846264338327950288;
  switch (kernel) {
    case SCTLGPU_LAPLACE3D_FXU:
    case SCTLGPU_LAPLACE3D_DXU: return 1.0 / (4.0 * pi);
    case SCTLGPU_STOKES3D_FXU: return 1.0 / (8.0 * pi);
    case SCTLGPU_STOKES3D_DXU: return 3.0 / (4.0 * pi);
    case SCTLGPU_LAPLACE3D_FXDU: return -1.0 / (4.0 * pi);        /* kernel_functions.hpp:88-90 */
    case SCTLGPU_LAPLACE3D_FXD2U: return 1.0 / (4.0 * pi);        /* :374-376 */
    case SCTLGPU_LAPLACE3D_DXDU: return 1.0 / (4.0 * pi);         /* :400-402 */
    case SCTLGPU_BIOTSAVART3D_FXU: return 1.0 / (4.0 * pi);       /* :424-426 */
    case SCTLGPU_BIOTSAVART3D_FXDU: return -1.0 / (4.0 * pi);     /* :459-461 */
    case SCTLGPU_HELMHOLTZ3D_FXU: return 1.0 / (4.0 * pi);        /* :499-501 */
    case SCTLGPU_HELMHOLTZ3D_DXU: return -1.0 / (4.0 * pi);       /* :537-539 */
    case SCTLGPU_HELMHOLTZ3D_FXDU: return 1.0 / (4.0 * pi);       /* :581-583 */
    case SCTLGPU_HELMHOLTZDIFF3D_FXDU: return 1.0 / (4.0 * pi);   /* :635-637 */
    case SCTLGPU_STOKES3D_FXT: return -3.0 / (4.0 * pi);          /* :228-230 */
    case SCTLGPU_STOKES3D_FSXU: return 1.0 / (8.0 * pi);          /* :272-274 */
    case SCTLGPU_STOKES3D_FXUP: return 1.0 / (8.0 * pi);          /* :333-335 */
    default: return 0.0;
  }
}

int sctlgpu_newton_steps(int mode, int digits) {
  if (mode != SCTLGPU_F64 && mode != SCTLGPU_F32 && mode != SCTLGPU_MIXED) return SCTLGPU_ERR_INVALID_MODE;
  return steps_for(mode, effective_digits(mode, digits));
}

int sctlgpu_eval(int kernel, int mode, int digits, int64_t nt, const void* r_trg, int64_t ns, const void* r_src,
                 const void* n_src, const void* v_src, void* v_trg, unsigned flags, void* stream) {
  return sctlgpu_eval_ctx(kernel, mode, digits, nt, r_trg, ns, r_src, n_src, v_src, v_trg, flags, nullptr, stream);
}

int sctlgpu_eval_ctx(int kernel, int mode, int digits, int64_t nt, const void* r_trg, int64_t ns, const void* r_src,
                     const void* n_src, const void* v_src, void* v_trg, unsigned flags, const void* ctx,
                     void* stream) {
  int nd, sd, td;
  int rc = check_common(kernel, mode, nt, r_trg, ns, r_src, n_src, &nd, &sd, &td);
  if (rc) return rc;
  double ctx_value;
  if ((rc = read_ctx(kernel, mode, ctx, &ctx_value))) return rc;
  if ((ns > 0 && !v_src) || (nt > 0 && !v_trg)) return SCTLGPU_ERR_NULL_POINTER;
  if (nt == 0) return SCTLGPU_OK;
  const bool dev_ptrs = flags & SCTLGPU_DEVICE_PTRS;
  const bool accumulate = flags & SCTLGPU_ACCUMULATE;
  const size_t real = mode == SCTLGPU_F32 ? sizeof(float) : sizeof(double);
  const size_t out_bytes = (size_t)nt * td * real;

  int dev;
  unsigned* status;
  int sms;
  if ((rc = device_state(&dev, &status, &sms))) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  if (!dev_ptrs && (rc = thread_stream(dev, &st))) return rc;

  if (ns == 0) {  // nothing to add; the reference leaves v_trg zeroed (or untouched when accumulating)
    if (accumulate) return SCTLGPU_OK;
    if (dev_ptrs) return record(cudaMemsetAsync(v_trg, 0, out_bytes, st));
    std::memset(v_trg, 0, out_bytes);
    return SCTLGPU_OK;
  }

  EvalCall c;
  c.kernel = kernel;
  c.ctx = ctx_value;
  c.nt = nt;
  c.ns = ns;
  c.accumulate = accumulate;
  c.stream = st;
  c.status = status;
  c.sms = sms;
  c.timing = thread_timing(dev);
  const int d = effective_digits(mode, digits);

  if (dev_ptrs) {
    c.r_trg = r_trg;
    c.r_src = r_src;
    c.n_src = nd ? n_src : nullptr;
    c.v_src = v_src;
    c.v_trg = v_trg;
    return record(run_eval(c, mode, d));
  }

  // Host pointers: stage through stream-ordered device buffers.
  const size_t b_trg = (size_t)nt * 3 * real, b_src = (size_t)ns * 3 * real, b_nrm = nd ? b_src : 0,
               b_den = (size_t)ns * sd * real;
  const size_t o_trg = 0, o_src = o_trg + (b_trg + 255) / 256 * 256, o_nrm = o_src + (b_src + 255) / 256 * 256,
               o_den = o_nrm + (b_nrm + 255) / 256 * 256, o_out = o_den + (b_den + 255) / 256 * 256,
               total = o_out + (out_bytes + 255) / 256 * 256;
  char* buf = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&buf, total, st);
  if (e != cudaSuccess) return record(e);
  do {
    if ((e = cudaMemcpyAsync(buf + o_trg, r_trg, b_trg, cudaMemcpyHostToDevice, st))) break;
    if ((e = cudaMemcpyAsync(buf + o_src, r_src, b_src, cudaMemcpyHostToDevice, st))) break;
    if (nd && (e = cudaMemcpyAsync(buf + o_nrm, n_src, b_nrm, cudaMemcpyHostToDevice, st))) break;
    if ((e = cudaMemcpyAsync(buf + o_den, v_src, b_den, cudaMemcpyHostToDevice, st))) break;
    if (accumulate && (e = cudaMemcpyAsync(buf + o_out, v_trg, out_bytes, cudaMemcpyHostToDevice, st))) break;
    c.r_trg = buf + o_trg;
    c.r_src = buf + o_src;
    c.n_src = nd ? buf + o_nrm : nullptr;
    c.v_src = buf + o_den;
    c.v_trg = buf + o_out;
    if ((e = run_eval(c, mode, d))) break;
    if ((e = cudaMemcpyAsync(v_trg, buf + o_out, out_bytes, cudaMemcpyDeviceToHost, st))) break;
  } while (0);
  cudaError_t e2 = cudaFreeAsync(buf, st);
  cudaError_t e3 = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = e2 != cudaSuccess ? e2 : e3;
  if (e != cudaSuccess) return record(e);
  return take_status(status, st);
}

int sctlgpu_kernel_matrix(int kernel, int mode, int digits, int64_t nt, const void* r_trg, int64_t ns,
                          const void* r_src, const void* n_src, void* M, unsigned flags, void* stream) {
  return sctlgpu_kernel_matrix_ctx(kernel, mode, digits, nt, r_trg, ns, r_src, n_src, M, flags, nullptr, stream);
}

int sctlgpu_kernel_matrix_ctx(int kernel, int mode, int digits, int64_t nt, const void* r_trg, int64_t ns,
                              const void* r_src, const void* n_src, void* M, unsigned flags, const void* ctx,
                              void* stream) {
  int nd, sd, td;
  int rc = check_common(kernel, mode, nt, r_trg, ns, r_src, n_src, &nd, &sd, &td);
  if (rc) return rc;
  double ctx_value;
  if ((rc = read_ctx(kernel, mode, ctx, &ctx_value))) return rc;
  if (nt == 0 || ns == 0) return SCTLGPU_OK;
  if (!M) return SCTLGPU_ERR_NULL_POINTER;
  if (overflows(nt * td, ns * sd)) return SCTLGPU_ERR_INVALID_SIZE;
  const bool dev_ptrs = flags & SCTLGPU_DEVICE_PTRS;
  const size_t real = mode == SCTLGPU_F32 ? sizeof(float) : sizeof(double);
  int dev;
  unsigned* status;
  int sms;
  if ((rc = device_state(&dev, &status, &sms))) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  if (!dev_ptrs && (rc = thread_stream(dev, &st))) return rc;

  KmatCall c;
  c.kernel = kernel;
  c.ctx = ctx_value;
  c.nt = nt;
  c.ns = ns;
  c.stream = st;
  c.sms = sms;
  c.timing = thread_timing(dev);
  const int d = effective_digits(mode, digits);
  if (dev_ptrs) {
    c.r_trg = r_trg;
    c.r_src = r_src;
    c.n_src = nd ? n_src : nullptr;
    c.M = M;
    return record(run_kmat(c, mode, d));
  }
  const size_t b_trg = (size_t)nt * 3 * real, b_src = (size_t)ns * 3 * real, b_nrm = nd ? b_src : 0,
               b_m = (size_t)ns * sd * (size_t)nt * td * real;
  const size_t o_trg = 0, o_src = (b_trg + 255) / 256 * 256, o_nrm = o_src + (b_src + 255) / 256 * 256,
               o_m = o_nrm + (b_nrm + 255) / 256 * 256, total = o_m + (b_m + 255) / 256 * 256;
  char* buf = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&buf, total, st);
  if (e != cudaSuccess) return record(e);
  do {
    if ((e = cudaMemcpyAsync(buf + o_trg, r_trg, b_trg, cudaMemcpyHostToDevice, st))) break;
    if ((e = cudaMemcpyAsync(buf + o_src, r_src, b_src, cudaMemcpyHostToDevice, st))) break;
    if (nd && (e = cudaMemcpyAsync(buf + o_nrm, n_src, b_nrm, cudaMemcpyHostToDevice, st))) break;
    c.r_trg = buf + o_trg;
    c.r_src = buf + o_src;
    c.n_src = nd ? buf + o_nrm : nullptr;
    c.M = buf + o_m;
    if ((e = run_kmat(c, mode, d))) break;
    if ((e = cudaMemcpyAsync(M, buf + o_m, b_m, cudaMemcpyDeviceToHost, st))) break;
  } while (0);
  cudaError_t e2 = cudaFreeAsync(buf, st);
  cudaError_t e3 = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = e2 != cudaSuccess ? e2 : e3;
  return record(e);
}

const char* sctlgpu_strerror(int status) {
  switch (status) {
    case SCTLGPU_OK: return "success";
    case SCTLGPU_ERR_INVALID_KERNEL: return "invalid kernel id";
    case SCTLGPU_ERR_INVALID_MODE: return "invalid arithmetic mode";
    case SCTLGPU_ERR_INVALID_SIZE: return "invalid or overflowing size";
    case SCTLGPU_ERR_NULL_POINTER: return "required array pointer is NULL";
    case SCTLGPU_ERR_CUDA: return "CUDA runtime error";
    case SCTLGPU_ERR_NO_DEVICE: return "no CUDA device available";
    case SCTLGPU_ERR_DEVICE_TIMEOUT: return "a bounded device-side wait timed out; results are invalid";
    case SCTLGPU_ERR_INVALID_ARGUMENT: return "invalid argument";
    case SCTLGPU_ERR_TOO_LARGE: return "request exceeds the entry point's fixed capacity";
    default: return "unknown status";
  }
}

const char* sctlgpu_last_cuda_error(void) { return tl_cuda_error.c_str(); }

int sctlgpu_device_status(void* stream) {
  int dev;
  unsigned* status;
  int sms;
  int rc = device_state(&dev, &status, &sms);
  if (rc) return rc;
  cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) return record(e);
  return take_status(status, (cudaStream_t)stream);
}

int sctlgpu_device_status_word(void* stream, unsigned* word) {
  if (!word) return SCTLGPU_ERR_NULL_POINTER;
  *word = 0;
  int dev;
  unsigned* status;
  int sms;
  int rc = device_state(&dev, &status, &sms);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(word, status, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(status, 0, sizeof(unsigned), s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? SCTLGPU_OK : record(e);
}

int64_t sctlgpu_launch_count(void) { return g_launches.load(); }

int sctlgpu_set_timing(int enable) {
  g_timing_enabled.store(enable ? 1 : 0);
  return SCTLGPU_OK;
}

double sctlgpu_last_kernel_ms(void) {
  if (!tl_timing.recorded) return -1.0;
  if (cudaEventSynchronize(tl_timing.stop) != cudaSuccess) return -1.0;
  float ms = -1.f;
  if (cudaEventElapsedTime(&ms, tl_timing.start, tl_timing.stop) != cudaSuccess) return -1.0;
  return (double)ms;
}

}  // extern "C"
