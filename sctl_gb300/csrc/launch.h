// Host-side interface between the C ABI (capi.cu) and the per-mode kernel
// translation units.  All pointers here are device pointers.
#pragma once

#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>

struct sctlgpu_near_plan_s;  // the C ABI's near plan (sctlgpu.h)

namespace sctlgpu {

struct BBox;

// Process-wide count of kernels launched by this library.
extern std::atomic<int64_t> g_launches;

struct Timing {
  bool enabled = false;
  cudaEvent_t start = nullptr, stop = nullptr;
  bool recorded = false;
};

struct EvalCall {
  int kernel;
  int64_t nt, ns;
  const void* r_trg;
  const void* r_src;
  const void* n_src;
  const void* v_src;
  void* v_trg;
  bool accumulate;
  cudaStream_t stream;
  unsigned* status;  // device status word
  int sms;           // multiprocessors of the current device
  Timing* timing;    // may be null
  double ctx = 0.0;  // kernel context (Helmholtz wavenumber)
};

struct KmatCall {
  int kernel;
  int64_t nt, ns;
  const void* r_trg;
  const void* r_src;
  const void* n_src;
  void* M;
  cudaStream_t stream;
  int sms;
  Timing* timing;
  double ctx = 0.0;  // kernel context (Helmholtz wavenumber)
};

// Direct sums.  `newton` is the number of Newton steps after the hardware seed.
cudaError_t eval_f64(const EvalCall& c, int newton);
cudaError_t eval_f32(const EvalCall& c, int newton);
cudaError_t eval_mixed_lo(const EvalCall& c, int newton);  // FP32 arithmetic on split coordinates
cudaError_t eval_mixed_df(const EvalCall& c);              // double-float arithmetic

// Kernel ids 4-15 (ext.cuh): FP64 or FP32 arithmetic.
cudaError_t eval_ext_f64(const EvalCall& c, int newton);
cudaError_t eval_ext_f32(const EvalCall& c, int newton);
cudaError_t kmat_ext_f64(const KmatCall& c, int newton);
cudaError_t kmat_ext_f32(const KmatCall& c, int newton);

// Kernel matrices.
cudaError_t kmat_f64(const KmatCall& c, int newton);
cudaError_t kmat_f32(const KmatCall& c, int newton);
// Mixed precision (digits up to the double-float limit): double-float entries rounded to FP64.
cudaError_t kmat_mixed_df(const KmatCall& c);

// Bounding box of targets and sources for the mixed-precision frame; `bb` is
// 64 bytes of device memory, initialised here.
cudaError_t compute_bbox(cudaStream_t s, int64_t nt, const double* r_trg, int64_t ns, const double* r_src, BBox* bb);

}  // namespace sctlgpu

namespace sctlgpu {

struct NearParams;
struct NearBlock;

// Per (kernel, arithmetic, Newton) entry points of the batched near-field path.
struct NearOps {
  size_t rec_bytes = 0;  // sizeof(Rec)
  int T = 1;             // targets per thread
  int occ = 1;           // resident CTAs per SM
  size_t smem = 0;       // dynamic shared memory of the persistent kernel
  // Records of two sources each (the packed double-float arithmetic): `pack` pairs the whole
  // list (source 2j with 2j + 1), `pack_blocks` pairs every block's sources separately, and the
  // kernel's block table counts pair records.
  bool paired = false;
  cudaError_t (*pack)(cudaStream_t, int64_t ns, const void* xs, const void* nrm, const void* f, const void* w,
                      void* recs, const BBox* bb, int sms) = nullptr;
  cudaError_t (*pack_blocks)(cudaStream_t, int64_t nblk, const NearBlock* pair_blocks, const NearBlock* src_blocks,
                             int64_t n_pairs, const void* xs, const void* nrm, const void* f, const void* w,
                             void* recs, const BBox* bb, int sms) = nullptr;
  cudaError_t (*launch)(cudaStream_t, unsigned ctas, const NearParams& p) = nullptr;
};

// Internal arithmetic of a batched plan.
enum { NEAR_F64 = 0, NEAR_F32 = 1, NEAR_MXLO = 2, NEAR_MXDF = 3 };
NearOps near_ops_f64(int kernel, int newton);
NearOps near_ops_f32(int kernel, int newton);
NearOps near_ops_mixed(int kernel, int imode, int newton);

// Runtime helpers of capi.cu shared with the other entry-point files.
int runtime_device(int* dev, unsigned** status, int* sms);
int runtime_record(cudaError_t e);
int runtime_effective_digits(int mode, int digits);
int runtime_steps(int mode, int digits);
int runtime_mixed_df_max_digits();
// SCTLGPU_MIXED's arithmetic at a digits value (after runtime_effective_digits).
enum { MIXED_ARITH_F32 = 0, MIXED_ARITH_DF = 1, MIXED_ARITH_F64 = 2 };
int runtime_mixed_arith(int digits);

// A near plan of the Stokes double layer with a symmetric 3 x 3 density per source (the
// treecode's proxies, KER_SDXU_SYM): n_src holds diag(S), v_src (2 S01, 2 S02, 2 S12).
// SCTLGPU_MIXED or SCTLGPU_F64 (SCTLGPU_ERR_INVALID_MODE otherwise); executed, queried and
// destroyed like any plan.
int near_plan_create_sym(::sctlgpu_near_plan_s** out, int mode, int digits, int64_t nblk, const void* blocks,
                         int64_t ns, int64_t nt, const int64_t* trg_map, int64_t n_out);

}  // namespace sctlgpu
