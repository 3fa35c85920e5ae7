// BF16 GEMMs on the 5th-generation tensor cores (tcgen05) with FP32
// accumulators in tensor memory, for the near-field correction MLP.
//
//   C[M x N] = act(A[M x K] . Bt[N x K]^T + bias)     (A, Bt row-major, K contiguous)
//
// One CTA of 128 threads owns a 128-row tile of C and all N (<= 256) columns.
// K is consumed in chunks of 64: every thread copies 16-byte pieces of the A
// and Bt chunks (cp.async) into shared memory in the canonical no-swizzle
// K-major layout of tcgen05 (8 x 16-byte core matrices; K-adjacent cores 128 B
// apart, 8-row groups 1024 B apart), one elected thread issues four
// tcgen05.mma (M=128, N, K=16) per chunk into the TMEM accumulator and commits
// them to an mbarrier, which gates the reuse of that chunk's buffer (two
// buffers: the copy of chunk k+1 overlaps the MMAs of chunk k).  The epilogue
// warps read their 32 TMEM lanes (tcgen05.ld 32x32b), add the bias, apply GELU
// and store FP32 and/or BF16.  Every mbarrier wait is bounded; TMEM is always
// released before the CTA exits.
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/sctlgpu.h"
#include "common.cuh"
#include "launch.h"

namespace sctlgpu {
namespace {

constexpr int TC_M = 128, TC_KC = 64, TC_THREADS = 128;
constexpr int TC_A_BYTES = TC_M * TC_KC * 2;   // 16 KB per chunk
constexpr int TC_B_BYTES = 256 * TC_KC * 2;    // up to 32 KB per chunk

// tcgen05 shared-memory matrix descriptor, no swizzle, K-major:
// start >> 4 in [0,14), leading-dimension byte offset >> 4 in [16,30) (between
// K-adjacent core matrices), stride-dimension byte offset >> 4 in [32,46)
// (between 8-row groups), bits [46,49) = 0b001, layout type 0 (no swizzle).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

// Instruction descriptor for kind::f16: D = F32 (bits 4-5 = 1), A = B = BF16
// (bits 7-9 and 10-12 = 1), both K-major, N >> 3 in bits 17-22, M >> 4 in 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst_smem)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, int accum) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum)
      : "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(smem)), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// Offset of element (row r, k) inside a chunk stored as 8x16B core matrices:
// core (r/8, k/8) at ((r/8)*8 + k/8) * 128 bytes, row r%8 at +16*(r%8).
__device__ __forceinline__ uint32_t core_off(int r, int k) {
  return (uint32_t)((((r >> 3) * (TC_KC / 8) + (k >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1));
}

__device__ __forceinline__ float gelu(float x) {  // tanh form
  const float c = 0.7978845608028654f;
  return 0.5f * x * (1.f + tanhf(c * (x + 0.044715f * x * x * x)));
}

struct TcParams {
  int M, N, K;              // M % 128 == 0, N % 16 == 0 and <= 256, K % 64 == 0
  const __nv_bfloat16* A;   // [M][K]
  const __nv_bfloat16* Bt;  // [N][K]
  const float* bias;        // [N] or null
  int act;                  // 0: none, 1: GELU
  float* C32;               // [M][N] FP32 output (after act), or null
  float* pre32;             // [M][N] FP32 pre-activation, or null
  __nv_bfloat16* C16;       // [M][N] BF16 output (after act), or null
  int accumulate32;         // C32 += result instead of =
  unsigned* status;
};

__global__ void __launch_bounds__(TC_THREADS) tc_gemm_kernel(TcParams p) {
  extern __shared__ __align__(1024) unsigned char tsm[];
  unsigned char* bufA[2] = {tsm, tsm + TC_A_BYTES};
  unsigned char* bufB[2] = {tsm + 2 * TC_A_BYTES, tsm + 2 * TC_A_BYTES + TC_B_BYTES};
  uint64_t* bars = reinterpret_cast<uint64_t*>(tsm + 2 * TC_A_BYTES + 2 * TC_B_BYTES);  // [2] chunk + [1] done
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 4);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * TC_M;
  const uint32_t ncols = p.N <= 32 ? 32 : p.N <= 64 ? 64 : p.N <= 128 ? 128 : 256;

  if (tid == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    mbar_init(&bars[2], 1);
    fence_mbar_init();
  }
  if (warp == 0) tmem_alloc(tmem_slot, ncols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  const uint32_t idesc = idesc_bf16(TC_M, p.N);
  const int nchunks = p.K / TC_KC;
  uint32_t use[2] = {0, 0};  // times each buffer was committed
  bool ok = true;
  for (int kc = 0; kc < nchunks; ++kc) {
    const int b = kc & 1;
    if (kc >= 2) {  // the MMAs that read this buffer two chunks ago must be complete
      if (!mbar_wait_bounded(&bars[b], (use[b] - 1) & 1, p.status)) ok = false;
    }
    // copy the A chunk (128 x 64) and the Bt chunk (N x 64) into core-matrix layout
    const int k0 = kc * TC_KC;
    for (int i = tid; i < TC_M * (TC_KC / 8); i += TC_THREADS) {
      const int r = i / (TC_KC / 8), kk = (i % (TC_KC / 8)) * 8;
      cp_async16(bufA[b] + core_off(r, kk), p.A + (size_t)(m0 + r) * p.K + k0 + kk);
    }
    for (int i = tid; i < p.N * (TC_KC / 8); i += TC_THREADS) {
      const int r = i / (TC_KC / 8), kk = (i % (TC_KC / 8)) * 8;
      cp_async16(bufB[b] + core_off(r, kk), p.Bt + (size_t)r * p.K + k0 + kk);
    }
    cp_async_wait_all();
    fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      const uint32_t a0 = smem_u32(bufA[b]), b0 = smem_u32(bufB[b]);
#pragma unroll
      for (int j = 0; j < TC_KC / 16; ++j) {
        const uint64_t ad = smem_desc(a0 + j * 256, 128, 1024);
        const uint64_t bd = smem_desc(b0 + j * 256, 128, 1024);
        tc_mma(tmem, ad, bd, idesc, (kc > 0 || j > 0) ? 1 : 0);
      }
      tc_commit(&bars[b]);
    }
    ++use[b];
  }
  if (tid == 0) tc_commit(&bars[2]);
  if (!mbar_wait_bounded(&bars[2], 0, p.status)) ok = false;
  // Drain the chunk barriers' last phases as well (their MMAs are complete once bars[2] fired).
  tc_fence_after();

  if (ok) {
    const int row = m0 + warp * 32 + lane;
    for (int c0 = 0; c0 < p.N; c0 += 16) {
      float v[16];
      tc_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const int col = c0 + i;
        float x = v[i] + (p.bias ? p.bias[col] : 0.f);
        if (p.pre32) p.pre32[(size_t)row * p.N + col] = x;
        if (p.act == 1) x = gelu(x);
        if (p.C32) {
          float* o = &p.C32[(size_t)row * p.N + col];
          *o = p.accumulate32 ? *o + x : x;
        }
        if (p.C16) p.C16[(size_t)row * p.N + col] = __float2bfloat16_rn(x);
      }
    }
  }
  if (!ok && tid == 0) mbar_wait_bounded(&bars[2], 0, nullptr);  // let in-flight MMAs land before TMEM is freed
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, ncols);
}

}  // namespace
}  // namespace sctlgpu

using namespace sctlgpu;

extern "C" int sctlgpu_tc_gemm_bf16(int M, int N, int K, const void* A, const void* Bt, const float* bias, int act,
                                    float* C32, float* pre32, void* C16, int accumulate32, void* stream) {
  if (M <= 0 || N <= 0 || K <= 0 || M % TC_M || N % 16 || N > 256 || K % TC_KC) return SCTLGPU_ERR_INVALID_SIZE;
  if (!A || !Bt || (!C32 && !C16 && !pre32)) return SCTLGPU_ERR_NULL_POINTER;
  if (act != 0 && act != 1) return SCTLGPU_ERR_INVALID_ARGUMENT;
  if (((uintptr_t)A | (uintptr_t)Bt) & 15) return SCTLGPU_ERR_INVALID_ARGUMENT;  // 16-byte copies
  int dev;
  unsigned* status;
  int sms;
  int rc = runtime_device(&dev, &status, &sms);
  if (rc) return rc;
  const size_t smem = 2 * TC_A_BYTES + 2 * TC_B_BYTES + 64;
  static bool attr[64] = {};
  if (!attr[dev]) {
    cudaFuncSetAttribute(tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr[dev] = true;
  }
  TcParams p;
  p.M = M;
  p.N = N;
  p.K = K;
  p.A = (const __nv_bfloat16*)A;
  p.Bt = (const __nv_bfloat16*)Bt;
  p.bias = bias;
  p.act = act;
  p.C32 = C32;
  p.pre32 = pre32;
  p.C16 = (__nv_bfloat16*)C16;
  p.accumulate32 = accumulate32;
  p.status = status;
  tc_gemm_kernel<<<M / TC_M, TC_THREADS, smem, (cudaStream_t)stream>>>(p);
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return runtime_record(cudaGetLastError());
}
