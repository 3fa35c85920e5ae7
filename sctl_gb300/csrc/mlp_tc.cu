// BF16 GEMMs on the 5th-generation tensor cores (tcgen05) with FP32
// accumulators in tensor memory, for the near-field correction MLP.
//
//   C[M x N] = act(A[M x K] . Bt[N x K]^T + bias)     (A, Bt row-major, K contiguous)
//
// One CTA of 128 threads owns a 128-row tile of C and all N (<= 256) columns,
// optionally a slice of K (split-K, partials reduced in a fixed order).  K is
// consumed in chunks of 64 through a ring of 4-8 shared-memory stages:
//   * one producer thread loads each chunk of A (128 x 64) and Bt (N x 64) with
//     TMA tensor copies (cp.async.bulk.tensor.2d, 128-byte swizzle) completing
//     on the stage's `full` mbarrier;
//   * one MMA thread waits for `full`, issues four tcgen05.mma (M=128, N, K=16)
//     from swizzled K-major shared-memory descriptors into the TMEM
//     accumulator, and commits them to the stage's `empty` mbarrier, which
//     hands the stage back to the producer;
//   * after the last chunk the MMA thread commits to `done`; all four warps
//     then read their 32 TMEM lanes (tcgen05.ld 32x32b), add the bias, apply
//     GELU and store FP32 and/or BF16 rows with 16-byte stores.
// Every mbarrier wait is bounded (a timeout sets the status word, skips the
// epilogue and drains the copies in flight); TMEM is always released.
#include <cmath>
#include <cstdint>
#include <mutex>
#include <random>
#include <vector>

#include <cuda.h>  // CUtensorMap and its enums; the encoder is fetched from the driver at run time
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/sctlgpu.h"
#include "common.cuh"
#include "launch.h"

namespace sctlgpu {
namespace {

constexpr int TC_M = 128, TC_KC = 64, TC_THREADS = 128;
constexpr int TC_A_BYTES = TC_M * TC_KC * 2;  // 16 KB per chunk
constexpr int TC_SMEM_BUDGET = 100 * 1024;     // stage ring (two CTAs per SM: one drains its tile while the other computes)

// tcgen05 shared-memory matrix descriptor for a K-major tile written by TMA
// with 128-byte swizzle: start >> 4 in [0,14), leading byte offset (unused
// for swizzled K-major, 16 B) in [16,30), stride byte offset >> 4 in [32,46)
// (1024 B between 8-row groups of 128-byte rows), version 1 at bit 46, layout
// SWIZZLE_128B (2) in [61,64).  Stepping K by 16 elements adds 32 bytes to the
// start address inside the swizzle atom.
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) | (1ull << 46) |
         (2ull << 61);
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

// 2-D TMA tile load (x = innermost coordinate, in elements) into shared memory.
__device__ __forceinline__ void tma_load_2d(void* smem_dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(smem_dst)),
      "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
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
  // optional fused epilogue: dot_out[row] += sum_{col < dot_cols} C[row][col] * dot_dens[dot_index[row]][col]
  const double* dot_dens;
  const int64_t* dot_index;
  int dot_cols;
  double* dot_out;
  unsigned* status;
  // split-K (gridDim.y slices): raw FP32 partials [slice][M][N], reduced afterwards
  float* partial;
  int stages;
};

__global__ void __launch_bounds__(TC_THREADS, 2)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, TcParams p) {
  extern __shared__ unsigned char tsm_raw[];
  unsigned char* tsm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(tsm_raw) + 1023) & ~(uintptr_t)1023);
  const int nst = p.stages;
  const uint32_t b_bytes = (uint32_t)p.N * TC_KC * 2;
  const uint32_t stage_bytes = TC_A_BYTES + b_bytes;  // multiple of 1024 (N % 16 == 0)
  uint64_t* full = reinterpret_cast<uint64_t*>(tsm + (size_t)nst * stage_bytes);
  uint64_t* empty = full + nst;
  uint64_t* done = empty + nst;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  int* s_err = reinterpret_cast<int*>(tmem_slot + 1);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * TC_M;
  const uint32_t ncols = p.N <= 32 ? 32 : p.N <= 64 ? 64 : p.N <= 128 ? 128 : 256;
  const int nchunks = p.K / TC_KC;
  const int per = (nchunks + (int)gridDim.y - 1) / (int)gridDim.y;
  const int c0 = (int)blockIdx.y * per;
  const int nk = max(0, min(nchunks, c0 + per) - c0);

  if (tid == 0) {
    for (int s = 0; s < nst; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    *s_err = 0;
    fence_mbar_init();
  }
  if (warp == 0) tmem_alloc(tmem_slot, ncols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  // Role lanes run alone; the rest of their warp waits at __syncwarp (not on an mbarrier
  // try_wait, which would suspend the warp the role lane runs in).
  if (warp == 0) {
    if (lane == 0) {  // producer
    int issued = 0;
    for (int i = 0; i < nk; ++i) {
      const int s = i % nst;
      const uint32_t use = (uint32_t)(i / nst);
      if (i >= nst && !mbar_wait_bounded(&empty[s], (use - 1) & 1, p.status)) {
        atomicExch(s_err, 1);
        break;
      }
      unsigned char* a = tsm + (size_t)s * stage_bytes;
      mbar_arrive_expect_tx(&full[s], stage_bytes);
      tma_load_2d(a, &mapA, (c0 + i) * TC_KC, m0, &full[s]);
      tma_load_2d(a + TC_A_BYTES, &mapB, (c0 + i) * TC_KC, 0, &full[s]);
      ++issued;
    }
    // Copies still in flight (only after a timeout): let them land before the CTA exits.
    for (int i = max(0, issued - nst); i < issued; ++i)
      mbar_wait_bounded(&full[i % nst], (uint32_t)((i / nst) & 1), nullptr);
    }
    __syncwarp();
  } else if (warp == 1) {
    if (lane == 0) {  // MMA issuer
    const uint32_t idesc = idesc_bf16(TC_M, p.N);
    for (int i = 0; i < nk; ++i) {
      const int s = i % nst;
      if (!mbar_wait_bounded(&full[s], (uint32_t)((i / nst) & 1), p.status)) {
        atomicExch(s_err, 1);
        break;
      }
      tc_fence_after();
      const uint32_t a0 = smem_u32(tsm + (size_t)s * stage_bytes), b0 = a0 + TC_A_BYTES;
#pragma unroll
      for (int j = 0; j < TC_KC / 16; ++j)
        tc_mma(tmem, smem_desc_sw128(a0 + j * 32), smem_desc_sw128(b0 + j * 32), idesc, (i > 0 || j > 0) ? 1 : 0);
      tc_commit(&empty[s]);
    }
    tc_commit(done);  // tracks every MMA issued above (arrives at once if none)
    }
    __syncwarp();
  }
  if (!mbar_wait_bounded(done, 0, p.status)) atomicExch(s_err, 1);
  if (tid == 32) {  // the MMA thread's last commits to the stage barriers have landed too
    for (int i = max(0, nk - nst); i < nk; ++i)
      mbar_wait_bounded(&empty[i % nst], (uint32_t)((i / nst) & 1), nullptr);
  }
  __syncthreads();
  tc_fence_after();
  const bool ok = *s_err == 0 && nk > 0;

  if (ok) {
    const int row = m0 + warp * 32 + lane;
    if (p.partial) {  // split-K slice: raw sums
      float* dst = p.partial + ((size_t)blockIdx.y * p.M + row) * p.N;
      for (int cb = 0; cb < p.N; cb += 16) {
        float v[16];
        tc_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)cb, v);
#pragma unroll
        for (int q = 0; q < 4; ++q)
          reinterpret_cast<float4*>(dst + cb)[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
      }
    } else {
      double dot = 0.0;
      const double* dv =
          (p.dot_out && p.dot_index[row] >= 0) ? p.dot_dens + p.dot_index[row] * p.dot_cols : nullptr;
      for (int cb = 0; cb < p.N; cb += 16) {
        float v[16], x[16];
        tc_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)cb, v);
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          v[i] += p.bias ? p.bias[cb + i] : 0.f;
          x[i] = p.act == 1 ? gelu(v[i]) : v[i];
        }
        const size_t o = (size_t)row * p.N + cb;
        if (p.pre32)
#pragma unroll
          for (int q = 0; q < 4; ++q)
            reinterpret_cast<float4*>(p.pre32 + o)[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
        if (p.C32) {
          float4* c = reinterpret_cast<float4*>(p.C32 + o);
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            float4 w = make_float4(x[4 * q], x[4 * q + 1], x[4 * q + 2], x[4 * q + 3]);
            if (p.accumulate32) {
              const float4 old = c[q];
              w.x += old.x;
              w.y += old.y;
              w.z += old.z;
              w.w += old.w;
            }
            c[q] = w;
          }
        }
        if (p.C16) {
          __nv_bfloat162 h[8];
#pragma unroll
          for (int q = 0; q < 8; ++q) h[q] = __floats2bfloat162_rn(x[2 * q], x[2 * q + 1]);
          uint4* d16 = reinterpret_cast<uint4*>(p.C16 + o);
          d16[0] = *reinterpret_cast<const uint4*>(&h[0]);
          d16[1] = *reinterpret_cast<const uint4*>(&h[4]);
        }
        if (dv)
#pragma unroll
          for (int i = 0; i < 16; ++i)
            if (cb + i < p.dot_cols) dot = fma((double)x[i], dv[cb + i], dot);
      }
      if (dv) p.dot_out[row] += dot;
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, ncols);
}

// C (+)= sum over slices of the split-K partials, in slice order.
__global__ void tc_splitk_reduce_kernel(int64_t n, int slices, const float* __restrict__ partial, int accumulate,
                                        float* __restrict__ C) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float acc = accumulate ? C[i] : 0.f;
    for (int s = 0; s < slices; ++s) acc += partial[(int64_t)s * n + i];
    C[i] = acc;
  }
}

// cuTensorMapEncodeTiled from the driver (no link-time dependency on libcuda).
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return (EncodeTiledFn) nullptr;
    return (EncodeTiledFn)f;
  }();
  return fn;
}

// Row-major BF16 matrix [rows][K] as a 2-D tensor map with box (64, box_rows), 128-byte swizzle.
cudaError_t make_map(CUtensorMap* map, const void* base, int rows, int K, int box_rows) {
  EncodeTiledFn enc = encode_tiled();
  if (!enc) return cudaErrorNotSupported;
  const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)K * 2};
  const cuuint32_t box[2] = {(cuuint32_t)TC_KC, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

int stages_for(int N) {
  const int stage = TC_A_BYTES + N * TC_KC * 2;
  return std::max(2, std::min(8, TC_SMEM_BUDGET / stage));
}

size_t smem_for(int N, int stages) { return 1024 + (size_t)stages * (TC_A_BYTES + N * TC_KC * 2) + 256; }

cudaError_t tc_gemm_launch(const TcParams& p0, cudaStream_t st) {
  TcParams p = p0;
  int dev = 0, sms = 0;
  unsigned* status = nullptr;
  if (runtime_device(&dev, &status, &sms) != SCTLGPU_OK) return cudaErrorNoDevice;
  CUtensorMap ma, mb;
  cudaError_t e = make_map(&ma, p.A, p.M, p.K, TC_M);
  if (e == cudaSuccess) e = make_map(&mb, p.Bt, p.N, p.K, p.N);
  if (e != cudaSuccess) return e;
  p.stages = stages_for(p.N);
  const size_t smem = smem_for(p.N, p.stages);
  static bool attr[64] = {};
  if (dev >= 0 && dev < 64 && !attr[dev]) {
    int n = 16;  // the largest ring over all N
    for (int N = 32; N <= 256; N += 16)
      if (smem_for(N, stages_for(N)) > smem_for(n, stages_for(n))) n = N;
    cudaFuncSetAttribute(tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_for(n, stages_for(n)));
    attr[dev] = true;
  }
  // Split K when the row tiles cannot fill the GPU and the epilogue is a plain FP32 store;
  // every slice gets at least one chunk.
  const int tiles = p.M / TC_M, chunks = p.K / TC_KC;
  const bool plain = p.C32 && !p.pre32 && !p.C16 && !p.bias && p.act == 0 && !p.dot_out;
  int slices = 1;
  if (plain && tiles < sms && chunks >= 8) {
    slices = std::min(std::max(1, sms / tiles), chunks / 4);
    const int per = (chunks + slices - 1) / slices;
    slices = (chunks + per - 1) / per;
  }
  p.partial = nullptr;
  float* part = nullptr;
  if (slices > 1) {
    if ((e = cudaMallocAsync((void**)&part, (size_t)slices * p.M * p.N * sizeof(float), st))) return e;
    p.partial = part;
  }
  tc_gemm_kernel<<<dim3((unsigned)tiles, (unsigned)slices), TC_THREADS, smem, st>>>(ma, mb, p);
  g_launches.fetch_add(1, std::memory_order_relaxed);
  e = cudaGetLastError();
  if (slices > 1) {
    if (e == cudaSuccess) {
      const int64_t n = (int64_t)p.M * p.N;
      tc_splitk_reduce_kernel<<<(unsigned)std::min<int64_t>((n + 255) / 256, (int64_t)sms * 8), 256, 0, st>>>(
          n, slices, part, p.accumulate32, p.C32);
      g_launches.fetch_add(1, std::memory_order_relaxed);
      e = cudaGetLastError();
    }
    cudaError_t e2 = cudaFreeAsync(part, st);
    if (e == cudaSuccess) e = e2;
  }
  return e;
}

TcParams gemm_params(int M, int N, int K, const __nv_bfloat16* A, const __nv_bfloat16* Bt, unsigned* status) {
  TcParams p{};
  p.M = M;
  p.N = N;
  p.K = K;
  p.A = A;
  p.Bt = Bt;
  p.status = status;
  return p;
}

// ------------------------------------------------------------ MLP kernels
__device__ __forceinline__ float gelu_grad(float x) {
  const float c = 0.7978845608028654f, k = 0.044715f;
  const float t = tanhf(c * (x + k * x * x * x));
  return 0.5f * (1.f + t) + 0.5f * x * (1.f - t * t) * c * (1.f + 3.f * k * x * x);
}

// x (FP32, B x in) -> BF16 (B x K0), zero padded
__global__ void mlp_input_kernel(int B, int in_dim, int K0, const float* __restrict__ x, __nv_bfloat16* __restrict__ x16) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (int64_t)B * K0;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / K0), c = (int)(i % K0);
    x16[i] = __float2bfloat16_rn(c < in_dim ? x[(int64_t)r * in_dim + c] : 0.f);
  }
}

// loss = sum (y - t)^2 / (B*out); dy = 2 (y - t) / (B*out) (zero in padded columns)
__global__ void mlp_loss_kernel(int B, int out_dim, int N, const float* __restrict__ y, const float* __restrict__ t,
                                __nv_bfloat16* __restrict__ dy16, float* __restrict__ db, float* __restrict__ loss) {
  float acc = 0.f;
  const float sc = 2.f / ((float)B * (float)out_dim);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (int64_t)B * N;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / N), c = (int)(i % N);
    float g = 0.f;
    if (c < out_dim) {
      const float d = y[i] - t[(int64_t)r * out_dim + c];
      acc += d * d;
      g = sc * d;
      atomicAdd(&db[c], g);
    }
    dy16[i] = __float2bfloat16_rn(g);
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, acc / ((float)B * (float)out_dim));
}

// dz = dh * gelu'(z) -> BF16, column sums into db
__global__ void mlp_gelu_back_kernel(int B, int N, const float* __restrict__ dh, const float* __restrict__ z,
                                     __nv_bfloat16* __restrict__ dz16, float* __restrict__ db) {
  const int c = blockIdx.y * 32 + (threadIdx.x & 31);
  const int rstep = blockDim.x / 32 * gridDim.x;
  float acc = 0.f;
  for (int r = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32; r < B; r += rstep) {
    const int64_t i = (int64_t)r * N + c;
    const float g = dh[i] * gelu_grad(z[i]);
    dz16[i] = __float2bfloat16_rn(g);
    acc += g;
  }
  atomicAdd(&db[c], acc);
}

// BF16 transpose: in (R x C) -> out (C x R); R, C multiples of 32
__global__ void mlp_transpose_kernel(int R, int C, const __nv_bfloat16* __restrict__ in, __nv_bfloat16* __restrict__ out) {
  __shared__ __nv_bfloat16 tile[32][33];
  const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) tile[j][threadIdx.x] = in[(int64_t)(r0 + j) * C + c0 + threadIdx.x];
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) out[(int64_t)(c0 + j) * R + r0 + threadIdx.x] = tile[threadIdx.x][j];
}

// Adam on the flat FP32 parameters
__global__ void mlp_adam_kernel(int64_t n, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                                float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
  }
}

// BF16 copies of a layer's weights: Wb (N x K) and Wt (K x N)
__global__ void mlp_cast_kernel(int N, int K, const float* __restrict__ W, __nv_bfloat16* __restrict__ Wb,
                                __nv_bfloat16* __restrict__ Wt) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (int64_t)N * K;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int n = (int)(i / K), k = (int)(i % K);
    const __nv_bfloat16 b = __float2bfloat16_rn(W[i]);
    Wb[i] = b;
    Wt[(int64_t)k * N + n] = b;
  }
}

}  // namespace
}  // namespace sctlgpu

using namespace sctlgpu;

// ------------------------------------------------------------------ MLP
// in -> 256 -> 256 -> 256 -> out, GELU between layers; K of layer 1 padded to 64,
// the output padded to 128 (zero rows), batch a multiple of 128.
struct sctlgpu_mlp_s {
  int in_dim = 0, out_dim = 0, max_batch = 0, step = 0;
  static constexpr int L = 4, H = 256, K0 = 64, NO = 128;
  int Nl[L] = {H, H, H, NO}, Kl[L] = {K0, H, H, H};
  int64_t off_w[L], off_b[L], n_params = 0;
  float *params = nullptr, *grads = nullptr, *adam_m = nullptr, *adam_v = nullptr, *loss = nullptr;
  __nv_bfloat16 *Wb[L] = {}, *Wt[L] = {};
  __nv_bfloat16 *x16 = nullptr, *h16[3] = {}, *dy16 = nullptr, *dz16[3] = {}, *tA = nullptr, *tB = nullptr;
  float *z[3] = {}, *y = nullptr, *dh = nullptr;
  char* arena = nullptr;
  int device = 0;
};

namespace {

unsigned* mlp_status() {
  int dev;
  unsigned* status = nullptr;
  int sms;
  if (runtime_device(&dev, &status, &sms)) return nullptr;
  return status;
}

cudaError_t mlp_refresh_bf16(sctlgpu_mlp_s* m, cudaStream_t st) {
  for (int l = 0; l < sctlgpu_mlp_s::L; ++l) {
    mlp_cast_kernel<<<256, 256, 0, st>>>(m->Nl[l], m->Kl[l], m->params + m->off_w[l], m->Wb[l], m->Wt[l]);
    g_launches.fetch_add(1, std::memory_order_relaxed);
  }
  return cudaGetLastError();
}

// Forward pass; fills z, h16 and y (FP32, B x NO).  Optional fused dot epilogue.
cudaError_t mlp_forward_dev(sctlgpu_mlp_s* m, int B, const float* x, cudaStream_t st, const double* dens,
                            const int64_t* index, double* dot_out) {
  unsigned* status = mlp_status();
  mlp_input_kernel<<<256, 256, 0, st>>>(B, m->in_dim, m->K0, x, m->x16);
  g_launches.fetch_add(1, std::memory_order_relaxed);
  const __nv_bfloat16* in = m->x16;
  for (int l = 0; l < 3; ++l) {
    TcParams p = gemm_params(B, m->Nl[l], m->Kl[l], in, m->Wb[l], status);
    p.bias = m->params + m->off_b[l];
    p.act = 1;
    p.pre32 = m->z[l];
    p.C16 = m->h16[l];
    cudaError_t e = tc_gemm_launch(p, st);
    if (e != cudaSuccess) return e;
    in = m->h16[l];
  }
  TcParams p = gemm_params(B, m->Nl[3], m->Kl[3], in, m->Wb[3], status);
  p.bias = m->params + m->off_b[3];
  p.C32 = m->y;
  p.dot_dens = dens;
  p.dot_index = index;
  p.dot_cols = m->out_dim;
  p.dot_out = dot_out;
  return tc_gemm_launch(p, st);
}

// Loss and gradients into m->grads (FP32), given targets t (B x out_dim).
cudaError_t mlp_backward_dev(sctlgpu_mlp_s* m, int B, const float* t, cudaStream_t st) {
  unsigned* status = mlp_status();
  const int H = sctlgpu_mlp_s::H, NO = sctlgpu_mlp_s::NO, K0 = sctlgpu_mlp_s::K0;
  cudaError_t e;
  if ((e = cudaMemsetAsync(m->grads, 0, m->n_params * sizeof(float), st))) return e;
  if ((e = cudaMemsetAsync(m->loss, 0, sizeof(float), st))) return e;
  mlp_loss_kernel<<<256, 256, 0, st>>>(B, m->out_dim, NO, m->y, t, m->dy16, m->grads + m->off_b[3], m->loss);
  g_launches.fetch_add(1, std::memory_order_relaxed);
  auto transpose = [&](int R, int C, const __nv_bfloat16* in, __nv_bfloat16* out) {
    mlp_transpose_kernel<<<dim3(C / 32, R / 32), dim3(32, 8), 0, st>>>(R, C, in, out);
    g_launches.fetch_add(1, std::memory_order_relaxed);
  };
  // dW4 = dy^T h3
  transpose(B, NO, m->dy16, m->tA);
  transpose(B, H, m->h16[2], m->tB);
  {
    TcParams p = gemm_params(NO, H, B, m->tA, m->tB, status);
    p.C32 = m->grads + m->off_w[3];
    if ((e = tc_gemm_launch(p, st))) return e;
  }
  const __nv_bfloat16* dcur = m->dy16;
  int kcur = NO;
  for (int l = 2; l >= 0; --l) {
    // dh_l = d_{l+1} W_{l+1}  (A: B x kcur, Bt = W_{l+1}^T: H x kcur)
    TcParams p = gemm_params(B, H, kcur, dcur, m->Wt[l + 1], status);
    p.C32 = m->dh;
    if ((e = tc_gemm_launch(p, st))) return e;
    mlp_gelu_back_kernel<<<dim3(64, H / 32), 256, 0, st>>>(B, H, m->dh, m->z[l], m->dz16[l], m->grads + m->off_b[l]);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    // dW_l = dz_l^T . (input of layer l)
    transpose(B, H, m->dz16[l], m->tA);
    const int Kin = l == 0 ? K0 : H;
    transpose(B, Kin, l == 0 ? m->x16 : m->h16[l - 1], m->tB);
    TcParams q = gemm_params(H, Kin, B, m->tA, m->tB, status);
    q.C32 = m->grads + m->off_w[l];
    if ((e = tc_gemm_launch(q, st))) return e;
    dcur = m->dz16[l];
    kcur = H;
  }
  return cudaGetLastError();
}

int mlp_check(sctlgpu_mlp_s* m, int B) {
  if (!m) return SCTLGPU_ERR_NULL_POINTER;
  if (B <= 0 || B % 128 || B > m->max_batch) return SCTLGPU_ERR_INVALID_SIZE;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev != m->device) return SCTLGPU_ERR_INVALID_ARGUMENT;
  return SCTLGPU_OK;
}

}  // namespace

extern "C" {

int sctlgpu_mlp_create(sctlgpu_mlp* out, int in_dim, int out_dim, int max_batch, uint64_t seed) {
  if (!out) return SCTLGPU_ERR_NULL_POINTER;
  *out = nullptr;
  if (in_dim < 1 || in_dim > sctlgpu_mlp_s::K0 || out_dim < 1 || out_dim > sctlgpu_mlp_s::NO || max_batch < 128 ||
      max_batch % 128 || max_batch > (1 << 24))
    return SCTLGPU_ERR_INVALID_SIZE;
  auto* m = new sctlgpu_mlp_s();
  m->in_dim = in_dim;
  m->out_dim = out_dim;
  m->max_batch = max_batch;
  cudaGetDevice(&m->device);
  const int L = sctlgpu_mlp_s::L, H = sctlgpu_mlp_s::H;
  int64_t o = 0;
  for (int l = 0; l < L; ++l) {
    m->off_w[l] = o;
    o += (int64_t)m->Nl[l] * m->Kl[l];
    m->off_b[l] = o;
    o += m->Nl[l];
  }
  m->n_params = o;
  // He-style initialisation (std 1/sqrt(fan_in) of the live inputs); padded rows / columns zero.
  std::vector<float> h(o, 0.f);
  std::mt19937_64 rng(seed);
  for (int l = 0; l < L; ++l) {
    const int fan = l == 0 ? in_dim : m->Kl[l];
    std::normal_distribution<float> nd(0.f, 1.f / std::sqrt((float)fan));
    for (int n = 0; n < m->Nl[l]; ++n)
      for (int k = 0; k < m->Kl[l]; ++k) {
        const bool live = (l > 0 || k < in_dim) && (l < L - 1 || n < out_dim);
        h[m->off_w[l] + (int64_t)n * m->Kl[l] + k] = live ? nd(rng) : 0.f;
      }
  }
  const int64_t B = max_batch;
  size_t bytes = 0;
  auto take = [&](size_t b) {
    const size_t at = bytes;
    bytes += (b + 255) / 256 * 256;
    return at;
  };
  const size_t o_p = take(o * 4), o_g = take(o * 4), o_m = take(o * 4), o_v = take(o * 4), o_l = take(4);
  size_t o_wb[L], o_wt[L];
  for (int l = 0; l < L; ++l) {
    o_wb[l] = take((size_t)m->Nl[l] * m->Kl[l] * 2);
    o_wt[l] = take((size_t)m->Nl[l] * m->Kl[l] * 2);
  }
  const size_t o_x = take(B * sctlgpu_mlp_s::K0 * 2), o_y = take(B * sctlgpu_mlp_s::NO * 4),
               o_dy = take(B * sctlgpu_mlp_s::NO * 2), o_dh = take(B * H * 4), o_ta = take(B * H * 2),
               o_tb = take(B * H * 2);
  size_t o_z[3], o_h[3], o_dz[3];
  for (int i = 0; i < 3; ++i) {
    o_z[i] = take(B * H * 4);
    o_h[i] = take(B * H * 2);
    o_dz[i] = take(B * H * 2);
  }
  cudaError_t e = cudaMalloc(&m->arena, bytes);
  if (e != cudaSuccess) {
    delete m;
    return runtime_record(e);
  }
  char* a = m->arena;
  m->params = (float*)(a + o_p);
  m->grads = (float*)(a + o_g);
  m->adam_m = (float*)(a + o_m);
  m->adam_v = (float*)(a + o_v);
  m->loss = (float*)(a + o_l);
  for (int l = 0; l < L; ++l) {
    m->Wb[l] = (__nv_bfloat16*)(a + o_wb[l]);
    m->Wt[l] = (__nv_bfloat16*)(a + o_wt[l]);
  }
  m->x16 = (__nv_bfloat16*)(a + o_x);
  m->y = (float*)(a + o_y);
  m->dy16 = (__nv_bfloat16*)(a + o_dy);
  m->dh = (float*)(a + o_dh);
  m->tA = (__nv_bfloat16*)(a + o_ta);
  m->tB = (__nv_bfloat16*)(a + o_tb);
  for (int i = 0; i < 3; ++i) {
    m->z[i] = (float*)(a + o_z[i]);
    m->h16[i] = (__nv_bfloat16*)(a + o_h[i]);
    m->dz16[i] = (__nv_bfloat16*)(a + o_dz[i]);
  }
  if ((e = cudaMemcpy(m->params, h.data(), o * 4, cudaMemcpyHostToDevice)) == cudaSuccess &&
      (e = cudaMemset(m->adam_m, 0, o * 4)) == cudaSuccess && (e = cudaMemset(m->adam_v, 0, o * 4)) == cudaSuccess &&
      (e = mlp_refresh_bf16(m, 0)) == cudaSuccess)
    e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    cudaFree(m->arena);
    delete m;
    return runtime_record(e);
  }
  *out = m;
  return SCTLGPU_OK;
}

int sctlgpu_mlp_destroy(sctlgpu_mlp m) {
  if (!m) return SCTLGPU_OK;
  cudaDeviceSynchronize();
  cudaFree(m->arena);
  delete m;
  return SCTLGPU_OK;
}

int64_t sctlgpu_mlp_num_params(sctlgpu_mlp m) { return m ? m->n_params : -1; }

int sctlgpu_mlp_get_params(sctlgpu_mlp m, float* host_out) {
  if (!m || !host_out) return SCTLGPU_ERR_NULL_POINTER;
  return runtime_record(cudaMemcpy(host_out, m->params, m->n_params * 4, cudaMemcpyDeviceToHost));
}

int sctlgpu_mlp_set_params(sctlgpu_mlp m, const float* host_in) {
  if (!m || !host_in) return SCTLGPU_ERR_NULL_POINTER;
  cudaError_t e = cudaMemcpy(m->params, host_in, m->n_params * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = mlp_refresh_bf16(m, 0);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  return runtime_record(e);
}

int sctlgpu_mlp_forward(sctlgpu_mlp m, int B, const float* x, float* y, void* stream) {
  int rc = mlp_check(m, B);
  if (rc) return rc;
  if (!x || !y) return SCTLGPU_ERR_NULL_POINTER;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = mlp_forward_dev(m, B, x, st, nullptr, nullptr, nullptr);
  if (e == cudaSuccess)
    e = cudaMemcpy2DAsync(y, m->out_dim * 4, m->y, sctlgpu_mlp_s::NO * 4, m->out_dim * 4, B, cudaMemcpyDeviceToDevice, st);
  return runtime_record(e);
}

int sctlgpu_mlp_forward_dot(sctlgpu_mlp m, int B, const float* x, const double* dens, const int64_t* index,
                            double* out, void* stream) {
  int rc = mlp_check(m, B);
  if (rc) return rc;
  if (!x || !dens || !index || !out) return SCTLGPU_ERR_NULL_POINTER;
  return runtime_record(mlp_forward_dev(m, B, x, (cudaStream_t)stream, dens, index, out));
}

int sctlgpu_mlp_train_step(sctlgpu_mlp m, int B, const float* x, const float* t, float lr, float* loss_host,
                           void* stream) {
  int rc = mlp_check(m, B);
  if (rc) return rc;
  if (!x || !t) return SCTLGPU_ERR_NULL_POINTER;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = mlp_forward_dev(m, B, x, st, nullptr, nullptr, nullptr);
  if (e == cudaSuccess) e = mlp_backward_dev(m, B, t, st);
  if (e != cudaSuccess) return runtime_record(e);
  m->step += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f / (1.f - std::pow(b1, (float)m->step)), c2 = 1.f / (1.f - std::pow(b2, (float)m->step));
  mlp_adam_kernel<<<256, 256, 0, st>>>(m->n_params, m->params, m->grads, m->adam_m, m->adam_v, lr, b1, b2, 1e-8f, c1, c2);
  g_launches.fetch_add(1, std::memory_order_relaxed);
  e = mlp_refresh_bf16(m, st);
  if (e == cudaSuccess && loss_host) {
    e = cudaMemcpyAsync(loss_host, m->loss, 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  }
  return runtime_record(e);
}

int sctlgpu_mlp_gradients(sctlgpu_mlp m, int B, const float* x, const float* t, float* grads_host, float* loss_host) {
  int rc = mlp_check(m, B);
  if (rc) return rc;
  if (!x || !t || !grads_host) return SCTLGPU_ERR_NULL_POINTER;
  cudaError_t e = mlp_forward_dev(m, B, x, 0, nullptr, nullptr, nullptr);
  if (e == cudaSuccess) e = mlp_backward_dev(m, B, t, 0);
  if (e == cudaSuccess) e = cudaMemcpy(grads_host, m->grads, m->n_params * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && loss_host) e = cudaMemcpy(loss_host, m->loss, 4, cudaMemcpyDeviceToHost);
  return runtime_record(e);
}

}  // extern "C"

extern "C" int sctlgpu_tc_gemm_bf16(int M, int N, int K, const void* A, const void* Bt, const float* bias, int act,
                                    float* C32, float* pre32, void* C16, int accumulate32, void* stream) {
  if (M <= 0 || N <= 0 || K <= 0 || M % TC_M || N % 16 || N > 256 || K % TC_KC) return SCTLGPU_ERR_INVALID_SIZE;
  if (!A || !Bt || (!C32 && !C16 && !pre32)) return SCTLGPU_ERR_NULL_POINTER;
  if (act != 0 && act != 1) return SCTLGPU_ERR_INVALID_ARGUMENT;
  // TMA sources and 16-byte epilogue stores need 16-byte aligned bases
  if (((uintptr_t)A | (uintptr_t)Bt | (uintptr_t)C32 | (uintptr_t)pre32 | (uintptr_t)C16) & 15)
    return SCTLGPU_ERR_INVALID_ARGUMENT;
  int dev;
  unsigned* status;
  int sms;
  int rc = runtime_device(&dev, &status, &sms);
  if (rc) return rc;
  TcParams p{};
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
  return runtime_record(tc_gemm_launch(p, (cudaStream_t)stream));
}
