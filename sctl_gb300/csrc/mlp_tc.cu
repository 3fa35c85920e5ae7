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
#include <cmath>
#include <cstdint>
#include <random>
#include <vector>

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
  // optional fused epilogue: dot_out[row] += sum_{col < dot_cols} C[row][col] * dot_dens[dot_index[row]][col]
  const double* dot_dens;
  const int64_t* dot_index;
  int dot_cols;
  double* dot_out;
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
    double dot = 0.0;
    const double* dv = (p.dot_out && p.dot_index[row] >= 0) ? p.dot_dens + p.dot_index[row] * p.dot_cols : nullptr;
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
        if (dv && col < p.dot_cols) dot = fma((double)x, dv[col], dot);
      }
    }
    if (dv) p.dot_out[row] += dot;
  }
  if (!ok && tid == 0) mbar_wait_bounded(&bars[2], 0, nullptr);  // let in-flight MMAs land before TMEM is freed
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, ncols);
}

cudaError_t tc_gemm_launch(const TcParams& p, cudaStream_t st) {
  const size_t smem = 2 * TC_A_BYTES + 2 * TC_B_BYTES + 64;
  static bool attr[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && !attr[dev]) {
    cudaFuncSetAttribute(tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr[dev] = true;
  }
  tc_gemm_kernel<<<p.M / TC_M, TC_THREADS, smem, st>>>(p);
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return cudaGetLastError();
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
