// Device-side building blocks shared by the sctlgpu kernels (sm_103a only):
// mbarrier + cp.async.bulk (TMA bulk copy) wrappers with bounded waits, the
// hardware rsqrt estimates, and double-float (two-FP32) error-free transforms.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ < 1000)
#error "sctlgpu is written for sm_103a (Blackwell Ultra); build with -gencode arch=compute_103a,code=sm_103a"
#endif

namespace sctlgpu {

// Device-side status word bits (one word per device, read by sctlgpu_device_status).
enum : unsigned { kStatusTimeout = 1u };

// Upper bound on mbarrier polls before a wait gives up (each poll may itself
// suspend for a bounded hardware time slice, so this is seconds, not cycles).
constexpr uint32_t kWaitLimit = 1u << 22;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Makes the mbarrier initialisation visible to the async (TMA) proxy.
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Orders this thread's prior generic-proxy shared-memory accesses before
// subsequent async-proxy (bulk copy) writes to the same buffer.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// 1-D bulk copy global -> shared (TMA engine), completion counted on `bar`.
// dst, src and bytes must be multiples of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for phase `parity` of `bar`.  Returns false (and raises the
// device status word) if the limit is reached; the caller then carries on
// with whatever the buffer holds, so every thread still reaches the same
// barriers and the kernel ends normally with an error the host reports.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, unsigned* status) {
  for (uint32_t i = 0; i < kWaitLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  if (status) atomicOr(status, kStatusTimeout);
  return false;
}

// ---------------------------------------------------------------- rsqrt seeds
// Hardware estimates (MUFU.RSQ / MUFU.RSQ64H); refinement is done by the
// callers with Newton steps whose count follows the reference's schedule.
__device__ __forceinline__ float rsqrt_seed(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ double rsqrt_seed(double x) {
  double y;
  asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  return y;
}

// Newton-Raphson for 1/sqrt(x): y <- y * (3/2 - (x/2) y^2), `hx` = x/2.
template <int N, class R>
__device__ __forceinline__ R newton_rsqrt(R y, R hx) {
#pragma unroll
  for (int i = 0; i < N; ++i) {
    const R t = hx * y;
    y = y * fma(-t, y, R(1.5));
  }
  return y;
}

// ------------------------------------------------------------- double-float
// Unnormalised pair h + l with |l| << |h|; error-free transforms after
// Knuth (TwoSum) and Dekker/FMA (TwoProduct).  The rounded products and sums
// these rely on are written as __fmul_rn / __fadd_rn: the compiler never
// merges those into a multiply-add, which would replace a rounded product
// feeding a TwoSum by the exact one and break the transformation.
struct f2 {
  float h, l;
};

__device__ __forceinline__ f2 two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = s - a;
  const float e = (a - (s - bb)) + (b - bb);
  return {s, e};
}
__device__ __forceinline__ f2 fast_two_sum(float a, float b) {  // requires |a| >= |b| or a == 0
  const float s = __fadd_rn(a, b);
  return {s, b - (s - a)};
}
__device__ __forceinline__ f2 two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return {p, fmaf(a, b, -p)};
}
__device__ __forceinline__ f2 df_norm(f2 x) { return fast_two_sum(x.h, x.l); }
__device__ __forceinline__ f2 df_mul(f2 x, f2 y) {
  const float p = __fmul_rn(x.h, y.h);
  float e = fmaf(x.h, y.h, -p);
  e = fmaf(x.h, y.l, e);
  e = fmaf(x.l, y.h, e);
  return {p, e};
}
__device__ __forceinline__ f2 df_mulf(f2 x, float y) {
  const float p = __fmul_rn(x.h, y);
  float e = fmaf(x.h, y, -p);
  e = fmaf(x.l, y, e);
  return {p, e};
}
__device__ __forceinline__ f2 df_add(f2 x, f2 y) {
  f2 s = two_sum(x.h, y.h);
  s.l += x.l + y.l;
  return s;
}
// acc += x, accumulator kept as an unnormalised pair.
__device__ __forceinline__ void df_acc(f2& acc, f2 x) {
  const f2 s = two_sum(acc.h, x.h);
  acc.h = s.h;
  acc.l += s.l + x.l;
}

// Kahan-compensated FP32 accumulator.
struct kahan {
  float s, c;
};
__device__ __forceinline__ void kahan_add(kahan& a, float x) {
  const float y = x - a.c;
  const float t = a.s + y;
  a.c = (t - a.s) - y;
  a.s = t;
}

}  // namespace sctlgpu
