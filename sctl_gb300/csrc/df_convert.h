// Correctly rounded double of a double-float value h + l, built with integer
// operations.  GB300 runs FP64 arithmetic and float->double conversions at a
// small fraction of its FP32/integer issue rate, so a kernel that writes one
// FP64 result per double-float value (a kernel matrix) would otherwise be
// bound by the two conversions and the FP64 add of (double)h + (double)l.
//
// Method: Fast2Sum gives s + e = h + l exactly with |e| <= ulp(s)/2.  The
// double image of s is its float bit pattern with the exponent rebiased
// (+896) and the mantissa moved up 29 bits.  Adding e is an integer
// adjustment of that pattern by round-to-nearest-even(|e| / ulp_d), with
// ulp_d the double ulp at |s| (half of it when |s| is a power of two and the
// adjustment points down, where the result lands in the binade below): one
// exact power-of-two scaling and one float-to-integer conversion.  The
// pattern's low 29 bits are zero, so rounding e alone and
// rounding the exact sum agree, ties included.  No FP64 instruction is
// issued, not even a predicated one: tiny, subnormal and huge values are
// rescaled by a power of two, zeros and non-finite values are selected.
//
// The same code compiles for the host (g++), where a unit test compares it
// with (double)h + (double)l over millions of cases.
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define SCTLGPU_DFC_HD __host__ __device__ __forceinline__
#else
#include <cmath>
#define SCTLGPU_DFC_HD inline
#endif

namespace sctlgpu {

SCTLGPU_DFC_HD uint32_t dfc_bits(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  uint32_t u;
  std::memcpy(&u, &x, 4);
  return u;
#endif
}
SCTLGPU_DFC_HD float dfc_float(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float x;
  std::memcpy(&x, &u, 4);
  return x;
#endif
}
SCTLGPU_DFC_HD uint32_t dfc_rint(float x) {  // round to nearest, ties to even (0 <= x < 2^31)
#if defined(__CUDA_ARCH__)
  return (uint32_t)__float2int_rn(x);
#else
  return (uint32_t)std::lrintf(x);
#endif
}
// Rounded sum that is never merged with a product into a multiply-add.
SCTLGPU_DFC_HD float dfc_add(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
SCTLGPU_DFC_HD double dfc_double(uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)b);
#else
  double x;
  std::memcpy(&x, &b, 8);
  return x;
#endif
}

// h + l with |l| no larger than |h| (any double-float pair from an
// error-free transformation), rounded to nearest-even as a double.
SCTLGPU_DFC_HD double df_to_double(float h, float l) {
  float s = dfc_add(h, l);
  float e = l - (s - h);
  uint32_t sb = dfc_bits(s);
  uint32_t E = (sb >> 23) & 0xffu;
  // Outside 64 <= E <= 253 (tiny, subnormal or huge |s|) both parts are rescaled
  // by 2^100 or 2^-100 -- exact -- and the double's exponent is corrected at the
  // end; the common path runs the same (branch-free) instructions.
  const int32_t bias = E < 64u ? -100 : (E > 253u && E < 255u ? 100 : 0);
  const float f = bias < 0 ? 0x1p100f : (bias > 0 ? 0x1p-100f : 1.0f);
  s *= f;
  e *= f;
  sb = dfc_bits(s);
  E = (sb >> 23) & 0xffu;
  const uint32_t eb = dfc_bits(e);
  const bool flip = ((sb ^ eb) >> 31) != 0u;  // e points towards zero
  const bool down = (sb & 0x7fffffu) == 0u && flip && (eb & 0x7fffffffu) != 0u;
  // n = round-half-even(|e| / ulp_d), ulp_d = 2^(E - 179) (half that below a power of two):
  // |e| * 2^k is exact (a power-of-two scaling, <= 2^28 since |e| <= ulp_f(s) / 2).
  const int32_t k = 179 - (int32_t)E + (down ? 1 : 0);
  const uint32_t n = dfc_rint(dfc_float(eb & 0x7fffffffu) * dfc_float((uint32_t)(k + 127) << 23));
  uint64_t mag = ((uint64_t)(sb & 0x7fffffffu) << 29) + ((uint64_t)(896 + bias) << 52);
  mag = flip ? mag - n : mag + n;
  if ((sb & 0x7fffffffu) == 0u) mag = 0u;                            // zero
  if (E == 255u) mag = (0x7ffull << 52) | ((sb & 0x7fffffu) ? (1ull << 51) : 0u);  // inf, NaN
  return dfc_double(mag | ((uint64_t)(sb >> 31) << 63));
}

}  // namespace sctlgpu
