// Correctly rounded double of a double-float value h + l, built with integer
// operations.  GB300 runs FP64 arithmetic and float->double conversions at a
// small fraction of its FP32/integer issue rate, so a kernel that writes one
// FP64 result per double-float value (a kernel matrix) would otherwise be
// bound by the two conversions and the FP64 add of (double)h + (double)l.
//
// Method: Fast2Sum gives s + e = h + l exactly with |e| <= ulp(s)/2.  The
// double image of s is its float bit pattern with the exponent rebiased
// (+896) and the mantissa moved up 29 bits.  Adding e is an integer
// adjustment of that pattern by round-to-nearest-even(e / ulp_d), with ulp_d
// the double ulp at |s| (half of it when |s| is a power of two and the
// adjustment points down, where the result lands in the binade below).  The
// pattern's low 29 bits are zero, so rounding e alone and rounding the exact
// sum agree, ties included.  Zero, subnormal, huge, infinite and NaN values
// of s take the FP64 route.
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
SCTLGPU_DFC_HD int32_t dfc_rint(float x) {  // round to nearest, ties to even (|x| < 2^31)
#if defined(__CUDA_ARCH__)
  return __float2int_rn(x);
#else
  return (int32_t)std::lrintf(x);
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
  const float s = dfc_add(h, l);
  const float e = l - (s - h);
  const uint32_t sb = dfc_bits(s);
  const uint32_t E = (sb >> 23) & 0xffu;
  // 64 <= E <= 253 keeps the scale factor below a normal float and |s| far from overflow.
  if (E < 64u || E > 253u) return (double)h + (double)l;
  const uint32_t neg = sb >> 31;
  const float em = neg ? -e : e;  // adjustment of |s|
  const bool down = (sb & 0x7fffffu) == 0u && em < 0.f;
  // e / ulp_d = e * 2^k, ulp_d = 2^(E - 127 - 52) (half that below a power of two)
  const int32_t k = 179 - (int32_t)E + (down ? 1 : 0);
  const float t = em * dfc_float((uint32_t)(k + 127) << 23);  // exact: scaling by a power of two
  const int32_t n = dfc_rint(t);                              // |t| <= 2^28
  uint64_t mag = ((uint64_t)(sb & 0x7fffffffu) << 29) + (896ull << 52);
  mag += (uint64_t)(int64_t)n;
  return dfc_double(mag | ((uint64_t)neg << 63));
}

}  // namespace sctlgpu
