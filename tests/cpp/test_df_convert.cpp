// Host check of df_to_double (sctl_gb300/csrc/df_convert.h): the integer
// construction of the rounded double of h + l must equal the FP64 sum
// (double)h + (double)l bit for bit.  Cases: random magnitudes and signs,
// low parts spread over the whole range below ulp(h)/2, exact ties at the
// double's half-ulp, powers of two with low parts pointing down, zeros.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <random>

#include "../../sctl_gb300/csrc/df_convert.h"

using sctlgpu::df_to_double;

static uint64_t bits(double x) {
  uint64_t b;
  std::memcpy(&b, &x, 8);
  return b;
}

int main() {
  std::mt19937_64 rng(12345);
  std::uniform_real_distribution<double> u01(0.0, 1.0);
  long n = 0, bad = 0;
  auto check = [&](float h, float l) {
    if (!(std::fabs(l) <= std::fabs(h)) && h != 0.f) return;
    // the pair as an error-free transformation leaves it: h = fl(h + l)
    const float s = h + l;
    const float e = l - (s - h);
    const double want = (double)s + (double)e;
    const double got = df_to_double(h, l);
    ++n;
    if (bits(want) != bits(got) && !(want == 0.0 && got == 0.0)) {
      if (bad < 10) std::printf("mismatch h=%a l=%a want=%a got=%a\n", h, l, want, got);
      ++bad;
    }
  };
  for (int it = 0; it < 4000000; ++it) {
    const int eh = (int)(u01(rng) * 160.0) - 80;
    float h = (float)std::ldexp(1.0 + u01(rng), eh);
    if (rng() & 1) h = -h;
    const float ulp = (float)std::ldexp(1.0, eh - 23);
    float l;
    switch (it % 5) {
      case 0:  // anywhere below half an ulp of h
        l = (float)((u01(rng) - 0.5) * ulp);
        break;
      case 1:  // much smaller low parts (rounding decided deep in the double)
        l = (float)((u01(rng) - 0.5) * std::ldexp((double)ulp, -(int)(u01(rng) * 40)));
        break;
      case 2: {  // exact ties at half a double ulp of h: (m + 1/2) * 2^(eh - 52)
        const long m = (long)(u01(rng) * (1 << 20)) - (1 << 19);
        l = (float)std::ldexp((double)m + 0.5, eh - 52);
        break;
      }
      case 3: {  // powers of two with a low part pointing down (result in the binade below)
        h = (float)std::ldexp(rng() & 1 ? -1.0 : 1.0, eh);
        const long m = (long)(u01(rng) * (1 << 20));
        l = (float)(-std::copysign(std::ldexp((double)m + ((rng() & 1) ? 0.5 : 0.0), eh - 53), (double)h));
        if (std::fabs(l) > 0.25f * ulp) l = (float)(-std::copysign(0.2 * ulp * u01(rng), (double)h));
        break;
      }
      default:  // largest mantissa of a binade, low part pointing up
        h = (float)std::copysign(std::ldexp(2.0 - std::ldexp(1.0, -23), eh), (double)h);
        l = (float)std::copysign(0.5 * ulp * u01(rng), (double)h);
        break;
    }
    check(h, l);
  }
  // tiny, subnormal and huge magnitudes (rescaled), zeros, infinities, NaN
  for (int it = 0; it < 1000000; ++it) {
    const int eh = (int)(u01(rng) * 300.0) - 150;  // 2^-150 .. 2^150 (subnormal .. overflow)
    float h = (float)std::ldexp(1.0 + u01(rng), eh);
    if (rng() & 1) h = -h;
    const float l = (float)((u01(rng) - 0.5) * std::ldexp(1.0, eh - 23));
    if (std::isfinite(h)) check(h, l);
  }
  check(0.f, 0.f);
  check(-0.f, 0.f);
  check(-0.f, -0.f);
  check(1e-30f, 1e-40f);
  check(3e38f, 1e30f);
  check(-3.4e38f, -1e31f);
  check(1.0f, -1e-30f);
  check(1.0f, 1e-45f);  // subnormal low part
  check(1e-45f, 0.f);   // subnormal
  check(-1.2e-38f, 1e-45f);
  {
    const float inf = std::numeric_limits<float>::infinity();
    const float nan = std::numeric_limits<float>::quiet_NaN();
    ++n;
    if (!(df_to_double(inf, 0.f) == (double)inf && df_to_double(-inf, 0.f) == -(double)inf)) ++bad;
    ++n;
    if (!std::isnan(df_to_double(nan, 0.f))) ++bad;
  }
  std::printf("%ld cases, %ld mismatches\n", n, bad);
  return bad == 0 ? 0 : 1;
}
