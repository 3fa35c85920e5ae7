// Tiled direct-sum kernels for GenericKernel::Eval (generic-kernel.txx:102-211)
// on sm_103a.
//
// Work decomposition: a CTA owns THREADS*T targets (held in registers, T per
// thread) and one contiguous chunk of the source list (grid.y splits the
// sources so small target counts still fill 152 SMs).  Sources arrive as
// packed records (see pack_*), staged into shared memory one tile at a time
// by the TMA bulk-copy engine (cp.async.bulk + mbarrier, double-buffered),
// and every thread sweeps the tile with broadcast shared-memory loads.  Each
// CTA writes one FP64 partial sum per (target, component); a final kernel
// adds the partials in a fixed order, applies uKerScaleFactor and
// (optionally) accumulates into v_trg -- so results are deterministic.
//
// Arithmetic modes (template MODE):
//   MODE_F64   FP64 everywhere; rsqrt.approx.f64 seed + Newton per digits.
//   MODE_F32   FP32 everywhere; rsqrt.approx.f32 seed + Newton per digits.
//   MODE_MXLO  FP64 inputs, FP32 arithmetic (digits <= 7): coordinates split
//              hi+lo on a common grid so x_t - y_s is formed to ~1e-14 of the
//              bounding box, Kahan-compensated FP32 accumulation.
//   MODE_MXDF  FP64 inputs, double-float arithmetic in the FP32 pipe (digits
//              8..11): exact hi differences, exact r^2 via TwoProduct/TwoSum,
//              one Newton step on the double-float residual, double-float
//              products and accumulation.  No FP64 instruction per pair: the
//              FP64 pipe of GB300 is a small fraction of its FP32 pipe.
#pragma once

#include <type_traits>

#include "common.cuh"

namespace sctlgpu {

enum { KER_LFXU = 0, KER_LDXU = 1, KER_SFXU = 2, KER_SDXU = 3 };
// Internal: the Stokes double layer of a symmetric 3 x 3 density S per source (the treecode's
// proxies carry the symmetric part of the moment sum_s L_k(y_s) n_s (x) f_s), u = 3/(4 pi) r
// (r . S r) / r^5 -- records hold diag(S) as the "normal" and (2 S01, 2 S02, 2 S12) as the
// "density".  Near-batch plans only (FP64, mixed FP32 and packed double-float arithmetic).
enum { KER_SDXU_SYM = 4 };
enum { MODE_F64 = 0, MODE_F32 = 1, MODE_MXLO = 2, MODE_MXDF = 3 };

template <int KER>
constexpr double scale_of() {  // uKerScaleFactor, kernel_functions.hpp:40,69,133,188
  constexpr double pi = 3.14159265358979323846264338327950288;
  return KER == 2 ? 1.0 / (8.0 * pi) : (KER == 3 || KER == 4) ? 3.0 / (4.0 * pi) : 1.0 / (4.0 * pi);
}

template <int KER>
struct KDims;
template <> struct KDims<KER_LFXU> { static constexpr int ND = 0, K0 = 1, K1 = 1; };
template <> struct KDims<KER_LDXU> { static constexpr int ND = 3, K0 = 1, K1 = 1; };
template <> struct KDims<KER_SFXU> { static constexpr int ND = 0, K0 = 3, K1 = 3; };
template <> struct KDims<KER_SDXU> { static constexpr int ND = 3, K0 = 3, K1 = 3; };
template <> struct KDims<KER_SDXU_SYM> { static constexpr int ND = 3, K0 = 3, K1 = 3; };

// Grid shared by all points of one mixed-precision call: x = o + xh + xl with
// xh a float on the grid g = L*2^-23 (|x-o| <= L, L a power of two), so the
// difference of two hi parts is exact in FP32.
struct MixedFrame {
  double o[3];
  double g, inv_g;
};

// Per-call bounding box accumulated on the device (order-preserving integer
// images of doubles so atomicMin/atomicMax work).
struct BBox {
  unsigned long long lo[3], hi[3];
};

__device__ __forceinline__ unsigned long long ordered_bits(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double from_ordered_bits(unsigned long long b) {
  return __longlong_as_double((long long)((b >> 63) ? (b & 0x7fffffffffffffffull) : ~b));
}

__device__ __forceinline__ MixedFrame frame_from_bbox(const BBox* bb) {
  MixedFrame f;
  double half = 0;
  for (int k = 0; k < 3; ++k) {
    const double lo = from_ordered_bits(bb->lo[k]), hi = from_ordered_bits(bb->hi[k]);
    f.o[k] = 0.5 * lo + 0.5 * hi;
    half = fmax(half, fmax(hi - f.o[k], f.o[k] - lo));
  }
  // L = smallest power of two >= half (with a margin for the rounding of o).
  int e;
  frexp(half * (1.0 + 1e-12) + 1e-300, &e);
  f.g = ldexp(1.0, e - 23);
  f.inv_g = ldexp(1.0, 23 - e);
  return f;
}

// Split a coordinate on the frame's grids: hi on g (|hi| <= 2^23 g), lo on
// g*2^-24 (|lo| <= g/2).  Both are exact floats, and so are the differences
// hi_t - hi_s and lo_t - lo_s of any two points: a coordinate difference is
// the exact sum of two floats, accurate to g*2^-25 (47 bits of the box).
__device__ __forceinline__ void split_coord(const MixedFrame& f, int k, double x, float& h, float& l) {
  const double d = x - f.o[k];
  const double q = rint(d * f.inv_g) * f.g;
  h = (float)q;
  l = (float)(rint((d - q) * f.inv_g * 16777216.0) * (f.g * (1.0 / 16777216.0)));
}
__device__ __forceinline__ void split_val(double x, float& h, float& l) {
  h = (float)x;
  l = (float)(x - (double)h);
}

// ------------------------------------------------------------------ records
// Packed source records (multiples of 16 bytes, so a tile is one bulk copy).
template <int KER, int MODE>
struct Rec;
// FP64
template <> struct Rec<KER_LFXU, MODE_F64> { double x, y, z, f; };
template <> struct Rec<KER_LDXU, MODE_F64> { double x, y, z, m0, m1, m2; };  // m = f n
template <> struct Rec<KER_SFXU, MODE_F64> { double x, y, z, f0, f1, f2; };
template <> struct Rec<KER_SDXU, MODE_F64> { double x, y, z, n0, n1, n2, f0, f1, f2, pad; };
// FP32
template <> struct Rec<KER_LFXU, MODE_F32> { float x, y, z, f; };
template <> struct Rec<KER_LDXU, MODE_F32> { float x, y, z, m0, m1, m2, pad0, pad1; };
template <> struct Rec<KER_SFXU, MODE_F32> { float x, y, z, f0, f1, f2, pad0, pad1; };
template <> struct Rec<KER_SDXU, MODE_F32> { float x, y, z, n0, n1, n2, f0, f1, f2, pad0, pad1, pad2; };
// Mixed (hi/lo pairs); the same records serve MODE_MXLO and MODE_MXDF.
template <> struct Rec<KER_LFXU, MODE_MXDF> { float xh, yh, zh, fh, xl, yl, zl, fl; };
template <> struct Rec<KER_LDXU, MODE_MXDF> { float xh, yh, zh, mh0, xl, yl, zl, ml0, mh1, mh2, ml1, ml2; };
template <> struct Rec<KER_SFXU, MODE_MXDF> { float xh, yh, zh, fh0, xl, yl, zl, fl0, fh1, fh2, fl1, fl2; };
template <> struct Rec<KER_SDXU, MODE_MXDF> {
  float xh, yh, zh, fh0, xl, yl, zl, fl0, fh1, fh2, fl1, fl2, nh0, nh1, nh2, p0, nl0, nl1, nl2, p1;
};
template <> struct Rec<KER_SDXU_SYM, MODE_F64> : Rec<KER_SDXU, MODE_F64> {};  // n: diag(S), f: 2 S_ij
template <> struct Rec<KER_SDXU_SYM, MODE_F32> : Rec<KER_SDXU, MODE_F32> {};
template <> struct Rec<KER_SDXU_SYM, MODE_MXDF> : Rec<KER_SDXU, MODE_MXDF> {};
template <int KER> struct Rec<KER, MODE_MXLO> : Rec<KER, MODE_MXDF> {};

// ----------------------------------------------------------------- packing
template <class Real>
__global__ void bbox_kernel(int64_t n, const Real* __restrict__ x, BBox* bb) {
  unsigned long long lo[3] = {~0ull, ~0ull, ~0ull}, hi[3] = {0, 0, 0};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    for (int k = 0; k < 3; ++k) {
      const unsigned long long b = ordered_bits((double)x[i * 3 + k]);
      lo[k] = b < lo[k] ? b : lo[k];
      hi[k] = b > hi[k] ? b : hi[k];
    }
  }
  for (int k = 0; k < 3; ++k) {
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long a = __shfl_xor_sync(0xffffffffu, lo[k], o);
      const unsigned long long b = __shfl_xor_sync(0xffffffffu, hi[k], o);
      lo[k] = a < lo[k] ? a : lo[k];
      hi[k] = b > hi[k] ? b : hi[k];
    }
  }
  if ((threadIdx.x & 31) == 0) {
    for (int k = 0; k < 3; ++k) {
      atomicMin(&bb->lo[k], lo[k]);
      atomicMax(&bb->hi[k], hi[k]);
    }
  }
}

// Packs AoS sources into records; `w` (optional) scales every density, the
// quadrature weight of a source node in a near-field correction.
template <int KER, int MODE, class Real>
__global__ void pack_sources_kernel(int64_t ns, const Real* __restrict__ xs, const Real* __restrict__ nrm,
                                    const Real* __restrict__ f, Rec<KER, MODE>* __restrict__ out, const BBox* bb,
                                    const Real* __restrict__ w = nullptr) {
  using R = Rec<KER, MODE>;
  MixedFrame fr;
  if (MODE == MODE_MXDF || MODE == MODE_MXLO) fr = frame_from_bbox(bb);
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < ns; s += (int64_t)gridDim.x * blockDim.x) {
    R r;
    memset(&r, 0, sizeof(R));
    if constexpr (MODE == MODE_F64 || MODE == MODE_F32) {
      const Real ws = w ? w[s] : Real(1);
      r.x = xs[s * 3 + 0];
      r.y = xs[s * 3 + 1];
      r.z = xs[s * 3 + 2];
      if constexpr (KER == KER_LFXU) {
        r.f = f[s] * ws;
      } else if constexpr (KER == KER_LDXU) {  // fold the density into the normal: m = f n
        const Real fs = f[s] * ws;
        r.m0 = fs * nrm[s * 3 + 0];
        r.m1 = fs * nrm[s * 3 + 1];
        r.m2 = fs * nrm[s * 3 + 2];
      } else if constexpr (KER == KER_SFXU) {
        r.f0 = f[s * 3 + 0] * ws;
        r.f1 = f[s * 3 + 1] * ws;
        r.f2 = f[s * 3 + 2] * ws;
      } else {
        r.n0 = nrm[s * 3 + 0];
        r.n1 = nrm[s * 3 + 1];
        r.n2 = nrm[s * 3 + 2];
        r.f0 = f[s * 3 + 0] * ws;
        r.f1 = f[s * 3 + 1] * ws;
        r.f2 = f[s * 3 + 2] * ws;
      }
    } else {
      const double ws = w ? (double)w[s] : 1.0;
      split_coord(fr, 0, (double)xs[s * 3 + 0], r.xh, r.xl);
      split_coord(fr, 1, (double)xs[s * 3 + 1], r.yh, r.yl);
      split_coord(fr, 2, (double)xs[s * 3 + 2], r.zh, r.zl);
      if constexpr (KER == KER_LFXU) {
        split_val((double)f[s] * ws, r.fh, r.fl);
      } else if constexpr (KER == KER_LDXU) {
        const double fs = (double)f[s] * ws;
        split_val(fs * (double)nrm[s * 3 + 0], r.mh0, r.ml0);
        split_val(fs * (double)nrm[s * 3 + 1], r.mh1, r.ml1);
        split_val(fs * (double)nrm[s * 3 + 2], r.mh2, r.ml2);
      } else {
        split_val((double)f[s * 3 + 0] * ws, r.fh0, r.fl0);
        split_val((double)f[s * 3 + 1] * ws, r.fh1, r.fl1);
        split_val((double)f[s * 3 + 2] * ws, r.fh2, r.fl2);
        if constexpr (KER == KER_SDXU || KER == KER_SDXU_SYM) {
          split_val((double)nrm[s * 3 + 0], r.nh0, r.nl0);
          split_val((double)nrm[s * 3 + 1], r.nh1, r.nl1);
          split_val((double)nrm[s * 3 + 2], r.nh2, r.nl2);
        }
      }
    }
    out[s] = r;
  }
}

// ------------------------------------------------------------ pair kernels
// Per-mode target state + per-pair update.  K1 = TrgDim accumulators.

template <int KER, int MODE, int NEWTON>
struct Pair;

// ---- plain FP64 / FP32 ---------------------------------------------------
template <int KER, class Real, int NEWTON>
struct PlainPair {
  static constexpr int K1 = KDims<KER>::K1;
  struct Trg {
    Real x[3];
    Real acc[K1];
  };
  template <class Src>
  __device__ static void load_trg(Trg& t, const Src* r, int64_t i, const MixedFrame&) {
    t.x[0] = (Real)r[i * 3 + 0];
    t.x[1] = (Real)r[i * 3 + 1];
    t.x[2] = (Real)r[i * 3 + 2];
#pragma unroll
    for (int k = 0; k < K1; ++k) t.acc[k] = 0;
  }
  __device__ __forceinline__ static void flush(Trg&) {}
  __device__ static double result(const Trg& t, int k) { return (double)t.acc[k]; }
  __device__ static void add_partial(Trg& t, int k, double v) { t.acc[k] += (Real)v; }

  template <class RecT>
  __device__ __forceinline__ static void apply(Trg& t, const RecT& s) {
    const Real d0 = t.x[0] - s.x, d1 = t.x[1] - s.y, d2 = t.x[2] - s.z;
    const Real r2 = fma(d2, d2, fma(d1, d1, d0 * d0));
    Real y = rsqrt_seed(r2);
    y = newton_rsqrt<NEWTON>(y, Real(0.5) * r2);
    y = r2 > Real(0) ? y : Real(0);
    if constexpr (KER == KER_LFXU) {
      t.acc[0] = fma(s.f, y, t.acc[0]);
    } else if constexpr (KER == KER_LDXU) {
      const Real dm = fma(d2, s.m2, fma(d1, s.m1, d0 * s.m0));
      t.acc[0] = fma(dm, y * y * y, t.acc[0]);
    } else if constexpr (KER == KER_SFXU) {
      const Real y3 = y * y * y;
      const Real fd = fma(d2, s.f2, fma(d1, s.f1, d0 * s.f0)) * y3;
      t.acc[0] = fma(s.f0, y, fma(d0, fd, t.acc[0]));
      t.acc[1] = fma(s.f1, y, fma(d1, fd, t.acc[1]));
      t.acc[2] = fma(s.f2, y, fma(d2, fd, t.acc[2]));
    } else {
      const Real y2 = y * y;
      const Real y5 = y2 * y2 * y;
      Real q;
      if constexpr (KER == KER_SDXU) {
        const Real dn = fma(d2, s.n2, fma(d1, s.n1, d0 * s.n0));
        const Real fd = fma(d2, s.f2, fma(d1, s.f1, d0 * s.f0));
        q = fd * dn;
      } else {  // r . S r: diag(S) in n, (2 S01, 2 S02, 2 S12) in f
        q = fma(s.n0 * d0, d0, fma(s.n1 * d1, d1, fma(s.n2 * d2, d2, fma(s.f0 * d0, d1, fma(s.f1 * d0, d2, s.f2 * d1 * d2)))));
      }
      const Real c = q * y5;
      t.acc[0] = fma(d0, c, t.acc[0]);
      t.acc[1] = fma(d1, c, t.acc[1]);
      t.acc[2] = fma(d2, c, t.acc[2]);
    }
  }
};
template <int KER, int NEWTON> struct Pair<KER, MODE_F64, NEWTON> : PlainPair<KER, double, NEWTON> {};
template <int KER, int NEWTON> struct Pair<KER, MODE_F32, NEWTON> : PlainPair<KER, float, NEWTON> {};

// ---- mixed, FP32 arithmetic (digits <= 7) ----------------------------------
template <int KER, int NEWTON>
struct Pair<KER, MODE_MXLO, NEWTON> {
  static constexpr int K1 = KDims<KER>::K1;
  struct Trg {
    float xh[3], xl[3];
    kahan acc[K1];   // compensated FP32 sum over the current source tile
    double tot[K1];  // FP64 sum of the tile sums
  };
  __device__ static void load_trg(Trg& t, const double* r, int64_t i, const MixedFrame& fr) {
#pragma unroll
    for (int k = 0; k < 3; ++k) split_coord(fr, k, r[i * 3 + k], t.xh[k], t.xl[k]);
#pragma unroll
    for (int k = 0; k < K1; ++k) {
      t.acc[k] = {0.f, 0.f};
      t.tot[k] = 0.0;
    }
  }
  __device__ __forceinline__ static void flush(Trg& t) {
#pragma unroll
    for (int k = 0; k < K1; ++k) {
      t.tot[k] += (double)t.acc[k].s - (double)t.acc[k].c;
      t.acc[k] = {0.f, 0.f};
    }
  }
  __device__ static double result(const Trg& t, int k) {
    return t.tot[k] + ((double)t.acc[k].s - (double)t.acc[k].c);
  }
  __device__ static void add_partial(Trg& t, int k, double v) { t.tot[k] += v; }

  template <class RecT>
  __device__ __forceinline__ static void apply(Trg& t, const RecT& s) {
    const float d0 = (t.xh[0] - s.xh) + (t.xl[0] - s.xl);
    const float d1 = (t.xh[1] - s.yh) + (t.xl[1] - s.yl);
    const float d2 = (t.xh[2] - s.zh) + (t.xl[2] - s.zl);
    const float r2 = fmaf(d2, d2, fmaf(d1, d1, d0 * d0));
    float y = rsqrt_seed(r2);
    y = newton_rsqrt<NEWTON>(y, 0.5f * r2);
    y = r2 > 0.f ? y : 0.f;
    if constexpr (KER == KER_LFXU) {
      kahan_add(t.acc[0], s.fh * y);
    } else if constexpr (KER == KER_LDXU) {
      const float dm = fmaf(d2, s.mh2, fmaf(d1, s.mh1, d0 * s.mh0));
      kahan_add(t.acc[0], dm * (y * y * y));
    } else if constexpr (KER == KER_SFXU) {
      const float y3 = y * y * y;
      const float fd = fmaf(d2, s.fh2, fmaf(d1, s.fh1, d0 * s.fh0)) * y3;
      kahan_add(t.acc[0], fmaf(s.fh0, y, d0 * fd));
      kahan_add(t.acc[1], fmaf(s.fh1, y, d1 * fd));
      kahan_add(t.acc[2], fmaf(s.fh2, y, d2 * fd));
    } else {
      const float y2 = y * y;
      const float y5 = y2 * y2 * y;
      float q;
      if constexpr (KER == KER_SDXU) {
        const float dn = fmaf(d2, s.nh2, fmaf(d1, s.nh1, d0 * s.nh0));
        const float fd = fmaf(d2, s.fh2, fmaf(d1, s.fh1, d0 * s.fh0));
        q = fd * dn;
      } else {  // r . S r: diag(S) in n, (2 S01, 2 S02, 2 S12) in f
        q = fmaf(s.nh0 * d0, d0, fmaf(s.nh1 * d1, d1, fmaf(s.nh2 * d2, d2,
                 fmaf(s.fh0 * d0, d1, fmaf(s.fh1 * d0, d2, s.fh2 * d1 * d2)))));
      }
      const float c = q * y5;
      kahan_add(t.acc[0], d0 * c);
      kahan_add(t.acc[1], d1 * c);
      kahan_add(t.acc[2], d2 * c);
    }
  }
};

// ---- mixed, double-float (digits 8..11) -------------------------------------
// Exact dot product a.b of double-float 3-vectors (a_i = ah_i + al_i), as a
// normalised pair; used where cancellation is expected (r.n near a surface).
__device__ __forceinline__ f2 df_dot3(const float (&ah)[3], const float (&al)[3], float bh0, float bh1, float bh2,
                                      float bl0, float bl1, float bl2) {
  const f2 p0 = two_prod(ah[0], bh0), p1 = two_prod(ah[1], bh1), p2 = two_prod(ah[2], bh2);
  const f2 s1 = two_sum(p0.h, p1.h);
  const f2 s2 = two_sum(s1.h, p2.h);
  float lo = (p0.l + p1.l) + (p2.l + s1.l) + s2.l;
  lo = fmaf(ah[0], bl0, fmaf(al[0], bh0, lo));
  lo = fmaf(ah[1], bl1, fmaf(al[1], bh1, lo));
  lo = fmaf(ah[2], bl2, fmaf(al[2], bh2, lo));
  return fast_two_sum(s2.h, lo);
}

template <int KER, int NEWTON>
struct Pair<KER, MODE_MXDF, NEWTON> {
  static constexpr int K1 = KDims<KER>::K1;
  struct Trg {
    float xh[3], xl[3];
    f2 acc[K1];      // double-float sum over the current source tile
    double tot[K1];  // FP64 sum of the tile sums
  };
  __device__ static void load_trg(Trg& t, const double* r, int64_t i, const MixedFrame& fr) {
#pragma unroll
    for (int k = 0; k < 3; ++k) split_coord(fr, k, r[i * 3 + k], t.xh[k], t.xl[k]);
#pragma unroll
    for (int k = 0; k < K1; ++k) {
      t.acc[k] = {0.f, 0.f};
      t.tot[k] = 0.0;
    }
  }
  // Once per tile: move the tile's double-float sum into FP64 so the pair
  // accumulator stays small and its rounding stays below 2^-48 of the result.
  __device__ __forceinline__ static void flush(Trg& t) {
#pragma unroll
    for (int k = 0; k < K1; ++k) {
      t.tot[k] += (double)t.acc[k].h + (double)t.acc[k].l;
      t.acc[k] = {0.f, 0.f};
    }
  }
  __device__ static double result(const Trg& t, int k) {
    return t.tot[k] + ((double)t.acc[k].h + (double)t.acc[k].l);
  }
  __device__ static void add_partial(Trg& t, int k, double v) { t.tot[k] += v; }

  template <class RecT>
  __device__ __forceinline__ static void apply(Trg& t, const RecT& s) {
    // r = x_t - y_s: hi and lo differences are exact (common grids); Fast2Sum
    // renormalises each component to D + d with |d| <= ulp(D)/2.
    float dh[3], dl[3];
    {
      const float sh[3] = {s.xh, s.yh, s.zh}, sl[3] = {s.xl, s.yl, s.zl};
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const f2 v = fast_two_sum(t.xh[i] - sh[i], t.xl[i] - sl[i]);
        dh[i] = v.h;
        dl[i] = v.l;
      }
    }
    // r^2 = R + Rl exactly up to the rounding of Rl.
    const f2 p0 = two_prod(dh[0], dh[0]), p1 = two_prod(dh[1], dh[1]), p2 = two_prod(dh[2], dh[2]);
    const f2 s1 = two_sum(p0.h, p1.h);
    const f2 s2 = two_sum(s1.h, p2.h);
    const float R = s2.h;
    float Rl = fmaf(dh[2], dl[2], fmaf(dh[1], dl[1], dh[0] * dl[0]));
    Rl = fmaf(2.f, Rl, (p0.l + p1.l) + (p2.l + s1.l) + s2.l);
    float y0 = rsqrt_seed(R);
    y0 = R > 0.f ? y0 : 0.f;
    // One Newton step on the exact residual rho = 1 - y0^2 (R + Rl).
    const f2 q = two_prod(y0, y0);
    float rho = fmaf(-q.h, R, 1.f);
    rho = fmaf(-q.l, R, rho);
    rho = fmaf(-q.h, Rl, rho);
    const f2 y = {y0, (0.5f * y0) * rho};  // 1/r = y.h + y.l
    if constexpr (KER == KER_LFXU) {
      df_acc(t.acc[0], df_mul(y, f2{s.fh, s.fl}));
    } else {
      // y^3 = y0^3 (1 + 3 rho / 2) to O(rho^2)
      const f2 y3 = [&] {
        f2 c = df_mulf(q, y0);
        c.l = fmaf(c.h, 1.5f * rho, c.l);
        return c;
      }();
      if constexpr (KER == KER_LDXU) {
        const f2 dm = df_dot3(dh, dl, s.mh0, s.mh1, s.mh2, s.ml0, s.ml1, s.ml2);
        df_acc(t.acc[0], df_mul(dm, y3));
      } else if constexpr (KER == KER_SFXU) {
        const f2 fd = df_mul(df_dot3(dh, dl, s.fh0, s.fh1, s.fh2, s.fl0, s.fl1, s.fl2), y3);
        const float fh[3] = {s.fh0, s.fh1, s.fh2}, fl[3] = {s.fl0, s.fl1, s.fl2};
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          df_acc(t.acc[i], df_mul(f2{fh[i], fl[i]}, y));
          df_acc(t.acc[i], df_mul(f2{dh[i], dl[i]}, fd));
        }
      } else {
        // y^5 = y0^5 (1 + 5 rho / 2)
        const f2 q2 = df_mul(q, q);
        f2 y5 = df_mulf(q2, y0);
        y5.l = fmaf(y5.h, 2.5f * rho, y5.l);
        const f2 dn = df_dot3(dh, dl, s.nh0, s.nh1, s.nh2, s.nl0, s.nl1, s.nl2);
        const f2 fd = df_dot3(dh, dl, s.fh0, s.fh1, s.fh2, s.fl0, s.fl1, s.fl2);
        const f2 c = df_mul(df_mul(fd, dn), y5);
#pragma unroll
        for (int i = 0; i < 3; ++i) df_acc(t.acc[i], df_mul(f2{dh[i], dl[i]}, c));
      }
    }
  }
};

// ----------------------------------------------------------- main kernel
__device__ __forceinline__ int64_t imin64(int64_t a, int64_t b) { return a < b ? a : b; }

struct DirectParams {
  int64_t nt, ns;
  const void* r_trg;   // AoS, Real (double for mixed)
  const void* recs;    // packed source records
  int64_t chunk;       // sources per grid.y slice (multiple of the tile size)
  double* partial;     // [grid.y][nt][K1]
  const BBox* bbox;    // mixed modes only
  unsigned* status;    // device status word
};

template <int KER, int MODE>
struct TileCfg {
  static constexpr int THREADS = 128;
  static constexpr int T = (MODE == MODE_F32) ? 4 : (MODE == MODE_MXDF && KER >= KER_SFXU) ? 1 : 2;
  static constexpr int S = 256;  // records per shared-memory tile
};

template <int KER, int MODE, int NEWTON>
__global__ void __launch_bounds__(TileCfg<KER, MODE>::THREADS)
    direct_sum_kernel(DirectParams p) {
  using P = Pair<KER, MODE, NEWTON>;
  using RecT = Rec<KER, MODE>;
  using Cfg = TileCfg<KER, MODE>;
  constexpr int THREADS = Cfg::THREADS, T = Cfg::T, S = Cfg::S, K1 = KDims<KER>::K1;
  static_assert(sizeof(RecT) % 16 == 0, "records must be a multiple of 16 bytes");

  extern __shared__ __align__(128) unsigned char smem_raw[];
  RecT* tiles = reinterpret_cast<RecT*>(smem_raw);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + 2 * S * sizeof(RecT));

  const int64_t t0 = (int64_t)blockIdx.x * THREADS * T;
  const int64_t s_begin = (int64_t)blockIdx.y * p.chunk;
  const int64_t s_end = imin64(p.ns, s_begin + p.chunk);
  const int64_t n_src = s_end - s_begin;
  const int ntiles = (int)((n_src + S - 1) / S);
  const RecT* src = reinterpret_cast<const RecT*>(p.recs) + s_begin;

  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int b = 0; b < 2 && b < ntiles; ++b) {
      const uint32_t cnt = (uint32_t)imin64((int64_t)S, n_src - (int64_t)b * S);
      mbar_arrive_expect_tx(&bars[b], cnt * (uint32_t)sizeof(RecT));
      bulk_g2s(tiles + b * S, src + (int64_t)b * S, cnt * (uint32_t)sizeof(RecT), &bars[b]);
    }
  }

  MixedFrame fr{};
  if constexpr (MODE == MODE_MXLO || MODE == MODE_MXDF) fr = frame_from_bbox(p.bbox);
  typename P::Trg tg[T];
  using TrgReal = typename std::conditional<MODE == MODE_F32, float, double>::type;
  const TrgReal* rt = reinterpret_cast<const TrgReal*>(p.r_trg);
#pragma unroll
  for (int j = 0; j < T; ++j) {
    const int64_t i = t0 + threadIdx.x + (int64_t)j * THREADS;
    P::load_trg(tg[j], rt, i < p.nt ? i : (p.nt - 1), fr);
  }

  bool timed_out = false;
  for (int k = 0; k < ntiles; ++k) {
    const int buf = k & 1;
    if (!mbar_wait_bounded(&bars[buf], (uint32_t)((k >> 1) & 1), p.status)) timed_out = true;
    const RecT* tile = tiles + buf * S;
    const int cnt = (int)imin64((int64_t)S, n_src - (int64_t)k * S);
#pragma unroll 2
    for (int s = 0; s < cnt; ++s) {
      const RecT rec = tile[s];
#pragma unroll
      for (int j = 0; j < T; ++j) P::apply(tg[j], rec);
    }
#pragma unroll
    for (int j = 0; j < T; ++j) P::flush(tg[j]);
    __syncthreads();  // every thread is done with this buffer
    if (threadIdx.x == 0 && k + 2 < ntiles) {
      fence_proxy_async_smem();
      const uint32_t c2 = (uint32_t)imin64((int64_t)S, n_src - (int64_t)(k + 2) * S);
      mbar_arrive_expect_tx(&bars[buf], c2 * (uint32_t)sizeof(RecT));
      bulk_g2s(tiles + buf * S, src + (int64_t)(k + 2) * S, c2 * (uint32_t)sizeof(RecT), &bars[buf]);
    }
  }
  if (timed_out && threadIdx.x == 0) {
    // Give copies still in flight (if any) a bounded chance to land before exit:
    // wait once more on the last phase each barrier was armed for.
    for (int b = 0; b < 2; ++b) {
      const int k_last = (ntiles - 1) - (((ntiles - 1) - b) & 1);
      if (k_last >= 0) mbar_wait_bounded(&bars[b], (uint32_t)((k_last >> 1) & 1), nullptr);
    }
  }

#pragma unroll
  for (int j = 0; j < T; ++j) {
    const int64_t i = t0 + threadIdx.x + (int64_t)j * THREADS;
    if (i < p.nt) {
#pragma unroll
      for (int k = 0; k < K1; ++k) p.partial[((int64_t)blockIdx.y * p.nt + i) * K1 + k] = P::result(tg[j], k);
    }
  }
}

template <class Real>
__global__ void reduce_partials_kernel(int64_t n, int nsplit, const double* __restrict__ partial, double scale,
                                       int accumulate, Real* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double acc = 0;
    for (int y = 0; y < nsplit; ++y) acc += partial[(int64_t)y * n + i];
    const double v = acc * scale;
    out[i] = accumulate ? (Real)((double)out[i] + v) : (Real)v;
  }
}

}  // namespace sctlgpu
