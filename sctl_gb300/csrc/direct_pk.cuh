// Double-float direct sums on the packed FP32 pipe (fma/add/mul .f32x2) for
// SCTLGPU_MIXED at digits 8..11: GenericKernel::Eval (generic-kernel.txx:102-211)
// for Laplace3D_FxU/DxU and Stokes3D_FxU/DxU (kernel_functions.hpp:43-47,72-78,
// 136-145,191-201) evaluated in error-free FP32 transformations.
//
// Why packed: the double-float evaluation is ~150 FP32 operations per
// interaction, nearly all on the FMA pipe (128 lanes per SM per clock on
// GB300).  Issued one FP32 operation per instruction, the kernel is bound by
// the instruction issue rate (4 warp-instructions per SM per clock), so every
// load, MUFU, select and loop instruction costs an FMA slot.  Here each thread
// evaluates TWO sources at once -- source records are stored in pairs, lane x
// = source 2j, lane y = source 2j+1 -- so every FP32 operation is one
// fma/add/mul.rn.f32x2 instruction for two interactions, issue pressure
// halves, and the FMA pipe itself becomes the bound (ncu on Stokes3D_DxU: FMA
// pipe 81 % busy, "math pipe throttle" the leading stall; the unpacked kernel
// issued 171 instructions per interaction at 83 % of the issue rate with the
// FMA pipe at 78 %).  FFMA2 does not raise the FP32 rate itself -- GB300
// executes it in two FMA-pipe cycles (76.4 vs 75.7 TFLOP/s measured) -- so the
// gain is the issue slots handed back to the FMA pipe: 1.05-1.12x.  Operations
// that do not pair (the rsqrt seeds, the r = 0 mask, the max/min ordering of
// the non-negative squares) run on the MUFU and ALU pipes.
//
// The arithmetic is the same error-free evaluation as Pair<KER, MODE_MXDF>
// (direct.cuh): exact coordinate differences on the mixed frame's grids
// renormalised by Fast2Sum, r^2 exact to 2^-48 (TwoProduct + ordered Fast2Sum of
// the three non-negative squares), one Newton step on the exact residual
// 1 - y0^2 r^2, compensated dot products (TwoProduct + TwoSum), double-float
// products that keep every first-order term, and a double-float accumulator per
// lane flushed to FP64 once per tile.  Per-interaction relative error stays
// near 2^-44; second-order terms (lo x lo, ~2^-48) are the only ones dropped.
#pragma once

#include "direct.cuh"

namespace sctlgpu {

// ------------------------------------------------------------ packed FP32
using v2 = float2;

__device__ __forceinline__ v2 vdup(float a) { return make_float2(a, a); }
__device__ __forceinline__ v2 vneg(v2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ v2 vadd(v2 a, v2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ v2 vsub(v2 a, v2 b) { return __fadd2_rn(a, vneg(b)); }
__device__ __forceinline__ v2 vmul(v2 a, v2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ v2 vfma(v2 a, v2 b, v2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ v2 vmax(v2 a, v2 b) { return make_float2(fmaxf(a.x, b.x), fmaxf(a.y, b.y)); }
__device__ __forceinline__ v2 vmin(v2 a, v2 b) { return make_float2(fminf(a.x, b.x), fminf(a.y, b.y)); }

// A double-float value per lane: h + l, |l| <= ~2^-23 |h| (not necessarily normalised).
struct dv2 {
  v2 h, l;
};

// TwoProduct a*b = p + e exactly.
__device__ __forceinline__ dv2 vtwo_prod(v2 a, v2 b) {
  const v2 p = vmul(a, b);
  return {p, vfma(a, b, vneg(p))};
}

// a + b = s + e exactly (Knuth's TwoSum, 6 operations, no ordering needed).
__device__ __forceinline__ dv2 vtwo_sum(v2 a, v2 b) {
  const v2 s = vadd(a, b);
  const v2 bb = vsub(s, a);
  return {s, vadd(vsub(a, vsub(s, bb)), vsub(b, bb))};
}

// Fast2Sum of two non-negative values ordered by max/min (ALU pipe).
__device__ __forceinline__ dv2 vtwo_sum_pos(v2 a, v2 b) {
  const v2 big = vmax(a, b), sml = vmin(a, b);
  const v2 s = vadd(big, sml);
  return {s, vsub(sml, vsub(s, big))};
}

// Double-float product keeping all first-order terms (x.l * y.l ~ 2^-48 dropped).
__device__ __forceinline__ dv2 vdf_mul(dv2 x, dv2 y) {
  const v2 p = vmul(x.h, y.h);
  v2 e = vfma(x.h, y.h, vneg(p));
  e = vfma(x.h, y.l, e);
  e = vfma(x.l, y.h, e);
  return {p, e};
}

// acc += x (accumulator kept unnormalised; its hi part collects every rounding error).
__device__ __forceinline__ void vdf_acc(dv2& acc, dv2 x) {
  const dv2 s = vtwo_sum(acc.h, x.h);
  acc.h = s.h;
  acc.l = vadd(acc.l, vadd(s.l, x.l));
}

// Compensated dot product a . r of a double-float 3-vector a = ah + al (per
// source) with r = D + d, as an unnormalised pair.
__device__ __forceinline__ dv2 vdot3(const v2 (&ah)[3], const v2 (&al)[3], const v2 (&D)[3], const v2 (&d)[3]) {
  const dv2 p0 = vtwo_prod(ah[0], D[0]), p1 = vtwo_prod(ah[1], D[1]), p2 = vtwo_prod(ah[2], D[2]);
  const dv2 s1 = vtwo_sum(p0.h, p1.h);
  const dv2 s2 = vtwo_sum(s1.h, p2.h);
  v2 lo = vadd(vadd(vadd(p0.l, p1.l), vadd(p2.l, s1.l)), s2.l);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    lo = vfma(ah[i], d[i], lo);
    lo = vfma(al[i], D[i], lo);
  }
  return {s2.h, lo};
}

// ------------------------------------------------------------ pair records
// Two sources per record, lane x = source 2j, lane y = source 2j+1; the same
// fields as Rec<KER, MODE_MXDF> (coordinates hi/lo on the frame's grids,
// densities -- m = f n for Laplace3D_DxU -- and normals as hi + lo floats).
template <int KER>
struct RecPk;
template <> struct RecPk<KER_LFXU> { v2 xh, yh, zh, xl, yl, zl, fh, fl; };
template <> struct RecPk<KER_LDXU> { v2 xh, yh, zh, xl, yl, zl, mh0, mh1, mh2, ml0, ml1, ml2; };
template <> struct RecPk<KER_SFXU> { v2 xh, yh, zh, xl, yl, zl, fh0, fh1, fh2, fl0, fl1, fl2; };
template <> struct RecPk<KER_SDXU> {
  v2 xh, yh, zh, xl, yl, zl, fh0, fh1, fh2, fl0, fl1, fl2, nh0, nh1, nh2, nl0, nl1, nl2;
};
template <> struct RecPk<KER_SDXU_SYM> : RecPk<KER_SDXU> {};  // n: diag(S), f: 2 S01, 2 S02, 2 S12

// The pair record of sources sa (lane x) and sa + 1 (lane y); without a real
// second source (real_b false) lane y is a copy of sa with zero densities (it
// adds exactly 0).
template <int KER>
__device__ __forceinline__ RecPk<KER> pair_record(const MixedFrame& fr, int64_t sa, bool real_b,
                                                  const double* __restrict__ xs, const double* __restrict__ nrm,
                                                  const double* __restrict__ f, const double* __restrict__ w) {
  float v[2][18];
#pragma unroll
  for (int lane = 0; lane < 2; ++lane) {
    const bool real = lane == 0 || real_b;
    const int64_t s = real ? sa + lane : sa;
    const double ws = real ? (w ? w[s] : 1.0) : 0.0;
#pragma unroll
    for (int k = 0; k < 3; ++k) split_coord(fr, k, xs[s * 3 + k], v[lane][k], v[lane][3 + k]);
    if constexpr (KER == KER_LFXU) {
      split_val(f[s] * ws, v[lane][6], v[lane][7]);
    } else if constexpr (KER == KER_LDXU) {
      const double fs = f[s] * ws;
#pragma unroll
      for (int k = 0; k < 3; ++k) split_val(fs * nrm[s * 3 + k], v[lane][6 + k], v[lane][9 + k]);
    } else {
#pragma unroll
      for (int k = 0; k < 3; ++k) split_val(f[s * 3 + k] * ws, v[lane][6 + k], v[lane][9 + k]);
      if constexpr (KER == KER_SDXU || KER == KER_SDXU_SYM) {
#pragma unroll
        for (int k = 0; k < 3; ++k) split_val(nrm[s * 3 + k], v[lane][12 + k], v[lane][15 + k]);
      }
    }
  }
  constexpr int NF = sizeof(RecPk<KER>) / sizeof(v2);
  RecPk<KER> r;
  v2* rv = reinterpret_cast<v2*>(&r);
#pragma unroll
  for (int q = 0; q < NF; ++q) rv[q] = make_float2(v[0][q], v[1][q]);
  return r;
}

// One pair record per thread: sources 2j and 2j + 1 of the list (`w`, when
// given, weights every density, as in pack_sources_kernel).
template <int KER>
__global__ void pack_pairs_kernel(int64_t ns, const double* __restrict__ xs, const double* __restrict__ nrm,
                                  const double* __restrict__ f, RecPk<KER>* __restrict__ out, const BBox* bb,
                                  const double* __restrict__ w = nullptr) {
  const MixedFrame fr = frame_from_bbox(bb);
  const int64_t npairs = (ns + 1) / 2;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < npairs; j += (int64_t)gridDim.x * blockDim.x)
    out[j] = pair_record<KER>(fr, 2 * j, 2 * j + 1 < ns, xs, nrm, f, w);
}

// ------------------------------------------------------------ pair kernel
template <int KER>
struct PairPk {
  static constexpr int K1 = KDims<KER>::K1;
  struct Trg {
    v2 xh[3], xl[3];  // the target's split coordinates in both lanes
    dv2 acc[K1];      // per-lane double-float sums over the current tile
    double tot[K1];   // FP64 sum of the tile sums
  };
  __device__ static void load_trg(Trg& t, const double* r, int64_t i, const MixedFrame& fr) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      float h, l;
      split_coord(fr, k, r[i * 3 + k], h, l);
      t.xh[k] = vdup(h);
      t.xl[k] = vdup(l);
    }
#pragma unroll
    for (int k = 0; k < K1; ++k) {
      t.acc[k] = {vdup(0.f), vdup(0.f)};
      t.tot[k] = 0.0;
    }
  }
  // Once per tile: the two lanes' double-float sums into the FP64 total.
  __device__ __forceinline__ static void flush(Trg& t) {
#pragma unroll
    for (int k = 0; k < K1; ++k) {
      const f2 s = two_sum(t.acc[k].h.x, t.acc[k].h.y);
      const float lo = (t.acc[k].l.x + t.acc[k].l.y) + s.l;
      t.tot[k] += (double)s.h + (double)lo;
      t.acc[k] = {vdup(0.f), vdup(0.f)};
    }
  }
  __device__ static double result(const Trg& t, int k) { return t.tot[k]; }
  __device__ static void add_partial(Trg& t, int k, double v) { t.tot[k] += v; }

  __device__ __forceinline__ static void apply(Trg& t, const RecPk<KER>& s) {
    // r = x_t - y_s = D + d: exact hi and lo differences (common grids), Fast2Sum.
    v2 D[3], d[3];
    {
      const v2 sh[3] = {s.xh, s.yh, s.zh}, sl[3] = {s.xl, s.yl, s.zl};
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const v2 dh = vsub(t.xh[i], sh[i]), dl = vsub(t.xl[i], sl[i]);
        D[i] = vadd(dh, dl);
        d[i] = vsub(dl, vsub(D[i], dh));
      }
    }
    // r^2 = R + Rl: the three squares exactly, summed largest-first.
    const dv2 P0 = vtwo_prod(D[0], D[0]), P1 = vtwo_prod(D[1], D[1]), P2 = vtwo_prod(D[2], D[2]);
    const dv2 S1 = vtwo_sum_pos(P0.h, P1.h);
    const dv2 S2 = vtwo_sum_pos(S1.h, P2.h);
    const v2 R = S2.h;
    v2 q = vmul(D[0], d[0]);
    q = vfma(D[1], d[1], q);
    q = vfma(D[2], d[2], q);
    v2 Rl = vadd(vadd(vadd(P0.l, P1.l), vadd(P2.l, S1.l)), S2.l);
    Rl = vfma(vdup(2.f), q, Rl);
    // Hardware rsqrt estimate, 0 for coincident points (r^2 == 0 contributes 0).
    const v2 y0 = make_float2(R.x > 0.f ? rsqrt_seed(R.x) : 0.f, R.y > 0.f ? rsqrt_seed(R.y) : 0.f);
    // One Newton step on the exact residual rho = 1 - y0^2 (R + Rl).
    const dv2 Q = vtwo_prod(y0, y0);
    v2 rho = vfma(vneg(Q.h), R, vdup(1.f));
    rho = vfma(vneg(Q.l), R, rho);
    rho = vfma(vneg(Q.h), Rl, rho);
    if constexpr (KER == KER_LFXU) {
      const dv2 y = {y0, vmul(vmul(vdup(0.5f), y0), rho)};  // 1/r = y0 (1 + rho/2)
      vdf_acc(t.acc[0], vdf_mul(y, dv2{s.fh, s.fl}));
    } else {
      // y^3 = y0^3 (1 + 3 rho / 2)
      dv2 y3 = vtwo_prod(Q.h, y0);
      y3.l = vfma(Q.l, y0, y3.l);
      y3.l = vfma(y3.h, vmul(vdup(1.5f), rho), y3.l);
      if constexpr (KER == KER_LDXU) {
        const v2 mh[3] = {s.mh0, s.mh1, s.mh2}, ml[3] = {s.ml0, s.ml1, s.ml2};
        vdf_acc(t.acc[0], vdf_mul(vdot3(mh, ml, D, d), y3));
      } else if constexpr (KER == KER_SFXU) {
        const v2 fh[3] = {s.fh0, s.fh1, s.fh2}, fl[3] = {s.fl0, s.fl1, s.fl2};
        const dv2 fd = vdf_mul(vdot3(fh, fl, D, d), y3);
        const dv2 y = {y0, vmul(vmul(vdup(0.5f), y0), rho)};
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          vdf_acc(t.acc[i], vdf_mul(dv2{fh[i], fl[i]}, y));
          vdf_acc(t.acc[i], vdf_mul(dv2{D[i], d[i]}, fd));
        }
      } else {
        // y^5 = y0^5 (1 + 5 rho / 2)
        dv2 q2 = vtwo_prod(Q.h, Q.h);
        q2.l = vfma(vadd(Q.h, Q.h), Q.l, q2.l);
        dv2 y5 = vtwo_prod(q2.h, y0);
        y5.l = vfma(q2.l, y0, y5.l);
        y5.l = vfma(y5.h, vmul(vdup(2.5f), rho), y5.l);
        dv2 c;
        if constexpr (KER == KER_SDXU) {
          const v2 nh[3] = {s.nh0, s.nh1, s.nh2}, nl[3] = {s.nl0, s.nl1, s.nl2};
          const v2 fh[3] = {s.fh0, s.fh1, s.fh2}, fl[3] = {s.fl0, s.fl1, s.fl2};
          const dv2 dn = vdot3(nh, nl, D, d);
          const dv2 fd = vdot3(fh, fl, D, d);
          c = vdf_mul(vdf_mul(fd, dn), y5);
        } else {
          // r . S r = sum_i S_ii r_i^2 + sum_{i<j} 2 S_ij r_i r_j: the six products r_i r_j in
          // double-float (hi products exact, first-order lo terms), weighted and summed by TwoSum
          const dv2 C01 = vtwo_prod(D[0], D[1]), C02 = vtwo_prod(D[0], D[2]), C12 = vtwo_prod(D[1], D[2]);
          const dv2 m[6] = {{P0.h, vfma(vadd(D[0], D[0]), d[0], P0.l)},
                            {P1.h, vfma(vadd(D[1], D[1]), d[1], P1.l)},
                            {P2.h, vfma(vadd(D[2], D[2]), d[2], P2.l)},
                            {C01.h, vfma(D[0], d[1], vfma(d[0], D[1], C01.l))},
                            {C02.h, vfma(D[0], d[2], vfma(d[0], D[2], C02.l))},
                            {C12.h, vfma(D[1], d[2], vfma(d[1], D[2], C12.l))}};
          const dv2 w[6] = {{s.nh0, s.nl0}, {s.nh1, s.nl1}, {s.nh2, s.nl2},
                            {s.fh0, s.fl0}, {s.fh1, s.fl1}, {s.fh2, s.fl2}};
          dv2 q = vdf_mul(w[0], m[0]);
#pragma unroll
          for (int k = 1; k < 6; ++k) {
            const dv2 tk = vdf_mul(w[k], m[k]);
            const dv2 sk = vtwo_sum(q.h, tk.h);
            q = {sk.h, vadd(vadd(q.l, tk.l), sk.l)};
          }
          c = vdf_mul(q, y5);
        }
#pragma unroll
        for (int i = 0; i < 3; ++i) vdf_acc(t.acc[i], vdf_mul(dv2{D[i], d[i]}, c));
      }
    }
  }
};

// Targets per thread (each against two sources per step): two for the kernels
// whose per-step chain is short enough to leave registers for a second
// independent chain (measured on GB300: Laplace3D_DxU +3 %, Stokes3D_FxU +4 %),
// one for the others (two lost 1-2 %).
template <int KER>
struct TileCfgPk {
  static constexpr int THREADS = 128;
  static constexpr int T = (KER == KER_LDXU || KER == KER_SFXU) ? 2 : 1;
  static constexpr int S = 128;  // pair records (256 sources) per shared-memory tile
};

// The tiled kernel of direct.cuh with pair records: `p.ns` and `p.chunk` count
// pair records.
template <int KER>
__global__ void __launch_bounds__(TileCfgPk<KER>::THREADS) direct_sum_pk_kernel(DirectParams p) {
  using P = PairPk<KER>;
  using RecT = RecPk<KER>;
  using Cfg = TileCfgPk<KER>;
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

  const MixedFrame fr = frame_from_bbox(p.bbox);
  typename P::Trg tg[T];
  const double* rt = reinterpret_cast<const double*>(p.r_trg);
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

}  // namespace sctlgpu
