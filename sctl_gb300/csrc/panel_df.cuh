// Double-float form of the near-singular panel quadrature (included by
// panel_quad.cu inside its namespace; same algorithm and parameters as the
// FP64 panel_near_kernel).  GB300's FP64 pipe is a small fraction of its FP32
// pipe and the FP64 kernel is bound by it, so the quadrature runs here on
// error-free transformations in FP32 (hi + lo pairs, ~2^-46 relative):
//
//  * the panel's node coordinates are stored relative to the target
//    (x_s - x_t, formed in FP64 once per pair), so interpolated positions
//    carry no cancellation and r = -(interpolated offset);
//  * the box-acceptance test runs in FP32 (it is a threshold, not a result);
//  * every accepted box: basis values at its Gauss points in double-float
//    (barycentric formula, Newton-refined reciprocals), tensor-product
//    interpolation of the 7 fields as 10-term double-float dot products, and
//    per Gauss node the kernel times the area element from the unnormalised
//    normal Xs x Xt: Laplace DxU (r . (Xs x Xt)) / r^3, Laplace FxU |Xs x Xt| / r
//    -- no normalisation of n is needed;
//  * per-lane double-float sums, combined in FP64 per pair.
#pragma once

#include <type_traits>

namespace dfq {

using sctlgpu::f2;
using sctlgpu::two_prod;
using sctlgpu::two_sum;

__device__ __forceinline__ f2 norm(f2 x) {
  const float s = __fadd_rn(x.h, x.l);
  return {s, x.l - (s - x.h)};
}
__device__ __forceinline__ f2 neg(f2 x) { return {-x.h, -x.l}; }
// Products keep the cross terms; sums are TwoSum on the high parts.
__device__ __forceinline__ f2 mul(f2 a, f2 b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  return {p, e};
}
__device__ __forceinline__ f2 mulf(f2 a, float b) {
  const float p = __fmul_rn(a.h, b);
  return {p, fmaf(a.l, b, fmaf(a.h, b, -p))};
}
__device__ __forceinline__ f2 add(f2 a, f2 b) {
  const f2 s = two_sum(a.h, b.h);
  return norm({s.h, s.l + a.l + b.l});
}
__device__ __forceinline__ f2 sub(f2 a, f2 b) { return add(a, neg(b)); }
// acc += a * b, accumulator left unnormalised (normalise after a short sum).
__device__ __forceinline__ void fma_acc(f2& acc, f2 a, f2 b) {
  const f2 p = mul(a, b);
  const f2 s = two_sum(acc.h, p.h);
  acc = {s.h, acc.l + (s.l + p.l)};
}
// 1 / d: FP32 reciprocal refined by one Newton step on the double-float residual.
__device__ __forceinline__ f2 rcp(f2 d) {
  const float y = 1.0f / d.h;
  float t = fmaf(-d.h, y, 1.0f);
  t = fmaf(-d.l, y, t);
  return norm({y, y * t});
}
__device__ __forceinline__ f2 from_double(double v) {
  const float h = (float)v;
  return {h, (float)(v - (double)h)};
}
__device__ __forceinline__ double to_double(f2 x) { return (double)x.h + (double)x.l; }
// 1/sqrt(R) and its powers from the hardware estimate and one Newton step on
// the exact residual rho = 1 - y0^2 R (|rho| ~ 2^-22): y = y0 (1 + rho/2).
__device__ __forceinline__ f2 rsqrt(f2 R, float* rho_out, float* y0_out) {
  float y0 = sctlgpu::rsqrt_seed(R.h);
  y0 = R.h > 0.f ? y0 : 0.f;
  const f2 q = two_prod(y0, y0);
  float rho = fmaf(-q.h, R.h, 1.f);
  rho = fmaf(-q.l, R.h, rho);
  rho = fmaf(-q.h, R.l, rho);
  *rho_out = rho;
  *y0_out = y0;
  return {y0, (0.5f * y0) * rho};
}

}  // namespace dfq

// Packed forms of the dfq operations (fma/add/mul.rn.f32x2): two quadrature
// nodes per lane, lane x and lane y, each with exactly the scalar sequence of
// roundings.  GB300 runs the double-float quadrature issue-bound on the FP32
// pipe; one f32x2 instruction per two nodes halves the issue slots.
namespace pdfq {

using v2 = float2;
struct d2 {
  v2 h, l;
};
__device__ __forceinline__ v2 dup(float a) { return make_float2(a, a); }
__device__ __forceinline__ v2 vneg(v2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ v2 vadd(v2 a, v2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ v2 vsub(v2 a, v2 b) { return __fadd2_rn(a, vneg(b)); }
__device__ __forceinline__ v2 vmul(v2 a, v2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ v2 vfma(v2 a, v2 b, v2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ d2 dupf2(sctlgpu::f2 x) { return {dup(x.h), dup(x.l)}; }
__device__ __forceinline__ d2 pair(sctlgpu::f2 x, sctlgpu::f2 y) { return {make_float2(x.h, y.h), make_float2(x.l, y.l)}; }
__device__ __forceinline__ d2 two_prod(v2 a, v2 b) {
  const v2 p = vmul(a, b);
  return {p, vfma(a, b, vneg(p))};
}
__device__ __forceinline__ d2 two_sum(v2 a, v2 b) {
  const v2 s = vadd(a, b);
  const v2 bb = vsub(s, a);
  return {s, vadd(vsub(a, vsub(s, bb)), vsub(b, bb))};
}
__device__ __forceinline__ d2 norm(d2 x) {
  const v2 s = vadd(x.h, x.l);
  return {s, vsub(x.l, vsub(s, x.h))};
}
__device__ __forceinline__ d2 neg(d2 x) { return {vneg(x.h), vneg(x.l)}; }
__device__ __forceinline__ d2 mul(d2 a, d2 b) {
  const v2 p = vmul(a.h, b.h);
  v2 e = vfma(a.h, b.h, vneg(p));
  e = vfma(a.h, b.l, e);
  e = vfma(a.l, b.h, e);
  return {p, e};
}
__device__ __forceinline__ d2 mulf(d2 a, v2 b) {
  const v2 p = vmul(a.h, b);
  return {p, vfma(a.l, b, vfma(a.h, b, vneg(p)))};
}
__device__ __forceinline__ d2 add(d2 a, d2 b) {
  const d2 s = two_sum(a.h, b.h);
  return norm({s.h, vadd(vadd(s.l, a.l), b.l)});
}
__device__ __forceinline__ d2 sub(d2 a, d2 b) { return add(a, neg(b)); }
__device__ __forceinline__ void fma_acc(d2& acc, d2 a, d2 b) {
  const d2 p = mul(a, b);
  const d2 s = two_sum(acc.h, p.h);
  acc = {s.h, vadd(acc.l, vadd(s.l, p.l))};
}

}  // namespace pdfq

// Per-warp shared state of the double-float kernel.  All boxes of one round
// have the same size (2^-depth), so only their corners are queued.  Gauss rows
// i and i + 4 of a box sit side by side (lane x, lane y) so that one lane
// integrates two nodes with f32x2 arithmetic and one 16-byte shared load per
// operand pair; the weights-mode arrays exist only in the weights-mode layout
// (smaller footprint = more resident warps for the potential mode).
struct PanelWarpSmemDFP {
  f2 F[4][PQ_NODES];  // x_s - x_t (3 components) and sigma at the panel nodes
  pdfq::d2 LsP[PQ_GL / 2][PQ_P], LdsP[PQ_GL / 2][PQ_P];  // basis and derivative along s, rows paired
  f2 Lt[PQ_GL][PQ_P], Ldt[PQ_GL][PQ_P];                  // along t
  pdfq::d2 AP[7][PQ_GL / 2][PQ_P];                        // L_s F (x,y,z,sigma) and L_s' F (x,y,z)
  float box[2][PQ_QUEUE][2];  // (s0, t0) of the boxes of this and the next round (dyadic: exact)
};
// Weights mode: K dA at the box's Gauss nodes, Kd . L_t, and the panel's 100 accumulated weights.
struct PanelWarpSmemDFPW : PanelWarpSmemDFP {
  f2 Kd[PQ_GL][PQ_GL];
  f2 T[PQ_GL][PQ_P];
  f2 W[PQ_NODES];
};
template <bool WEIGHTS>
using DFSmem = typename std::conditional<WEIGHTS, PanelWarpSmemDFPW, PanelWarpSmemDFP>::type;

__constant__ float c_gl_xh[PQ_GL], c_gl_xl[PQ_GL];        // Gauss-Legendre nodes, double-float
__constant__ float c_gl_wh[PQ_GL], c_gl_wl[PQ_GL];        // and weights
__constant__ float c_ch_xh[PQ_P], c_ch_xl[PQ_P];          // Chebyshev nodes, double-float
__constant__ float c_ch_wh[PQ_P], c_ch_wl[PQ_P];          // barycentric weights, double-float

// Double-float Lagrange basis and its derivative (barycentric formula, Newton-
// refined reciprocals) at the 16 points s = b0 + bz * g of a box (8 along s, 8
// along t; b0, bz dyadic, so exact), spread over the whole warp: two lanes per
// point, each lane five of the ten terms; the partial sums (and a node hit,
// where the basis is a unit vector and the derivative a differentiation-matrix
// row) are exchanged with the partner lane.  Writes
// the s-rows into the paired layout and the t-rows into Lt / Ldt.
template <class SM>
__device__ __forceinline__ void basis_df_warp(SM& sm, int lane, float bs, float bt, float bz) {
  constexpr int H = PQ_GL / 2, K = PQ_P / 2;
  const int pt = lane >> 1, a0 = (lane & 1) * K;
  const int i = pt % PQ_GL;
  const f2 g = {c_gl_xh[i], c_gl_xl[i]};
  const f2 s = dfq::add({pt < PQ_GL ? bs : bt, 0.f}, dfq::mulf(g, bz));
  int hit = -1;
#pragma unroll
  for (int k = 0; k < K; ++k)
    if (s.h == c_ch_xh[a0 + k] && s.l == c_ch_xl[a0 + k]) hit = a0 + k;
  hit = max(hit, __shfl_xor_sync(0xffffffffu, hit, 1));
  f2 l[K], d[K];
  if (hit >= 0) {  // at a node: l is a unit vector, l' the differentiation-matrix row
    f2 diag = {0.f, 0.f};
    const f2 xh = {c_ch_xh[hit], c_ch_xl[hit]}, iwh = dfq::rcp({c_ch_wh[hit], c_ch_wl[hit]});
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int a = a0 + k;
      l[k] = {(a == hit) ? 1.f : 0.f, 0.f};
      d[k] = {0.f, 0.f};
      if (a != hit) {
        const f2 w = dfq::mul({c_ch_wh[a], c_ch_wl[a]}, iwh);
        d[k] = dfq::mul(w, dfq::rcp(dfq::sub(xh, {c_ch_xh[a], c_ch_xl[a]})));
        diag = dfq::sub(diag, d[k]);
      }
    }
    diag = dfq::add(diag, {__shfl_xor_sync(0xffffffffu, diag.h, 1), __shfl_xor_sync(0xffffffffu, diag.l, 1)});
#pragma unroll
    for (int k = 0; k < K; ++k)
      if (a0 + k == hit) d[k] = diag;
  } else {
    f2 T = {0.f, 0.f}, U = {0.f, 0.f}, r[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int a = a0 + k;
      r[k] = dfq::rcp(dfq::sub(s, {c_ch_xh[a], c_ch_xl[a]}));
      const f2 t = dfq::mul({c_ch_wh[a], c_ch_wl[a]}, r[k]);
      l[k] = t;
      T = dfq::add(T, t);
      U = dfq::add(U, dfq::mul(t, r[k]));
    }
    T = dfq::add(T, {__shfl_xor_sync(0xffffffffu, T.h, 1), __shfl_xor_sync(0xffffffffu, T.l, 1)});
    U = dfq::add(U, {__shfl_xor_sync(0xffffffffu, U.h, 1), __shfl_xor_sync(0xffffffffu, U.l, 1)});
    const f2 iT = dfq::rcp(T), UT = dfq::mul(U, iT);
#pragma unroll
    for (int k = 0; k < K; ++k) {
      l[k] = dfq::mul(l[k], iT);
      d[k] = dfq::mul(l[k], dfq::sub(UT, r[k]));
    }
  }
  const int rr = i % H, y = i >= H ? 1 : 0;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    const int a = a0 + k;
    if (pt < PQ_GL) {
      // d2 = {h.x, h.y, l.x, l.y}: row i's words sit at offsets y and 2 + y
      float* ls = reinterpret_cast<float*>(&sm.LsP[rr][a]) + y;
      float* ld = reinterpret_cast<float*>(&sm.LdsP[rr][a]) + y;
      ls[0] = l[k].h;
      ls[2] = l[k].l;
      ld[0] = d[k].h;
      ld[2] = d[k].l;
    } else {
      sm.Lt[i][a] = l[k];
      sm.Ldt[i][a] = d[k];
    }
  }
}

template <int KER, bool WEIGHTS, class SM>
__device__ __forceinline__ void leaf_pk(SM& sm, int lane, float bs, float bt, float bz, pdfq::d2& acc) {
  constexpr int H = PQ_GL / 2;
  basis_df_warp(sm, lane, bs, bt, bz);
  __syncwarp();
  for (int e = lane; e < 7 * H * PQ_P; e += 32) {
    const int m = e / (H * PQ_P), r = (e / PQ_P) % H, b = e % PQ_P;
    if (WEIGHTS && m == 3) continue;  // no density in weights mode
    const int c = m < 4 ? m : m - 4;
    const pdfq::d2* L = m < 4 ? sm.LsP[r] : sm.LdsP[r];
    pdfq::d2 v = {};
#pragma unroll
    for (int a = 0; a < PQ_P; ++a) pdfq::fma_acc(v, L[a], pdfq::dupf2(sm.F[c][a * PQ_P + b]));
    sm.AP[m][r][b] = pdfq::norm(v);
  }
  __syncwarp();
  const int r = lane / PQ_GL, j = lane % PQ_GL;  // nodes (r, j) and (r + 4, j)
  pdfq::d2 X[3] = {}, Xs[3] = {}, Xt[3] = {}, sg = {};
#pragma unroll 1
  for (int b = 0; b < PQ_P; ++b) {
    const pdfq::d2 lt = pdfq::dupf2(sm.Lt[j][b]), ldt = pdfq::dupf2(sm.Ldt[j][b]);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const pdfq::d2 ac = sm.AP[c][r][b];
      pdfq::fma_acc(X[c], ac, lt);
      pdfq::fma_acc(Xt[c], ac, ldt);
      pdfq::fma_acc(Xs[c], sm.AP[4 + c][r][b], lt);
    }
    if (!WEIGHTS) pdfq::fma_acc(sg, sm.AP[3][r][b], lt);
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    X[c] = pdfq::norm(X[c]);  // X = x_s - x_t = -r
    Xs[c] = pdfq::norm(Xs[c]);
    Xt[c] = pdfq::norm(Xt[c]);
  }
  using pdfq::add;
  using pdfq::mul;
  using pdfq::sub;
  const pdfq::d2 n0 = sub(mul(Xs[1], Xt[2]), mul(Xs[2], Xt[1]));
  const pdfq::d2 n1 = sub(mul(Xs[2], Xt[0]), mul(Xs[0], Xt[2]));
  const pdfq::d2 n2 = sub(mul(Xs[0], Xt[1]), mul(Xs[1], Xt[0]));
  const pdfq::d2 R = add(add(mul(X[0], X[0]), mul(X[1], X[1])), mul(X[2], X[2]));
  // 1/sqrt(R): hardware estimate per lane, one Newton step on the exact residual (dfq::rsqrt)
  float2 y0 = make_float2(sctlgpu::rsqrt_seed(R.h.x), sctlgpu::rsqrt_seed(R.h.y));
  y0.x = R.h.x > 0.f ? y0.x : 0.f;
  y0.y = R.h.y > 0.f ? y0.y : 0.f;
  const pdfq::d2 q = pdfq::two_prod(y0, y0);
  float2 rho = pdfq::vfma(pdfq::vneg(q.h), R.h, pdfq::dup(1.f));
  rho = pdfq::vfma(pdfq::vneg(q.l), R.h, rho);
  rho = pdfq::vfma(pdfq::vneg(q.h), R.l, rho);
  const pdfq::d2 yv = {y0, pdfq::vmul(pdfq::vmul(pdfq::dup(0.5f), y0), rho)};
  const pdfq::d2 wi = pdfq::pair({c_gl_wh[r], c_gl_wl[r]}, {c_gl_wh[r + H], c_gl_wl[r + H]});
  const pdfq::d2 w = pdfq::mulf(mul(wi, pdfq::dupf2({c_gl_wh[j], c_gl_wl[j]})), pdfq::dup(bz * bz));
  pdfq::d2 kda;
  if (KER == 0) {  // single layer: |n| / r
    const pdfq::d2 J2 = add(add(mul(n0, n0), mul(n1, n1)), mul(n2, n2));
    const float2 jh = make_float2(sqrtf(J2.h.x), sqrtf(J2.h.y));
    const pdfq::d2 jp = pdfq::two_prod(jh, jh);
    const float2 jl = make_float2(jh.x > 0.f ? ((J2.h.x - jp.h.x - jp.l.x) + J2.l.x) / (2.f * jh.x) : 0.f,
                                  jh.y > 0.f ? ((J2.h.y - jp.h.y - jp.l.y) + J2.l.y) / (2.f * jh.y) : 0.f);
    kda = mul(mul(pdfq::norm({jh, jl}), yv), w);
  } else {  // double layer: (r . n) / r^3 with r = -X
    const pdfq::d2 rn = pdfq::neg(add(add(mul(X[0], n0), mul(X[1], n1)), mul(X[2], n2)));
    pdfq::d2 y3 = pdfq::mulf(pdfq::two_prod(y0, y0), y0);  // y0^3 (1 + 3 rho / 2)
    y3.l = pdfq::vfma(y3.h, pdfq::vmul(pdfq::dup(1.5f), rho), y3.l);
    kda = mul(mul(rn, y3), w);
  }
  if constexpr (WEIGHTS) {
    const pdfq::d2 k = pdfq::norm(kda);
    sm.Kd[r][j] = {k.h.x, k.l.x};
    sm.Kd[r + H][j] = {k.h.y, k.l.y};
    __syncwarp();
    for (int e = lane; e < PQ_GL * PQ_P; e += 32) {  // T = Kd . L_t
      const int i = e / PQ_P, b = e % PQ_P;
      f2 v = {0.f, 0.f};
#pragma unroll
      for (int jj = 0; jj < PQ_GL; ++jj) dfq::fma_acc(v, sm.Kd[i][jj], sm.Lt[jj][b]);
      sm.T[i][b] = dfq::norm(v);
    }
    __syncwarp();
    for (int e = lane; e < PQ_NODES; e += 32) {  // W += L_s^T T, rows i and i + 4 from one packed entry
      const int a = e / PQ_P, b = e % PQ_P;
      f2 v = sm.W[e];
#pragma unroll
      for (int i = 0; i < H; ++i) {
        const pdfq::d2 ls = sm.LsP[i][a];
        dfq::fma_acc(v, {ls.h.x, ls.l.x}, sm.T[i][b]);
        dfq::fma_acc(v, {ls.h.y, ls.l.y}, sm.T[i + H][b]);
      }
      sm.W[e] = dfq::norm(v);
    }
  } else {
    pdfq::fma_acc(acc, kda, pdfq::norm(sg));
    acc = pdfq::norm(acc);
  }
}

template <int KER, bool WEIGHTS>
__global__ void __launch_bounds__(32 * PQ_WARPS, WEIGHTS ? 3 : 4) panel_near_kernel_df(PanelParams p) {
  extern __shared__ __align__(16) unsigned char pq_smem_df[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  DFSmem<WEIGHTS>& sm = reinterpret_cast<DFSmem<WEIGHTS>*>(pq_smem_df)[warp];
  for (int64_t pr = next_pair(p, lane); pr < p.n_pairs; pr = next_pair(p, lane)) {
    const int64_t tix = p.pair_trg[pr], pix = p.pair_panel[pr];
    const int64_t oix = p.trg_map ? (tix >= 0 && tix < p.nt ? p.trg_map[tix] : -1) : tix;
    if (tix < 0 || tix >= p.nt || pix < 0 || pix >= p.n_panels || oix < 0 || oix >= p.n_out) {
      if (lane == 0 && p.status) atomicOr(p.status, 4u);
      continue;
    }
    const double xt[3] = {p.r_trg[tix * 3], p.r_trg[tix * 3 + 1], p.r_trg[tix * 3 + 2]};
    __syncwarp();
    double acc_smooth = 0.0;
    for (int q = lane; q < PQ_NODES; q += 32) {
      const double* xq = p.X + (pix * PQ_NODES + q) * 3;
      const double rx = xq[0] - xt[0], ry = xq[1] - xt[1], rz = xq[2] - xt[2];
      sm.F[0][q] = dfq::from_double(rx);
      sm.F[1][q] = dfq::from_double(ry);
      sm.F[2][q] = dfq::from_double(rz);
      if (!WEIGHTS) {
        const double sg = p.sigma[pix * PQ_NODES + q];
        sm.F[3][q] = dfq::from_double(sg);
        if (p.subtract_smooth) {  // the panel's own smooth-rule part (FP64, once per pair)
          const double r[3] = {-rx, -ry, -rz};
          const double n[3] = {p.N[(pix * PQ_NODES + q) * 3], p.N[(pix * PQ_NODES + q) * 3 + 1],
                               p.N[(pix * PQ_NODES + q) * 3 + 2]};
          acc_smooth -= kernel_val<KER>(r, n) * sg * p.Q[pix * PQ_NODES + q];
        }
      } else {
        if constexpr (WEIGHTS) sm.W[q] = {0.f, 0.f};
      }
    }
    __syncwarp();
    pdfq::d2 acc = {};  // potential mode: the lane's two node sums
    int cur = 0, ncur = 1;
    if (lane == 0) {
      sm.box[0][0][0] = 0.0f;
      sm.box[0][0][1] = 0.0f;
    }
    __syncwarp();
    for (int depth = 0; depth <= p.max_depth && ncur > 0; ++depth) {
      int nnext = 0;
      const float bz = ldexpf(1.0f, -depth);  // every box of this round has this size
      // Integrates the accepted boxes of one group of 32 (acc_mask over the lanes holding them),
      // in lane order, as soon as the group is classified: no leaf queue in shared memory.
      auto integrate_leaves = [&](unsigned acc_mask, float lbs, float lbt) {
        for (unsigned mk = acc_mask; mk; mk &= mk - 1u) {
          const int src = __ffs(mk) - 1;
          const float bs = __shfl_sync(0xffffffffu, lbs, src), bt = __shfl_sync(0xffffffffu, lbt, src);
          leaf_pk<KER, WEIGHTS>(sm, lane, bs, bt, bz, acc);
          __syncwarp();
        }
      };
      for (int base = 0; base < ncur; base += 32) {
        const int i = base + lane;
        bool accept = false, far = true, valid = i < ncur;
        float bs = 0, bt = 0;
        if (valid) {
          bs = sm.box[cur][i][0];
          bt = sm.box[cur][i][1];
          far = box_far_enough([&](int c, int q) { return sm.F[c][q].h; }, bs, bt, bz, (float)p.alpha);
          accept = far || depth == p.max_depth;
        }
        {  // boxes whose four children no longer fit in the next level's queue are integrated
           // unrefined (flagged) rather than dropped
          const unsigned want = __ballot_sync(0xffffffffu, valid && !accept);
          if (valid && !accept && nnext + 4 * __popc(want & ((1u << lane) - 1u)) + 4 > PQ_QUEUE) accept = true;
          if (lane == 0 && p.status && nnext + 4 * __popc(want) > PQ_QUEUE) atomicOr(p.status, 2u);
        }
        const unsigned acc_mask = __ballot_sync(0xffffffffu, valid && accept);
        const unsigned ref_mask = __ballot_sync(0xffffffffu, valid && !accept);
        const unsigned lt_mask = (1u << lane) - 1u;
        if (valid && !accept) {
          const int slot = nnext + 4 * __popc(ref_mask & lt_mask);
          const float h = 0.5f * bz;
          for (int c = 0; c < 4; ++c)
            if (slot + c < PQ_QUEUE) {
              sm.box[cur ^ 1][slot + c][0] = bs + (c & 1) * h;
              sm.box[cur ^ 1][slot + c][1] = bt + (c >> 1) * h;
            }
        }
        nnext += 4 * __popc(ref_mask);  // <= PQ_QUEUE by the room check
        __syncwarp();
        integrate_leaves(acc_mask, bs, bt);
      }
      __syncwarp();
      cur ^= 1;
      ncur = nnext;
    }
    if constexpr (WEIGHTS) {
      __syncwarp();
      for (int q = lane; q < PQ_NODES; q += 32) p.out[pr * PQ_NODES + q] = dfq::to_double(sm.W[q]) * p.scale;
    } else {
      double v = ((double)acc.h.x + (double)acc.l.x) + ((double)acc.h.y + (double)acc.l.y) + acc_smooth;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) atomicAdd(&p.out[oix], v * p.scale);
    }
  }
}
