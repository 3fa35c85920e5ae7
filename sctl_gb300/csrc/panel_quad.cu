// Near-singular panel quadrature for the Laplace double layer (and single
// layer) on p x p Chebyshev panels: the "upsampled" near-field path of a
// boundary element list (the NearInterac plugin contract,
// boundary_integral.hpp:164-239), done adaptively on the GPU.
//
// For a (target, panel) pair the kernel refines the panel's parameter square
// [0,1]^2 level by level (a box is accepted once its distance to the target is
// at least `alpha` times its physical diameter; the legacy quadrature's dyadic
// refinement toward the target, boundary_quadrature.hpp:364-478, is the model),
// integrates every accepted box with an 8 x 8 Gauss-Legendre rule on geometry
// and density interpolated from the panel's nodes (barycentric Lagrange,
// as LagrangeInterp does on the CPU), and subtracts the panel's own smooth-rule
// contribution (the KNearSubtract convention, boundary_integral.txx:1165-1240).
// The result is the correction that turns the far-field smooth sum into the
// accurate value; it is added into v_out[map[target]].
//
// One warp per pair, pairs taken from a device work queue; each round, each
// lane tests one queued box (FP32 interpolation at the box centre: a
// threshold), then the lanes share the Gauss nodes of the accepted boxes.
// Node coordinates are kept relative to the target, so r needs no
// cancellation.  This file holds the FP64 form (behind
// sctlgpu_panel_arithmetic(SCTLGPU_F64)); panel_df.cuh the default
// double-float form with the same refinement.  Loops are bounded by the depth
// and queue limits; leaves are integrated whenever their buffer fills, and a
// level whose children would overflow the queue integrates the rest unrefined
// (status bit 2) instead of dropping them.
#include <cstdint>
#include <cuda_runtime.h>

#include <atomic>

#include "../../include/sctlgpu.h"
#include "common.cuh"
#include "launch.h"

namespace sctlgpu {
namespace {

constexpr int PQ_P = 10;          // panel order
constexpr int PQ_NODES = PQ_P * PQ_P;
// Gauss-Legendre points per box side.  With alpha = 1 the nearest singularity
// of an accepted box's integrand lies >= 2.8 half-sides from its centre; 8
// points keep the torus near field within 1e-10 (max, relative) of a rule
// refined twice as far (10 points: 2e-12 at 1.4x the time), and 64 nodes fill
// two full warp rounds.
constexpr int PQ_GL = 8;
constexpr int PQ_WARPS = 4;       // warps per CTA
constexpr int PQ_QUEUE = 256;     // boxes per round (per warp)
constexpr int PQ_MAX_DEPTH = 22;  // box corners k * 2^-depth stay exact in FP32

// Per-warp shared state (dynamic shared memory).
struct PanelWarpSmem {
  double F[4][PQ_NODES];          // x, y, z, sigma at the panel nodes (a-major: F[c][a*P+b])
  float Fo[3][PQ_NODES];          // (float)(x_q - x_t): the box test's node offsets
  double Ls[PQ_GL][PQ_P], Lds[PQ_GL][PQ_P], Lt[PQ_GL][PQ_P], Ldt[PQ_GL][PQ_P];  // basis at a box's Gauss points
  double A[7][PQ_GL][PQ_P];       // L_s F (x,y,z,sigma) and L_s' F (x,y,z)
  double Kd[PQ_GL][PQ_GL];        // weights mode: K * dA at a box's Gauss nodes
  double T[PQ_GL][PQ_P];          // weights mode: Kd . L_t
  double W[PQ_NODES];             // weights mode: accumulated node weights
  float box[2][PQ_QUEUE][3];      // (s0, t0, size) of the boxes of this and the next round (dyadic: exact)
  float leaf[PQ_QUEUE][3];
};

__constant__ double c_gl_x[PQ_GL], c_gl_w[PQ_GL];
// First-kind Chebyshev points of [0,1] (ChebQuadRule's nodes) and their
// barycentric weights (-1)^a sin((2a+1) pi / 2P), computed once on the host.
__constant__ double c_ch_x[PQ_P], c_ch_w[PQ_P];

__constant__ float c_ch_xf[PQ_P], c_ch_wf[PQ_P];  // FP32 copies for the box test

// FP32 barycentric basis and derivative (box test only).
__device__ __forceinline__ void basis_f32(float s, float (&l)[PQ_P], float (&d)[PQ_P]) {
  int hit = -1;
#pragma unroll
  for (int a = 0; a < PQ_P; ++a)
    if (s == c_ch_xf[a]) hit = a;
  if (hit >= 0) {
#pragma unroll
    for (int a = 0; a < PQ_P; ++a) {
      l[a] = (a == hit) ? 1.f : 0.f;
      d[a] = 0.f;
    }
    float diag = 0.f;
    const float xh = c_ch_xf[hit], iwh = 1.f / c_ch_wf[hit];
#pragma unroll
    for (int a = 0; a < PQ_P; ++a)
      if (a != hit) {
        d[a] = (c_ch_wf[a] * iwh) / (xh - c_ch_xf[a]);
        diag -= d[a];
      }
#pragma unroll
    for (int a = 0; a < PQ_P; ++a)
      if (a == hit) d[a] = diag;
    return;
  }
  float T = 0.f, U = 0.f, r[PQ_P], t[PQ_P];
#pragma unroll
  for (int a = 0; a < PQ_P; ++a) {
    r[a] = 1.f / (s - c_ch_xf[a]);
    t[a] = c_ch_wf[a] * r[a];
    T += t[a];
    U += t[a] * r[a];
  }
  const float iT = 1.f / T, UT = U * iT;
#pragma unroll
  for (int a = 0; a < PQ_P; ++a) {
    l[a] = t[a] * iT;
    d[a] = l[a] * (UT - r[a]);
  }
}

// The box test of both arithmetic forms (a threshold, so FP32 suffices, and the
// FP64 and double-float kernels refine identically): offset and tangents
// interpolated at the box centre from the FP32 node offsets off(c, q) =
// x_q - x_t; the box is far enough when that offset is at least alpha times
// the box's physical diameter.
template <class Off>
__device__ __forceinline__ bool box_far_enough(Off off, float bs, float bt, float bz, float alpha) {
  float ls[PQ_P], ds[PQ_P], lt[PQ_P], dt[PQ_P];
  basis_f32(bs + 0.5f * bz, ls, ds);
  basis_f32(bt + 0.5f * bz, lt, dt);
  float X[3], Xs[3], Xt[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    float v = 0.f, vs = 0.f, vt = 0.f;
#pragma unroll
    for (int a = 0; a < PQ_P; ++a) {
      float r0 = 0.f, rt = 0.f;
#pragma unroll
      for (int b = 0; b < PQ_P; ++b) {
        const float f = off(c, a * PQ_P + b);
        r0 = fmaf(lt[b], f, r0);
        rt = fmaf(dt[b], f, rt);
      }
      v = fmaf(ls[a], r0, v);
      vs = fmaf(ds[a], r0, vs);
      vt = fmaf(ls[a], rt, vt);
    }
    X[c] = v;
    Xs[c] = vs;
    Xt[c] = vt;
  }
  const float sl = Xs[0] * Xs[0] + Xs[1] * Xs[1] + Xs[2] * Xs[2];
  const float tl = Xt[0] * Xt[0] + Xt[1] * Xt[1] + Xt[2] * Xt[2];
  const float diam = bz * sqrtf(sl + tl);
  const float d = sqrtf(X[0] * X[0] + X[1] * X[1] + X[2] * X[2]);
  return d >= alpha * diam;
}


struct Basis {
  double l[PQ_P], d[PQ_P];
};

// Barycentric Lagrange basis on the first-kind Chebyshev points of [0,1] and
// its derivative: l_a(s) = (w_a/(s-x_a)) / sum_b w_b/(s-x_b),
// l_a'(s) = l_a(s) * (sum_b w_b/(s-x_b)^2 / sum_b w_b/(s-x_b) - 1/(s-x_a)).
__device__ __forceinline__ void basis(double s, Basis& B) {
  int hit = -1;
#pragma unroll
  for (int a = 0; a < PQ_P; ++a)
    if (s == c_ch_x[a]) hit = a;
  if (hit >= 0) {  // at a node: l is a unit vector; l' from the differentiation matrix row
#pragma unroll
    for (int a = 0; a < PQ_P; ++a) {
      B.l[a] = (a == hit) ? 1.0 : 0.0;
      B.d[a] = 0.0;
    }
    double diag = 0.0;
    const double xh = c_ch_x[hit], iwh = 1.0 / c_ch_w[hit];
#pragma unroll
    for (int a = 0; a < PQ_P; ++a)
      if (a != hit) {
        B.d[a] = (c_ch_w[a] * iwh) / (xh - c_ch_x[a]);
        diag -= B.d[a];
      }
#pragma unroll
    for (int a = 0; a < PQ_P; ++a)  // static indices keep B in registers
      if (a == hit) B.d[a] = diag;
    return;
  }
  double T = 0.0, U = 0.0, t[PQ_P], r[PQ_P];
#pragma unroll
  for (int a = 0; a < PQ_P; ++a) {
    r[a] = 1.0 / (s - c_ch_x[a]);
    t[a] = c_ch_w[a] * r[a];
    T += t[a];
    U += t[a] * r[a];
  }
  const double iT = 1.0 / T, UT = U * iT;
#pragma unroll
  for (int a = 0; a < PQ_P; ++a) {
    B.l[a] = t[a] * iT;
    B.d[a] = B.l[a] * (UT - r[a]);  // d/ds of t_a/T = (-t_a r T + t_a U) / T^2
  }
}

template <int KER>
__device__ __forceinline__ double kernel_val(const double r[3], const double n[3]) {
  const double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
  if (!(r2 > 0)) return 0.0;
  const double ri = 1.0 / sqrt(r2);
  if (KER == 0) return ri;  // Laplace3D_FxU
  return (r[0] * n[0] + r[1] * n[1] + r[2] * n[2]) * ri * ri * ri;
}

struct PanelParams {
  int64_t n_pairs, n_panels, nt, n_out;
  const int64_t* pair_trg;
  const int64_t* pair_panel;
  const int64_t* trg_map;   // output index of a target (or null: identity)
  const double* r_trg;      // AoS targets
  const double* X;          // [np][100][3] node coordinates
  const double* N;          // [np][100][3] unit normals
  const double* Q;          // [np][100]    smooth-rule weights
  const double* sigma;      // [np][100]    density
  double alpha;
  int max_depth;
  int subtract_smooth;
  double scale;
  double* out;
  unsigned* status;
  unsigned long long* next;  // work queue head: the next pair a warp takes
};

// The next (target, panel) pair for this warp: pairs are taken from a device
// counter as warps finish (their costs differ by orders of magnitude).
__device__ __forceinline__ int64_t next_pair(const PanelParams& p, int lane) {
  unsigned long long v = 0;
  if (lane == 0) v = atomicAdd(p.next, 1ull);
  return (int64_t)__shfl_sync(0xffffffffu, v, 0);
}

// WEIGHTS = false: potential correction added into out[target].  WEIGHTS =
// true: the accurate weights W_ab = int_P K(x_t - y) l_a(s) l_b(t) dA(y) of the
// pair's panel (times scale) are written to out[pair * 100 + a * 10 + b]; per
// box W += L_s^T (K dA) L_t.
template <int KER, bool WEIGHTS>
__global__ void __launch_bounds__(32 * PQ_WARPS) panel_near_kernel(PanelParams p) {
  extern __shared__ __align__(16) unsigned char pq_smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  PanelWarpSmem& sm = reinterpret_cast<PanelWarpSmem*>(pq_smem)[warp];
  for (int64_t pr = next_pair(p, lane); pr < p.n_pairs; pr = next_pair(p, lane)) {
    const int64_t tix = p.pair_trg[pr], pix = p.pair_panel[pr];
    const int64_t oix = p.trg_map ? (tix >= 0 && tix < p.nt ? p.trg_map[tix] : -1) : tix;
    if (tix < 0 || tix >= p.nt || pix < 0 || pix >= p.n_panels || oix < 0 || oix >= p.n_out) {
      if (lane == 0 && p.status) atomicOr(p.status, 4u);  // index out of range: pair skipped
      continue;
    }
    const double xt[3] = {p.r_trg[tix * 3], p.r_trg[tix * 3 + 1], p.r_trg[tix * 3 + 2]};
    __syncwarp();
    for (int q = lane; q < PQ_NODES; q += 32) {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        sm.F[c][q] = p.X[(pix * PQ_NODES + q) * 3 + c] - xt[c];  // relative to the target: no cancellation in r
        sm.Fo[c][q] = (float)sm.F[c][q];
      }
      sm.F[3][q] = p.sigma[pix * PQ_NODES + q];
    }
    __syncwarp();
    double acc = 0.0;
    if (WEIGHTS)
      for (int q = lane; q < PQ_NODES; q += 32) sm.W[q] = 0.0;
    // Smooth-rule part of this panel, to be subtracted (unless the caller
    // subtracts it in the arithmetic of its far field).
    for (int q = lane; q < PQ_NODES && p.subtract_smooth && !WEIGHTS; q += 32) {
      const double r[3] = {-sm.F[0][q], -sm.F[1][q], -sm.F[2][q]};
      const double n[3] = {p.N[(pix * PQ_NODES + q) * 3], p.N[(pix * PQ_NODES + q) * 3 + 1],
                           p.N[(pix * PQ_NODES + q) * 3 + 2]};
      acc -= kernel_val<KER>(r, n) * sm.F[3][q] * p.Q[pix * PQ_NODES + q];
    }
    // Level-by-level refinement.
    int cur = 0, ncur = 1, nleaf = 0;
    if (lane == 0) {
      sm.box[0][0][0] = 0.0f;
      sm.box[0][0][1] = 0.0f;
      sm.box[0][0][2] = 1.0f;
    }
    __syncwarp();
    for (int depth = 0; depth <= p.max_depth && ncur > 0; ++depth) {
      // each lane tests boxes of the current round
      int nnext = 0;
      nleaf = 0;
      auto integrate_leaves = [&]() {
        // Integrate this round's leaves.  Per box, tensor-product interpolation:
        // basis matrices at the box's Gauss points (lanes 0-19), then A = L_s F and
        // L_s' F (stage 1), then every node from two 10-term dot products per field.
        for (int lf = 0; lf < nleaf; ++lf) {
          const double bs = sm.leaf[lf][0], bt = sm.leaf[lf][1], bz = sm.leaf[lf][2];
          if (lane < 2 * PQ_GL) {
            const int i = lane % PQ_GL;
            Basis Bq;
            basis((lane < PQ_GL ? bs : bt) + bz * c_gl_x[i], Bq);
  #pragma unroll
            for (int a = 0; a < PQ_P; ++a) {
              if (lane < PQ_GL) {
                sm.Ls[i][a] = Bq.l[a];
                sm.Lds[i][a] = Bq.d[a];
              } else {
                sm.Lt[i][a] = Bq.l[a];
                sm.Ldt[i][a] = Bq.d[a];
              }
            }
          }
          __syncwarp();
          for (int e = lane; e < 7 * PQ_GL * PQ_P; e += 32) {
            const int m = e / (PQ_GL * PQ_P), i = (e / PQ_P) % PQ_GL, b = e % PQ_P;
            const int c = m < 4 ? m : m - 4;  // m = 0..3: L_s F_c ; m = 4..6: L_s' F_c
            const double* L = m < 4 ? sm.Ls[i] : sm.Lds[i];
            double v = 0.0;
  #pragma unroll
            for (int a = 0; a < PQ_P; ++a) v = fma(L[a], sm.F[c][a * PQ_P + b], v);
            sm.A[m][i][b] = v;
          }
          __syncwarp();
          for (int g = lane; g < PQ_GL * PQ_GL; g += 32) {
            const int i = g / PQ_GL, j = g % PQ_GL;
            double X[3] = {0, 0, 0}, Xs[3] = {0, 0, 0}, Xt[3] = {0, 0, 0}, sg = 0;
  #pragma unroll
            for (int b = 0; b < PQ_P; ++b) {
              const double lt = sm.Lt[j][b], ldt = sm.Ldt[j][b];
  #pragma unroll
              for (int c = 0; c < 3; ++c) {
                X[c] = fma(sm.A[c][i][b], lt, X[c]);
                Xt[c] = fma(sm.A[c][i][b], ldt, Xt[c]);
                Xs[c] = fma(sm.A[4 + c][i][b], lt, Xs[c]);
              }
              sg = fma(sm.A[3][i][b], lt, sg);
            }
            double n[3] = {Xs[1] * Xt[2] - Xs[2] * Xt[1], Xs[2] * Xt[0] - Xs[0] * Xt[2],
                           Xs[0] * Xt[1] - Xs[1] * Xt[0]};
            const double J = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
            const double iJ = 1.0 / J;
            n[0] *= iJ;
            n[1] *= iJ;
            n[2] *= iJ;
            const double r[3] = {-X[0], -X[1], -X[2]};  // X = x_s - x_t
            const double kda = kernel_val<KER>(r, n) * J * (bz * bz * c_gl_w[i] * c_gl_w[j]);
            if (WEIGHTS)
              sm.Kd[i][j] = kda;
            else
              acc += kda * sg;
          }
          __syncwarp();
          if (WEIGHTS) {
            for (int e = lane; e < PQ_GL * PQ_P; e += 32) {
              const int i = e / PQ_P, b = e % PQ_P;
              double v = 0.0;
  #pragma unroll
              for (int j = 0; j < PQ_GL; ++j) v = fma(sm.Kd[i][j], sm.Lt[j][b], v);
              sm.T[i][b] = v;
            }
            __syncwarp();
            for (int e = lane; e < PQ_NODES; e += 32) {  // each entry owned by one lane
              const int a = e / PQ_P, b = e % PQ_P;
              double v = sm.W[e];
  #pragma unroll
              for (int i = 0; i < PQ_GL; ++i) v = fma(sm.Ls[i][a], sm.T[i][b], v);
              sm.W[e] = v;
            }
            __syncwarp();
          }
        }
        nleaf = 0;
      };
      for (int base = 0; base < ncur; base += 32) {
        // a batch adds at most 32 leaves: flush the leaves when they might not fit
        if (nleaf + 32 > PQ_QUEUE) {
          __syncwarp();
          integrate_leaves();
          __syncwarp();
        }
        const int i = base + lane;
        bool accept = false, far = true, valid = i < ncur;
        double bs = 0, bt = 0, bz = 0;
        if (valid) {
          bs = sm.box[cur][i][0];
          bt = sm.box[cur][i][1];
          bz = sm.box[cur][i][2];
          far = box_far_enough([&](int c, int q) { return sm.Fo[c][q]; }, (float)bs, (float)bt, (float)bz,
                               (float)p.alpha);
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
        if (valid && accept) {
          const int slot = nleaf + __popc(acc_mask & lt_mask);
          if (slot < PQ_QUEUE) {
            sm.leaf[slot][0] = (float)bs;
            sm.leaf[slot][1] = (float)bt;
            sm.leaf[slot][2] = (float)bz;
          }
        }
        if (valid && !accept) {
          const int slot = nnext + 4 * __popc(ref_mask & lt_mask);
          const double h = 0.5 * bz;
          for (int c = 0; c < 4; ++c)
            if (slot + c < PQ_QUEUE) {
              sm.box[cur ^ 1][slot + c][0] = (float)(bs + (c & 1) * h);
              sm.box[cur ^ 1][slot + c][1] = (float)(bt + (c >> 1) * h);
              sm.box[cur ^ 1][slot + c][2] = (float)h;
            }
        }
        nleaf += __popc(acc_mask);  // <= PQ_QUEUE by the flush above
        nnext += 4 * __popc(ref_mask);  // <= PQ_QUEUE by the room check
      }
      __syncwarp();
      integrate_leaves();
      cur ^= 1;
      ncur = nnext;
    }
    if (WEIGHTS) {
      __syncwarp();
      for (int q = lane; q < PQ_NODES; q += 32) p.out[pr * PQ_NODES + q] = sm.W[q] * p.scale;
    } else {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (lane == 0) atomicAdd(&p.out[oix], acc * p.scale);
    }
  }
}

#include "panel_df.cuh"

// Arithmetic of the panel entries: SCTLGPU_MIXED (double-float, default) or SCTLGPU_F64.
std::atomic<int> g_panel_mode{SCTLGPU_MIXED};

// Gauss-Legendre nodes and weights on [0,1] (Newton iteration on P_n).
void gauss_legendre01(int n, double* x, double* w) {
  const double pi = 3.14159265358979323846264338327950288;
  for (int i = 0; i < n; ++i) {
    double z = cos(pi * (i + 0.75) / (n + 0.5)), dp = 0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1, p1 = z;
      for (int k = 2; k <= n; ++k) {
        const double p2 = ((2.0 * k - 1) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp = n * (z * p1 - p0) / (z * z - 1);
      const double dz = p1 / dp;
      z -= dz;
      if (fabs(dz) < 1e-16) break;
    }
    x[n - 1 - i] = 0.5 * (1 + z);
    w[n - 1 - i] = 1.0 / ((1 - z * z) * dp * dp);  // 2/((1-z^2) P'^2) on [-1,1], halved for [0,1]
  }
}

int ensure_gl(int dev) {
  static bool have_gl[64] = {};
  if (dev < 0 || dev >= 64) return SCTLGPU_ERR_NO_DEVICE;
  if (!have_gl[dev]) {
    double gx[PQ_GL], gw[PQ_GL], cx[PQ_P], cw[PQ_P];
    gauss_legendre01(PQ_GL, gx, gw);
    const double pi = 3.14159265358979323846264338327950288;
    for (int a = 0; a < PQ_P; ++a) {
      cx[a] = 0.5 - 0.5 * cos((2.0 * a + 1.0) * pi / (2.0 * PQ_P));
      cw[a] = ((a & 1) ? -1.0 : 1.0) * sin((2.0 * a + 1.0) * pi / (2.0 * PQ_P));
    }
    cudaError_t e = cudaMemcpyToSymbol(c_gl_x, gx, sizeof(gx));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_gl_w, gw, sizeof(gw));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_ch_x, cx, sizeof(cx));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_ch_w, cw, sizeof(cw));
    // double-float (hi + lo) and FP32 copies for the double-float kernel
    float gxh[PQ_GL], gxl[PQ_GL], gwh[PQ_GL], gwl[PQ_GL], cxh[PQ_P], cxl[PQ_P], cwh[PQ_P], cwl[PQ_P];
    auto split = [](double v, float* h, float* l) {
      *h = (float)v;
      *l = (float)(v - (double)*h);
    };
    for (int i = 0; i < PQ_GL; ++i) {
      split(gx[i], &gxh[i], &gxl[i]);
      split(gw[i], &gwh[i], &gwl[i]);
    }
    for (int a = 0; a < PQ_P; ++a) {
      split(cx[a], &cxh[a], &cxl[a]);
      split(cw[a], &cwh[a], &cwl[a]);
    }
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_gl_xh, gxh, sizeof(gxh));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_gl_xl, gxl, sizeof(gxl));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_gl_wh, gwh, sizeof(gwh));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_gl_wl, gwl, sizeof(gwl));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_ch_xh, cxh, sizeof(cxh));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_ch_xl, cxl, sizeof(cxl));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_ch_wh, cwh, sizeof(cwh));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_ch_wl, cwl, sizeof(cwl));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_ch_xf, cxh, sizeof(cxh));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_ch_wf, cwh, sizeof(cwh));
    if (e != cudaSuccess) return runtime_record(e);
    have_gl[dev] = true;
  }
  return SCTLGPU_OK;
}

int launch_panel_kernels(int kernel, bool weights, const PanelParams& p, unsigned grid, int dev, cudaStream_t st);

int launch_panel(int kernel, bool weights, const PanelParams& p0, unsigned grid, int dev, cudaStream_t st) {
  PanelParams p = p0;
  cudaError_t qe = cudaMallocAsync((void**)&p.next, sizeof(unsigned long long), st);
  if (qe == cudaSuccess) qe = cudaMemsetAsync(p.next, 0, sizeof(unsigned long long), st);
  if (qe != cudaSuccess) return runtime_record(qe);
  const int rc = launch_panel_kernels(kernel, weights, p, grid, dev, st);
  const cudaError_t fe = cudaFreeAsync(p.next, st);
  return rc != SCTLGPU_OK ? rc : runtime_record(fe);
}

int launch_panel_kernels(int kernel, bool weights, const PanelParams& p, unsigned grid, int dev, cudaStream_t st) {
  const size_t smem = PQ_WARPS * sizeof(PanelWarpSmem);
  const size_t smem_p = PQ_WARPS * sizeof(DFSmem<false>), smem_w = PQ_WARPS * sizeof(DFSmem<true>);
  static bool attr[64] = {};
  if (!attr[dev]) {
    cudaFuncSetAttribute(panel_near_kernel<0, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(panel_near_kernel<1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(panel_near_kernel<0, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(panel_near_kernel<1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(panel_near_kernel_df<0, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_p);
    cudaFuncSetAttribute(panel_near_kernel_df<1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_p);
    cudaFuncSetAttribute(panel_near_kernel_df<0, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_w);
    cudaFuncSetAttribute(panel_near_kernel_df<1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_w);
    attr[dev] = true;
  }
  if (g_panel_mode.load() == SCTLGPU_MIXED) {
    if (kernel == SCTLGPU_LAPLACE3D_FXU) {
      if (weights)
        panel_near_kernel_df<0, true><<<grid, 32 * PQ_WARPS, smem_w, st>>>(p);
      else
        panel_near_kernel_df<0, false><<<grid, 32 * PQ_WARPS, smem_p, st>>>(p);
    } else {
      if (weights)
        panel_near_kernel_df<1, true><<<grid, 32 * PQ_WARPS, smem_w, st>>>(p);
      else
        panel_near_kernel_df<1, false><<<grid, 32 * PQ_WARPS, smem_p, st>>>(p);
    }
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return runtime_record(cudaGetLastError());
  }
  if (kernel == SCTLGPU_LAPLACE3D_FXU) {
    if (weights)
      panel_near_kernel<0, true><<<grid, 32 * PQ_WARPS, smem, st>>>(p);
    else
      panel_near_kernel<0, false><<<grid, 32 * PQ_WARPS, smem, st>>>(p);
  } else {
    if (weights)
      panel_near_kernel<1, true><<<grid, 32 * PQ_WARPS, smem, st>>>(p);
    else
      panel_near_kernel<1, false><<<grid, 32 * PQ_WARPS, smem, st>>>(p);
  }
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return runtime_record(cudaGetLastError());
}

}  // namespace
}  // namespace sctlgpu

using namespace sctlgpu;

extern "C" int sctlgpu_panel_near_correction(int kernel, int64_t n_pairs, const int64_t* pair_trg,
                                             const int64_t* pair_panel, int64_t nt, const double* r_trg,
                                             int64_t n_panels, const double* X, const double* N, const double* Q,
                                             const double* sigma, const int64_t* trg_map, int64_t n_out, double alpha,
                                             int max_depth, int subtract_smooth, double* v_out, void* stream) {
  if (kernel != SCTLGPU_LAPLACE3D_FXU && kernel != SCTLGPU_LAPLACE3D_DXU) return SCTLGPU_ERR_INVALID_KERNEL;
  if (n_pairs < 0 || max_depth < 0 || nt < 0 || n_panels < 0 || (trg_map && n_out < 0)) return SCTLGPU_ERR_INVALID_SIZE;
  if (!(alpha > 0)) return SCTLGPU_ERR_INVALID_ARGUMENT;
  if (n_pairs == 0) return SCTLGPU_OK;
  if (!pair_trg || !pair_panel || !r_trg || !X || !N || !Q || !sigma || !v_out) return SCTLGPU_ERR_NULL_POINTER;
  int dev;
  unsigned* status;
  int sms;
  int rc = runtime_device(&dev, &status, &sms);
  if (rc) return rc;
  if ((rc = ensure_gl(dev))) return rc;
  PanelParams p;
  p.n_pairs = n_pairs;
  p.n_panels = n_panels;
  p.nt = nt;
  p.n_out = trg_map ? n_out : nt;
  p.pair_trg = pair_trg;
  p.pair_panel = pair_panel;
  p.trg_map = trg_map;
  p.r_trg = r_trg;
  p.X = X;
  p.N = N;
  p.Q = Q;
  p.sigma = sigma;
  p.alpha = alpha;
  p.max_depth = max_depth < PQ_MAX_DEPTH ? max_depth : PQ_MAX_DEPTH;
  p.subtract_smooth = subtract_smooth ? 1 : 0;
  p.scale = sctlgpu_scale_factor(kernel);
  p.out = v_out;
  p.status = status;
  const int64_t ctas = (n_pairs + PQ_WARPS - 1) / PQ_WARPS;
  const unsigned grid = (unsigned)(ctas < (int64_t)sms * 16 ? ctas : (int64_t)sms * 16);
  return launch_panel(kernel, false, p, grid, dev, (cudaStream_t)stream);
}

extern "C" int sctlgpu_panel_near_weights(int kernel, int64_t n_pairs, const int64_t* pair_trg,
                                          const int64_t* pair_panel, int64_t nt, const double* r_trg,
                                          int64_t n_panels, const double* X, double alpha, int max_depth,
                                          double* w_out, void* stream) {
  if (kernel != SCTLGPU_LAPLACE3D_FXU && kernel != SCTLGPU_LAPLACE3D_DXU) return SCTLGPU_ERR_INVALID_KERNEL;
  if (n_pairs < 0 || max_depth < 0 || nt < 0 || n_panels < 0) return SCTLGPU_ERR_INVALID_SIZE;
  if (!(alpha > 0)) return SCTLGPU_ERR_INVALID_ARGUMENT;
  if (n_pairs == 0) return SCTLGPU_OK;
  if (!pair_trg || !pair_panel || !r_trg || !X || !w_out) return SCTLGPU_ERR_NULL_POINTER;
  int dev;
  unsigned* status;
  int sms;
  int rc = runtime_device(&dev, &status, &sms);
  if (rc) return rc;
  if ((rc = ensure_gl(dev))) return rc;
  PanelParams p{};
  p.n_pairs = n_pairs;
  p.n_panels = n_panels;
  p.nt = nt;
  p.n_out = nt;
  p.pair_trg = pair_trg;
  p.pair_panel = pair_panel;
  p.r_trg = r_trg;
  p.X = X;
  p.N = X;       // unused in weights mode
  p.Q = X;       // unused in weights mode
  p.sigma = X;   // unused in weights mode (the interpolated sigma is not needed)
  p.alpha = alpha;
  p.max_depth = max_depth < PQ_MAX_DEPTH ? max_depth : PQ_MAX_DEPTH;
  p.scale = sctlgpu_scale_factor(kernel);
  p.out = w_out;
  p.status = status;
  const int64_t ctas = (n_pairs + PQ_WARPS - 1) / PQ_WARPS;
  const unsigned grid = (unsigned)(ctas < (int64_t)sms * 16 ? ctas : (int64_t)sms * 16);
  return launch_panel(kernel, true, p, grid, dev, (cudaStream_t)stream);
}

extern "C" int sctlgpu_panel_arithmetic(int mode) {
  if (mode != SCTLGPU_F64 && mode != SCTLGPU_MIXED) return SCTLGPU_ERR_INVALID_MODE;
  return g_panel_mode.exchange(mode);
}
