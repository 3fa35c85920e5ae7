// Far field by a barycentric Lagrange treecode: the role ParticleFMM::Eval
// (fmm-wrapper.txx:542-549) gives EvalPVFMM (fmm-wrapper.txx:854-1038) for
// 40,000 targets or more -- U(x_t) = sum_s K(x_t, y_s) q_s to `digits`, with
// work below the O(N M) of the direct sum.  The algorithm is not PVFMM's (an
// FMM with equivalent densities and M2L translations): it is a particle-cluster
// treecode whose cluster approximations are themselves direct sums, so every
// interaction runs in the batched near-field kernels of near_plan.cu with the
// arithmetic `digits` selects there.
//
//  * host: an octree over the sources (tight boxes split at their centres,
//    leaves of <= leaf_max sources) and one over the targets whose leaves are
//    the target batches (<= batch_max).  Sources are laid out leaf by leaf and
//    every leaf is padded to an even count with zero-charge slots, so every
//    cluster's slot range starts and ends on a pair boundary: the plan pairs
//    the whole slot list once (packed double-float records) for all blocks.
//  * traversal per batch from the root: a cluster is approximated when
//    (r_batch + r_cluster) < theta |c_batch - c_cluster| and it holds more
//    sources than proxy slots, a leaf is summed directly, anything else descends.
//  * an approximated cluster carries proxy sources at the tensor-product
//    Chebyshev points (second kind) of its box -- order + 1 along its longest
//    side, fewer along a much thinner side (tc_grid) -- and with the
//    Lagrange basis L_k, K(x, y) ~ sum_k L_k(y) K(x, z_k) for y in the box, so
//    the proxies carry the moments M_k = sum_s L_k(y_s) q_s of the cluster's
//    source charges q_s: the density (single layers), the density times the
//    normal (Laplace double layer: the moment is the proxy's normal), or
//    normal (x) density (Stokes double layer: three proxies per point with
//    unit normals e_c and densities M_k[c][:] would do; instead one proxy per
//    point carries the symmetric density sym(M_k), which gives the same field
//    since (r.n)(r.f) = r . (n (x) f) r, evaluated by KER_SDXU_SYM in a second
//    plan).
//  * device, per evaluation: densities gathered into slot order, moments per
//    (cluster, 256-slot chunk) -- in double-float on the FP32 pipe when the
//    plan's arithmetic is FP32 or double-float, else in FP64 -- reduced per
//    cluster in chunk order (deterministic), then one execution of the
//    near-field plan over the (batch, leaf range) and (batch, proxy range)
//    blocks.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <atomic>
#include <numeric>
#include <thread>
#include <type_traits>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/sctlgpu.h"
#include "common.cuh"
#include "launch.h"

namespace sctlgpu {
namespace {

constexpr int TC_MAX_NP = 16;   // Chebyshev points per dimension (order + 1)
constexpr int TC_CHUNK = 256;   // source slots per moment work item
constexpr int TC_THREADS = 256;
constexpr int TC_MAX_BATCH = 2048;
constexpr double TC_DIRECT_FRACTION = 0.75;  // treecode interactions above this share of Ns * Nt: direct sum
// Cost of one symmetric-density proxy of the Stokes double layer (KER_SDXU_SYM: r . S r, six
// double-float products) in Stokes double-layer interactions (two compensated dot products);
// measured on GB300: 179 against 227 G interactions/s.
constexpr double TC_SYM_COST = 1.25;
constexpr double TC_PART_BYTES = 1e9;  // partial moments held at once (2^20 sources, degree 11: 0.7-2 GB in all)  // targets per batch (the downward pass keeps a batch's sums in shared memory)

struct TcNode {
  int64_t b = 0, e = 0;    // points [b, e) of the tree's permutation
  int64_t sb = 0, se = 0;  // slots [sb, se) (sources: leaves padded to even counts)
  double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0}, c[3] = {0, 0, 0}, r = 0;
  int32_t child0 = -1, nchild = 0;  // children are consecutive nodes
  int32_t parent = -1;
  int64_t proxy = -1;  // sources: first proxy slot; targets: first proxy entry of the target list
  int32_t g[3] = {1, 1, 1};  // Chebyshev points per dimension of the node's interpolation grid
  int32_t npts = 1;          // g[0] * g[1] * g[2]
};

void set_box(const double* X, const std::vector<int64_t>& perm, TcNode& nd) {
  for (int d = 0; d < 3; ++d) {
    nd.lo[d] = INFINITY;
    nd.hi[d] = -INFINITY;
  }
  for (int64_t i = nd.b; i < nd.e; ++i)
    for (int d = 0; d < 3; ++d) {
      const double v = X[perm[i] * 3 + d];
      nd.lo[d] = std::min(nd.lo[d], v);
      nd.hi[d] = std::max(nd.hi[d], v);
    }
  double r2 = 0;
  for (int d = 0; d < 3; ++d) {
    nd.c[d] = 0.5 * (nd.lo[d] + nd.hi[d]);
    r2 += 0.25 * (nd.hi[d] - nd.lo[d]) * (nd.hi[d] - nd.lo[d]);
  }
  nd.r = std::sqrt(r2);
}

// Splits node `id` of `nodes` at its box centre into its non-empty octants
// (children appended consecutively, in octant order, which is also their order
// in `perm`), the children's tight boxes gathered while the points are moved.
// Returns false for a node that stays a leaf.
bool split_node(const double* X, std::vector<int64_t>& perm, std::vector<int64_t>& tmp, std::vector<TcNode>& nodes,
                int32_t id, int depth, int64_t leaf_max) {
  const TcNode nd = nodes[id];
  if (nd.e - nd.b <= leaf_max || depth >= 60) return false;
  if (nd.hi[0] == nd.lo[0] && nd.hi[1] == nd.lo[1] && nd.hi[2] == nd.lo[2]) return false;  // coincident points
  int64_t cnt[8] = {0, 0, 0, 0, 0, 0, 0, 0}, off[8];
  auto octant = [&](const double* x) {
    return (x[0] > nd.c[0] ? 1 : 0) | (x[1] > nd.c[1] ? 2 : 0) | (x[2] > nd.c[2] ? 4 : 0);
  };
  for (int64_t i = nd.b; i < nd.e; ++i) ++cnt[octant(X + perm[i] * 3)];
  off[0] = nd.b;
  for (int o = 1; o < 8; ++o) off[o] = off[o - 1] + cnt[o - 1];
  int64_t pos[8];
  std::copy(off, off + 8, pos);
  double lo[8][3], hi[8][3];
  for (int o = 0; o < 8; ++o)
    for (int d = 0; d < 3; ++d) {
      lo[o][d] = INFINITY;
      hi[o][d] = -INFINITY;
    }
  for (int64_t i = nd.b; i < nd.e; ++i) {
    const double* x = X + perm[i] * 3;
    const int o = octant(x);
    for (int d = 0; d < 3; ++d) {
      lo[o][d] = std::min(lo[o][d], x[d]);
      hi[o][d] = std::max(hi[o][d], x[d]);
    }
    tmp[pos[o]++] = perm[i];
  }
  std::copy(tmp.begin() + nd.b, tmp.begin() + nd.e, perm.begin() + nd.b);
  nodes[id].child0 = (int32_t)nodes.size();
  for (int o = 0; o < 8; ++o) {
    if (!cnt[o]) continue;
    TcNode ch;
    ch.parent = id;
    ch.b = off[o];
    ch.e = off[o] + cnt[o];
    double r2 = 0;
    for (int d = 0; d < 3; ++d) {
      ch.lo[d] = lo[o][d];
      ch.hi[d] = hi[o][d];
      ch.c[d] = 0.5 * (ch.lo[d] + ch.hi[d]);
      r2 += 0.25 * (ch.hi[d] - ch.lo[d]) * (ch.hi[d] - ch.lo[d]);
    }
    ch.r = std::sqrt(r2);
    nodes.push_back(ch);
    ++nodes[id].nchild;
  }
  return true;
}

// Octree on tight boxes: nodes with more than `leaf_max` points are split (split_node).  The
// first levels are split in order until there are subtrees for every host thread; those are
// built concurrently (disjoint ranges of `perm`) and appended in order, so the node numbering
// keeps children consecutive and after their parent.  (Binary trees split at the median along
// the longest side -- leaves of exactly leaf_max points -- were measured: 5-15 % faster at
// digits 10, but their elongated boxes let the acceptance test admit targets closer to the
// long side, and 3000 coincident targets met 3e-10 against 1e-10.)
void build_octree(const double* X, int64_t n, int64_t leaf_max, std::vector<int64_t>& perm,
                  std::vector<TcNode>& nodes) {
  perm.resize((size_t)n);
  std::iota(perm.begin(), perm.end(), (int64_t)0);
  nodes.assign(1, TcNode{});
  nodes[0].b = 0;
  nodes[0].e = n;
  if (n == 0) return;
  set_box(X, perm, nodes[0]);
  std::vector<int64_t> tmp((size_t)n);
  const int nthreads = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  // breadth-first to a frontier of >= 4 subtrees per thread (or until nothing splits)
  std::vector<std::pair<int32_t, int>> frontier{{0, 0}};
  while (frontier.size() < (size_t)4 * nthreads) {
    std::vector<std::pair<int32_t, int>> next;
    bool any = false;
    for (const auto& [id, depth] : frontier) {
      if (split_node(X, perm, tmp, nodes, id, depth, leaf_max)) {
        any = true;
        for (int k = 0; k < nodes[id].nchild; ++k) next.push_back({nodes[id].child0 + k, depth + 1});
      }
    }
    if (!any) return;
    frontier.swap(next);
  }
  // each frontier node's subtree in a local node list (local node 0 = the frontier node)
  std::vector<std::vector<TcNode>> local(frontier.size());
  std::atomic<size_t> next_task{0};
  auto work = [&] {
    for (size_t f = next_task++; f < frontier.size(); f = next_task++) {
      std::vector<TcNode>& L = local[f];
      L.assign(1, nodes[frontier[f].first]);
      L[0].child0 = -1;
      L[0].nchild = 0;
      std::vector<std::pair<int32_t, int>> stack{{0, frontier[f].second}};
      while (!stack.empty()) {
        const auto [id, depth] = stack.back();
        stack.pop_back();
        if (!split_node(X, perm, tmp, L, id, depth, leaf_max)) continue;
        for (int k = L[id].nchild - 1; k >= 0; --k) stack.push_back({L[id].child0 + k, depth + 1});
      }
    }
  };
  std::vector<std::thread> pool;
  for (int w = 1; w < nthreads; ++w) pool.emplace_back(work);
  work();
  for (auto& th : pool) th.join();
  for (size_t f = 0; f < frontier.size(); ++f) {  // append, renumbering local ids
    const int32_t g = frontier[f].first, base = (int32_t)nodes.size() - 1;  // local id i >= 1 -> base + i
    const std::vector<TcNode>& L = local[f];
    if (L[0].nchild == 0) continue;
    nodes[g].child0 = base + L[0].child0;
    nodes[g].nchild = L[0].nchild;
    for (size_t i = 1; i < L.size(); ++i) {
      TcNode nd = L[i];
      nd.parent = nd.parent == 0 ? g : base + nd.parent;
      if (nd.nchild) nd.child0 += base;
      nodes.push_back(nd);
    }
  }
}

// Interpolation box of a cluster: exactly its tight box, so every proxy lies
// inside the bounding box of the input points.  That keeps the mixed-precision
// frame of the plan (derived from the bounding box of everything it sees)
// identical to the frame of any other plan or direct sum over the same sources
// and targets, so that terms a caller subtracts later (the smooth-rule
// correction of near panels) cancel term by term.  A side of zero extent maps
// every point to t = -1 (inv = 0): all weight on the proxies at that coordinate.
void interp_box(const TcNode& C, double lo[3], double inv[3]) {
  for (int d = 0; d < 3; ++d) {
    lo[d] = C.lo[d];
    const double ext = C.hi[d] - C.lo[d];
    inv[d] = ext > 0 ? 2.0 / ext : 0.0;
  }
}
// Coordinate of Chebyshev point x in [-1, 1] on [lo, hi], with both ends exact
// and every point inside [lo, hi].
double cheb_coord(double lo, double hi, double x) {
  return x >= 0 ? hi - 0.5 * (1.0 - x) * (hi - lo) : lo + 0.5 * (1.0 + x) * (hi - lo);
}

// Points per dimension of a cluster's interpolation grid.  Tensor-product Chebyshev
// interpolation errs by about the sum over the dimensions of rho_k^-(points_k - 1), where
// rho_k = s_k + sqrt(s_k^2 - 1) and s_k = (r / theta) / h_k is the closest distance the
// acceptance test admits (r / theta from the centre) in half-widths h_k of that side.  The
// longest side keeps the full order; a thinner side -- a patch of a surface seen edge-on -- gets
// the fewest points whose term stays below a third of the longest side's, and a side of zero
// extent one point (its coordinate is the same for every point of the cluster: exact).  (A
// tenth measured the same errors and ran 3-10 % slower; equal terms raised the sphere/ball error
// at digits 10 from 3e-12 to 1.7e-11.)
void tc_grid(TcNode& C, int order, double theta) {
  double h[3], hmax = 0;
  for (int d = 0; d < 3; ++d) {
    h[d] = 0.5 * (C.hi[d] - C.lo[d]);
    hmax = std::max(hmax, h[d]);
  }
  auto lrho = [](double s) { return std::log(s + std::sqrt(std::max(0.0, s * s - 1.0))); };
  const double reach = C.r / theta;
  const double need = hmax > 0 ? order * lrho(reach / hmax) + std::log(3.0) : 0.0;
  C.npts = 1;
  for (int d = 0; d < 3; ++d) {
    int p = 0;
    if (h[d] > 0) {
      const double l = lrho(reach / h[d]);
      p = l > 0 ? (int)std::ceil(need / l) : order;
      p = std::min(order, std::max(1, p));
    }
    C.g[d] = p + 1;
    C.npts *= p + 1;
  }
}

struct TcLayout {
  int order = 0, np = 0, npts = 0, per_point = 1;  // np, npts: the largest grid (order + 1 per dimension)
  // Stokes double layer: one proxy per grid point carrying the symmetric part of its moment
  // (evaluated by KER_SDXU_SYM, cost pw each) instead of three with unit normals
  bool sym = false;
  double pw = 1.0;
  double theta = 0;
  std::vector<TcNode> src, trg;
  std::vector<int64_t> sperm, tperm;
  std::vector<int64_t> slot_src;  // source slot -> source index, -1 = padding
  int64_t n_src_slots = 0, n_slots = 0;
  std::vector<int32_t> clusters;  // approximated source clusters (node ids) in proxy order
  std::vector<int32_t> tclusters; // target clusters with proxies (node ids) in proxy order
  int64_t n_trg_slots = 0;        // sorted targets, then the target clusters' proxies
  std::vector<int32_t> batches;   // target leaves in target order
  std::vector<int32_t> anc_ptr, anc;  // per batch: its target clusters with proxies (indices of tclusters)
  std::vector<sctlgpu_block> blocks;
  int64_t pp = 0, approx = 0;     // interactions of the direct blocks and of the proxy blocks
  bool dual = true;
  bool direct = false;   // the traversal saves too little: evaluations run the direct sum
  double theta_trg = 0;  // acceptance for target-side interpolation (<= theta)
};

// Proxy slots of a source cluster: its grid points times the proxies per point, padded to an
// even count (pair boundaries).
int64_t tc_proxy_slots(const TcLayout& L, const TcNode& C) { return ((int64_t)C.npts * L.per_point + 1) / 2 * 2; }

// Chebyshev points of the second kind of every degree (x_m = cos(pi m / p), m = 0..p) and their
// barycentric weights (-1)^m, halved at the ends; degree 0 is the single point 1 with weight 1.
struct TcCheb {
  double x[TC_MAX_NP][TC_MAX_NP], w[TC_MAX_NP][TC_MAX_NP];
  float xh[TC_MAX_NP][TC_MAX_NP], xl[TC_MAX_NP][TC_MAX_NP], wf[TC_MAX_NP][TC_MAX_NP];  // double-float points
};
const TcCheb& tc_cheb() {
  static const TcCheb tab = [] {
    TcCheb t{};
    for (int p = 0; p < TC_MAX_NP; ++p)
      for (int m = 0; m <= p; ++m) {
        t.x[p][m] = p ? std::cos(M_PI * m / p) : 1.0;
        t.w[p][m] = p ? (m % 2 ? -1.0 : 1.0) * ((m == 0 || m == p) ? 0.5 : 1.0) : 1.0;
        t.xh[p][m] = (float)t.x[p][m];
        t.xl[p][m] = (float)(t.x[p][m] - (double)t.xh[p][m]);
        t.wf[p][m] = (float)t.w[p][m];  // +-1 or +-1/2: exact
      }
    return t;
  }();
  return tab;
}

// Default (order, theta) per digits: Chebyshev interpolation of K(x, .) on a box
// seen from distance >= r / theta converges like rho^-order with
// rho = s + sqrt(s^2 - 1), s ~ sqrt(3) / theta per dimension.
void tc_defaults(int digits, int* order, double* theta) {
  static const int ord[16] = {3, 3, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 15};
  static const double th[16] = {0.7, 0.7, 0.7, 0.7, 0.65, 0.6, 0.6, 0.55, 0.55, 0.5, 0.5, 0.5, 0.45, 0.45, 0.4, 0.4};
  const int d = std::min(15, std::max(0, digits < 0 ? 15 : digits));
  if (*order <= 0) *order = ord[d];
  if (*theta <= 0) *theta = th[d];
}

int tc_build_layout(int kernel, int64_t ns, const double* r_src, int64_t nt, const double* r_trg, int order,
                    double theta, double theta_trg, int64_t leaf_max, int64_t batch_max, bool dual, bool sym,
                    TcLayout& L) {
  if (order < 1 || order >= TC_MAX_NP || !(theta > 0) || theta >= 1.0) return SCTLGPU_ERR_INVALID_ARGUMENT;
  if (batch_max > TC_MAX_BATCH || theta_trg > theta) return SCTLGPU_ERR_INVALID_ARGUMENT;
  L.dual = dual;
  L.theta_trg = theta_trg > 0 ? theta_trg : theta;
  L.order = order;
  L.np = order + 1;
  L.npts = L.np * L.np * L.np;
  L.sym = sym && kernel == SCTLGPU_STOKES3D_DXU;
  L.per_point = kernel == SCTLGPU_STOKES3D_DXU && !L.sym ? 3 : 1;
  L.pw = L.sym ? TC_SYM_COST : 1.0;
  L.theta = theta;
  if (leaf_max <= 0) leaf_max = std::max<int64_t>(64, (int64_t)std::ceil(L.npts * L.per_point * L.pw));
  if (batch_max <= 0) batch_max = 512;
  {  // the two trees are independent
    std::thread tt([&] { build_octree(r_trg, nt, batch_max, L.tperm, L.trg); });
    build_octree(r_src, ns, leaf_max, L.sperm, L.src);
    tt.join();
  }
  for (TcNode& nd : L.src) tc_grid(nd, order, theta);
  for (TcNode& nd : L.trg) tc_grid(nd, order, L.theta_trg);
  // source slots: leaves in permutation order, each padded to an even count
  std::vector<int32_t> leaves;
  for (int32_t i = 0; i < (int32_t)L.src.size(); ++i)
    if (L.src[i].nchild == 0 && L.src[i].e > L.src[i].b) leaves.push_back(i);
  std::sort(leaves.begin(), leaves.end(), [&](int32_t a, int32_t b) { return L.src[a].b < L.src[b].b; });
  int64_t cur = 0;
  L.slot_src.clear();
  for (int32_t id : leaves) {
    TcNode& nd = L.src[id];
    nd.sb = cur;
    for (int64_t i = nd.b; i < nd.e; ++i) L.slot_src.push_back(L.sperm[i]);
    if ((nd.e - nd.b) % 2) L.slot_src.push_back(-1);
    cur = (int64_t)L.slot_src.size();
    nd.se = cur;
  }
  for (int32_t i = (int32_t)L.src.size() - 1; i >= 0; --i) {  // children come after their parent
    TcNode& nd = L.src[i];
    if (nd.nchild) {
      nd.sb = L.src[nd.child0].sb;
      nd.se = L.src[nd.child0 + nd.nchild - 1].se;
    }
  }
  L.n_src_slots = cur;
  // Traversal over (target node, source node) pairs.  With `dual`, from the two roots; a pair
  // that passes the acceptance test takes the cheapest of: direct (targets x sources),
  // targets x source proxies, target proxies x sources, target proxies x source proxies, where
  // a side may use its proxies only when it holds more points than proxies; otherwise the
  // larger node (by radius) is split, and two leaves are summed directly.  Without `dual`,
  // every batch starts from the source root and only the source side is ever approximated.
  struct Rec {
    int32_t t, s;
    char kind;  // 0 direct, 1 source proxies, 2 target proxies, 3 both
  };
  std::vector<Rec> recs;
  std::vector<char> sused(L.src.size(), 0), tused(L.trg.size(), 0);
  std::vector<std::pair<int32_t, int32_t>> st;
  L.batches.clear();
  for (int32_t i = 0; i < (int32_t)L.trg.size(); ++i)
    if (L.trg[i].nchild == 0 && L.trg[i].e > L.trg[i].b) L.batches.push_back(i);
  std::sort(L.batches.begin(), L.batches.end(), [&](int32_t a, int32_t b) { return L.trg[a].b < L.trg[b].b; });
  if (ns > 0 && nt > 0) {
    if (L.dual)
      st.push_back({0, 0});
    else
      for (auto it = L.batches.rbegin(); it != L.batches.rend(); ++it) st.push_back({*it, 0});
  }
  while (!st.empty()) {
    const auto [ti, si] = st.back();
    st.pop_back();
    const TcNode &T = L.trg[ti], &S = L.src[si];
    if (T.e == T.b || S.e == S.b) continue;
    const double dx = T.c[0] - S.c[0], dy = T.c[1] - S.c[1], dz = T.c[2] - S.c[2];
    const double dist = std::sqrt(dx * dx + dy * dy + dz * dz);
    const int64_t nT = T.e - T.b, nS = S.e - S.b, sS = S.se - S.sb;
    const int64_t Ps = (int64_t)S.npts * L.per_point, Pt = T.npts;  // the clusters' proxies
    const double Pc = (double)Ps * L.pw;                              // the source proxies' cost
    if (T.r + S.r < theta * dist) {
      // target-side interpolation (a target cluster's proxies) only under the stricter theta_trg
      const bool src_ok = (double)nS > Pc, trg_ok = L.dual && nT > Pt && T.r + S.r < L.theta_trg * dist;
      double best = (double)nT * sS;
      char kind = 0;
      if (src_ok && (double)nT * Pc < best) best = (double)nT * Pc, kind = 1;
      if (trg_ok && (double)Pt * sS < best) best = (double)Pt * sS, kind = 2;
      if (src_ok && trg_ok && (double)Pt * Pc < best) best = (double)Pt * Pc, kind = 3;
      recs.push_back({ti, si, kind});
      if (kind & 1) sused[si] = 1;
      if (kind & 2) tused[ti] = 1;
      continue;
    }
    const bool tl = T.nchild == 0 || !L.dual, sl = S.nchild == 0;
    if (tl && sl) {
      recs.push_back({ti, si, 0});
    } else if (sl || (!tl && T.r >= S.r)) {
      for (int k = T.nchild - 1; k >= 0; --k) st.push_back({T.child0 + k, si});
    } else {
      for (int k = S.nchild - 1; k >= 0; --k) st.push_back({ti, S.child0 + k});
    }
  }
  // proxies: source clusters in node order (siblings adjacent), then target clusters
  L.clusters.clear();
  int64_t pcur = L.n_src_slots;
  for (int32_t i = 0; i < (int32_t)L.src.size(); ++i)
    if (sused[i]) {
      L.src[i].proxy = pcur;
      pcur += tc_proxy_slots(L, L.src[i]);
      L.clusters.push_back(i);
    }
  L.n_slots = pcur;
  L.tclusters.clear();
  std::vector<int32_t> tindex(L.trg.size(), -1);
  int64_t tcur = nt;
  for (int32_t i = 0; i < (int32_t)L.trg.size(); ++i)
    if (tused[i]) {
      L.trg[i].proxy = tcur;
      tcur += L.trg[i].npts;
      tindex[i] = (int32_t)L.tclusters.size();
      L.tclusters.push_back(i);
    }
  L.n_trg_slots = tcur;
  // per batch, its ancestors (and itself) that carry target proxies
  L.anc_ptr.assign(1, 0);
  L.anc.clear();
  for (int32_t b : L.batches) {
    for (int32_t a = b; a >= 0; a = L.trg[a].parent)
      if (tindex[a] >= 0) L.anc.push_back(tindex[a]);
    L.anc_ptr.push_back((int32_t)L.anc.size());
  }
  // blocks: per target range, contiguous source ranges merged
  struct Blk {
    int64_t t0, tn, s0, s1;
  };
  std::vector<Blk> bl;
  bl.reserve(recs.size());
  for (const Rec& r : recs) {
    const TcNode &T = L.trg[r.t], &S = L.src[r.s];
    const bool tp = r.kind & 2, sp = r.kind & 1;
    bl.push_back({tp ? T.proxy : T.b, tp ? (int64_t)T.npts : T.e - T.b, sp ? S.proxy : S.sb,
                  sp ? S.proxy + tc_proxy_slots(L, S) : S.se});  // with the zero-charge padding slot
  }
  std::sort(bl.begin(), bl.end(), [](const Blk& a, const Blk& b) {
    return a.t0 != b.t0 ? a.t0 < b.t0 : (a.tn != b.tn ? a.tn < b.tn : a.s0 < b.s0);
  });
  std::vector<Blk> merged;
  for (size_t k = 0; k < bl.size();) {
    Blk cur = bl[k];
    size_t j = k + 1;
    while (j < bl.size() && bl[j].t0 == cur.t0 && bl[j].tn == cur.tn && bl[j].s0 == cur.s1 &&
           (bl[j].s0 < L.n_src_slots) == (cur.s0 < L.n_src_slots))
      cur.s1 = bl[j++].s1;
    merged.push_back(cur);
    k = j;
  }
  // then blocks over the same sources whose target ranges adjoin (sibling batches or target
  // clusters that accepted the same source nodes): fewer, fuller blocks (the lanes of an item
  // take up to 128 or 256 targets; batches average 130-270)
  std::sort(merged.begin(), merged.end(), [](const Blk& a, const Blk& b) {
    return a.s0 != b.s0 ? a.s0 < b.s0 : (a.s1 != b.s1 ? a.s1 < b.s1 : a.t0 < b.t0);
  });
  L.blocks.clear();
  L.pp = L.approx = 0;
  for (size_t k = 0; k < merged.size();) {
    Blk cur = merged[k];
    size_t j = k + 1;
    while (j < merged.size() && merged[j].s0 == cur.s0 && merged[j].s1 == cur.s1 &&
           merged[j].t0 == cur.t0 + cur.tn && (merged[j].t0 < nt) == (cur.t0 < nt))
      cur.tn += merged[j++].tn;
    const bool direct = cur.t0 < nt && cur.s0 < L.n_src_slots;
    L.blocks.push_back({cur.s0, cur.s1 - cur.s0, cur.t0, cur.tn});
    (direct ? L.pp : L.approx) += (cur.s1 - cur.s0) * cur.tn;
    k = j;
  }
  // Below ~25 % saved interactions the proxies' overheads (moments, downward pass, smaller
  // blocks) eat the gain: such geometries are evaluated by the direct sum.
  L.direct = (double)(L.pp + L.approx) > TC_DIRECT_FRACTION * (double)ns * (double)nt;
  return SCTLGPU_OK;
}

// ------------------------------------------------------------------ device

struct TcCluster {
  double lo[3], inv[3];  // interpolation box: t = (y - lo) * inv - 1 in [-1, 1]
  int64_t proxy;         // first proxy slot
  int32_t item0, item1;  // moment work items [item0, item1)
  int32_t g[3];          // grid points per dimension
};
struct TcItem {
  int32_t cluster;
  int32_t n;   // slots of the chunk
  int64_t s0;  // first slot
};
struct TcMomParams {
  const TcCluster* clusters;
  const TcItem* items;
  const double* r;  // slot coordinates
  const double* n;  // slot normals (double-layer kernels)
  const double* v;  // slot densities
  double* part;     // per item of the pass: npts x Q partial moments
  int item0, item1; // the pass's items [item0, item1)
  double* pn;       // proxy normals (Laplace double layer)
  double* pv;       // proxy densities
  int np;           // the largest grid's points per dimension (shared-memory stride)
  const TcCheb* cheb;
  int sym;          // Stokes double layer: one symmetric-density proxy per point (else three)
};

template <int KER>
struct TcCharge;
template <>
struct TcCharge<SCTLGPU_LAPLACE3D_FXU> {
  static constexpr int Q = 1;
};
template <>
struct TcCharge<SCTLGPU_LAPLACE3D_DXU> {
  static constexpr int Q = 3;
};
template <>
struct TcCharge<SCTLGPU_STOKES3D_FXU> {
  static constexpr int Q = 3;
};
template <>
struct TcCharge<SCTLGPU_STOKES3D_DXU> {
  static constexpr int Q = 9;
};

__global__ void tc_gather_kernel(int64_t n_slots, int sd, const int64_t* slot_src, const double* v_src, double* v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_slots * sd;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = slot_src[i / sd];
    v[i] = s >= 0 ? v_src[s * sd + i % sd] : 0.0;
  }
}

// Barycentric Lagrange basis at t (second-kind Chebyshev points x, weights w).
__device__ __forceinline__ void tc_lagrange(double t, int np, const double* x, const double* w, double* L) {
  int hit = -1;
  double sum = 0;
  for (int m = 0; m < np; ++m) {
    const double d = t - x[m];
    if (d == 0.0) hit = m;
    const double q = d != 0.0 ? w[m] / d : 0.0;
    L[m] = q;
    sum += q;
  }
  if (hit >= 0) {
    for (int m = 0; m < np; ++m) L[m] = m == hit ? 1.0 : 0.0;
  } else {
    const double inv = 1.0 / sum;
    for (int m = 0; m < np; ++m) L[m] *= inv;
  }
}

// Partial moments of one chunk: M_k = sum_s L_k(y_s) q_s over <= 256 slots.
template <int KER>
__global__ void __launch_bounds__(TC_THREADS) tc_moments_kernel(TcMomParams p) {
  constexpr int Q = TcCharge<KER>::Q;
  extern __shared__ double tc_sm[];
  const int np = p.np, npmax3 = np * np * np;
  double* Ls = tc_sm;                          // [TC_CHUNK][3][np]
  double* qs = tc_sm + TC_CHUNK * 3 * np;      // [TC_CHUNK][Q]
  const TcItem it = p.items[p.item0 + blockIdx.x];
  const TcCluster C = p.clusters[it.cluster];
  const int g0 = C.g[0], g1 = C.g[1], g2 = C.g[2], npts = g0 * g1 * g2;
  for (int s = threadIdx.x; s < TC_CHUNK; s += blockDim.x) {
    const bool valid = s < it.n;
    const int64_t slot = it.s0 + s;
    for (int d = 0; d < 3; ++d) {
      double t = valid ? (p.r[slot * 3 + d] - C.lo[d]) * C.inv[d] - 1.0 : 0.0;
      t = fmin(1.0, fmax(-1.0, t));
      tc_lagrange(t, C.g[d], p.cheb->x[C.g[d] - 1], p.cheb->w[C.g[d] - 1], Ls + (s * 3 + d) * np);
    }
    double q[Q];
    for (int c = 0; c < Q; ++c) q[c] = 0.0;
    if (valid) {
      if constexpr (KER == SCTLGPU_LAPLACE3D_FXU) {
        q[0] = p.v[slot];
      } else if constexpr (KER == SCTLGPU_LAPLACE3D_DXU) {
        for (int c = 0; c < 3; ++c) q[c] = p.n[slot * 3 + c] * p.v[slot];
      } else if constexpr (KER == SCTLGPU_STOKES3D_FXU) {
        for (int c = 0; c < 3; ++c) q[c] = p.v[slot * 3 + c];
      } else {  // normal (x) density
        for (int c = 0; c < 3; ++c)
          for (int d = 0; d < 3; ++d) q[c * 3 + d] = p.n[slot * 3 + c] * p.v[slot * 3 + d];
      }
    }
    for (int c = 0; c < Q; ++c) qs[s * Q + c] = q[c];
  }
  __syncthreads();
  for (int k = threadIdx.x; k < npts; k += blockDim.x) {
    const int i = k / (g1 * g2), j = (k / g2) % g1, l = k % g2;
    double acc[Q];
    for (int c = 0; c < Q; ++c) acc[c] = 0.0;
    for (int s = 0; s < it.n; ++s) {
      const double wgt = Ls[(s * 3) * np + i] * Ls[(s * 3 + 1) * np + j] * Ls[(s * 3 + 2) * np + l];
#pragma unroll
      for (int c = 0; c < Q; ++c) acc[c] = fma(wgt, qs[s * Q + c], acc[c]);
    }
    double* out = p.part + ((int64_t)blockIdx.x * npmax3 + k) * Q;
#pragma unroll
    for (int c = 0; c < Q; ++c) out[c] = acc[c];
  }
}

// The same in double-float on the FP32 pipe (GB300's FP64 pipe is ~1/64 of it): for plans
// whose arithmetic is FP32 or double-float, whose own per-interaction error is far above the
// ~2^-44 of these moments.
__device__ __forceinline__ f2 tc_rcp(f2 d) {  // 1 / d: FP32 estimate, one Newton step on the exact residual
  const float y = 1.0f / d.h;
  float t = fmaf(-d.h, y, 1.0f);
  t = fmaf(-d.l, y, t);
  return fast_two_sum(y, y * t);
}
__device__ __forceinline__ f2 tc_split(double v) {
  const float h = (float)v;
  return {h, (float)(v - (double)h)};
}
// Barycentric Lagrange basis at t in double-float, for the np points of degree np - 1 of C.
__device__ __forceinline__ void tc_lagrange_df(double tt, int np, const TcCheb* C, f2* L) {
  const float *xh = C->xh[np - 1], *xl = C->xl[np - 1], *wf = C->wf[np - 1];
  const f2 t = tc_split(tt);
  int hit = -1;
  f2 sum = {0.f, 0.f};
  for (int m = 0; m < np; ++m) {
    const f2 d = df_norm(df_add(t, {-xh[m], -xl[m]}));
    if (d.h == 0.f) hit = m;
    const f2 q = d.h != 0.f ? df_mulf(tc_rcp(d), wf[m]) : f2{0.f, 0.f};
    L[m] = q;
    df_acc(sum, q);
  }
  if (hit >= 0) {
    for (int m = 0; m < np; ++m) L[m] = {m == hit ? 1.f : 0.f, 0.f};
  } else {
    const f2 inv = tc_rcp(df_norm(sum));
    for (int m = 0; m < np; ++m) L[m] = df_norm(df_mul(L[m], inv));
  }
}

template <int KER>
__global__ void __launch_bounds__(TC_THREADS) tc_moments_df_kernel(TcMomParams p) {
  constexpr int Q = TcCharge<KER>::Q;
  extern __shared__ double tc_sm[];
  const int np = p.np, npmax3 = np * np * np;
  f2* Ls = reinterpret_cast<f2*>(tc_sm);  // [TC_CHUNK][3][np]
  f2* qs = Ls + TC_CHUNK * 3 * np;        // [TC_CHUNK][Q]
  const TcItem it = p.items[p.item0 + blockIdx.x];
  const TcCluster C = p.clusters[it.cluster];
  const int g1 = C.g[1], g2 = C.g[2], npts = C.g[0] * g1 * g2;
  for (int s = threadIdx.x; s < TC_CHUNK; s += blockDim.x) {
    const bool valid = s < it.n;
    const int64_t slot = it.s0 + s;
    for (int d = 0; d < 3; ++d) {
      double t = valid ? (p.r[slot * 3 + d] - C.lo[d]) * C.inv[d] - 1.0 : 0.0;
      t = fmin(1.0, fmax(-1.0, t));
      tc_lagrange_df(t, C.g[d], p.cheb, Ls + (s * 3 + d) * np);
    }
    double q[Q];
    for (int c = 0; c < Q; ++c) q[c] = 0.0;
    if (valid) {
      if constexpr (KER == SCTLGPU_LAPLACE3D_FXU) {
        q[0] = p.v[slot];
      } else if constexpr (KER == SCTLGPU_LAPLACE3D_DXU) {
        for (int c = 0; c < 3; ++c) q[c] = p.n[slot * 3 + c] * p.v[slot];
      } else if constexpr (KER == SCTLGPU_STOKES3D_FXU) {
        for (int c = 0; c < 3; ++c) q[c] = p.v[slot * 3 + c];
      } else {
        for (int c = 0; c < 3; ++c)
          for (int d = 0; d < 3; ++d) q[c * 3 + d] = p.n[slot * 3 + c] * p.v[slot * 3 + d];
      }
    }
    for (int c = 0; c < Q; ++c) qs[s * Q + c] = tc_split(q[c]);
  }
  __syncthreads();
  for (int k = threadIdx.x; k < npts; k += blockDim.x) {
    const int i = k / (g1 * g2), j = (k / g2) % g1, l = k % g2;
    f2 acc[Q];
    for (int c = 0; c < Q; ++c) acc[c] = {0.f, 0.f};
    for (int s = 0; s < it.n; ++s) {
      const f2 wgt = df_mul(df_mul(Ls[(s * 3) * np + i], Ls[(s * 3 + 1) * np + j]), Ls[(s * 3 + 2) * np + l]);
#pragma unroll
      for (int c = 0; c < Q; ++c) df_acc(acc[c], df_mul(wgt, qs[s * Q + c]));
    }
    double* out = p.part + ((int64_t)blockIdx.x * npmax3 + k) * Q;
#pragma unroll
    for (int c = 0; c < Q; ++c) out[c] = (double)acc[c].h + (double)acc[c].l;
  }
}

// Moments of every approximated cluster (its chunks in order) into the proxy slots.
template <int KER>
__global__ void tc_reduce_kernel(TcMomParams p, int n_clusters) {
  constexpr int Q = TcCharge<KER>::Q;
  const int npmax3 = p.np * p.np * p.np;
  const int c = blockIdx.y;
  if (c >= n_clusters) return;
  const TcCluster C = p.clusters[c];
  const int npts = C.g[0] * C.g[1] * C.g[2];
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < npts; k += gridDim.x * blockDim.x) {
    // this pass's items of the cluster, in order; the pass holding the cluster's first item
    // writes, later passes add (the same order of additions as one pass)
    const int i0 = max(C.item0, p.item0), i1 = min(C.item1, p.item1);
    if (i0 >= i1) continue;
    double m[Q];
    for (int q = 0; q < Q; ++q) m[q] = 0.0;
    for (int it = i0; it < i1; ++it) {
      const double* src = p.part + ((int64_t)(it - p.item0) * npmax3 + k) * Q;
#pragma unroll
      for (int q = 0; q < Q; ++q) m[q] += src[q];
    }
    const bool first = C.item0 >= p.item0;
    auto put = [&](double* dst, double v) { *dst = first ? v : *dst + v; };
    if constexpr (KER == SCTLGPU_LAPLACE3D_FXU) {
      put(&p.pv[C.proxy + k], m[0]);
    } else if constexpr (KER == SCTLGPU_LAPLACE3D_DXU) {
      for (int q = 0; q < 3; ++q) put(&p.pn[(C.proxy + k) * 3 + q], m[q]);
    } else if constexpr (KER == SCTLGPU_STOKES3D_FXU) {
      for (int q = 0; q < 3; ++q) put(&p.pv[(C.proxy + k) * 3 + q], m[q]);
    } else if (p.sym) {  // proxy k: diag(M_k) as the normal, its symmetrised off-diagonal pairs
      const int64_t o = (C.proxy + k) * 3;
      for (int c = 0; c < 3; ++c) put(&p.pn[o + c], m[c * 4]);
      put(&p.pv[o + 0], m[1] + m[3]);
      put(&p.pv[o + 1], m[2] + m[6]);
      put(&p.pv[o + 2], m[5] + m[7]);
    } else {  // proxy (k, c): normal e_c, density M_k[c][:]
      for (int q = 0; q < Q; ++q) put(&p.pv[(C.proxy + 3 * k + q / 3) * 3 + q % 3], m[q]);
    }
  }
}

// Moments in passes of at most `pass_items` chunks (the partial buffer's capacity).
template <int KER>
cudaError_t tc_launch_moments(TcMomParams p, int n_items, int pass_items, int n_clusters, bool df, cudaStream_t st) {
  constexpr int Q = TcCharge<KER>::Q;
  if (n_items == 0) return cudaSuccess;
  // f2 and double tiles: both fit the same byte count (8 bytes per value)
  const size_t smem = (size_t)TC_CHUNK * (3 * p.np + Q) * sizeof(double);
  auto kern = df ? tc_moments_df_kernel<KER> : tc_moments_kernel<KER>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int npts = p.np * p.np * p.np;
  for (int i0 = 0; i0 < n_items; i0 += pass_items) {
    p.item0 = i0;
    p.item1 = std::min(n_items, i0 + pass_items);
    kern<<<p.item1 - p.item0, TC_THREADS, smem, st>>>(p);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    tc_reduce_kernel<KER><<<dim3((npts + 255) / 256, n_clusters), 256, 0, st>>>(p, n_clusters);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// Downward pass and output: every sorted target k gets its plan sum u[k] plus, for each of
// its target clusters A with proxies (its batch and the batch's ancestors),
// sum_k L_k(x) u[A's proxy k] -- the interpolation of the potentials the plan accumulated at
// A's Chebyshev points -- and is written (or added) to out[perm[k]].  One CTA per batch, one
// warp per target: the lanes split the rows (i, j) of the cluster's grid, in double-float (DF) or
// FP64.
struct TcTrgBox {
  double lo[3], inv[3];
  int64_t proxy;  // first proxy entry of the target list
  int32_t g[3];   // grid points per dimension
};
struct TcL2PParams {
  const TcTrgBox* boxes;
  const int64_t* bt0;  // per batch: first sorted target
  const int32_t* btn;  // per batch: targets
  const int32_t* anc_ptr;
  const int32_t* anc;
  const double* r;      // sorted target coordinates
  const double* u;      // plan results over the target list (targets, then proxies)
  const int64_t* perm;  // sorted target -> output index
  double* out;
  int accumulate;
  int np;  // the largest grid's points per dimension (shared-memory size)
  const TcCheb* cheb;
};

template <int TD, bool DF>
__global__ void __launch_bounds__(TC_THREADS) tc_l2p_kernel(TcL2PParams p) {
  using V = typename std::conditional<DF, f2, double>::type;
  extern __shared__ double tc_sm[];
  const int npmax3 = p.np * p.np * p.np;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  V* P = reinterpret_cast<V*>(tc_sm);                         // [npts][TD] proxy potentials of one cluster
  V* Lw = P + (size_t)npmax3 * TD + warp * 3 * TC_MAX_NP;     // per warp: [3][points] basis values
  double* acc_t = tc_sm + (size_t)npmax3 * TD + nwarps * 3 * TC_MAX_NP;  // [batch_max][TD] target sums
  const int b = blockIdx.x;
  const int64_t t0 = p.bt0[b];
  const int tn = p.btn[b];
  for (int e = threadIdx.x; e < tn * TD; e += blockDim.x) acc_t[e] = p.u[t0 * TD + e];
  for (int a = p.anc_ptr[b]; a < p.anc_ptr[b + 1]; ++a) {
    const TcTrgBox* A = p.boxes + p.anc[a];  // read in place (indexed by lane below)
    const int g0 = A->g[0], g1 = A->g[1], g2 = A->g[2], g01 = g0 * g1, npts = g01 * g2;
    const int64_t aproxy = A->proxy;
    __syncthreads();
    for (int e = threadIdx.x; e < npts * TD; e += blockDim.x) {  // stored [l][i, j][c]
      const double v = p.u[aproxy * TD + e];
      const int kk = e / TD, c = e - kk * TD, ij = kk / g2, l = kk - ij * g2;
      V* dst = P + ((size_t)l * g01 + ij) * TD + c;
      if constexpr (DF)
        *dst = tc_split(v);
      else
        *dst = v;
    }
    __syncthreads();
    for (int t = warp; t < tn; t += nwarps) {  // one warp per target
      const int64_t k = t0 + t;
      if (lane < 3) {
        double tt = (p.r[k * 3 + lane] - A->lo[lane]) * A->inv[lane] - 1.0;
        tt = fmin(1.0, fmax(-1.0, tt));
        const int gd = A->g[lane];
        if constexpr (DF)
          tc_lagrange_df(tt, gd, p.cheb, Lw + lane * TC_MAX_NP);
        else
          tc_lagrange(tt, gd, p.cheb->x[gd - 1], p.cheb->w[gd - 1], Lw + lane * TC_MAX_NP);
      }
      __syncwarp();
      // sum_i L_i(x) sum_j L_j(y) sum_l L_l(z) P[i][j][l]: the lanes split the (i, j) rows
      V acc[TD];
      for (int c = 0; c < TD; ++c) acc[c] = V{};
      for (int ij = lane; ij < g01; ij += 32) {
        const int i = ij / g1, j = ij - i * g1;
        V part[TD];
        for (int c = 0; c < TD; ++c) part[c] = V{};
        for (int l = 0; l < g2; ++l) {
          const V z = Lw[2 * TC_MAX_NP + l];
          const V* pl = P + ((size_t)l * g01 + ij) * TD;
#pragma unroll
          for (int c = 0; c < TD; ++c) {
            if constexpr (DF)
              df_acc(part[c], df_mul(z, pl[c]));
            else
              part[c] = fma(z, pl[c], part[c]);
          }
        }
        if constexpr (DF) {
          const f2 xy = df_mul(Lw[i], Lw[TC_MAX_NP + j]);
#pragma unroll
          for (int c = 0; c < TD; ++c) df_acc(acc[c], df_mul(xy, two_sum(part[c].h, part[c].l)));
        } else {
          const double xy = Lw[i] * Lw[TC_MAX_NP + j];
#pragma unroll
          for (int c = 0; c < TD; ++c) acc[c] = fma(xy, part[c], acc[c]);
        }
      }
#pragma unroll
      for (int c = 0; c < TD; ++c) {
        double v;
        if constexpr (DF)
          v = (double)acc[c].h + (double)acc[c].l;
        else
          v = acc[c];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) acc_t[t * TD + c] += v;
      }
      __syncwarp();
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < tn * TD; e += blockDim.x) {
    const int t = e / TD, c = e % TD;
    double* o = p.out + p.perm[t0 + t] * TD + c;
    *o = p.accumulate ? *o + acc_t[e] : acc_t[e];
  }
}

cudaError_t tc_launch_l2p(const TcL2PParams& p, int td, bool df, int n_batches, int batch_max, cudaStream_t st) {
  if (n_batches == 0) return cudaSuccess;
  const size_t smem =
      ((size_t)p.np * p.np * p.np * td + (TC_THREADS / 32) * 3 * TC_MAX_NP + (size_t)batch_max * td) * sizeof(double);
  auto kern = td == 3 ? (df ? tc_l2p_kernel<3, true> : tc_l2p_kernel<3, false>)
                      : (df ? tc_l2p_kernel<1, true> : tc_l2p_kernel<1, false>);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  kern<<<n_batches, TC_THREADS, smem, st>>>(p);
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return cudaGetLastError();
}

}  // namespace
}  // namespace sctlgpu

using namespace sctlgpu;

struct sctlgpu_treecode_s {
  int kernel = 0, mode = 0, digits = 0, ND = 0, SD = 0, TD = 0;
  bool df = false;  // moments and downward pass in double-float (plans in FP32 or double-float arithmetic)
  int device = 0, sms = 1, batch_max = 0;
  TcLayout L;
  int64_t ns = 0, nt = 0, n_items = 0, n_pieces = 0;
  int pass_items = 1;  // moment chunks per pass
  double *d_trg = nullptr, *d_r = nullptr, *d_n = nullptr, *d_v = nullptr, *d_part = nullptr, *d_u = nullptr;
  double *h_in = nullptr, *h_out = nullptr;  // device staging of host-array executions (allocated on first use)
  double *d_xs = nullptr, *d_xn = nullptr, *d_xt = nullptr;  // the direct form: inputs in their own order
  int64_t *d_slot_src = nullptr, *d_tperm = nullptr, *d_bt0 = nullptr;
  int32_t *d_btn = nullptr, *d_anc_ptr = nullptr, *d_anc = nullptr;
  TcCluster* d_clusters = nullptr;
  TcItem* d_items = nullptr;
  TcTrgBox* d_boxes = nullptr;
  TcCheb* d_cheb = nullptr;
  sctlgpu_near_plan plan = nullptr;
  sctlgpu_near_plan plan_sym = nullptr;  // the symmetric-density proxies' blocks (Stokes double layer)
};

namespace {

void tc_free(sctlgpu_treecode_s* T) {
  if (T->plan) sctlgpu_near_plan_destroy(T->plan);
  if (T->plan_sym) sctlgpu_near_plan_destroy(T->plan_sym);
  for (void* q : {(void*)T->d_trg, (void*)T->d_r, (void*)T->d_n, (void*)T->d_v, (void*)T->d_part, (void*)T->d_u,
                  (void*)T->h_in, (void*)T->h_out, (void*)T->d_xs, (void*)T->d_xn, (void*)T->d_xt,
                  (void*)T->d_slot_src, (void*)T->d_tperm, (void*)T->d_bt0, (void*)T->d_btn, (void*)T->d_anc_ptr,
                  (void*)T->d_anc, (void*)T->d_clusters, (void*)T->d_items, (void*)T->d_boxes, (void*)T->d_cheb})
    cudaFree(q);
  delete T;
}

int tc_check_common(int kernel, int64_t ns, const double* r_src, int64_t nt, const double* r_trg) {
  if (kernel < 0 || kernel > SCTLGPU_STOKES3D_DXU) return SCTLGPU_ERR_INVALID_KERNEL;
  if (ns < 0 || nt < 0 || ns > (INT64_C(1) << 40) || nt > (INT64_C(1) << 40)) return SCTLGPU_ERR_INVALID_SIZE;
  if ((ns && !r_src) || (nt && !r_trg)) return SCTLGPU_ERR_NULL_POINTER;
  for (int64_t i = 0; i < 3 * ns; ++i)
    if (!std::isfinite(r_src[i])) return SCTLGPU_ERR_INVALID_ARGUMENT;
  for (int64_t i = 0; i < 3 * nt; ++i)
    if (!std::isfinite(r_trg[i])) return SCTLGPU_ERR_INVALID_ARGUMENT;
  return SCTLGPU_OK;
}

int tc_layout_from(int kernel, int digits, int64_t ns, const double* r_src, int64_t nt, const double* r_trg,
                   const sctlgpu_treecode_params* prm, TcLayout& L, int* batch_max) {
  int order = prm ? prm->order : 0;
  double theta = prm ? prm->theta : 0.0;
  tc_defaults(digits, &order, &theta);
  const double theta_trg = prm ? prm->theta_trg : 0.0;
  const int64_t leaf = prm ? prm->leaf_max : 0;
  const bool dual = !prm || prm->dual != 0;
  const bool sym = true;  // the Stokes double layer's proxies: one symmetric density per point
  if (prm && prm->batch_max > 0) {
    if (batch_max) *batch_max = prm->batch_max;
    return tc_build_layout(kernel, ns, r_src, nt, r_trg, order, theta, theta_trg, leaf, prm->batch_max, dual, sym,
                           L);
  }
  // Batches of 512 and of 256 targets (built concurrently): the one with fewer interactions, the
  // larger on a near tie (fewer blocks).  Targets filling a volume favour 256 (sphere/ball: 0.147
  // vs 0.166 of Ns * Nt at digits 10, 7-17 % faster), targets hugging a surface tie (torus).
  TcLayout S;
  int rc_s = SCTLGPU_OK;
  std::thread small;
  if (nt > 512)
    small = std::thread([&] {
      rc_s = tc_build_layout(kernel, ns, r_src, nt, r_trg, order, theta, theta_trg, leaf, 256, dual, sym, S);
    });
  int rc = tc_build_layout(kernel, ns, r_src, nt, r_trg, order, theta, theta_trg, leaf, 512, dual, sym, L);
  if (small.joinable()) small.join();
  if (rc) return rc;
  if (batch_max) *batch_max = 512;
  if (nt > 512) {
    if (rc_s) return rc_s;
    if ((double)S.pp + S.pw * (double)S.approx < 0.97 * ((double)L.pp + L.pw * (double)L.approx)) {
      L = std::move(S);
      if (batch_max) *batch_max = 256;
    }
  }
  return SCTLGPU_OK;
}

void tc_sizes(const TcLayout& L, int64_t* sizes) {
  sizes[0] = (int64_t)L.blocks.size();
  sizes[1] = L.n_src_slots;
  sizes[2] = L.n_slots;
  sizes[3] = (int64_t)L.clusters.size();
  sizes[4] = L.pp;
  sizes[5] = L.approx;
  sizes[6] = L.order;
  sizes[7] = L.n_trg_slots;
  sizes[8] = (int64_t)L.tclusters.size();
  sizes[9] = L.direct ? 1 : 0;
}

}  // namespace

extern "C" {

int sctlgpu_treecode_layout(int kernel, int64_t ns, const double* r_src, int64_t nt, const double* r_trg,
                            const sctlgpu_treecode_params* prm, int digits, int64_t* sizes, double* theta_out,
                            sctlgpu_block* blocks, int64_t* slot_src, int64_t* trg_order, int64_t* clusters,
                            int64_t* trg_clusters) {
  int rc = tc_check_common(kernel, ns, r_src, nt, r_trg);
  if (rc) return rc;
  if (!sizes) return SCTLGPU_ERR_NULL_POINTER;
  TcLayout L;
  if ((rc = tc_layout_from(kernel, digits, ns, r_src, nt, r_trg, prm, L, nullptr))) return rc;
  tc_sizes(L, sizes);
  if (theta_out) *theta_out = L.theta;
  if (blocks) std::copy(L.blocks.begin(), L.blocks.end(), blocks);
  if (slot_src) {
    std::copy(L.slot_src.begin(), L.slot_src.end(), slot_src);
    for (int64_t i = L.n_src_slots; i < L.n_slots; ++i) slot_src[i] = -2;  // proxy slots
  }
  if (trg_order) std::copy(L.tperm.begin(), L.tperm.end(), trg_order);
  if (clusters)
    for (size_t k = 0; k < L.clusters.size(); ++k) {
      const TcNode& C = L.src[L.clusters[k]];
      const int64_t row[7] = {C.sb, C.se, C.proxy, C.proxy + tc_proxy_slots(L, C), C.g[0], C.g[1], C.g[2]};
      std::copy(row, row + 7, clusters + 7 * k);
    }
  if (trg_clusters)
    for (size_t k = 0; k < L.tclusters.size(); ++k) {
      const TcNode& C = L.trg[L.tclusters[k]];
      const int64_t row[7] = {C.b, C.e, C.proxy, C.proxy + C.npts, C.g[0], C.g[1], C.g[2]};
      std::copy(row, row + 7, trg_clusters + 7 * k);
    }
  return SCTLGPU_OK;
}

int sctlgpu_treecode_create(sctlgpu_treecode* out, int kernel, int mode, int digits, int64_t ns, const double* r_src,
                            const double* n_src, int64_t nt, const double* r_trg, const sctlgpu_treecode_params* prm) {
  if (!out) return SCTLGPU_ERR_NULL_POINTER;
  *out = nullptr;
  int rc = tc_check_common(kernel, ns, r_src, nt, r_trg);
  if (rc) return rc;
  if (mode != SCTLGPU_F64 && mode != SCTLGPU_MIXED) return SCTLGPU_ERR_INVALID_MODE;  // FP64 results, scattered
  int nd, sd, td;
  if (sctlgpu_kernel_dims(kernel, nullptr, &nd, &sd, &td) != SCTLGPU_OK) return SCTLGPU_ERR_INVALID_KERNEL;
  if (nd && ns && !n_src) return SCTLGPU_ERR_NULL_POINTER;
  int dev;
  unsigned* status;
  int sms;
  if ((rc = runtime_device(&dev, &status, &sms))) return rc;
  auto* T = new sctlgpu_treecode_s();
  T->kernel = kernel;
  T->mode = mode;
  T->digits = digits;
  T->ND = nd;
  T->SD = sd;
  T->TD = td;
  T->device = dev;
  T->sms = sms;
  T->ns = ns;
  T->nt = nt;
  T->df = mode == SCTLGPU_MIXED && runtime_mixed_arith(runtime_effective_digits(mode, digits)) != MIXED_ARITH_F64;
  TcLayout& L = T->L;
  if ((rc = tc_layout_from(kernel, digits, ns, r_src, nt, r_trg, prm, L, &T->batch_max))) {
    delete T;
    return rc;
  }
  if (L.direct) {  // the direct sum over the inputs as given
    cudaError_t e = cudaSuccess;
    auto up = [&](double** dst, const double* src, int64_t n) {
      if (e != cudaSuccess) return;
      e = cudaMalloc((void**)dst, std::max<size_t>((size_t)n * sizeof(double), 16));
      if (e == cudaSuccess && n) e = cudaMemcpy(*dst, src, (size_t)n * sizeof(double), cudaMemcpyHostToDevice);
    };
    up(&T->d_xs, r_src, 3 * ns);
    if (nd) up(&T->d_xn, n_src, 3 * ns);
    up(&T->d_xt, r_trg, 3 * nt);
    if (e != cudaSuccess) {
      tc_free(T);
      return runtime_record(e);
    }
    *out = T;
    return SCTLGPU_OK;
  }
  // source slots: sources (sorted, padded), then the source proxies
  const int64_t S = L.n_slots;
  std::vector<double> hr((size_t)S * 3, 0.0), hn(nd ? (size_t)S * 3 : 0, 0.0), hv((size_t)S * sd, 0.0);
  for (int64_t i = 0; i < L.n_src_slots; ++i) {
    int64_t s = L.slot_src[i];
    const bool pad = s < 0;
    if (pad) s = L.slot_src[i - 1];  // padding sits on its leaf's last source, with zero charge
    for (int d = 0; d < 3; ++d) hr[i * 3 + d] = r_src[s * 3 + d];
    if (nd && !pad)
      for (int d = 0; d < 3; ++d) hn[i * 3 + d] = n_src[s * 3 + d];
  }
  const TcCheb& cb = tc_cheb();
  // coordinates of grid point k of a cluster's grid
  auto grid_point = [&](const TcNode& C, int k, double* x) {
    const int ijk[3] = {k / (C.g[1] * C.g[2]), (k / C.g[2]) % C.g[1], k % C.g[2]};
    for (int d = 0; d < 3; ++d) x[d] = cheb_coord(C.lo[d], C.hi[d], cb.x[C.g[d] - 1][ijk[d]]);
  };
  std::vector<TcCluster> hc;
  std::vector<TcItem> hi;
  for (int32_t id : L.clusters) {
    const TcNode& C = L.src[id];
    TcCluster tc{};
    interp_box(C, tc.lo, tc.inv);
    tc.proxy = C.proxy;
    for (int d = 0; d < 3; ++d) tc.g[d] = C.g[d];
    tc.item0 = (int32_t)hi.size();
    for (int64_t s0 = C.sb; s0 < C.se; s0 += TC_CHUNK)
      hi.push_back({(int32_t)hc.size(), (int32_t)std::min<int64_t>(TC_CHUNK, C.se - s0), s0});
    tc.item1 = (int32_t)hi.size();
    const int64_t slots = tc_proxy_slots(L, C);
    for (int k = 0; k < slots; ++k) {
      const int pt = std::min(k / L.per_point, C.npts - 1);  // the padding slot repeats the last point
      const int64_t slot = C.proxy + k;
      grid_point(C, pt, hr.data() + slot * 3);
      const bool real = k < C.npts * L.per_point;
      if (kernel == SCTLGPU_LAPLACE3D_DXU && real) hv[slot] = 1.0;  // the moment is the proxy's normal
      if (kernel == SCTLGPU_STOKES3D_DXU && !L.sym && real) hn[slot * 3 + k % 3] = 1.0;  // normal e_c
    }
    hc.push_back(tc);
  }
  T->n_items = (int64_t)hi.size();
  const int64_t npts = L.npts, Q = kernel == SCTLGPU_STOKES3D_DXU ? 9 : (kernel == SCTLGPU_LAPLACE3D_FXU ? 1 : 3);
  // partial moments per chunk, reduced per cluster in chunk order; at most TC_PART_BYTES of
  // them at a time (more chunks: several passes)
  const double part_bytes = prm && prm->moment_bytes > 0 ? prm->moment_bytes : TC_PART_BYTES;
  T->pass_items = (int)std::max<int64_t>(
      1, std::min<int64_t>(T->n_items, (int64_t)(part_bytes / (double)(npts * Q * sizeof(double)))));
  // target list: sorted targets, then the target clusters' proxies (their Chebyshev points)
  const int64_t NT = L.n_trg_slots;
  std::vector<double> htrg((size_t)NT * 3);
  for (int64_t k = 0; k < nt; ++k)
    for (int d = 0; d < 3; ++d) htrg[k * 3 + d] = r_trg[L.tperm[k] * 3 + d];
  std::vector<TcTrgBox> hb;
  for (int32_t id : L.tclusters) {
    const TcNode& C = L.trg[id];
    TcTrgBox tb{};
    interp_box(C, tb.lo, tb.inv);
    tb.proxy = C.proxy;
    for (int d = 0; d < 3; ++d) tb.g[d] = C.g[d];
    for (int k = 0; k < C.npts; ++k) grid_point(C, k, htrg.data() + (C.proxy + k) * 3);
    hb.push_back(tb);
  }
  // downward-pass work: every batch in pieces of <= batch_max targets (a leaf of coincident
  // targets can hold more), each with the batch's list of target clusters
  std::vector<int64_t> hbt0;
  std::vector<int32_t> hbtn, hanc_ptr{0}, hanc;
  for (size_t bi = 0; bi < L.batches.size(); ++bi) {
    const TcNode& B = L.trg[L.batches[bi]];
    for (int64_t off = B.b; off < B.e; off += T->batch_max) {
      hbt0.push_back(off);
      hbtn.push_back((int32_t)std::min<int64_t>(T->batch_max, B.e - off));
      for (int32_t a = L.anc_ptr[bi]; a < L.anc_ptr[bi + 1]; ++a) hanc.push_back(L.anc[a]);
      hanc_ptr.push_back((int32_t)hanc.size());
    }
  }
  T->n_pieces = (int64_t)hbt0.size();
  cudaError_t e = cudaSuccess;
  auto up = [&](void** dst, const void* src, size_t bytes) {
    if (e != cudaSuccess) return;
    e = cudaMalloc(dst, std::max<size_t>(bytes, 16));
    if (e == cudaSuccess && bytes) e = cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice);
  };
  up((void**)&T->d_trg, htrg.data(), htrg.size() * sizeof(double));
  up((void**)&T->d_r, hr.data(), hr.size() * sizeof(double));
  if (nd) up((void**)&T->d_n, hn.data(), hn.size() * sizeof(double));
  up((void**)&T->d_v, hv.data(), hv.size() * sizeof(double));
  up((void**)&T->d_slot_src, L.slot_src.data(), L.slot_src.size() * sizeof(int64_t));
  up((void**)&T->d_clusters, hc.data(), hc.size() * sizeof(TcCluster));
  up((void**)&T->d_items, hi.data(), hi.size() * sizeof(TcItem));
  up((void**)&T->d_tperm, L.tperm.data(), L.tperm.size() * sizeof(int64_t));
  up((void**)&T->d_boxes, hb.data(), hb.size() * sizeof(TcTrgBox));
  up((void**)&T->d_cheb, &cb, sizeof(TcCheb));
  up((void**)&T->d_bt0, hbt0.data(), hbt0.size() * sizeof(int64_t));
  up((void**)&T->d_btn, hbtn.data(), hbtn.size() * sizeof(int32_t));
  up((void**)&T->d_anc_ptr, hanc_ptr.data(), hanc_ptr.size() * sizeof(int32_t));
  up((void**)&T->d_anc, hanc.data(), hanc.size() * sizeof(int32_t));
  if (e == cudaSuccess)
    e = cudaMalloc((void**)&T->d_part, std::max<size_t>(16, (size_t)T->pass_items * npts * Q * sizeof(double)));
  if (e == cudaSuccess) e = cudaMalloc((void**)&T->d_u, std::max<size_t>(16, (size_t)NT * td * sizeof(double)));
  if (e != cudaSuccess) {
    tc_free(T);
    return runtime_record(e);
  }
  // the plan accumulates into d_u over the whole target list (identity map: the scattered,
  // zero-initialised form of the plan); with symmetric-density proxies their blocks form a
  // second plan that adds to the first one's sums
  std::vector<int64_t> ident((size_t)NT);
  std::iota(ident.begin(), ident.end(), (int64_t)0);
  std::vector<sctlgpu_block> pb, sb;
  for (const sctlgpu_block& b : L.blocks) (L.sym && b.src_begin >= L.n_src_slots ? sb : pb).push_back(b);
  rc = sctlgpu_near_plan_create(&T->plan, kernel, mode, digits, (int64_t)pb.size(), pb.data(), S, NT,
                                NT ? ident.data() : nullptr, NT);
  if (!rc && !sb.empty())
    rc = near_plan_create_sym(&T->plan_sym, mode, digits, (int64_t)sb.size(), sb.data(), S, NT, ident.data(), NT);
  if (rc) {
    tc_free(T);
    return rc;
  }
  *out = T;
  return SCTLGPU_OK;
}

static int tc_execute_device(sctlgpu_treecode T, const double* v_src, double* v_out, unsigned flags, void* stream);

int sctlgpu_treecode_execute(sctlgpu_treecode T, const double* v_src, double* v_out, unsigned flags, void* stream) {
  if (!T) return SCTLGPU_ERR_NULL_POINTER;
  if (flags & ~(unsigned)(SCTLGPU_ACCUMULATE | SCTLGPU_DEVICE_PTRS)) return SCTLGPU_ERR_INVALID_ARGUMENT;
  if ((T->ns && !v_src) || (T->nt && !v_out)) return SCTLGPU_ERR_NULL_POINTER;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev != T->device) return SCTLGPU_ERR_INVALID_ARGUMENT;
  if (flags & SCTLGPU_DEVICE_PTRS) return tc_execute_device(T, v_src, v_out, flags, stream);
  // host arrays: staged through device buffers kept with the treecode, synchronous
  cudaStream_t st = (cudaStream_t)stream;
  const size_t bin = (size_t)T->ns * T->SD * sizeof(double), bout = (size_t)T->nt * T->TD * sizeof(double);
  cudaError_t e = cudaSuccess;
  if (!T->h_in && (e = cudaMalloc((void**)&T->h_in, std::max<size_t>(bin, 16))) != cudaSuccess) return runtime_record(e);
  if (!T->h_out && (e = cudaMalloc((void**)&T->h_out, std::max<size_t>(bout, 16))) != cudaSuccess)
    return runtime_record(e);
  if (bin && (e = cudaMemcpyAsync(T->h_in, v_src, bin, cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return runtime_record(e);
  if ((flags & SCTLGPU_ACCUMULATE) && bout &&
      (e = cudaMemcpyAsync(T->h_out, v_out, bout, cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return runtime_record(e);
  const int rc = tc_execute_device(T, T->h_in, T->h_out, flags | SCTLGPU_DEVICE_PTRS, stream);
  if (rc) return rc;
  if (bout && (e = cudaMemcpyAsync(v_out, T->h_out, bout, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
    return runtime_record(e);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return runtime_record(e);
  int rc2 = T->plan ? sctlgpu_near_plan_status(T->plan, stream) : SCTLGPU_OK;
  if (!rc2 && T->plan_sym) rc2 = sctlgpu_near_plan_status(T->plan_sym, stream);
  return rc2;
}

static int tc_execute_device(sctlgpu_treecode T, const double* v_src, double* v_out, unsigned flags, void* stream) {
  if (T->L.direct)
    return sctlgpu_eval(T->kernel, T->mode, T->digits, T->nt, T->d_xt, T->ns, T->d_xs, T->d_xn, v_src, v_out,
                        (flags & SCTLGPU_ACCUMULATE) | SCTLGPU_DEVICE_PTRS, stream);
  cudaStream_t st = (cudaStream_t)stream;
  const TcLayout& L = T->L;
  cudaError_t e = cudaSuccess;
  if (T->nt == 0) return SCTLGPU_OK;
  if (L.n_src_slots) {
    const int64_t work = L.n_src_slots * T->SD;
    tc_gather_kernel<<<(unsigned)std::min<int64_t>((work + 255) / 256, (int64_t)T->sms * 16), 256, 0, st>>>(
        L.n_src_slots, T->SD, T->d_slot_src, v_src, T->d_v);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    if ((e = cudaGetLastError()) != cudaSuccess) return runtime_record(e);
  }
  TcMomParams p{};
  p.clusters = T->d_clusters;
  p.items = T->d_items;
  p.r = T->d_r;
  p.n = T->d_n;
  p.v = T->d_v;
  p.part = T->d_part;
  p.pn = T->d_n;
  p.pv = T->d_v;
  p.np = L.np;
  p.cheb = T->d_cheb;
  p.sym = L.sym ? 1 : 0;
  TcL2PParams q{};
  q.boxes = T->d_boxes;
  q.bt0 = T->d_bt0;
  q.btn = T->d_btn;
  q.anc_ptr = T->d_anc_ptr;
  q.anc = T->d_anc;
  q.r = T->d_trg;
  q.u = T->d_u;
  q.perm = T->d_tperm;
  q.out = v_out;
  q.accumulate = (flags & SCTLGPU_ACCUMULATE) ? 1 : 0;
  q.np = L.np;
  q.cheb = T->d_cheb;
  const int nc = (int)L.clusters.size(), ni = (int)T->n_items;
  switch (T->kernel) {
    case SCTLGPU_LAPLACE3D_FXU: e = tc_launch_moments<SCTLGPU_LAPLACE3D_FXU>(p, ni, T->pass_items, nc, T->df, st); break;
    case SCTLGPU_LAPLACE3D_DXU: e = tc_launch_moments<SCTLGPU_LAPLACE3D_DXU>(p, ni, T->pass_items, nc, T->df, st); break;
    case SCTLGPU_STOKES3D_FXU: e = tc_launch_moments<SCTLGPU_STOKES3D_FXU>(p, ni, T->pass_items, nc, T->df, st); break;
    default: e = tc_launch_moments<SCTLGPU_STOKES3D_DXU>(p, ni, T->pass_items, nc, T->df, st); break;
  }
  if (e != cudaSuccess) return runtime_record(e);
  int rc = sctlgpu_near_plan_execute(T->plan, T->d_trg, T->d_r, T->d_n, T->d_v, nullptr, T->d_u, SCTLGPU_DEVICE_PTRS,
                                     stream);
  if (rc) return rc;
  if (T->plan_sym &&
      (rc = sctlgpu_near_plan_execute(T->plan_sym, T->d_trg, T->d_r, T->d_n, T->d_v, nullptr, T->d_u,
                                      SCTLGPU_DEVICE_PTRS | SCTLGPU_ACCUMULATE, stream)))
    return rc;
  e = tc_launch_l2p(q, T->TD, T->df, (int)T->n_pieces, T->batch_max, st);
  return e == cudaSuccess ? SCTLGPU_OK : runtime_record(e);
}

int sctlgpu_treecode_info(sctlgpu_treecode T, int64_t* stats, double* theta) {
  if (!T || !stats) return SCTLGPU_ERR_NULL_POINTER;
  tc_sizes(T->L, stats);
  if (theta) *theta = T->L.theta;
  return SCTLGPU_OK;
}

int sctlgpu_treecode_status(sctlgpu_treecode T, void* stream) {
  if (!T) return SCTLGPU_ERR_NULL_POINTER;
  if (!T->plan) {  // the direct form: the runtime's status word
    const cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    return e == cudaSuccess ? sctlgpu_device_status(stream) : runtime_record(e);
  }
  int rc = sctlgpu_near_plan_status(T->plan, stream);
  if (!rc && T->plan_sym) rc = sctlgpu_near_plan_status(T->plan_sym, stream);
  return rc;
}

int sctlgpu_treecode_destroy(sctlgpu_treecode T) {
  if (!T) return SCTLGPU_OK;
  cudaDeviceSynchronize();
  tc_free(T);
  return SCTLGPU_OK;
}

}  // extern "C"
