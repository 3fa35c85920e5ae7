// Near lists on the GPU: the GPU form of BuildNearList
// (boundary_integral.txx:50-522, single rank).
//
// Definition kept from the reference: target t is near element e when some
// source node s of e has |x_t - x_s|^2 < rad_s^2 (rad = the node's near
// distance, dist_far of GetFarFieldNodes).  Outputs, as the reference:
//   near_elem_cnt/dsp  -- per element, its near targets (element-major list,
//                         sorted by (element, target index));
//   near_trg_idx       -- the element-major list's target indices (the
//                         reference stores their coordinates, Xtrg_near);
//   near_scatter_index -- for every entry of the target-major order, its
//                         position in the element-major list (ScatterForward
//                         turns element-major data into target-major data);
//   near_trg_cnt/dsp   -- per target, its entries in the target-major order
//                         (dsp 0 for targets without entries, as the reference).
//
// The reference searches a sample-sorted Morton tree (neighbour cells at a
// depth set by each node's radius).  Here:
//   1. one warp per element: its bounding sphere (centre c_e, radius R_e =
//      max_s |x_s - c_e| + rad_s) and its nodes relative to c_e in FP32;
//   2. a uniform grid (cell h ~ 2 mean R_e, at least max R_e / 8) hashed into
//      buckets; every element is entered into the cells its sphere's box
//      overlaps (counting sort into buckets);
//   3. one thread per target looks up its own cell only, tests each listed
//      element: sphere test (FP64), node tests in FP32 with a margin, and the
//      reference's FP64 test for nodes inside the margin; count pass, scan,
//      fill pass; each target's elements are sorted (short lists);
//   4. the element-major order is a stable LSD radix sort (8-bit digits,
//      warp match-any ranks) of the target-major list by element.
// Everything is deterministic.  The build synchronises its stream once (the
// number of pairs sizes the outputs).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>
#include <vector>

#include "../../include/sctlgpu.h"
#include "launch.h"

namespace sctlgpu {
namespace {

constexpr int NL_T = 256;                    // threads per CTA
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = NL_T * SCAN_ITEMS;  // 2048
constexpr int RS_TILE = 4096;                // radix-sort tile (one warp)
constexpr int CELL_BITS = 21;                // per grid coordinate

// --------------------------------------------------------------- scan (int64)
__global__ void __launch_bounds__(NL_T) scan_tile_kernel(const int64_t* in, int64_t* out, int64_t n,
                                                         int64_t* tile_sums) {
  __shared__ int64_t warp_tot[NL_T / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
  int64_t v[SCAN_ITEMS], s = 0;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    v[i] = base + i < n ? in[base + i] : 0;
    s += v[i];
  }
  int64_t incl = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) warp_tot[w] = incl;
  __syncthreads();
  if (w == 0) {
    int64_t t = lane < NL_T / 32 ? warp_tot[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < NL_T / 32) warp_tot[lane] = t;
  }
  __syncthreads();
  int64_t run = incl - s + (w > 0 ? warp_tot[w - 1] : 0);
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    if (base + i < n) out[base + i] = run;
    run += v[i];
  }
  if (tile_sums && threadIdx.x == NL_T - 1) tile_sums[blockIdx.x] = warp_tot[NL_T / 32 - 1];
}

__global__ void scan_add_kernel(int64_t* out, int64_t n, const int64_t* tile_offs) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] += tile_offs[i / SCAN_TILE];
}

unsigned grid_for(int64_t n, int sms) {
  const int64_t b = (n + NL_T - 1) / NL_T;
  const int64_t cap = (int64_t)sms * 16;
  return (unsigned)std::max<int64_t>(1, std::min(b, cap));
}

// Exclusive prefix sum of n int64 values (in may equal out).
cudaError_t exclusive_scan(const int64_t* in, int64_t* out, int64_t n, cudaStream_t st, int sms) {
  if (n <= 0) return cudaSuccess;
  const int64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (tiles == 1) {
    scan_tile_kernel<<<1, NL_T, 0, st>>>(in, out, n, nullptr);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
  }
  int64_t* sums = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&sums, tiles * sizeof(int64_t), st);
  if (e != cudaSuccess) return e;
  scan_tile_kernel<<<(unsigned)tiles, NL_T, 0, st>>>(in, out, n, sums);
  g_launches.fetch_add(1, std::memory_order_relaxed);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = exclusive_scan(sums, sums, tiles, st, sms);
  if (e == cudaSuccess) {
    scan_add_kernel<<<grid_for(n, sms), NL_T, 0, st>>>(out, n, sums);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    e = cudaGetLastError();
  }
  cudaFreeAsync(sums, st);
  return e;
}

// ------------------------------------------------------------------ elements
struct alignas(32) Sphere {
  double x, y, z, w;  // centre and radius (w < 0: no pairs)
};

struct GridInfo {
  double o[3];  // grid origin
  double h;     // cell size
  double ih;    // 1 / h
  int64_t nbuckets;
};

__device__ __forceinline__ uint64_t cell_key(int64_t ix, int64_t iy, int64_t iz) {
  return ((uint64_t)ix << (2 * CELL_BITS)) | ((uint64_t)iy << CELL_BITS) | (uint64_t)iz;
}
__device__ __forceinline__ uint64_t bucket_of(uint64_t key, int64_t nb) {
  uint64_t x = key * 0x9E3779B97F4A7C15ull;  // multiplicative hash (Fibonacci), high bits mixed down
  x ^= x >> 29;
  return x & (uint64_t)(nb - 1);
}

// Element spheres [c, R] (R < 0: no nodes or invalid ranges) and FP32 node data
// (x_s - c_e, rad_s^2).  Also the sum and max of R (ordered-bit atomics).
__global__ void elem_sphere_kernel(int64_t n_elem, const int64_t* cnt, const int64_t* dsp, int64_t ns,
                                   const double* xs, const double* rad, Sphere* sph, float4* node32,
                                   double* sum_r, unsigned long long* max_r_bits, unsigned* status) {
  const int lane = threadIdx.x & 31;
  const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t e = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); e < n_elem; e += nw) {
    const int64_t c0 = cnt[e], d0 = dsp[e];
    if (c0 <= 0 || d0 < 0 || d0 + c0 > ns) {
      if (lane == 0) {
        sph[e] = Sphere{0, 0, 0, -1.0};
        if (c0 < 0 || d0 < 0 || d0 + c0 > ns) atomicOr(status, 4u);
      }
      continue;
    }
    double sx = 0, sy = 0, sz = 0;
    for (int64_t j = lane; j < c0; j += 32) {
      sx += xs[(d0 + j) * 3];
      sy += xs[(d0 + j) * 3 + 1];
      sz += xs[(d0 + j) * 3 + 2];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sx += __shfl_xor_sync(0xffffffffu, sx, o);
      sy += __shfl_xor_sync(0xffffffffu, sy, o);
      sz += __shfl_xor_sync(0xffffffffu, sz, o);
    }
    const double cx = sx / (double)c0, cy = sy / (double)c0, cz = sz / (double)c0;
    double R = 0.0;
    bool bad = false;
    for (int64_t j = lane; j < c0; j += 32) {
      const int64_t s = d0 + j;
      const double dx = xs[s * 3] - cx, dy = xs[s * 3 + 1] - cy, dz = xs[s * 3 + 2] - cz;
      const double r = rad[s];
      if (!(r >= 0.0) || !isfinite(dx + dy + dz)) bad = true;
      R = fmax(R, sqrt(dx * dx + dy * dy + dz * dz) + fmax(r, 0.0));
      node32[s] = make_float4((float)dx, (float)dy, (float)dz, (float)(r * r));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) R = fmax(R, __shfl_xor_sync(0xffffffffu, R, o));
    bad = __any_sync(0xffffffffu, bad);
    if (lane == 0) {
      if (bad) {
        atomicOr(status, 4u);  // negative or non-finite radius / coordinates: element skipped
        sph[e] = Sphere{cx, cy, cz, -1.0};
      } else {
        R = R * (1.0 + 1e-12) + 1e-300;  // covers the rounding of c and of the norms
        sph[e] = Sphere{cx, cy, cz, R};
        atomicAdd(sum_r, R);
        atomicMax(max_r_bits, (unsigned long long)__double_as_longlong(R));  // R > 0: bit order = value order
        atomicAdd(max_r_bits + 1, 1ull);                                     // live elements
      }
    }
  }
}

__device__ __forceinline__ bool elem_box(const Sphere& s, const GridInfo& g, int64_t lo[3], int64_t hi[3]) {
  if (!(s.w > 0)) return false;
  const double c[3] = {s.x, s.y, s.z};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    lo[k] = (int64_t)floor((c[k] - s.w - g.o[k]) * g.ih);
    hi[k] = (int64_t)floor((c[k] + s.w - g.o[k]) * g.ih);
    const int64_t top = (1ll << CELL_BITS) - 1;
    lo[k] = lo[k] < 0 ? 0 : (lo[k] > top ? top : lo[k]);
    hi[k] = hi[k] < 0 ? 0 : (hi[k] > top ? top : hi[k]);
  }
  return true;
}

__global__ void elem_cells_count_kernel(int64_t n_elem, const Sphere* sph, GridInfo g, int64_t* ecnt) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n_elem; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t lo[3], hi[3];
    ecnt[e] = elem_box(sph[e], g, lo, hi) ? (hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1) : 0;
  }
}

__global__ void elem_cells_fill_kernel(int64_t n_elem, const Sphere* sph, GridInfo g, const int64_t* eoff,
                                       uint64_t* ekey, int32_t* eelem, int64_t* bcnt) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n_elem; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t lo[3], hi[3];
    if (!elem_box(sph[e], g, lo, hi)) continue;
    int64_t k = eoff[e];
    for (int64_t ix = lo[0]; ix <= hi[0]; ++ix)
      for (int64_t iy = lo[1]; iy <= hi[1]; ++iy)
        for (int64_t iz = lo[2]; iz <= hi[2]; ++iz, ++k) {
          const uint64_t key = cell_key(ix, iy, iz);
          ekey[k] = key;
          eelem[k] = (int32_t)e;
          atomicAdd((unsigned long long*)&bcnt[bucket_of(key, g.nbuckets)], 1ull);
        }
  }
}

__global__ void bucket_place_kernel(int64_t n_entries, const uint64_t* ekey, const int32_t* eelem, GridInfo g,
                                    const int64_t* boff, int64_t* bcur, uint64_t* bkey, int32_t* belem) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_entries; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t b = bucket_of(ekey[i], g.nbuckets);
    const int64_t pos = boff[b] + (int64_t)atomicAdd((unsigned long long*)&bcur[b], 1ull);
    bkey[pos] = ekey[i];
    belem[pos] = eelem[i];
  }
}

// ------------------------------------------------------------------- targets
struct TrgParams {
  int64_t nt, ns;
  const double* xt;
  const double* xs;
  const double* rad;
  const int64_t* cnt;
  const int64_t* dsp;
  const Sphere* sph;
  const float4* node32;
  const int64_t* boff;  // [nbuckets + 1]
  const uint64_t* bkey;
  const int32_t* belem;
  GridInfo g;
};

// The reference's test, node_dist2(src, trg) < rad^2, in FP64 without contraction.
__device__ __forceinline__ bool exact_near(const double* xt, const double* xs, double r) {
  const double dx = __dsub_rn(xs[0], xt[0]), dy = __dsub_rn(xs[1], xt[1]), dz = __dsub_rn(xs[2], xt[2]);
  double d2 = __dmul_rn(dx, dx);
  d2 = __dadd_rn(d2, __dmul_rn(dy, dy));
  d2 = __dadd_rn(d2, __dmul_rn(dz, dz));
  return d2 < __dmul_rn(r, r);
}

__device__ bool elem_near(const TrgParams& p, int64_t e, const double x[3]) {
  const Sphere s = p.sph[e];
  if (!(s.w > 0)) return false;
  // Every operation explicitly rounded: the count and fill passes must take identical decisions.
  const double rx = __dsub_rn(x[0], s.x), ry = __dsub_rn(x[1], s.y), rz = __dsub_rn(x[2], s.z);
  const double R2 = __dmul_rn(s.w, s.w);
  const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(rx, rx), __dmul_rn(ry, ry)), __dmul_rn(rz, rz));
  if (r2 >= __dmul_rn(R2, 1.0 + 1e-12)) return false;  // outside the element's sphere
  const float fx = __double2float_rn(rx), fy = __double2float_rn(ry), fz = __double2float_rn(rz);
  const float margin = __fmul_rn(1e-5f, __double2float_rn(R2));  // >> the FP32 rounding of d2 (terms <= ~4 R^2)
  const int64_t c0 = p.cnt[e], d0 = p.dsp[e];
  for (int64_t j = 0; j < c0; ++j) {
    const float4 nd = p.node32[d0 + j];
    const float ax = __fsub_rn(fx, nd.x), ay = __fsub_rn(fy, nd.y), az = __fsub_rn(fz, nd.z);
    const float d2 = __fmaf_rn(ax, ax, __fmaf_rn(ay, ay, __fmul_rn(az, az)));
    if (d2 < __fsub_rn(nd.w, margin)) return true;
    if (d2 <= __fadd_rn(nd.w, margin) && exact_near(x, p.xs + (d0 + j) * 3, p.rad[d0 + j])) return true;
  }
  return false;
}

template <bool FILL>
__global__ void __launch_bounds__(NL_T) trg_pairs_kernel(TrgParams p, int64_t* tcnt, const int64_t* toff,
                                                         int32_t* pair_e, int64_t* pair_t, unsigned* status) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < p.nt; t += (int64_t)gridDim.x * blockDim.x) {
    const double x[3] = {p.xt[t * 3], p.xt[t * 3 + 1], p.xt[t * 3 + 2]};
    int64_t ic[3];
    bool inside = true;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double f = floor((x[k] - p.g.o[k]) * p.g.ih);
      inside = inside && f >= 0.0 && f < (double)(1ll << CELL_BITS);
      ic[k] = inside ? (int64_t)f : 0;
    }
    int64_t n = 0;
    if (inside) {
      const uint64_t key = cell_key(ic[0], ic[1], ic[2]);
      const uint64_t b = bucket_of(key, p.g.nbuckets);
      const int64_t base = FILL ? toff[t] : 0;
      const int64_t cap = FILL ? tcnt[t] : 0;
      for (int64_t i = p.boff[b]; i < p.boff[b + 1]; ++i) {
        if (p.bkey[i] != key) continue;
        const int32_t e = p.belem[i];
        if (!elem_near(p, e, x)) continue;
        if (FILL) {
          if (n >= cap) {  // cannot happen (same decisions as the count pass); never write past the segment
            atomicOr(status, 2u);
            break;
          }
          // insertion into the target's sorted element list
          int64_t k = base + n;
          while (k > base && pair_e[k - 1] > e) {
            pair_e[k] = pair_e[k - 1];
            --k;
          }
          pair_e[k] = e;
          pair_t[base + n] = t;
        }
        ++n;
      }
    }
    if (!FILL) tcnt[t] = n;
  }
}

// ------------------------------------------------------------ radix sort
__global__ void radix_hist_kernel(const int32_t* keys, int64_t n, int shift, int64_t ntiles, int64_t* hist) {
  __shared__ unsigned c[256];
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    c[threadIdx.x] = 0;
    __syncthreads();
    const int64_t a = tile * RS_TILE, b = std::min<int64_t>(n, a + RS_TILE);
    for (int64_t i = a + threadIdx.x; i < b; i += blockDim.x) atomicAdd(&c[(keys[i] >> shift) & 255], 1u);
    __syncthreads();
    hist[(int64_t)threadIdx.x * ntiles + tile] = c[threadIdx.x];
    __syncthreads();
  }
}

// One warp per tile, items in order: stable ranks from match-any groups.
__global__ void radix_scatter_kernel(const int32_t* kin, const int64_t* vin, int32_t* kout, int64_t* vout, int64_t n,
                                     int shift, int64_t ntiles, const int64_t* offs) {
  __shared__ int64_t base[256];
  const int lane = threadIdx.x;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    for (int d = lane; d < 256; d += 32) base[d] = offs[(int64_t)d * ntiles + tile];
    __syncwarp();
    const int64_t a = tile * RS_TILE, b = std::min<int64_t>(n, a + RS_TILE);
    for (int64_t c = a; c < b; c += 32) {
      const int64_t i = c + lane;
      const bool act = i < b;
      const int32_t k = act ? kin[i] : 0;
      const int d = act ? ((k >> shift) & 255) : 256 + lane;
      const unsigned peers = __match_any_sync(0xffffffffu, d);
      const int rank = __popc(peers & ((1u << lane) - 1u));
      const int64_t pos = act ? base[d] + rank : 0;
      __syncwarp();
      if (act) {
        kout[pos] = k;
        vout[pos] = vin ? vin[i] : i;
        if (lane == __ffs(peers) - 1) base[d] += __popc(peers);
      }
      __syncwarp();
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------- outputs
__global__ void elem_count_kernel(int64_t n, const int32_t* pair_e, int64_t* ecnt) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    atomicAdd((unsigned long long*)&ecnt[pair_e[i]], 1ull);
}

__global__ void finish_kernel(int64_t n, const int64_t* perm, const int64_t* pair_t, int64_t* trg_idx,
                              int64_t* scatter) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = perm ? perm[k] : k;
    trg_idx[k] = pair_t[i];
    scatter[i] = k;
  }
}

__global__ void widen_kernel(int64_t n, const int32_t* in, int64_t* out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = in[i];
}

// Element of every element-major entry: the last element whose offset is <= the
// entry's position (an element without entries shares its offset with the next
// element, so the last such element is the one that owns the entry).
__global__ void elem_index_kernel(int64_t n_near, int64_t n_elem, const int64_t* __restrict__ dsp,
                                  int64_t* __restrict__ out) {
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n_near; j += (int64_t)gridDim.x * blockDim.x) {
    int64_t lo = 0, hi = n_elem - 1;  // dsp[lo] <= j always holds (dsp[0] == 0)
    while (lo < hi) {
      const int64_t mid = (lo + hi + 1) >> 1;
      if (dsp[mid] <= j) lo = mid; else hi = mid - 1;
    }
    out[j] = lo;
  }
}

__global__ void trg_dsp_fix_kernel(int64_t nt, const int64_t* tcnt, int64_t* tdsp) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += (int64_t)gridDim.x * blockDim.x)
    if (tcnt[t] == 0) tdsp[t] = 0;
}

}  // namespace
}  // namespace sctlgpu

using namespace sctlgpu;

struct sctlgpu_near_list_s {
  int device = 0;
  int64_t nt = 0, n_elem = 0, n_near = 0;
  int64_t* elem_cnt = nullptr;
  int64_t* elem_dsp = nullptr;
  int64_t* trg_idx = nullptr;
  int64_t* scatter = nullptr;
  int64_t* trg_cnt = nullptr;
  int64_t* trg_dsp = nullptr;
  int64_t* trg_elem = nullptr;  // target-major element indices
  unsigned status = 0;
};

namespace {

void free_list(sctlgpu_near_list_s* L) {
  if (!L) return;
  int cur = 0;
  cudaGetDevice(&cur);
  cudaSetDevice(L->device);
  for (int64_t* p : {L->elem_cnt, L->elem_dsp, L->trg_idx, L->scatter, L->trg_cnt, L->trg_dsp, L->trg_elem})
    if (p) cudaFree(p);
  cudaSetDevice(cur);
  delete L;
}

// Device copy of a caller array (or the pointer itself for device inputs).
template <class T>
cudaError_t stage(const T* src, int64_t n, bool dev_ptrs, cudaStream_t st, const T** out, std::vector<void*>& owned) {
  if (dev_ptrs || n == 0) {
    *out = src;
    return cudaSuccess;
  }
  void* d = nullptr;
  cudaError_t e = cudaMallocAsync(&d, n * sizeof(T), st);
  if (e != cudaSuccess) return e;
  owned.push_back(d);
  *out = (const T*)d;
  return cudaMemcpyAsync(d, src, n * sizeof(T), cudaMemcpyHostToDevice, st);
}

}  // namespace

extern "C" int sctlgpu_near_list_build(sctlgpu_near_list* out, int64_t nt, const double* r_trg, int64_t n_elem,
                                       const int64_t* elem_nds_cnt, const int64_t* elem_nds_dsp, int64_t ns,
                                       const double* r_src, const double* src_radius, unsigned flags,
                                       void* stream) {
  if (!out) return SCTLGPU_ERR_NULL_POINTER;
  *out = nullptr;
  if (nt < 0 || n_elem < 0 || ns < 0 || n_elem >= (1ll << 31) || nt > (1ll << 40) || ns > (1ll << 40))
    return SCTLGPU_ERR_INVALID_SIZE;
  if ((nt && !r_trg) || (n_elem && (!elem_nds_cnt || !elem_nds_dsp)) || (ns && (!r_src || !src_radius)))
    return SCTLGPU_ERR_NULL_POINTER;
  if (flags & ~(unsigned)SCTLGPU_DEVICE_PTRS) return SCTLGPU_ERR_INVALID_ARGUMENT;
  int dev;
  unsigned* status;
  int sms;
  int rc = runtime_device(&dev, &status, &sms);
  if (rc) return rc;
  const bool dp = (flags & SCTLGPU_DEVICE_PTRS) != 0;
  cudaStream_t st = (cudaStream_t)stream;

  auto* L = new sctlgpu_near_list_s();
  L->device = dev;
  L->nt = nt;
  L->n_elem = n_elem;
  std::vector<void*> tmp;  // stream-ordered scratch, freed at the end
  auto scratch = [&](size_t bytes, void** p) {
    cudaError_t e = cudaMallocAsync(p, std::max<size_t>(bytes, 16), st);
    if (e == cudaSuccess) tmp.push_back(*p);
    return e;
  };
  cudaError_t e = cudaSuccess;
  do {
    if ((e = cudaMalloc(&L->elem_cnt, std::max<int64_t>(n_elem + 1, 1) * 8))) break;
    if ((e = cudaMalloc(&L->elem_dsp, std::max<int64_t>(n_elem + 1, 1) * 8))) break;
    if ((e = cudaMalloc(&L->trg_cnt, std::max<int64_t>(nt + 1, 1) * 8))) break;
    if ((e = cudaMalloc(&L->trg_dsp, std::max<int64_t>(nt + 1, 1) * 8))) break;
    if ((e = cudaMemsetAsync(L->elem_cnt, 0, std::max<int64_t>(n_elem + 1, 1) * 8, st))) break;
    if ((e = cudaMemsetAsync(L->elem_dsp, 0, std::max<int64_t>(n_elem + 1, 1) * 8, st))) break;
    if ((e = cudaMemsetAsync(L->trg_cnt, 0, std::max<int64_t>(nt + 1, 1) * 8, st))) break;
    if ((e = cudaMemsetAsync(L->trg_dsp, 0, std::max<int64_t>(nt + 1, 1) * 8, st))) break;
    if (nt == 0 || n_elem == 0 || ns == 0) break;

    const double *xt, *xs, *rad;
    const int64_t *cnt, *dsp;
    if ((e = stage(r_trg, nt * 3, dp, st, &xt, tmp))) break;
    if ((e = stage(r_src, ns * 3, dp, st, &xs, tmp))) break;
    if ((e = stage(src_radius, ns, dp, st, &rad, tmp))) break;
    if ((e = stage(elem_nds_cnt, n_elem, dp, st, &cnt, tmp))) break;
    if ((e = stage(elem_nds_dsp, n_elem, dp, st, &dsp, tmp))) break;

    // 1. element spheres, FP32 node data, sum / max of R; bounding box of targets and nodes
    Sphere* sph;
    float4* node32;
    double* stats;  // [0] sum R, [1] max R bits
    BBox* bb;
    if ((e = scratch(n_elem * sizeof(Sphere), (void**)&sph))) break;
    if ((e = scratch(ns * sizeof(float4), (void**)&node32))) break;
    if ((e = scratch(64, (void**)&stats))) break;
    if ((e = scratch(64, (void**)&bb))) break;
    if ((e = cudaMemsetAsync(stats, 0, 64, st))) break;
    elem_sphere_kernel<<<grid_for(n_elem * 32, sms), NL_T, 0, st>>>(n_elem, cnt, dsp, ns, xs, rad, sph, node32, stats,
                                                                   (unsigned long long*)(stats + 1), status);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    if ((e = cudaGetLastError())) break;
    if ((e = compute_bbox(st, nt, xt, ns, xs, bb))) break;
    double hs[3];
    double hb[8];
    if ((e = cudaMemcpyAsync(hs, stats, 24, cudaMemcpyDeviceToHost, st))) break;
    if ((e = cudaMemcpyAsync(hb, bb, 64, cudaMemcpyDeviceToHost, st))) break;
    if ((e = cudaStreamSynchronize(st))) break;
    double max_r;
    std::memcpy(&max_r, &hs[1], 8);
    const int64_t live = (int64_t)((const unsigned long long*)hs)[2];
    if (!(max_r > 0)) break;  // no element with nodes: no pairs
    // bbox: ordered-bit min/max encoded by compute_bbox; decode on the host
    double lo[3], hi[3];
    {
      const uint64_t* u = (const uint64_t*)hb;
      auto dec = [](uint64_t v) {
        const uint64_t b = (v & 0x8000000000000000ull) ? (v ^ 0x8000000000000000ull) : ~v;
        double d;
        std::memcpy(&d, &b, 8);
        return d;
      };
      for (int k = 0; k < 3; ++k) {
        lo[k] = dec(u[k]);
        hi[k] = dec(u[3 + k]);
      }
    }
    const double mean_r = hs[0] / (double)std::max<int64_t>(1, live);
    double ext = 0;
    for (int k = 0; k < 3; ++k) ext = std::max(ext, hi[k] - lo[k]);
    ext += 2 * max_r;
    double h = std::max({2.0 * mean_r, max_r / 8.0, ext * std::ldexp(1.0, -(CELL_BITS - 2)), 1e-300});
    GridInfo g;
    for (int k = 0; k < 3; ++k) g.o[k] = lo[k] - max_r - h;
    g.h = h;
    g.ih = 1.0 / h;

    // 2. elements into grid cells, cells into hash buckets
    int64_t* ecnt;
    if ((e = scratch((n_elem + 1) * 8, (void**)&ecnt))) break;
    if ((e = cudaMemsetAsync(ecnt, 0, (n_elem + 1) * 8, st))) break;
    elem_cells_count_kernel<<<grid_for(n_elem, sms), NL_T, 0, st>>>(n_elem, sph, g, ecnt);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    if ((e = exclusive_scan(ecnt, ecnt, n_elem + 1, st, sms))) break;
    int64_t n_entries = 0;
    if ((e = cudaMemcpyAsync(&n_entries, ecnt + n_elem, 8, cudaMemcpyDeviceToHost, st))) break;
    if ((e = cudaStreamSynchronize(st))) break;
    int64_t nb = 1024;
    while (nb < 2 * n_entries) nb <<= 1;
    g.nbuckets = nb;
    uint64_t *ekey, *bkey;
    int32_t *eelem, *belem;
    int64_t *bcnt, *bcur;
    if ((e = scratch(n_entries * 8, (void**)&ekey))) break;
    if ((e = scratch(n_entries * 4, (void**)&eelem))) break;
    if ((e = scratch(n_entries * 8, (void**)&bkey))) break;
    if ((e = scratch(n_entries * 4, (void**)&belem))) break;
    if ((e = scratch((nb + 1) * 8, (void**)&bcnt))) break;
    if ((e = scratch(nb * 8, (void**)&bcur))) break;
    if ((e = cudaMemsetAsync(bcnt, 0, (nb + 1) * 8, st))) break;
    if ((e = cudaMemsetAsync(bcur, 0, nb * 8, st))) break;
    elem_cells_fill_kernel<<<grid_for(n_elem, sms), NL_T, 0, st>>>(n_elem, sph, g, ecnt, ekey, eelem, bcnt);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    if ((e = exclusive_scan(bcnt, bcnt, nb + 1, st, sms))) break;
    bucket_place_kernel<<<grid_for(n_entries, sms), NL_T, 0, st>>>(n_entries, ekey, eelem, g, bcnt, bcur, bkey, belem);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    if ((e = cudaGetLastError())) break;

    // 3. per-target near elements: count, scan, fill (sorted per target)
    TrgParams tp;
    tp.nt = nt;
    tp.ns = ns;
    tp.xt = xt;
    tp.xs = xs;
    tp.rad = rad;
    tp.cnt = cnt;
    tp.dsp = dsp;
    tp.sph = sph;
    tp.node32 = node32;
    tp.boff = bcnt;
    tp.bkey = bkey;
    tp.belem = belem;
    tp.g = g;
    trg_pairs_kernel<false><<<grid_for(nt, sms), NL_T, 0, st>>>(tp, L->trg_cnt, nullptr, nullptr, nullptr, status);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    int64_t* toff;
    if ((e = scratch((nt + 1) * 8, (void**)&toff))) break;
    if ((e = exclusive_scan(L->trg_cnt, toff, nt + 1, st, sms))) break;
    if ((e = cudaMemcpyAsync(&L->n_near, toff + nt, 8, cudaMemcpyDeviceToHost, st))) break;
    if ((e = cudaStreamSynchronize(st))) break;
    const int64_t nn = L->n_near;
    int32_t *pe, *pe2;
    int64_t *pt, *perm, *perm2;
    if ((e = scratch(nn * 4, (void**)&pe))) break;
    if ((e = scratch(nn * 4, (void**)&pe2))) break;
    if ((e = scratch(nn * 8, (void**)&pt))) break;
    if ((e = scratch(nn * 8, (void**)&perm))) break;
    if ((e = scratch(nn * 8, (void**)&perm2))) break;
    if ((e = cudaMalloc(&L->trg_idx, std::max<int64_t>(nn, 1) * 8))) break;
    if ((e = cudaMalloc(&L->scatter, std::max<int64_t>(nn, 1) * 8))) break;
    if ((e = cudaMalloc(&L->trg_elem, std::max<int64_t>(nn, 1) * 8))) break;
    trg_pairs_kernel<true><<<grid_for(nt, sms), NL_T, 0, st>>>(tp, L->trg_cnt, toff, pe, pt, status);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    if ((e = cudaGetLastError())) break;
    if ((e = cudaMemcpyAsync(L->trg_dsp, toff, nt * 8, cudaMemcpyDeviceToDevice, st))) break;
    trg_dsp_fix_kernel<<<grid_for(nt, sms), NL_T, 0, st>>>(nt, L->trg_cnt, L->trg_dsp);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    if (nn == 0) break;

    // 4. element-major order: stable radix sort of the target-major list by element
    elem_count_kernel<<<grid_for(nn, sms), NL_T, 0, st>>>(nn, pe, L->elem_cnt);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    if ((e = exclusive_scan(L->elem_cnt, L->elem_dsp, n_elem + 1, st, sms))) break;
    widen_kernel<<<grid_for(nn, sms), NL_T, 0, st>>>(nn, pe, L->trg_elem);  // before the sort reuses pe
    g_launches.fetch_add(1, std::memory_order_relaxed);
    const int64_t ntiles = (nn + RS_TILE - 1) / RS_TILE;
    int64_t* hist;
    if ((e = scratch((256 * ntiles + 1) * 8, (void**)&hist))) break;
    int32_t *kin = pe, *kout = pe2;
    int64_t *vin = nullptr, *vout = perm;
    int passes = 0;
    for (int shift = 0; shift < 31 && ((n_elem - 1) >> shift) > 0; shift += 8) {
      radix_hist_kernel<<<(unsigned)std::min<int64_t>(ntiles, (int64_t)sms * 8), 256, 0, st>>>(kin, nn, shift, ntiles,
                                                                                                hist);
      g_launches.fetch_add(1, std::memory_order_relaxed);
      if ((e = exclusive_scan(hist, hist, 256 * ntiles, st, sms))) break;
      radix_scatter_kernel<<<(unsigned)std::min<int64_t>(ntiles, (int64_t)sms * 32), 32, 0, st>>>(
          kin, vin, kout, vout, nn, shift, ntiles, hist);
      g_launches.fetch_add(1, std::memory_order_relaxed);
      if ((e = cudaGetLastError())) break;
      std::swap(kin, kout);
      vin = vout;
      vout = (vout == perm) ? perm2 : perm;
      ++passes;
    }
    if (e) break;
    const int64_t* order = vin;  // element-major position -> target-major index
    if (passes == 0) {           // a single element: the target-major order is already element-major
      finish_kernel<<<grid_for(nn, sms), NL_T, 0, st>>>(nn, nullptr, pt, L->trg_idx, L->scatter);
    } else {
      finish_kernel<<<grid_for(nn, sms), NL_T, 0, st>>>(nn, order, pt, L->trg_idx, L->scatter);
    }
    g_launches.fetch_add(1, std::memory_order_relaxed);
    if ((e = cudaGetLastError())) break;
  } while (false);
  for (void* p : tmp) cudaFreeAsync(p, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    free_list(L);
    return runtime_record(e);
  }
  *out = L;
  return SCTLGPU_OK;
}

extern "C" int sctlgpu_near_list_sizes(sctlgpu_near_list L, int64_t* n_near, int64_t* nt, int64_t* n_elem) {
  if (!L) return SCTLGPU_ERR_NULL_POINTER;
  if (n_near) *n_near = L->n_near;
  if (nt) *nt = L->nt;
  if (n_elem) *n_elem = L->n_elem;
  return SCTLGPU_OK;
}

extern "C" int sctlgpu_near_list_get(sctlgpu_near_list L, int64_t* near_elem_cnt, int64_t* near_elem_dsp,
                                     int64_t* near_trg_idx, int64_t* near_scatter_index, int64_t* near_trg_cnt,
                                     int64_t* near_trg_dsp, int64_t* near_trg_elem, void* stream) {
  if (!L) return SCTLGPU_ERR_NULL_POINTER;
  int cur = 0;
  cudaGetDevice(&cur);
  if (cur != L->device) return SCTLGPU_ERR_INVALID_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaSuccess;
  auto cp = [&](int64_t* dst, const int64_t* src, int64_t n) {
    if (e == cudaSuccess && dst && n > 0) e = cudaMemcpyAsync(dst, src, n * 8, cudaMemcpyDefault, st);
  };
  cp(near_elem_cnt, L->elem_cnt, L->n_elem);
  cp(near_elem_dsp, L->elem_dsp, L->n_elem);
  cp(near_trg_idx, L->trg_idx, L->n_near);
  cp(near_scatter_index, L->scatter, L->n_near);
  cp(near_trg_cnt, L->trg_cnt, L->nt);
  cp(near_trg_dsp, L->trg_dsp, L->nt);
  cp(near_trg_elem, L->trg_elem, L->n_near);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return runtime_record(e);
}

extern "C" int sctlgpu_near_list_elem_index(sctlgpu_near_list L, int64_t* near_elem_idx, void* stream) {
  if (!L) return SCTLGPU_ERR_NULL_POINTER;
  if (L->n_near == 0) return SCTLGPU_OK;
  if (!near_elem_idx) return SCTLGPU_ERR_NULL_POINTER;
  int cur = 0;
  cudaGetDevice(&cur);
  if (cur != L->device) return SCTLGPU_ERR_INVALID_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, L->device);
  cudaPointerAttributes pa{};
  cudaError_t e = cudaPointerGetAttributes(&pa, near_elem_idx);
  const bool on_device = e == cudaSuccess && (pa.type == cudaMemoryTypeDevice || pa.type == cudaMemoryTypeManaged);
  (void)cudaGetLastError();  // a plain host pointer is not an error here
  int64_t* dst = near_elem_idx;
  if (!on_device) {
    e = cudaMallocAsync((void**)&dst, L->n_near * 8, st);
    if (e != cudaSuccess) return runtime_record(e);
  }
  elem_index_kernel<<<grid_for(L->n_near, sms > 0 ? sms : 1), NL_T, 0, st>>>(L->n_near, L->n_elem, L->elem_dsp, dst);
  g_launches.fetch_add(1, std::memory_order_relaxed);
  e = cudaGetLastError();
  if (!on_device) {
    if (e == cudaSuccess) e = cudaMemcpyAsync(near_elem_idx, dst, L->n_near * 8, cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(dst, st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return runtime_record(e);
}

extern "C" int sctlgpu_near_list_destroy(sctlgpu_near_list L) {
  if (!L) return SCTLGPU_OK;
  int cur = 0;
  cudaGetDevice(&cur);
  cudaSetDevice(L->device);
  cudaDeviceSynchronize();
  cudaSetDevice(cur);
  free_list(L);
  return SCTLGPU_OK;
}
