/*
 * sctlgpu -- GB300 (sm_103a) particle-kernel direct sums behind a C ABI.
 *
 * Drop-in for the hot path of SCTL's GenericKernel (include/sctl/generic-kernel.hpp):
 * the Eval / KernelMatrix direct sums for Laplace3D_FxU, Laplace3D_DxU,
 * Stokes3D_FxU and Stokes3D_DxU (include/sctl/kernel_functions.hpp:32-218).
 *
 * Conventions (identical to the reference unless stated):
 *   - coordinates, normals and densities are array-of-structures, exactly as
 *     SCTL's Vector<Real> holds them: r_trg[nt*3], r_src[ns*3], n_src[ns*3]
 *     (only for kernels with NormalDim()==3), v_src[ns*SrcDim], v_trg[nt*TrgDim];
 *   - pairs with r^2 == 0 contribute nothing (the approx_rsqrt mask);
 *   - the kernel's scale factor (1/4pi, 1/4pi, 1/8pi, 3/4pi) is applied once
 *     after summation;
 *   - digits follows the reference: -1 (or >= 16) means full precision of the
 *     arithmetic type, otherwise the number of significant digits requested;
 *   - errors are returned as status codes (the reference aborts through
 *     SCTL_ASSERT; the C++ shim in sctlgpu.hpp restores that behaviour).
 *
 * Pointers are host pointers unless SCTLGPU_DEVICE_PTRS is set.  With host
 * pointers the call is synchronous (copies in, computes, copies out).  With
 * device pointers the work is enqueued on `stream` (a cudaStream_t, or NULL
 * for the legacy default stream) and the call returns without synchronising.
 * All entry points are thread-safe.
 */
#ifndef SCTLGPU_H_
#define SCTLGPU_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SCTLGPU_VERSION 1

/* Kernel ids: the micro-kernels of kernel_functions.hpp (aliases at :669-684).  Ids 0-3 are
 * the hot path (every mode, near plans, the allocation-free entry); ids 4-15 run Eval and
 * KernelMatrix in FP64 and FP32 (SCTLGPU_MIXED runs them on the FP64 path). */
enum sctlgpu_kernel {
  SCTLGPU_LAPLACE3D_FXU = 0,        /* sctl::Laplace3D_FxU        kernel_functions.hpp:32-59   */
  SCTLGPU_LAPLACE3D_DXU = 1,        /* sctl::Laplace3D_DxU        kernel_functions.hpp:61-79   */
  SCTLGPU_STOKES3D_FXU = 2,         /* sctl::Stokes3D_FxU         kernel_functions.hpp:125-178 */
  SCTLGPU_STOKES3D_DXU = 3,         /* sctl::Stokes3D_DxU         kernel_functions.hpp:180-218 */
  SCTLGPU_LAPLACE3D_FXDU = 4,       /* sctl::Laplace3D_FxdU       kernel_functions.hpp:81-123  */
  SCTLGPU_LAPLACE3D_FXD2U = 5,      /* sctl::Laplace3D_Fxd2U      kernel_functions.hpp:366-390 */
  SCTLGPU_LAPLACE3D_DXDU = 6,       /* sctl::Laplace3D_DxdU       kernel_functions.hpp:392-414 */
  SCTLGPU_BIOTSAVART3D_FXU = 7,     /* sctl::BiotSavart3D_FxU     kernel_functions.hpp:416-449 */
  SCTLGPU_BIOTSAVART3D_FXDU = 8,    /* sctl::BiotSavart3D_FxdU    kernel_functions.hpp:451-483 */
  SCTLGPU_HELMHOLTZ3D_FXU = 9,      /* sctl::Helmholtz3D_FxU      kernel_functions.hpp:491-527 (needs ctx) */
  SCTLGPU_HELMHOLTZ3D_DXU = 10,     /* sctl::Helmholtz3D_DxU      kernel_functions.hpp:529-571 (needs ctx) */
  SCTLGPU_HELMHOLTZ3D_FXDU = 11,    /* sctl::Helmholtz3D_FxdU     kernel_functions.hpp:573-620 (needs ctx) */
  SCTLGPU_HELMHOLTZDIFF3D_FXDU = 12,/* sctl::HelmholtzDiff3D_FxdU kernel_functions.hpp:627-659 (needs ctx) */
  SCTLGPU_STOKES3D_FXT = 13,        /* sctl::Stokes3D_FxT         kernel_functions.hpp:220-262 */
  SCTLGPU_STOKES3D_FSXU = 14,       /* sctl::Stokes3D_FSxU        kernel_functions.hpp:264-323 */
  SCTLGPU_STOKES3D_FXUP = 15        /* sctl::Stokes3D_FxUP        kernel_functions.hpp:325-364 */
};
#define SCTLGPU_NUM_KERNELS 16

/* Arithmetic modes. */
enum sctlgpu_mode {
  SCTLGPU_F64 = 0,   /* Real = double: FP64 arithmetic throughout (GenericKernel<...>::Eval<double,...>). */
  SCTLGPU_F32 = 1,   /* Real = float:  FP32 arithmetic throughout (GenericKernel<...>::Eval<float,...>).  */
  SCTLGPU_MIXED = 2  /* Real = double in and out; FP32 arithmetic up to 7 digits, double-float (two-FP32)
                        error-free transformations for 8..11 digits, the FP64 path beyond. */
};

/* Flags. */
#define SCTLGPU_ACCUMULATE 1u  /* v_trg += result (the reference's Eval when v_trg is already sized); else v_trg = result */
#define SCTLGPU_DEVICE_PTRS 2u /* every array argument is a device pointer; asynchronous on `stream` */

/* Status codes. */
enum sctlgpu_status {
  SCTLGPU_OK = 0,
  SCTLGPU_ERR_INVALID_KERNEL = -1,
  SCTLGPU_ERR_INVALID_MODE = -2,
  SCTLGPU_ERR_INVALID_SIZE = -3,    /* negative counts, or counts whose arrays would overflow int64 */
  SCTLGPU_ERR_NULL_POINTER = -4,    /* a required array is NULL while its count is > 0 */
  SCTLGPU_ERR_CUDA = -5,            /* a CUDA runtime call failed; sctlgpu_last_cuda_error() has the text */
  SCTLGPU_ERR_NO_DEVICE = -6,
  SCTLGPU_ERR_DEVICE_TIMEOUT = -7,  /* a bounded device-side wait gave up; results are not valid */
  SCTLGPU_ERR_INVALID_ARGUMENT = -8,
  SCTLGPU_ERR_TOO_LARGE = -9        /* the request exceeds a fixed capacity of the entry point */
};

/*
 * GenericKernel::CoordDim / NormalDim / SrcDim / TrgDim (generic-kernel.hpp:54-74).
 * Any output pointer may be NULL.
 */
int sctlgpu_kernel_dims(int kernel, int* coord_dim, int* normal_dim, int* src_dim, int* trg_dim);

/* uKerScaleFactor<double>() of the kernel (kernel_functions.hpp:40,69,88,133,188,...). */
double sctlgpu_scale_factor(int kernel);

/*
 * Direct sum  v_trg[t*TrgDim+k] (+)= scale * sum_s K(x_t - y_s, n_s) . f_s.
 * Replaces GenericKernel<uK>::Eval<Real,enable_openmp>(v_trg, r_trg, r_src, n_src, v_src, digits, self)
 * (generic-kernel.hpp:99, generic-kernel.txx:72-211), the function ParticleFMM stores in
 * S2TData::ker_s2t_eval_omp (fmm-wrapper.txx:153-154,450-451) and calls in EvalDirect
 * (fmm-wrapper.txx:618).  Arrays are double for SCTLGPU_F64 / SCTLGPU_MIXED, float for
 * SCTLGPU_F32.  n_src may be NULL for kernels with NormalDim()==0.
 */
int sctlgpu_eval(int kernel, int mode, int digits,
                 int64_t nt, const void* r_trg,
                 int64_t ns, const void* r_src, const void* n_src, const void* v_src,
                 void* v_trg, unsigned flags, void* stream);

/*
 * Dense kernel matrix M[(s*SrcDim+k0)*(nt*TrgDim) + t*TrgDim+k1] = scale * K_{k0,k1}(x_t - y_s, n_s),
 * row-major, source-major, overwritten.  Replaces GenericKernel<uK>::KernelMatrix<Real,omp,digits>
 * (generic-kernel.hpp:124, generic-kernel.txx:213-329), which BoundaryIntegralOp calls per near
 * block in SetupNear (boundary_integral.txx:1197,1211).
 */
int sctlgpu_kernel_matrix(int kernel, int mode, int digits,
                          int64_t nt, const void* r_trg,
                          int64_t ns, const void* r_src, const void* n_src,
                          void* M, unsigned flags, void* stream);

/*
 * sctlgpu_eval / sctlgpu_kernel_matrix with the kernel's context, as the reference's
 * GenericKernel::SetCtxPtr (generic-kernel.hpp:79) provides it to uKerMatrix /
 * uKerApply: for the Helmholtz kernels (ids 9-12) `ctx` points to the wavenumber, a
 * host value of the call's real type (double, or float for SCTLGPU_F32); other
 * kernels ignore it.  The entries without ctx refuse the Helmholtz kernels
 * (SCTLGPU_ERR_NULL_POINTER).
 */
int sctlgpu_eval_ctx(int kernel, int mode, int digits,
                     int64_t nt, const void* r_trg,
                     int64_t ns, const void* r_src, const void* n_src, const void* v_src,
                     void* v_trg, unsigned flags, const void* ctx, void* stream);
int sctlgpu_kernel_matrix_ctx(int kernel, int mode, int digits,
                              int64_t nt, const void* r_trg,
                              int64_t ns, const void* r_src, const void* n_src,
                              void* M, unsigned flags, const void* ctx, void* stream);

/*
 * Batched near-field direct sums: many independent blocks of uneven sizes in one
 * persistent launch, captured in a CUDA graph.  Replaces BoundaryIntegralOp's
 * per-block near-field loops -- KNearSubtract's KernelMatrix per near block
 * (boundary_integral.txx:1165-1240) and ComputeNearInterac's per-block apply
 * plus ScatterForward / per-target sum (:1311-1381) -- done matrix-free: block b
 * adds  scale * sum_{s in b} K(x_t - y_s, n_s) * w_s * f_s  to each of its targets.
 *
 * Sources and targets of all blocks are concatenated arrays (AoS, as for
 * sctlgpu_eval); a block names its ranges in them.  With trg_map (nt entries,
 * output index of every target) results are added into v_out[trg_map[t]]
 * (n_out outputs; several blocks may feed one output, as in the reference's
 * scatter), otherwise v_out has one entry per target.  w_src (optional, one
 * weight per source) multiplies the densities: quadrature weights of upsampled
 * nodes, or negative smooth-quadrature weights for the subtraction.
 *
 * A plan fixes the block structure (the reference's Setup / ComputePotential
 * split): creation validates the blocks, cuts them into work items sized by
 * the autotuned table, sorts them by cost and uploads them; execution
 * replays a captured CUDA graph (re-captured when the array pointers change).
 * Execution takes device pointers and is asynchronous on `stream`.
 */
typedef struct sctlgpu_block {
  int64_t src_begin, src_count; /* sources [src_begin, src_begin+src_count) */
  int64_t trg_begin, trg_count; /* targets [trg_begin, trg_begin+trg_count) */
} sctlgpu_block;
typedef struct sctlgpu_near_plan_s* sctlgpu_near_plan;

int sctlgpu_near_plan_create(sctlgpu_near_plan* plan, int kernel, int mode, int digits,
                             int64_t nblk, const sctlgpu_block* blocks, /* host array */
                             int64_t ns, int64_t nt,
                             const int64_t* trg_map, int64_t n_out); /* host array or NULL */
/*
 * Same, with a target index list (the reference's near lists): block target
 * ranges select entries of trg_index (n_index entries, each a target in
 * [0, nt)), and results are added into v_out[trg_map ? trg_map[k] : trg_index[k]]
 * for list entry k.  Because the coordinate arrays are the full target and
 * source sets, a mixed-precision plan uses the same frame as a sctlgpu_eval of
 * those arrays, so a smooth-rule subtraction cancels the far field's terms
 * consistently (the KNearSubtract convention, boundary_integral.txx:1165-1240).
 */
int sctlgpu_near_plan_create_indexed(sctlgpu_near_plan* plan, int kernel, int mode, int digits,
                                     int64_t nblk, const sctlgpu_block* blocks, int64_t ns, int64_t nt,
                                     const int64_t* trg_index, int64_t n_index,
                                     const int64_t* trg_map, int64_t n_out);
int sctlgpu_near_plan_execute(sctlgpu_near_plan plan, const void* r_trg, const void* r_src, const void* n_src,
                              const void* v_src, const void* w_src, void* v_out, unsigned flags, void* stream);
/* Work items, interactions per execution, and CUDA-graph kernel nodes of a plan. */
int sctlgpu_near_plan_info(sctlgpu_near_plan plan, int64_t* n_items, int64_t* interactions, int* graph_kernels);
/* Synchronises `stream` and returns SCTLGPU_ERR_DEVICE_TIMEOUT if a bounded device wait of the plan gave up. */
int sctlgpu_near_plan_status(sctlgpu_near_plan plan, void* stream);
/* Waits for the device (the plan's graph may still be running), then frees the plan. */
int sctlgpu_near_plan_destroy(sctlgpu_near_plan plan);

/*
 * Near-singular correction of p x p (p = 10) Chebyshev panels -- the plugin point
 * of ElementListBase::NearInterac / EvalNearInterac (boundary_integral.hpp:164-239)
 * for a surface given only by its panel nodes.  For every (target, panel) pair
 * the panel's geometry and density are interpolated from its nodes and
 * integrated with adaptive dyadic refinement (boxes accepted at distance >=
 * alpha x diameter, 8 x 8 Gauss-Legendre per box, at most max_depth levels),
 * the panel's smooth-rule part (nodes X, normals N, weights Q) is subtracted
 * when subtract_smooth != 0 (KNearSubtract, boundary_integral.txx:1165-1240; pass
 * 0 and subtract with a near plan in the far field's arithmetic when the far field
 * is mixed precision), and scale x the result is
 * atomically added to v_out[trg_map ? trg_map[t] : t].  Kernels: Laplace3D_FxU,
 * Laplace3D_DxU (double arrays; arithmetic per sctlgpu_panel_arithmetic); device
 * pointers, asynchronous on `stream`.  Out-of-range pair indices are skipped (status
 * bit 4).  Each warp queues at most 256 boxes per level, which holds the refinement
 * for alpha <= ~2.5 (alpha = 1: ~1e-10 relative on the torus workload; alpha = 2:
 * ~1e-13); when a level would overflow, boxes are integrated unrefined instead of
 * dropped and status bit 2 is set.
 */
int sctlgpu_panel_near_correction(int kernel, int64_t n_pairs, const int64_t* pair_trg, const int64_t* pair_panel,
                                  int64_t nt, const double* r_trg, int64_t n_panels, const double* X,
                                  const double* N, const double* Q, const double* sigma,
                                  const int64_t* trg_map, int64_t n_out, double alpha, int max_depth,
                                  int subtract_smooth, double* v_out, void* stream);

/*
 * Accurate near-singular weights of (target, panel) pairs: for each pair the
 * 100 values scale * int_P K(x_t - y) l_a(s) l_b(t) dA(y) (l the Lagrange basis of
 * the panel's 10 x 10 Chebyshev nodes) are written to w_out[pair * 100 + a * 10 + b],
 * by the same adaptive refinement as sctlgpu_panel_near_correction.  These are
 * the weights a NearInterac plugin returns (boundary_integral.hpp:164-221) and the
 * training labels of the correction network.  Device pointers, asynchronous.
 */
int sctlgpu_panel_near_weights(int kernel, int64_t n_pairs, const int64_t* pair_trg, const int64_t* pair_panel,
                               int64_t nt, const double* r_trg, int64_t n_panels, const double* X,
                               double alpha, int max_depth, double* w_out, void* stream);

/*
 * Far-field densities (replaces the density weighting of
 * BoundaryIntegralOp::ComputeFarField, boundary_integral.txx:1266-1285):
 * f_far[i*dof + k] = f[i*dof + k] * w[i] for i < n, k < dof.  Device pointers,
 * asynchronous on `stream`; f_far may alias f.
 */
int sctlgpu_far_densities(int64_t n, int dof, const double* f, const double* w, double* f_far, void* stream);

/*
 * Near lists (replaces BuildNearList, boundary_integral.txx:50-522, single rank).
 * Target t is near element e when some node s of e (nodes elem_nds_dsp[e] ..
 * elem_nds_dsp[e] + elem_nds_cnt[e] - 1 of r_src) has |x_t - x_s|^2 < src_radius[s]^2,
 * the reference's test.  The handle holds, on the device:
 *   near_elem_cnt/dsp[n_elem]   near targets per element (element-major list sorted by
 *                               (element, target));
 *   near_trg_idx[n_near]        the element-major list's target indices (the reference
 *                               returns their coordinates, Xtrg_near = r_trg[near_trg_idx]);
 *   near_scatter_index[n_near]  for entry i of the target-major order, its position in
 *                               the element-major list (the reference's ScatterForward
 *                               index; entries of one target in element order);
 *   near_trg_cnt/dsp[nt]        per target, its entries in the target-major order (dsp 0
 *                               where cnt is 0, as the reference);
 *   near_trg_elem[n_near]       the target-major order's element indices.
 * Inputs are host arrays, or device arrays with SCTLGPU_DEVICE_PTRS.  The build
 * synchronises `stream`.  Nodes with a negative or non-finite radius, and elements with
 * invalid node ranges, are skipped and set bit 4 of the device status word.
 */
typedef struct sctlgpu_near_list_s* sctlgpu_near_list;
int sctlgpu_near_list_build(sctlgpu_near_list* out, int64_t nt, const double* r_trg, int64_t n_elem,
                            const int64_t* elem_nds_cnt, const int64_t* elem_nds_dsp, int64_t ns,
                            const double* r_src, const double* src_radius, unsigned flags, void* stream);
int sctlgpu_near_list_sizes(sctlgpu_near_list list, int64_t* n_near, int64_t* nt, int64_t* n_elem);
/* Copies the arrays out (host or device destinations; NULL skips one), synchronously. */
int sctlgpu_near_list_get(sctlgpu_near_list list, int64_t* near_elem_cnt, int64_t* near_elem_dsp,
                          int64_t* near_trg_idx, int64_t* near_scatter_index, int64_t* near_trg_cnt,
                          int64_t* near_trg_dsp, int64_t* near_trg_elem, void* stream);
/* The element of every element-major entry (near_elem_idx[n_near]; the reference
 * expands near_elem_cnt the same way when it walks the element-major list,
 * boundary_integral.txx:1009-1032): with near_trg_idx, the (element, target)
 * pairs sorted by element.  Host or device destination; synchronous. */
int sctlgpu_near_list_elem_index(sctlgpu_near_list list, int64_t* near_elem_idx, void* stream);
int sctlgpu_near_list_destroy(sctlgpu_near_list list);

/*
 * Far field by a barycentric Lagrange treecode.  Replaces ParticleFMM::Eval's
 * fast path, EvalPVFMM (fmm-wrapper.txx:854-1038; Eval at :542-549 takes it for
 * 40,000 targets or more): v_out = scale * sum_s K(x_t - y_s, n_s) . f_s for
 * the four hot-path kernels, with work below the direct sum's Ns * Nt.  The
 * algorithm differs from PVFMM's (a barycentric Lagrange treecode over a
 * source and a target tree: separated clusters are replaced by proxies at
 * the tensor-product Chebyshev points of their boxes, up to order+1 per
 * dimension (fewer along a side much thinner than the longest, one along a side
 * of zero extent) -- source proxies carry interpolated moments,
 * target proxies collect potentials that a downward pass interpolates to the
 * targets -- and everything else is summed directly); every
 * interaction runs in the batched near-field kernels with `mode` / `digits`
 * arithmetic (SCTLGPU_F64 or SCTLGPU_MIXED).
 *
 * create: the geometry (host arrays; the reference's SetSrcCoord / SetTrgCoord,
 * fmm-wrapper.txx:505-540): source coordinates and normals (double-layer
 * kernels), target coordinates; builds both trees, the interaction blocks and
 * the device-side plans.  params may be NULL: order and theta then follow
 * `digits`, leaf_max = the cost of a full grid's proxies ((order+1)^3; the
 * Stokes double layer's proxies carry the symmetric part of their moment and
 * cost 1.25 interactions each), batch_max = 512 or 256, whichever leaves
 * fewer interactions (512 unless 256 saves 3 %).
 * execute: v_src (ns * SrcDim, source order as given; SetDensitySL / DL) ->
 * v_out (nt * TrgDim, target order as given); flags may hold
 * SCTLGPU_ACCUMULATE.  Host arrays (synchronous, staged through device buffers
 * kept with the treecode; also reports a device-side timeout), or device arrays
 * with SCTLGPU_DEVICE_PTRS (asynchronous on `stream`).  A treecode's device buffers
 * are reused by every execution: executions of one treecode must not overlap
 * (one stream, or one treecode per concurrent stream).
 * info / layout: sizes[10] = {blocks, source slots (leaves padded to even
 * counts), all source slots (with proxies), source clusters with proxies,
 * direct interactions, interactions through proxies, order, target list
 * (targets, then target proxies), target clusters with proxies, 1 when the
 * traversal saves less than a quarter of Ns * Nt and evaluations run the
 * direct sum instead}, and the acceptance parameter.  layout is the host-only part of create (no device
 * needed): the blocks (sources index the source slots, targets the target
 * list), the source of every slot (-1 padding, -2 proxy), the target order,
 * per source cluster with proxies {slot begin, end, proxy slot begin, end,
 * grid points along x, y, z} and per target cluster with proxies {target begin,
 * end, proxy begin, end, grid points along x, y, z} (7 entries each); any
 * output may be NULL.
 */
typedef struct sctlgpu_treecode_params {
  double theta;  /* a pair of clusters is separated when (r_trg + r_src) < theta * distance; <= 0: from digits */
  int order;     /* interpolation degree per dimension, 1..15; <= 0: from digits */
  int leaf_max;  /* sources per leaf; <= 0: the cost of a full grid's proxies */
  int batch_max; /* targets per batch, <= 2048; <= 0: 512 or 256 (fewer interactions) */
  int dual;      /* nonzero: target clusters interpolate too (cluster-cluster interactions, a downward pass);
                    0: particle-cluster only */
  double theta_trg; /* acceptance of target-side interpolation, <= theta; <= 0: theta */
  double moment_bytes; /* device scratch for partial moments (more is done in passes); <= 0: 1e9 */
} sctlgpu_treecode_params;
typedef struct sctlgpu_treecode_s* sctlgpu_treecode;
int sctlgpu_treecode_create(sctlgpu_treecode* tc, int kernel, int mode, int digits, int64_t ns, const double* r_src,
                            const double* n_src, int64_t nt, const double* r_trg,
                            const sctlgpu_treecode_params* params);
int sctlgpu_treecode_execute(sctlgpu_treecode tc, const double* v_src, double* v_out, unsigned flags, void* stream);
int sctlgpu_treecode_info(sctlgpu_treecode tc, int64_t* sizes, double* theta);
/* Synchronises `stream`; SCTLGPU_ERR_DEVICE_TIMEOUT if a bounded device wait gave up. */
int sctlgpu_treecode_status(sctlgpu_treecode tc, void* stream);
int sctlgpu_treecode_destroy(sctlgpu_treecode tc);
int sctlgpu_treecode_layout(int kernel, int64_t ns, const double* r_src, int64_t nt, const double* r_trg,
                            const sctlgpu_treecode_params* params, int digits, int64_t* sizes, double* theta,
                            sctlgpu_block* blocks, int64_t* slot_src, int64_t* trg_order, int64_t* clusters,
                            int64_t* trg_clusters);

/*
 * Applies precomputed near-interaction matrices and sums them per target:
 * replaces BoundaryIntegralOp::ComputeNearInterac's per-block GEMV, ScatterForward
 * and per-target accumulation (boundary_integral.txx:1311-1381) with one pass.
 *
 *   U[t*k1 + c] += sum over j in [trg_dsp[t], trg_dsp[t+1]) of
 *                  sum_i K[pair_kdsp[p] + c*n + i] * F[elem_nds_dsp[e]*k0 + i],
 *   p = trg_pair[j] (or j when trg_pair is NULL), e = pair_elem[p],
 *   n = elem_nds_cnt[e] * k0.
 *
 * k0 = SrcDim, k1 = TrgDim (1, 2, 3, 4 or 9).  A pair's block is k1 rows of n entries
 * (row-major), as one target's rows of the reference's target-major K_near.  Each
 * target's pairs are summed in the given order by one warp (deterministic).  Indices
 * out of range skip the pair and set bit 4 of the device status word.  Device
 * pointers, asynchronous on `stream`; targets without pairs are left untouched.
 */
int sctlgpu_near_matrix_apply(int k0, int k1, int64_t n_trg, const int64_t* trg_dsp, int64_t n_near,
                              const int64_t* trg_pair, int64_t n_pairs, const int64_t* pair_elem,
                              const int64_t* pair_kdsp, int64_t n_elem, const int64_t* elem_nds_dsp,
                              const int64_t* elem_nds_cnt, int64_t n_k, const double* K, int64_t n_f,
                              const double* F, double* U, void* stream);

/*
 * The same application with the blocks stored as float pairs: K2[2i], K2[2i+1] = hi, lo
 * of weight i (hi + lo = the FP64 weight to ~2^-48; same 8 bytes per weight, made once by
 * sctlgpu_to_float_pairs, in place if wanted), accumulated in double-float on the FP32
 * pipe -- GB300's FP64 pipe cannot keep up with one FP64 multiply-add per 8 bytes at HBM
 * speed.  Results within ~1e-14 relative of the FP64 application.  K2 8-byte aligned.
 */
int sctlgpu_near_matrix_apply_pairs(int k0, int k1, int64_t n_trg, const int64_t* trg_dsp, int64_t n_near,
                                    const int64_t* trg_pair, int64_t n_pairs, const int64_t* pair_elem,
                                    const int64_t* pair_kdsp, int64_t n_elem, const int64_t* elem_nds_dsp,
                                    const int64_t* elem_nds_cnt, int64_t n_k, const float* K2, int64_t n_f,
                                    const double* F, double* U, void* stream);

/*
 * The index chain of the two entry points above (target-major entry -> pair ->
 * element -> nodes), resolved once for stored matrices (SetupNear keeps the same
 * structure for every ComputeNearInterac): resolved[2j] = K offset of entry j,
 * resolved[2j+1] = (F offset << 20) | F length, or -1 where an index is out of range
 * (that entry is skipped and flagged when applied).  Device arrays, asynchronous.
 */
int sctlgpu_near_matrix_resolve(int k0, int k1, int64_t n_near, const int64_t* trg_pair, int64_t n_pairs,
                                const int64_t* pair_elem, const int64_t* pair_kdsp, int64_t n_elem,
                                const int64_t* elem_nds_dsp, const int64_t* elem_nds_cnt, int64_t n_k, int64_t n_f,
                                int64_t* resolved, void* stream);
/* ComputeNearInterac from resolved entries: one coalesced 16-byte load per entry instead of the
 * chain of dependent index loads.  Exactly one of K (FP64 blocks) and K2 (float pairs) non-NULL. */
int sctlgpu_near_matrix_apply_resolved(int k0, int k1, int64_t n_trg, const int64_t* trg_dsp, int64_t n_near,
                                       const int64_t* resolved, int64_t n_k, const double* K, const float* K2,
                                       int64_t n_f, const double* F, double* U, void* stream);

/* x[0..n) -> out[2i], out[2i+1] = hi, lo float pair of x[i] (device pointers, 8-byte
 * aligned; out may be x itself), asynchronous on `stream`. */
int sctlgpu_to_float_pairs(int64_t n, const double* x, float* out, void* stream);

/*
 * Arithmetic of sctlgpu_panel_near_correction / sctlgpu_panel_near_weights for the whole
 * process: SCTLGPU_MIXED (default; double-float error-free transformations on the FP32
 * pipe, within ~1e-13 of the FP64 form) or SCTLGPU_F64.  Returns the previous mode, or
 * SCTLGPU_ERR_INVALID_MODE.
 */
int sctlgpu_panel_arithmetic(int mode);

/*
 * C[M x N] = act(A[M x K] . Bt[N x K]^T + bias) on the tcgen05 tensor cores: A and Bt
 * row-major BF16 (K contiguous, 16-byte aligned), FP32 accumulation in tensor memory,
 * act 0 = none, 1 = GELU (tanh form).  Outputs (any may be NULL, not all): C32 (FP32,
 * after act; added into when accumulate32), pre32 (FP32 before act), C16 (BF16 after
 * act).  M % 128 == 0, N % 16 == 0 and N <= 256, K % 64 == 0.  The building block of
 * the near-field correction MLP; no counterpart in the reference.  Device pointers,
 * asynchronous on `stream`.
 */
int sctlgpu_tc_gemm_bf16(int M, int N, int K, const void* A, const void* Bt, const float* bias, int act,
                         float* C32, float* pre32, void* C16, int accumulate32, void* stream);

/*
 * The near-field correction network: in_dim -> 256 -> 256 -> 256 -> out_dim
 * (in_dim <= 64, out_dim <= 128), GELU between layers, BF16 weights and
 * activations with FP32 accumulation on the tcgen05 tensor cores, FP32 master
 * weights and Adam.  No counterpart in the reference (it predicts the weights a
 * NearInterac plugin returns, boundary_integral.hpp:164-221).  Batches are
 * multiples of 128 up to max_batch; x, y, t are FP32 device arrays (row-major,
 * B x in_dim / B x out_dim).  Parameters are one flat FP32 vector: per layer
 * W (N x K, row-major; layer-1 K padded to 64, last-layer N padded to 128) then b.
 */
typedef struct sctlgpu_mlp_s* sctlgpu_mlp;
int sctlgpu_mlp_create(sctlgpu_mlp* mlp, int in_dim, int out_dim, int max_batch, uint64_t seed);
int sctlgpu_mlp_destroy(sctlgpu_mlp mlp);
int64_t sctlgpu_mlp_num_params(sctlgpu_mlp mlp);
int sctlgpu_mlp_get_params(sctlgpu_mlp mlp, float* host_out);
int sctlgpu_mlp_set_params(sctlgpu_mlp mlp, const float* host_in);
int sctlgpu_mlp_forward(sctlgpu_mlp mlp, int B, const float* x, float* y, void* stream);
/* Inference with the output dotted in the last GEMM's epilogue:
 * out[b] += sum_j y[b][j] * dens[index[b] * out_dim + j]  (rows with index[b] < 0 are skipped). */
int sctlgpu_mlp_forward_dot(sctlgpu_mlp mlp, int B, const float* x, const double* dens, const int64_t* index,
                            double* out, void* stream);
/* One Adam step on the mean squared error against t; loss_host (optional) receives the loss (synchronises). */
int sctlgpu_mlp_train_step(sctlgpu_mlp mlp, int B, const float* x, const float* t, float lr, float* loss_host,
                           void* stream);
/* Gradient of the loss with respect to the flat parameters (host output), for checks.  Synchronous. */
int sctlgpu_mlp_gradients(sctlgpu_mlp mlp, int B, const float* x, const float* t, float* grads_host,
                          float* loss_host);

/*
 * Runs (or returns the cached result of) the tile autotuner for the batched
 * path on the current device: for each block-size class it times the source
 * split factors 1, 2, 4, 8 on synthetic blocks and keeps the fastest.  Fills
 * splits[i] for the SCTLGPU_NEAR_CLASSES classes (target-count buckets
 * <=24, <=48, <=96, <=192, larger; each for source counts <=512 and larger).
 * Environment SCTLGPU_NEAR_AUTOTUNE=0 replaces the measurement by the
 * lane-filling rule.
 */
#define SCTLGPU_NEAR_CLASSES 10
int sctlgpu_near_autotune(int kernel, int mode, int digits, int* splits);

/*
 * sctlgpu_eval with SCTLGPU_MIXED and device pointers, for callers that cannot
 * allocate device memory.  This entry point has no counterpart in the
 * reference.  sctlgpu_eval takes its scratch (packed sources, partial sums)
 * from the stream-ordered allocator; some callers must not allocate at all:
 * a host whose device memory is owned by another allocator or pool it may not
 * bypass, code running after its caller has frozen allocations, or a real-time
 * loop that cannot risk an allocation stall or an out-of-memory error.  This
 * variant allocates nothing: it works in one fixed scratch array of
 * SCTLGPU_NOALLOC_SCRATCH_BYTES (64 MiB) that every GPU loading the library
 * holds until the process exits.
 *   - Arrays are device pointers (double); flags may hold SCTLGPU_ACCUMULATE
 *     (SCTLGPU_DEVICE_PTRS is implied).  Digits are routed as for SCTLGPU_MIXED.
 *   - Returns SCTLGPU_ERR_TOO_LARGE, before launching anything, when the packed
 *     sources plus partial sums do not fit: 512 B + ns * (32, 48, 48, 80 bytes
 *     for Laplace FxU, Laplace DxU, Stokes FxU, Stokes DxU) + nt * TrgDim * 8 B
 *     must stay within the array (e.g. 2^20 Laplace FxU sources and 2^20
 *     targets fit; 2^20 Stokes DxU sources do not).
 *   - The first call on a device looks up the array's device address; make it
 *     before any stream capture.
 *   - All calls share the array and it keeps the last call's contents: calls
 *     whose work overlaps on the GPU race and give wrong results, so order
 *     them (one stream, or synchronise between them).
 *   - The call waits for `stream` to finish before it returns, and reports a
 *     device-side wait timeout as SCTLGPU_ERR_DEVICE_TIMEOUT.
 */
#define SCTLGPU_NOALLOC_SCRATCH_BYTES (64u << 20)
int sctlgpu_eval_mixed_noalloc(int kernel, int digits,
                               int64_t nt, const double* r_trg,
                               int64_t ns, const double* r_src, const double* n_src, const double* v_src,
                               double* v_trg, unsigned flags, void* stream);

/* Human-readable text for a status code. */
const char* sctlgpu_strerror(int status);

/* Text of the last CUDA error seen by this thread (empty if none). */
const char* sctlgpu_last_cuda_error(void);

/*
 * Reads and clears the device-side status word of the current device after
 * synchronising `stream` (what asynchronous calls made with SCTLGPU_DEVICE_PTRS
 * report).  Returns SCTLGPU_OK or SCTLGPU_ERR_DEVICE_TIMEOUT (any bit set).
 */
int sctlgpu_device_status(void* stream);

/*
 * The same, with the word itself in *word: bit 1 a bounded wait gave up (tile copy or
 * work queue), bit 2 a panel refinement was cut short (boxes integrated unrefined),
 * bit 4 an index out of range was skipped (near plans, panel pairs, near matrices).
 */
int sctlgpu_device_status_word(void* stream, unsigned* word);

/* Number of kernels this library has launched in this process (all threads). */
int64_t sctlgpu_launch_count(void);

/*
 * Kernel timing: when enabled, the direct-sum and kernel-matrix entry points
 * record CUDA events on their launch stream around their main kernel, and
 * sctlgpu_last_kernel_ms() returns that kernel's duration for the calling
 * thread's most recent call (synchronising on the end event).  Off by default.
 */
int sctlgpu_set_timing(int enable);
double sctlgpu_last_kernel_ms(void);

/*
 * Number of Newton steps the evaluation uses for (mode, digits): the
 * reference's schedule mylog2(floor(digits / seed_digits)) with the seed
 * accuracy of sm_103a's rsqrt.approx (intrin-wrapper.hpp:560-562).
 */
int sctlgpu_newton_steps(int mode, int digits);

#ifdef __cplusplus
}
#endif

#endif /* SCTLGPU_H_ */
