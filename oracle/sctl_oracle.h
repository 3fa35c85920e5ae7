/*
 * CPU oracle for the particle-kernel direct sums -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of SCTL's GenericKernel::Eval / KernelMatrix for the
 * micro-kernels of include/sctl/kernel_functions.hpp (the four hot-path ones,
 * include/sctl/generic-kernel.txx:102-211 and :213-329, kernel_functions.hpp:
 * 32-218, and the other twelve, :81-659) and of BuildNearList's near test.
 * The CUDA path's results are compared against it in the tests, and it is the
 * timed CPU baseline ("port"); nothing in the product library links or calls
 * it.  It is pinned against outputs of the reference itself
 * (fixtures under tests/golden/, generated by tests/golden/make_golden.py from
 * the reference headers) and against the reference's known-answer tests
 * (src/test-kernel_functions.cpp:36-132, src/test-generic-kernel.cpp:55-103).
 */
#ifndef SCTL_ORACLE_H_
#define SCTL_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Kernel ids, same numbering as include/sctlgpu.h. */
enum { ORACLE_LAPLACE3D_FXU = 0, ORACLE_LAPLACE3D_DXU = 1, ORACLE_STOKES3D_FXU = 2, ORACLE_STOKES3D_DXU = 3 };

/* CoordDim / NormalDim / SrcDim / TrgDim (generic-kernel.txx:48-62). Returns 0, or -1 for an unknown id. */
int oracle_kernel_dims(int kernel, int* coord_dim, int* normal_dim, int* src_dim, int* trg_dim);

/* uKerScaleFactor<double>() of the micro-kernel (kernel_functions.hpp:40,69,133,188). */
double oracle_scale_factor(int kernel);

/*
 * v_trg[t*TrgDim+k] += scale * sum_s K(x_t - y_s, n_s) f_s   (generic-kernel.txx:102-211).
 * Accumulates into v_trg, like the reference does once v_trg has the right size.
 * Pairs with r^2 == 0 contribute nothing (approx_rsqrt mask, kernel_functions.hpp:45).
 * nthreads <= 0 uses every OpenMP thread.  1/sqrt is evaluated exactly (the
 * reference's generic scalar path, intrin-wrapper.hpp:563-577).
 */
int oracle_eval_f64(int kernel, int64_t nt, const double* r_trg, int64_t ns, const double* r_src,
                    const double* n_src, const double* v_src, double* v_trg, int nthreads);
int oracle_eval_f32(int kernel, int64_t nt, const float* r_trg, int64_t ns, const float* r_src,
                    const float* n_src, const float* v_src, float* v_trg, int nthreads);

/*
 * Long-double accumulation variant of oracle_eval_f64 (x86-64: 64-bit mantissa;
 * aarch64: IEEE quad), used as the tighter oracle for the error columns.
 */
int oracle_eval_ld(int kernel, int64_t nt, const double* r_trg, int64_t ns, const double* r_src,
                   const double* n_src, const double* v_src, double* v_trg, int nthreads);

/*
 * M[(s*SrcDim+k0)*(nt*TrgDim) + t*TrgDim+k1] = scale * K_{k0,k1}(x_t - y_s, n_s)
 * (generic-kernel.txx:213-329; source-major, already scaled).  Overwrites M.
 */
int oracle_kernel_matrix_f64(int kernel, int64_t nt, const double* r_trg, int64_t ns, const double* r_src,
                             const double* n_src, double* M, int nthreads);
int oracle_kernel_matrix_f32(int kernel, int64_t nt, const float* r_trg, int64_t ns, const float* r_src,
                             const float* n_src, float* M, int nthreads);

/*
 * The reference's Newton schedule: mylog2(floor(digits / seed_digits))
 * (intrin-wrapper.hpp:560-562 with :1562-1566, :3384).  digits == -1 means
 * floor(SigBits*log10(2)) of the type (vec.txx:376): 15 for double, 6 for float.
 */
int oracle_newton_steps(int digits, int is_double, double seed_digits);

/*
 * Newton refinement of y0 ~ 1/sqrt(x) with SCTL's deferred scaling
 * (intrin-wrapper.hpp:540-558): y <- y*(x*y*y + c1_k), c1_k = -3*2^(3^k-1),
 * final scale c2 = (-1/2)^((3^(n-1)-1)*3/2+1).  Returns 0 for x == 0.
 */
double oracle_rsqrt_newton(double x, double y0, int steps);

/* Number of OpenMP threads an oracle call with nthreads <= 0 would use. */
int oracle_max_threads(void);

/* BuildNearList's near test (boundary_integral.txx:50-522; the test itself is
 * node_dist2(src, trg) < rad * rad at :394): target t is near element e when
 * some node s of e has |x_s - x_t|^2 < rad_s^2, squared distance summed
 * x, y, z in FP64 without contraction.  Brute force over all (element, target)
 * pairs, written element-major sorted by (element, target): pair_elem[k],
 * pair_trg[k].  With pair arrays NULL only counts.  Returns the number of
 * pairs, or -1 when more than `cap`. */
/* The other twelve micro-kernels (ids 4-15, kernel_functions.hpp:81-659): Eval and
 * KernelMatrix from each kernel's uKerMatrix, exact 1/sqrt, in float, double or long
 * double; mu is the Helmholtz wavenumber (ids 9-12).  Same layouts as above. */
int oracle_xdims(int kernel, int* nd, int* sd, int* td);
double oracle_xscale(int kernel);
int oracle_xeval(int kernel, int precision /* 0 double, 1 float, 2 long double */, int64_t nt, const void* r_trg,
                 int64_t ns, const void* r_src, const void* n_src, const void* v_src, double mu, void* v_trg,
                 int nthreads);
int oracle_xkmat(int kernel, int precision /* 0 double, 1 float */, int64_t nt, const void* r_trg, int64_t ns,
                 const void* r_src, const void* n_src, double mu, void* M, int nthreads);

int64_t oracle_near_pairs(int64_t nt, const double* r_trg, int64_t n_elem, const int64_t* elem_nds_cnt,
                          const int64_t* elem_nds_dsp, const double* r_src, const double* src_radius, int64_t cap,
                          int64_t* pair_elem, int64_t* pair_trg);

#ifdef __cplusplus
}
#endif

#endif
