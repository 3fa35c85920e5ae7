/*
 * CPU oracle for the particle-kernel direct sums -- TEST INFRASTRUCTURE ONLY
 * (see sctl_oracle.h).  Restates include/sctl/generic-kernel.txx:102-329 and
 * the four micro-kernels of include/sctl/kernel_functions.hpp.
 *
 * Structure mirrors the reference's hot loop (generic-kernel.txx:175-188):
 * SIMD lanes run over a block of targets, the source loop is sequential, and
 * each lane accumulates in the working precision in source order.  The lanes
 * here are a fixed block of ORACLE_TB targets that the compiler vectorises.
 */
#include "sctl_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_TB 8

static const double kPi = 3.14159265358979323846264338327950288;

int oracle_kernel_dims(int kernel, int* cd, int* nd, int* sd, int* td) {
  int c = 3, n, s, t;
  switch (kernel) {
    case ORACLE_LAPLACE3D_FXU: n = 0; s = 1; t = 1; break;
    case ORACLE_LAPLACE3D_DXU: n = 3; s = 1; t = 1; break;
    case ORACLE_STOKES3D_FXU: n = 0; s = 3; t = 3; break;
    case ORACLE_STOKES3D_DXU: n = 3; s = 3; t = 3; break;
    default: return -1;
  }
  if (cd) *cd = c;
  if (nd) *nd = n;
  if (sd) *sd = s;
  if (td) *td = t;
  return 0;
}

double oracle_scale_factor(int kernel) {
  switch (kernel) {
    case ORACLE_LAPLACE3D_FXU: return 1.0 / (4.0 * kPi);  /* kernel_functions.hpp:40-42 */
    case ORACLE_LAPLACE3D_DXU: return 1.0 / (4.0 * kPi);  /* :69-71 */
    case ORACLE_STOKES3D_FXU: return 1.0 / (8.0 * kPi);   /* :133-135 */
    case ORACLE_STOKES3D_DXU: return 3.0 / (4.0 * kPi);   /* :188-190 */
    default: return 0.0;
  }
}

int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

static int resolve_threads(int nthreads) { return nthreads > 0 ? nthreads : oracle_max_threads(); }

int oracle_newton_steps(int digits, int is_double, double seed_digits) {
  /* vec.txx:376: digits == -1 -> floor(SigBits * log10 2). */
  if (digits < 0 || digits >= 16) digits = is_double ? 15 : 6;
  if (!(seed_digits > 0)) return 0;
  long q = (long)((double)digits / seed_digits);
  int n = 0; /* mylog2, intrin-wrapper.hpp:560-562 */
  while (q >= 1) { n++; q /= 2; }
  return n;
}

double oracle_rsqrt_newton(double x, double y, int steps) {
  if (x == 0) return 0;
  if (steps <= 0) return y;
  /* Deferred-scaling Newton: the unscaled iterate grows by (-2)^... each step,
   * so step k uses c1_k = -3 * 2^(3^k - 1) and one final scale c2. */
  long p3 = 1; /* 3^k */
  for (int k = 0; k < steps; k++) {
    const double c1 = -3.0 * ldexp(1.0, (int)(p3 - 1));
    y = y * fma(x, y * y, c1);
    if (k + 1 < steps) p3 *= 3;
  }
  /* c2 = (-0.5)^((3^(n-1)-1)*3/2+1) */
  const long e = (p3 - 1) * 3 / 2 + 1;
  const double c2 = ((e & 1) ? -1.0 : 1.0) * ldexp(1.0, (int)-e);
  return y * c2;
}

/* ------------------------------------------------------------------ Eval */

#define DEFINE_EVAL(NAME, REAL, ACC, SQRT)                                                        \
  int NAME(int kernel, int64_t nt, const REAL* r_trg, int64_t ns, const REAL* r_src,             \
           const REAL* n_src, const REAL* v_src, REAL* v_trg, int nthreads) {                     \
    int nd, sd, td;                                                                               \
    if (oracle_kernel_dims(kernel, NULL, &nd, &sd, &td)) return -1;                               \
    if (nt < 0 || ns < 0) return -2;                                                              \
    const ACC scale = (ACC)oracle_scale_factor(kernel);                                           \
    const int64_t nblk = (nt + ORACLE_TB - 1) / ORACLE_TB;                                        \
    _Pragma("omp parallel for schedule(static) num_threads(resolve_threads(nthreads))")           \
    for (int64_t b = 0; b < nblk; b++) {                                                          \
      ACC xt[3][ORACLE_TB], vt[3][ORACLE_TB];                                                     \
      const int64_t t0 = b * ORACLE_TB;                                                           \
      const int cnt = (int)((nt - t0) < ORACLE_TB ? (nt - t0) : ORACLE_TB);                       \
      for (int k = 0; k < 3; k++)                                                                 \
        for (int l = 0; l < ORACLE_TB; l++) {                                                     \
          xt[k][l] = l < cnt ? (ACC)r_trg[(t0 + l) * 3 + k] : (ACC)0;                             \
          vt[k][l] = 0;                                                                           \
        }                                                                                         \
      for (int64_t s = 0; s < ns; s++) {                                                          \
        const ACC xs0 = (ACC)r_src[s * 3 + 0], xs1 = (ACC)r_src[s * 3 + 1], xs2 = (ACC)r_src[s * 3 + 2]; \
        ACC ns0 = 0, ns1 = 0, ns2 = 0;                                                            \
        if (nd) { ns0 = (ACC)n_src[s * 3 + 0]; ns1 = (ACC)n_src[s * 3 + 1]; ns2 = (ACC)n_src[s * 3 + 2]; } \
        const ACC f0 = (ACC)v_src[s * sd + 0];                                                    \
        const ACC f1 = sd > 1 ? (ACC)v_src[s * sd + 1] : (ACC)0;                                  \
        const ACC f2 = sd > 1 ? (ACC)v_src[s * sd + 2] : (ACC)0;                                  \
        switch (kernel) {                                                                         \
          case ORACLE_LAPLACE3D_FXU: /* kernel_functions.hpp:43-47, then FMA generic-kernel.txx:115-119 */ \
            for (int l = 0; l < ORACLE_TB; l++) {                                                 \
              const ACC d0 = xt[0][l] - xs0, d1 = xt[1][l] - xs1, d2 = xt[2][l] - xs2;            \
              const ACC r2 = d0 * d0 + d1 * d1 + d2 * d2;                                         \
              const ACC rinv = r2 > 0 ? (ACC)1 / SQRT(r2) : (ACC)0;                               \
              vt[0][l] += rinv * f0;                                                              \
            }                                                                                     \
            break;                                                                                \
          case ORACLE_LAPLACE3D_DXU: /* kernel_functions.hpp:72-78 */                             \
            for (int l = 0; l < ORACLE_TB; l++) {                                                 \
              const ACC d0 = xt[0][l] - xs0, d1 = xt[1][l] - xs1, d2 = xt[2][l] - xs2;            \
              const ACC r2 = d0 * d0 + d1 * d1 + d2 * d2;                                         \
              const ACC rinv = r2 > 0 ? (ACC)1 / SQRT(r2) : (ACC)0;                               \
              const ACC rdotn = d0 * ns0 + d1 * ns1 + d2 * ns2;                                   \
              const ACC rinv3 = rinv * rinv * rinv;                                               \
              vt[0][l] += (rdotn * rinv3) * f0;                                                   \
            }                                                                                     \
            break;                                                                                \
          case ORACLE_STOKES3D_FXU: /* fused apply, kernel_functions.hpp:166-176 */               \
            for (int l = 0; l < ORACLE_TB; l++) {                                                 \
              const ACC d0 = xt[0][l] - xs0, d1 = xt[1][l] - xs1, d2 = xt[2][l] - xs2;            \
              const ACC r2 = d0 * d0 + d1 * d1 + d2 * d2;                                         \
              const ACC rinv = r2 > 0 ? (ACC)1 / SQRT(r2) : (ACC)0;                               \
              const ACC rinv3 = rinv * rinv * rinv;                                               \
              const ACC fdr = (f0 * d0 + f1 * d1 + f2 * d2) * rinv3;                              \
              vt[0][l] += f0 * rinv + d0 * fdr;                                                   \
              vt[1][l] += f1 * rinv + d1 * fdr;                                                   \
              vt[2][l] += f2 * rinv + d2 * fdr;                                                   \
            }                                                                                     \
            break;                                                                                \
          default: /* Stokes3D_DxU fused apply, kernel_functions.hpp:205-217 */                   \
            for (int l = 0; l < ORACLE_TB; l++) {                                                 \
              const ACC d0 = xt[0][l] - xs0, d1 = xt[1][l] - xs1, d2 = xt[2][l] - xs2;            \
              const ACC r2 = d0 * d0 + d1 * d1 + d2 * d2;                                         \
              const ACC rinv = r2 > 0 ? (ACC)1 / SQRT(r2) : (ACC)0;                               \
              const ACC rinv2 = rinv * rinv;                                                      \
              const ACC rinv5 = rinv2 * rinv2 * rinv;                                             \
              const ACC rdn = (d0 * ns0 + d1 * ns1 + d2 * ns2) * rinv5;                           \
              const ACC c = (f0 * d0 + f1 * d1 + f2 * d2) * rdn;                                  \
              vt[0][l] += d0 * c;                                                                 \
              vt[1][l] += d1 * c;                                                                 \
              vt[2][l] += d2 * c;                                                                 \
            }                                                                                     \
            break;                                                                                \
        }                                                                                         \
      }                                                                                           \
      for (int l = 0; l < cnt; l++) /* v_trg += Vt_ * scale, generic-kernel.txx:204-208 */        \
        for (int k = 0; k < td; k++) v_trg[(t0 + l) * td + k] += (REAL)(vt[k][l] * scale);        \
    }                                                                                             \
    return 0;                                                                                     \
  }

DEFINE_EVAL(oracle_eval_f64, double, double, sqrt)
DEFINE_EVAL(oracle_eval_f32, float, float, sqrtf)
DEFINE_EVAL(oracle_eval_ld, double, long double, sqrtl)

/* ---------------------------------------------------------- KernelMatrix */

#define DEFINE_KMAT(NAME, REAL, SQRT)                                                             \
  int NAME(int kernel, int64_t nt, const REAL* r_trg, int64_t ns, const REAL* r_src,             \
           const REAL* n_src, REAL* M, int nthreads) {                                            \
    int nd, sd, td;                                                                               \
    if (oracle_kernel_dims(kernel, NULL, &nd, &sd, &td)) return -1;                               \
    if (nt < 0 || ns < 0) return -2;                                                              \
    const REAL scale = (REAL)oracle_scale_factor(kernel);                                         \
    const int64_t ld = nt * td;                                                                   \
    _Pragma("omp parallel for schedule(static) num_threads(resolve_threads(nthreads))")           \
    for (int64_t s = 0; s < ns; s++) {                                                            \
      const REAL xs0 = r_src[s * 3], xs1 = r_src[s * 3 + 1], xs2 = r_src[s * 3 + 2];              \
      REAL n0 = 0, n1 = 0, n2 = 0;                                                                \
      if (nd) { n0 = n_src[s * 3]; n1 = n_src[s * 3 + 1]; n2 = n_src[s * 3 + 2]; }                \
      for (int64_t t = 0; t < nt; t++) {                                                          \
        const REAL r[3] = {r_trg[t * 3] - xs0, r_trg[t * 3 + 1] - xs1, r_trg[t * 3 + 2] - xs2};   \
        const REAL r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];                                  \
        const REAL rinv = r2 > 0 ? (REAL)1 / SQRT(r2) : (REAL)0;                                  \
        REAL u[3][3];                                                                             \
        switch (kernel) {                                                                         \
          case ORACLE_LAPLACE3D_FXU: u[0][0] = rinv; break;                                       \
          case ORACLE_LAPLACE3D_DXU:                                                              \
            u[0][0] = (r[0] * n0 + r[1] * n1 + r[2] * n2) * (rinv * rinv * rinv);                 \
            break;                                                                                \
          case ORACLE_STOKES3D_FXU: { /* kernel_functions.hpp:136-145 */                          \
            const REAL rinv3 = rinv * rinv * rinv;                                                \
            for (int i = 0; i < 3; i++)                                                           \
              for (int j = 0; j < 3; j++) u[i][j] = (i == j ? rinv : (REAL)0) + r[i] * r[j] * rinv3; \
          } break;                                                                                \
          default: { /* Stokes3D_DxU, kernel_functions.hpp:191-201 */                             \
            const REAL rinv2 = rinv * rinv;                                                       \
            const REAL rinv5 = rinv2 * rinv2 * rinv;                                              \
            const REAL rdn = (r[0] * n0 + r[1] * n1 + r[2] * n2) * rinv5;                         \
            for (int i = 0; i < 3; i++)                                                           \
              for (int j = 0; j < 3; j++) u[i][j] = r[i] * r[j] * rdn;                            \
          } break;                                                                                \
        }                                                                                         \
        for (int k0 = 0; k0 < sd; k0++)                                                           \
          for (int k1 = 0; k1 < td; k1++) M[(s * sd + k0) * ld + t * td + k1] = u[k0][k1] * scale; \
      }                                                                                           \
    }                                                                                             \
    return 0;                                                                                     \
  }

DEFINE_KMAT(oracle_kernel_matrix_f64, double, sqrt)
DEFINE_KMAT(oracle_kernel_matrix_f32, float, sqrtf)

/* ---------------------------------------------------------------- near lists */
static int near_test(const double* xt, const double* xs, double r) {
  /* node_dist2: dist2 += dX * dX over x, y, z, then dist2 < rad * rad */
  volatile double d2 = 0.0;
  for (int k = 0; k < 3; ++k) {
    volatile double dx = xs[k] - xt[k];
    volatile double sq = dx * dx;
    d2 = d2 + sq;
  }
  volatile double r2 = r * r;
  return d2 < r2;
}

int64_t oracle_near_pairs(int64_t nt, const double* r_trg, int64_t n_elem, const int64_t* elem_nds_cnt,
                          const int64_t* elem_nds_dsp, const double* r_src, const double* src_radius, int64_t cap,
                          int64_t* pair_elem, int64_t* pair_trg) {
  int64_t* cnt = (int64_t*)calloc((size_t)(n_elem > 0 ? n_elem : 1), sizeof(int64_t));
  if (!cnt) return -1;
#pragma omp parallel for schedule(dynamic)
  for (int64_t e = 0; e < n_elem; ++e) {
    int64_t c = 0;
    for (int64_t t = 0; t < nt; ++t)
      for (int64_t j = 0; j < elem_nds_cnt[e]; ++j) {
        const int64_t s = elem_nds_dsp[e] + j;
        if (near_test(r_trg + t * 3, r_src + s * 3, src_radius[s])) {
          ++c;
          break;
        }
      }
    cnt[e] = c;
  }
  int64_t total = 0;
  for (int64_t e = 0; e < n_elem; ++e) total += cnt[e];
  if (pair_elem && pair_trg) {
    if (total > cap) {
      free(cnt);
      return -1;
    }
    int64_t off = 0;
    for (int64_t e = 0; e < n_elem; ++e) {
      const int64_t o = off;
      off += cnt[e];
      cnt[e] = o;
    }
#pragma omp parallel for schedule(dynamic)
    for (int64_t e = 0; e < n_elem; ++e) {
      int64_t k = cnt[e];
      for (int64_t t = 0; t < nt; ++t)
        for (int64_t j = 0; j < elem_nds_cnt[e]; ++j) {
          const int64_t s = elem_nds_dsp[e] + j;
          if (near_test(r_trg + t * 3, r_src + s * 3, src_radius[s])) {
            pair_elem[k] = e;
            pair_trg[k] = t;
            ++k;
            break;
          }
        }
    }
  }
  free(cnt);
  return total;
}

/* ------------------------------------------------- kernel ids 4-15 (uKerMatrix forms) */
int oracle_xdims(int kernel, int* nd, int* sd, int* td) {
  static const int D[16][3] = {{0, 1, 1}, {3, 1, 1}, {0, 3, 3}, {3, 3, 3}, {0, 1, 3}, {0, 1, 9}, {3, 1, 3}, {0, 3, 3},
                               {0, 3, 9}, {0, 2, 2}, {3, 2, 2}, {0, 2, 6}, {0, 2, 6}, {0, 3, 9}, {0, 4, 3}, {0, 3, 4}};
  if (kernel < 0 || kernel > 15) return -1;
  *nd = D[kernel][0];
  *sd = D[kernel][1];
  *td = D[kernel][2];
  return 0;
}

double oracle_xscale(int kernel) {
  switch (kernel) {
    case 4: return -1.0 / (4.0 * kPi);  /* kernel_functions.hpp:88-90 */
    case 5: return 1.0 / (4.0 * kPi);   /* :374-376 */
    case 6: return 1.0 / (4.0 * kPi);   /* :400-402 */
    case 7: return 1.0 / (4.0 * kPi);   /* :424-426 */
    case 8: return -1.0 / (4.0 * kPi);  /* :459-461 */
    case 9: return 1.0 / (4.0 * kPi);   /* :499-501 */
    case 10: return -1.0 / (4.0 * kPi); /* :537-539 */
    case 11: return 1.0 / (4.0 * kPi);  /* :581-583 */
    case 12: return 1.0 / (4.0 * kPi);  /* :635-637 */
    case 13: return -3.0 / (4.0 * kPi); /* :228-230 */
    case 14: return 1.0 / (8.0 * kPi);  /* :272-274 */
    case 15: return 1.0 / (8.0 * kPi);  /* :333-335 */
    default: return oracle_scale_factor(kernel);
  }
}

/* u[k0][k1] of kernel `kernel` at r (target minus source), normal n, wavenumber mu. */
#define DEFINE_XUMAT(NAME, REAL, SQRT, SIN, COS)                                                    \
  static void NAME(int kernel, const REAL r[3], const REAL n[3], REAL mu, REAL u[4][9]) {           \
    const REAL r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];                                        \
    const REAL rinv = r2 > 0 ? (REAL)1 / SQRT(r2) : (REAL)0;                                        \
    const REAL rinv2 = rinv * rinv, rinv3 = rinv2 * rinv;                                           \
    for (int a = 0; a < 4; a++)                                                                     \
      for (int b = 0; b < 9; b++) u[a][b] = 0;                                                      \
    switch (kernel) {                                                                               \
      case 4: /* Laplace3D_FxdU :91-98 */                                                           \
        for (int i = 0; i < 3; i++) u[0][i] = r[i] * rinv3;                                         \
        break;                                                                                      \
      case 5: { /* Laplace3D_Fxd2U :377-389 */                                                      \
        const REAL t5 = (REAL)3 * rinv3 * rinv2;                                                    \
        for (int i = 0; i < 3; i++)                                                                 \
          for (int j = 0; j < 3; j++) u[0][i * 3 + j] = t5 * r[i] * r[j] - (i == j ? rinv3 : (REAL)0); \
      } break;                                                                                      \
      case 6: { /* Laplace3D_DxdU :404-413 */                                                       \
        const REAL rdotn = r[0] * n[0] + r[1] * n[1] + r[2] * n[2];                                 \
        const REAL t5 = (REAL)3 * rdotn * rinv3 * rinv2;                                            \
        for (int i = 0; i < 3; i++) u[0][i] = n[i] * rinv3 - r[i] * t5;                             \
      } break;                                                                                      \
      case 7: /* BiotSavart3D_FxU :427-434: v = f x r / r^3 */                                      \
        u[0][1] = -r[2] * rinv3; u[0][2] = r[1] * rinv3;                                            \
        u[1][0] = r[2] * rinv3;  u[1][2] = -r[0] * rinv3;                                           \
        u[2][0] = -r[1] * rinv3; u[2][1] = r[0] * rinv3;                                            \
        break;                                                                                      \
      case 8: { /* BiotSavart3D_FxdU :462-479: (grad of f x r / r^3), 3 x 9 */                      \
        const REAL t5 = (REAL)3 * rinv3 * rinv2;                                                    \
        for (int j = 0; j < 3; j++) { /* derivative direction j: d/dx_j (r_m / r^3) */               \
          REAL g[3]; /* g[m] = delta_mj / r^3 - 3 r_m r_j / r^5 (the reference's sign convention) */ \
          for (int m = 0; m < 3; m++) g[m] = (m == j ? rinv3 : (REAL)0) - t5 * r[m] * r[j];         \
          /* column block c of the source density f_c: v_i = sum eps(i, c, m) ... */                \
          u[1][0 * 3 + j] = -g[2]; u[2][0 * 3 + j] = g[1];                                          \
          u[0][1 * 3 + j] = g[2];  u[2][1 * 3 + j] = -g[0];                                         \
          u[0][2 * 3 + j] = -g[1]; u[1][2 * 3 + j] = g[0];                                          \
        }                                                                                           \
      } break;                                                                                      \
      case 9: case 10: case 11: case 12: { /* Helmholtz :502-511, :540-552, :584-597, :638-658 */ \
        REAL sn, cs, cm1;                                                                           \
        if (kernel == 12) {                                                                         \
          const REAL h = r2 * rinv * mu * (REAL)0.5;                                                \
          const REAL sh = SIN(h), ch = COS(h);                                                      \
          sn = (REAL)2 * sh * ch; cm1 = -(REAL)2 * sh * sh; cs = (REAL)1 + cm1;                     \
        } else {                                                                                    \
          const REAL x = r2 * rinv * mu;                                                            \
          sn = SIN(x); cs = COS(x); cm1 = cs;                                                       \
        }                                                                                           \
        if (kernel == 9) {                                                                          \
          u[0][0] = cs * rinv; u[0][1] = sn * rinv; u[1][0] = -u[0][1]; u[1][1] = u[0][0];          \
        } else if (kernel == 10) {                                                                  \
          const REAL ndotr = n[0] * r[0] + n[1] * r[1] + n[2] * r[2];                               \
          u[0][0] = (-mu * sn - cs * rinv) * rinv2 * ndotr;                                         \
          u[0][1] = (mu * cs - sn * rinv) * rinv2 * ndotr;                                          \
          u[1][0] = -u[0][1]; u[1][1] = u[0][0];                                                    \
        } else {                                                                                    \
          const REAL G0 = (-mu * sn - cm1 * rinv) * rinv2, G1 = (mu * cs - sn * rinv) * rinv2;      \
          for (int i = 0; i < 3; i++) {                                                             \
            u[0][i * 2] = G0 * r[i]; u[0][i * 2 + 1] = G1 * r[i];                                   \
            u[1][i * 2] = -u[0][i * 2 + 1]; u[1][i * 2 + 1] = u[0][i * 2];                          \
          }                                                                                         \
        }                                                                                           \
      } break;                                                                                      \
      case 13: { /* Stokes3D_FxT :231-244 */                                                        \
        const REAL rinv5 = rinv2 * rinv2 * rinv;                                                    \
        for (int i = 0; i < 3; i++)                                                                 \
          for (int j = 0; j < 3; j++)                                                               \
            for (int k = 0; k < 3; k++) u[i][j * 3 + k] = r[i] * r[j] * r[k] * rinv5;              \
      } break;                                                                                      \
      case 14: case 15: /* Stokes3D_FSxU :275-287, Stokes3D_FxUP :336-348 */                        \
        for (int i = 0; i < 3; i++)                                                                 \
          for (int j = 0; j < 3; j++) u[i][j] = (i == j ? rinv : (REAL)0) + r[i] * r[j] * rinv3;    \
        for (int j = 0; j < 3; j++) {                                                               \
          if (kernel == 14) u[3][j] = r[j] * rinv3; else u[j][3] = r[j] * rinv3;                    \
        }                                                                                           \
        break;                                                                                      \
      default: break;                                                                               \
    }                                                                                               \
  }

DEFINE_XUMAT(xumat_d, double, sqrt, sin, cos)
DEFINE_XUMAT(xumat_f, float, sqrtf, sinf, cosf)
DEFINE_XUMAT(xumat_l, long double, sqrtl, sinl, cosl)

#define DEFINE_XEVAL(NAME, REAL, UMAT)                                                              \
  static int NAME(int kernel, int64_t nt, const REAL* xt, int64_t ns, const REAL* xs, const REAL* xn, \
                  const REAL* f, REAL mu, REAL* out, const double scale, int nthreads, int mat) {    \
    int nd, sd, td;                                                                                 \
    if (oracle_xdims(kernel, &nd, &sd, &td) || kernel < 4) return -1;                               \
    _Pragma("omp parallel for schedule(static) num_threads(resolve_threads(nthreads))")             \
    for (int64_t t = 0; t < nt; t++) {                                                              \
      REAL v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};                                                      \
      for (int64_t s = 0; s < ns; s++) {                                                            \
        const REAL r[3] = {xt[t * 3] - xs[s * 3], xt[t * 3 + 1] - xs[s * 3 + 1], xt[t * 3 + 2] - xs[s * 3 + 2]}; \
        REAL n[3] = {0, 0, 0};                                                                      \
        if (nd) { n[0] = xn[s * 3]; n[1] = xn[s * 3 + 1]; n[2] = xn[s * 3 + 2]; }                   \
        REAL u[4][9];                                                                               \
        UMAT(kernel, r, n, mu, u);                                                                  \
        if (mat) {                                                                                  \
          for (int a = 0; a < sd; a++)                                                              \
            for (int b = 0; b < td; b++)                                                            \
              out[(s * sd + a) * (nt * td) + t * td + b] = (REAL)(u[a][b] * (REAL)scale);           \
        } else {                                                                                    \
          for (int b = 0; b < td; b++)                                                              \
            for (int a = 0; a < sd; a++) v[b] += u[a][b] * f[s * sd + a];                           \
        }                                                                                           \
      }                                                                                             \
      if (!mat)                                                                                     \
        for (int b = 0; b < td; b++) out[t * td + b] += v[b] * (REAL)scale;                         \
    }                                                                                               \
    return 0;                                                                                       \
  }

DEFINE_XEVAL(xeval_d, double, xumat_d)
DEFINE_XEVAL(xeval_f, float, xumat_f)
DEFINE_XEVAL(xeval_l, long double, xumat_l)

int oracle_xeval(int kernel, int precision, int64_t nt, const void* r_trg, int64_t ns, const void* r_src,
                 const void* n_src, const void* v_src, double mu, void* v_trg, int nthreads) {
  const double sc = oracle_xscale(kernel);
  if (precision == 1)
    return xeval_f(kernel, nt, (const float*)r_trg, ns, (const float*)r_src, (const float*)n_src,
                   (const float*)v_src, (float)mu, (float*)v_trg, sc, nthreads, 0);
  if (precision == 2) { /* inputs and outputs double, arithmetic long double */
    int nd, sd, td;
    if (oracle_xdims(kernel, &nd, &sd, &td)) return -1;
    long double *xt = malloc(sizeof(long double) * (size_t)(nt * 3 + 1)), *xs = malloc(sizeof(long double) * (size_t)(ns * 3 + 1)),
                *xn = malloc(sizeof(long double) * (size_t)(ns * 3 + 1)), *f = malloc(sizeof(long double) * (size_t)(ns * sd + 1)),
                *o = calloc((size_t)(nt * td + 1), sizeof(long double));
    for (int64_t i = 0; i < nt * 3; i++) xt[i] = ((const double*)r_trg)[i];
    for (int64_t i = 0; i < ns * 3; i++) xs[i] = ((const double*)r_src)[i];
    for (int64_t i = 0; i < ns * 3; i++) xn[i] = nd ? ((const double*)n_src)[i] : 0.0L;
    for (int64_t i = 0; i < ns * sd; i++) f[i] = ((const double*)v_src)[i];
    const int rc = xeval_l(kernel, nt, xt, ns, xs, xn, f, (long double)mu, o, sc, nthreads, 0);
    for (int64_t i = 0; i < nt * td; i++) ((double*)v_trg)[i] += (double)o[i];
    free(xt); free(xs); free(xn); free(f); free(o);
    return rc;
  }
  return xeval_d(kernel, nt, (const double*)r_trg, ns, (const double*)r_src, (const double*)n_src,
                 (const double*)v_src, mu, (double*)v_trg, sc, nthreads, 0);
}

int oracle_xkmat(int kernel, int precision, int64_t nt, const void* r_trg, int64_t ns, const void* r_src,
                 const void* n_src, double mu, void* M, int nthreads) {
  const double sc = oracle_xscale(kernel);
  if (precision == 1)
    return xeval_f(kernel, nt, (const float*)r_trg, ns, (const float*)r_src, (const float*)n_src, NULL, (float)mu,
                   (float*)M, sc, nthreads, 1);
  return xeval_d(kernel, nt, (const double*)r_trg, ns, (const double*)r_src, (const double*)n_src, NULL, mu,
                 (double*)M, sc, nthreads, 1);
}
