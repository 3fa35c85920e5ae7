// Thin C-ABI wrapper around the REFERENCE's own header-only implementation --
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/Makefile against the reference
// headers (include/sctl/*) into oracle/_ref/libsctlref.so; used to pin the
// restated oracle (sctl_oracle.c) and to generate tests/golden fixtures.  It
// calls the reference's public API exactly as ParticleFMM does:
//   GenericKernel<uK>::Eval<Real,true>(v_trg, r_trg, r_src, n_src, v_src, digits, self)
//   (generic-kernel.hpp:99, called through a function pointer at fmm-wrapper.txx:618)
// and GenericKernel<uK>::KernelMatrix<Real,omp,digits>(M, Xt, Xs, Xn)
//   (generic-kernel.hpp:124, called by boundary_integral.txx:1197,1211).
#include <cstdint>
#include <cstring>
#include <type_traits>

#include "sctl.hpp"

namespace {

// The Helmholtz kernels read their wavenumber through the kernel object's ctx
// pointer (GenericKernel::SetCtxPtr, generic-kernel.hpp:79), as a value of the
// evaluation's real type.
double g_ctx_d = 0.0;
float g_ctx_f = 0.0f;

template <class Real>
void* ctx_for() {
  return std::is_same<Real, float>::value ? (void*)&g_ctx_f : (void*)&g_ctx_d;
}

template <class Kernel, class Real>
int eval_impl(int digits, int64_t nt, const Real* r_trg, int64_t ns, const Real* r_src, const Real* n_src,
              const Real* v_src, Real* v_trg, int omp) {
  Kernel ker;
  ker.SetCtxPtr(ctx_for<Real>());
  const sctl::Long nd = Kernel::NormalDim(), sd = Kernel::SrcDim(), td = Kernel::TrgDim();
  sctl::Vector<Real> Xt(nt * 3, sctl::Ptr2Itr<Real>((Real*)r_trg, nt * 3), false);
  sctl::Vector<Real> Xs(ns * 3, sctl::Ptr2Itr<Real>((Real*)r_src, ns * 3), false);
  sctl::Vector<Real> Xn;
  if (nd) Xn.ReInit(ns * nd, sctl::Ptr2Itr<Real>((Real*)n_src, ns * nd), false);
  sctl::Vector<Real> Vs(ns * sd, sctl::Ptr2Itr<Real>((Real*)v_src, ns * sd), false);
  // v_trg has the right size, so Eval accumulates into it (generic-kernel.txx:129-132).
  sctl::Vector<Real> Vt(nt * td, sctl::Ptr2Itr<Real>(v_trg, nt * td), false);
  if (omp)
    Kernel::template Eval<Real, true>(Vt, Xt, Xs, Xn, Vs, digits, (sctl::ConstIterator<char>)sctl::Ptr2ConstItr<char>(&ker, sizeof(ker)));
  else
    Kernel::template Eval<Real, false>(Vt, Xt, Xs, Xn, Vs, digits, (sctl::ConstIterator<char>)sctl::Ptr2ConstItr<char>(&ker, sizeof(ker)));
  return 0;
}

template <class Kernel, class Real>
int kmat_impl(int64_t nt, const Real* r_trg, int64_t ns, const Real* r_src, const Real* n_src, Real* M) {
  Kernel ker;
  ker.SetCtxPtr(ctx_for<Real>());
  const sctl::Long nd = Kernel::NormalDim(), sd = Kernel::SrcDim(), td = Kernel::TrgDim();
  sctl::Vector<Real> Xt(nt * 3, sctl::Ptr2Itr<Real>((Real*)r_trg, nt * 3), false);
  sctl::Vector<Real> Xs(ns * 3, sctl::Ptr2Itr<Real>((Real*)r_src, ns * 3), false);
  sctl::Vector<Real> Xn;
  if (nd) Xn.ReInit(ns * nd, sctl::Ptr2Itr<Real>((Real*)n_src, ns * nd), false);
  sctl::Matrix<Real> Mat(ns * sd, nt * td, sctl::Ptr2Itr<Real>(M, ns * sd * nt * td), false);
  ker.template KernelMatrix<Real, true>(Mat, Xt, Xs, Xn);
  return 0;
}

template <class Real>
int eval_dispatch(int kernel, int digits, int64_t nt, const Real* r_trg, int64_t ns, const Real* r_src,
                  const Real* n_src, const Real* v_src, Real* v_trg, int omp) {
  switch (kernel) {
    case 0: return eval_impl<sctl::Laplace3D_FxU, Real>(digits, nt, r_trg, ns, r_src, n_src, v_src, v_trg, omp);
    case 1: return eval_impl<sctl::Laplace3D_DxU, Real>(digits, nt, r_trg, ns, r_src, n_src, v_src, v_trg, omp);
    case 2: return eval_impl<sctl::Stokes3D_FxU, Real>(digits, nt, r_trg, ns, r_src, n_src, v_src, v_trg, omp);
    case 3: return eval_impl<sctl::Stokes3D_DxU, Real>(digits, nt, r_trg, ns, r_src, n_src, v_src, v_trg, omp);
    case 4: return eval_impl<sctl::Laplace3D_FxdU, Real>(digits, nt, r_trg, ns, r_src, n_src, v_src, v_trg, omp);
    case 5: return eval_impl<sctl::Laplace3D_Fxd2U, Real>(digits, nt, r_trg, ns, r_src, n_src, v_src, v_trg, omp);
    case 6: return eval_impl<sctl::Laplace3D_DxdU, Real>(digits, nt, r_trg, ns, r_src, n_src, v_src, v_trg, omp);
    case 7: return eval_impl<sctl::BiotSavart3D_FxU, Real>(digits, nt, r_trg, ns, r_src, n_src, v_src, v_trg, omp);
    case 8: return eval_impl<sctl::BiotSavart3D_FxdU, Real>(digits, nt, r_trg, ns, r_src, n_src, v_src, v_trg, omp);
    case 9: return eval_impl<sctl::Helmholtz3D_FxU, Real>(digits, nt, r_trg, ns, r_src, n_src, v_src, v_trg, omp);
    case 10: return eval_impl<sctl::Helmholtz3D_DxU, Real>(digits, nt, r_trg, ns, r_src, n_src, v_src, v_trg, omp);
    case 11: return eval_impl<sctl::Helmholtz3D_FxdU, Real>(digits, nt, r_trg, ns, r_src, n_src, v_src, v_trg, omp);
    case 12: return eval_impl<sctl::HelmholtzDiff3D_FxdU, Real>(digits, nt, r_trg, ns, r_src, n_src, v_src, v_trg, omp);
    case 13: return eval_impl<sctl::Stokes3D_FxT, Real>(digits, nt, r_trg, ns, r_src, n_src, v_src, v_trg, omp);
    case 14: return eval_impl<sctl::Stokes3D_FSxU, Real>(digits, nt, r_trg, ns, r_src, n_src, v_src, v_trg, omp);
    case 15: return eval_impl<sctl::Stokes3D_FxUP, Real>(digits, nt, r_trg, ns, r_src, n_src, v_src, v_trg, omp);
    default: return -1;
  }
}

template <class Real>
int kmat_dispatch(int kernel, int64_t nt, const Real* r_trg, int64_t ns, const Real* r_src, const Real* n_src, Real* M) {
  switch (kernel) {
    case 0: return kmat_impl<sctl::Laplace3D_FxU, Real>(nt, r_trg, ns, r_src, n_src, M);
    case 1: return kmat_impl<sctl::Laplace3D_DxU, Real>(nt, r_trg, ns, r_src, n_src, M);
    case 2: return kmat_impl<sctl::Stokes3D_FxU, Real>(nt, r_trg, ns, r_src, n_src, M);
    case 3: return kmat_impl<sctl::Stokes3D_DxU, Real>(nt, r_trg, ns, r_src, n_src, M);
    case 4: return kmat_impl<sctl::Laplace3D_FxdU, Real>(nt, r_trg, ns, r_src, n_src, M);
    case 5: return kmat_impl<sctl::Laplace3D_Fxd2U, Real>(nt, r_trg, ns, r_src, n_src, M);
    case 6: return kmat_impl<sctl::Laplace3D_DxdU, Real>(nt, r_trg, ns, r_src, n_src, M);
    case 7: return kmat_impl<sctl::BiotSavart3D_FxU, Real>(nt, r_trg, ns, r_src, n_src, M);
    case 8: return kmat_impl<sctl::BiotSavart3D_FxdU, Real>(nt, r_trg, ns, r_src, n_src, M);
    case 9: return kmat_impl<sctl::Helmholtz3D_FxU, Real>(nt, r_trg, ns, r_src, n_src, M);
    case 10: return kmat_impl<sctl::Helmholtz3D_DxU, Real>(nt, r_trg, ns, r_src, n_src, M);
    case 11: return kmat_impl<sctl::Helmholtz3D_FxdU, Real>(nt, r_trg, ns, r_src, n_src, M);
    case 12: return kmat_impl<sctl::HelmholtzDiff3D_FxdU, Real>(nt, r_trg, ns, r_src, n_src, M);
    case 13: return kmat_impl<sctl::Stokes3D_FxT, Real>(nt, r_trg, ns, r_src, n_src, M);
    case 14: return kmat_impl<sctl::Stokes3D_FSxU, Real>(nt, r_trg, ns, r_src, n_src, M);
    case 15: return kmat_impl<sctl::Stokes3D_FxUP, Real>(nt, r_trg, ns, r_src, n_src, M);
    default: return -1;
  }
}

}  // namespace

extern "C" {

int ref_eval(int kernel, int is_double, int digits, int64_t nt, const void* r_trg, int64_t ns, const void* r_src,
             const void* n_src, const void* v_src, void* v_trg, int omp) {
  if (is_double)
    return eval_dispatch<double>(kernel, digits, nt, (const double*)r_trg, ns, (const double*)r_src,
                                 (const double*)n_src, (const double*)v_src, (double*)v_trg, omp);
  return eval_dispatch<float>(kernel, digits, nt, (const float*)r_trg, ns, (const float*)r_src, (const float*)n_src,
                              (const float*)v_src, (float*)v_trg, omp);
}

int ref_kernel_matrix(int kernel, int is_double, int64_t nt, const void* r_trg, int64_t ns, const void* r_src,
                      const void* n_src, void* M) {
  if (is_double)
    return kmat_dispatch<double>(kernel, nt, (const double*)r_trg, ns, (const double*)r_src, (const double*)n_src,
                                 (double*)M);
  return kmat_dispatch<float>(kernel, nt, (const float*)r_trg, ns, (const float*)r_src, (const float*)n_src, (float*)M);
}

// BuildNearList<double,3> (boundary_integral.txx:50-522) on one rank
// (Comm::Self), as BoundaryIntegralOp::SetupNear calls it (:948).  The first
// call computes and keeps the result and returns the number of near entries;
// ref_near_list_get copies it out.
static sctl::Vector<double> g_xtrg_near, g_xn_near;
static sctl::Vector<sctl::Long> g_elem_cnt, g_elem_dsp, g_scatter, g_trg_cnt, g_trg_dsp;

int64_t ref_near_list(int64_t nt, const double* r_trg, int64_t n_elem, const int64_t* elem_nds_cnt,
                      const int64_t* elem_nds_dsp, int64_t ns, const double* r_src, const double* src_radius) {
  sctl::Vector<double> Xt(nt * 3, sctl::Ptr2Itr<double>((double*)r_trg, nt * 3), false);
  sctl::Vector<double> Xn;
  sctl::Vector<double> Xs(ns * 3, sctl::Ptr2Itr<double>((double*)r_src, ns * 3), false);
  sctl::Vector<double> rad(ns, sctl::Ptr2Itr<double>((double*)src_radius, ns), false);
  sctl::Vector<sctl::Long> cnt(n_elem), dsp(n_elem);
  for (int64_t i = 0; i < n_elem; ++i) {
    cnt[i] = elem_nds_cnt[i];
    dsp[i] = elem_nds_dsp[i];
  }
  sctl::BuildNearList<double, 3>(g_xtrg_near, g_xn_near, g_elem_cnt, g_elem_dsp, g_scatter, g_trg_cnt, g_trg_dsp, Xt,
                                 Xn, Xs, rad, cnt, dsp, sctl::Comm::Self());
  return (int64_t)g_scatter.Dim();
}

int ref_near_list_get(double* xtrg_near, int64_t* elem_cnt, int64_t* elem_dsp, int64_t* scatter, int64_t* trg_cnt,
                      int64_t* trg_dsp) {
  for (sctl::Long i = 0; i < g_xtrg_near.Dim(); ++i) xtrg_near[i] = g_xtrg_near[i];
  for (sctl::Long i = 0; i < g_elem_cnt.Dim(); ++i) elem_cnt[i] = g_elem_cnt[i];
  for (sctl::Long i = 0; i < g_elem_dsp.Dim(); ++i) elem_dsp[i] = g_elem_dsp[i];
  for (sctl::Long i = 0; i < g_scatter.Dim(); ++i) scatter[i] = g_scatter[i];
  for (sctl::Long i = 0; i < g_trg_cnt.Dim(); ++i) trg_cnt[i] = g_trg_cnt[i];
  for (sctl::Long i = 0; i < g_trg_dsp.Dim(); ++i) trg_dsp[i] = g_trg_dsp[i];
  return 0;
}

// Wavenumber seen by the Helmholtz kernels (both real types).
void ref_set_ctx(double mu) {
  g_ctx_d = mu;
  g_ctx_f = (float)mu;
}

// Which SIMD path the reference was compiled for (DefaultVecLen, vec.txx:27-42).
int ref_vec_len(int is_double) {
  return is_double ? (int)sctl::DefaultVecLen<double>() : (int)sctl::DefaultVecLen<float>();
}

}  // extern "C"
