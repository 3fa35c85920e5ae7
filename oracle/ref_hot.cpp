// The REFERENCE's own GenericKernel::Eval for one of the four hot-path kernels
// and one real type -- TEST AND BASELINE INFRASTRUCTURE ONLY.  Compiled by
// oracle/Makefile (target `hot`) against the installed reference headers
// (baseline/_ref/include/sctl) once per (kernel, real type) so the eight
// translation units build in parallel in seconds; ref_hot_main.cpp dispatches.
// The call is the static digits dispatcher through the kernel object pointer,
// exactly as ParticleFMM::EvalDirect calls it through ker_s2t_eval_omp
// (fmm-wrapper.txx:153-154,450-451,618; generic-kernel.hpp:99,
// generic-kernel.txx:72-100), with OpenMP enabled.
#include <cstdint>

#include "sctl.hpp"

#ifndef SCTLREF_KERNEL
#error "define SCTLREF_KERNEL (Laplace3D_FxU, Laplace3D_DxU, Stokes3D_FxU or Stokes3D_DxU)"
#endif
#ifndef SCTLREF_REAL
#error "define SCTLREF_REAL (double or float)"
#endif
#define SCTLREF_CAT2(a, b, c) a##_##b##_##c
#define SCTLREF_CAT(a, b, c) SCTLREF_CAT2(a, b, c)

extern "C" int SCTLREF_CAT(ref_hot_eval, SCTLREF_KERNEL, SCTLREF_REAL)(int digits, int64_t nt, const SCTLREF_REAL* r_trg,
                                                                       int64_t ns, const SCTLREF_REAL* r_src,
                                                                       const SCTLREF_REAL* n_src,
                                                                       const SCTLREF_REAL* v_src, SCTLREF_REAL* v_trg) {
  using Real = SCTLREF_REAL;
  using Kernel = sctl::SCTLREF_KERNEL;
  Kernel ker;
  const sctl::Long nd = Kernel::NormalDim(), sd = Kernel::SrcDim(), td = Kernel::TrgDim();
  sctl::Vector<Real> Xt(nt * 3, sctl::Ptr2Itr<Real>((Real*)r_trg, nt * 3), false);
  sctl::Vector<Real> Xs(ns * 3, sctl::Ptr2Itr<Real>((Real*)r_src, ns * 3), false);
  sctl::Vector<Real> Xn;
  if (nd) Xn.ReInit(ns * nd, sctl::Ptr2Itr<Real>((Real*)n_src, ns * nd), false);
  sctl::Vector<Real> Vs(ns * sd, sctl::Ptr2Itr<Real>((Real*)v_src, ns * sd), false);
  // v_trg has Nt * TrgDim entries, so Eval adds into it (generic-kernel.txx:129-132).
  sctl::Vector<Real> Vt(nt * td, sctl::Ptr2Itr<Real>(v_trg, nt * td), false);
  Kernel::template Eval<Real, true>(Vt, Xt, Xs, Xn, Vs, digits,
                                    (sctl::ConstIterator<char>)sctl::Ptr2ConstItr<char>(&ker, sizeof(ker)));
  return 0;
}
