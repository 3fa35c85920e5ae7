// Compile-only check against the reference's own headers: the drop-in's
// static Eval converts to ParticleFMM's S2TData::ker_s2t_eval_omp pointer type
// (fmm-wrapper.txx:153-154) and the member Eval / KernelMatrix instantiate with
// sctl::Vector / sctl::Matrix.
#include "sctl/common.hpp"
#include "sctl/iterator.hpp"
#include "sctl/iterator.txx"
#include "sctl/matrix.hpp"
#include "sctl/matrix.txx"
#include "sctl/vector.hpp"
#include "sctl/vector.txx"

#include "sctlgpu.hpp"

template <class Real>
using KerS2TEval = void (*)(sctl::Vector<Real>& v_trg, const sctl::Vector<Real>& r_trg,
                            const sctl::Vector<Real>& r_src, const sctl::Vector<Real>& n_src,
                            const sctl::Vector<Real>& v_src, sctl::Integer digits, sctl::ConstIterator<char> self);

KerS2TEval<double> p0 = &sctlgpu::Laplace3D_FxU::Eval<double, true, sctl::Vector<double>, sctl::ConstIterator<char>>;
KerS2TEval<double> p1 = &sctlgpu::Laplace3D_DxU::Eval<double, true, sctl::Vector<double>, sctl::ConstIterator<char>>;
KerS2TEval<float> p2 = &sctlgpu::Stokes3D_FxU::Eval<float, false, sctl::Vector<float>, sctl::ConstIterator<char>>;
KerS2TEval<double> p3 = &sctlgpu::Stokes3D_DxU::Eval<double, true, sctl::Vector<double>, sctl::ConstIterator<char>>;
// a kernel that reads its context through `self` (the Helmholtz wavenumber)
KerS2TEval<double> p4 = &sctlgpu::Helmholtz3D_FxdU::Eval<double, true, sctl::Vector<double>, sctl::ConstIterator<char>>;
KerS2TEval<float> p5 = &sctlgpu::Stokes3D_FxT::Eval<float, true, sctl::Vector<float>, sctl::ConstIterator<char>>;

void instantiate_members() {
  sctlgpu::Stokes3D_DxU k;
  sctl::Vector<double> v, x, y, n, f;
  sctl::Matrix<double> M;
  k.Eval<double, false>(v, x, y, n, f);
  k.KernelMatrix<double, false>(M, x, y, n);
  static_assert(sctlgpu::Stokes3D_DxU::NormalDim() == 3 && sctlgpu::Laplace3D_FxU::SrcDim() == 1, "dims");
}
