// C++ drop-in for sctl::GenericKernel<uKernel> on the GB300 direct-sum path.
//
// sctlgpu::GpuKernel<KID> offers the members of GenericKernel that
// BoundaryIntegralOp and ParticleFMM use (include/sctl/generic-kernel.hpp):
//
//   static constexpr CoordDim/NormalDim/SrcDim/TrgDim()            (:54-74)
//   template <class Real, bool omp> static void Eval(v_trg, r_trg, r_src, n_src, v_src, digits, self)   (:99)
//   template <class Real, bool omp=false, Integer digits=-1> void Eval(v_trg, r_trg, r_src, n_src, v_src) const (:112)
//   template <class Real, bool omp=false, Integer digits=-1> void KernelMatrix(M, Xt, Xs, Xn) const     (:124)
//
// with the same argument meaning: AoS coordinates, v_trg re-initialised and
// zeroed when its size is wrong and otherwise accumulated into
// (generic-kernel.txx:129-132), M re-initialised when mis-sized
// (generic-kernel.txx:220-223).  The vector/matrix types are template
// parameters, so sctl::Vector<Real> / sctl::Matrix<Real> (or any type with
// Dim(), operator[], ReInit and SetZero) work unchanged, and
//
//   &sctlgpu::Laplace3D_DxU::Eval<double, true, sctl::Vector<double>, sctl::ConstIterator<char>>
//
// has exactly the type of ParticleFMM's S2TData::ker_s2t_eval_omp
// (fmm-wrapper.txx:153-154).  Failures abort like SCTL_ASSERT
// (common.hpp:98-105) unless SCTLGPU_ON_ERROR is defined to something else.
#ifndef SCTLGPU_HPP_
#define SCTLGPU_HPP_

#include <cstdio>
#include <cstdlib>
#include <string>
#include <type_traits>
#include <vector>

#include "sctlgpu.h"

#ifndef SCTLGPU_ON_ERROR
#define SCTLGPU_ON_ERROR(rc, what)                                                              \
  do {                                                                                          \
    std::fprintf(stderr, "sctlgpu: %s failed: %s %s\n", what, sctlgpu_strerror(rc),              \
                 rc == SCTLGPU_ERR_CUDA ? sctlgpu_last_cuda_error() : "");                       \
    std::abort();                                                                               \
  } while (0)
#endif

namespace sctlgpu {

// Arithmetic used for Real = double (Real = float always runs SCTLGPU_F32).
// SCTLGPU_F64 reproduces the reference's FP64 Eval; SCTLGPU_MIXED trades the
// FP64 pipe for double-float FP32 arithmetic at the same digits.
inline int& double_mode() {
  static int mode = SCTLGPU_F64;
  return mode;
}
inline void set_double_mode(int mode) { double_mode() = mode; }

template <int KID>
class GpuKernel {
  // NormalDim, SrcDim, TrgDim of every kernel id (kernel_functions.hpp with generic-kernel.hpp:54-74).
  static constexpr long kDims[SCTLGPU_NUM_KERNELS][3] = {
      {0, 1, 1}, {3, 1, 1}, {0, 3, 3}, {3, 3, 3}, {0, 1, 3}, {0, 1, 9}, {3, 1, 3}, {0, 3, 3},
      {0, 3, 9}, {0, 2, 2}, {3, 2, 2}, {0, 2, 6}, {0, 2, 6}, {0, 3, 9}, {0, 4, 3}, {0, 3, 4}};
  static constexpr bool kNeedsCtx = KID >= SCTLGPU_HELMHOLTZ3D_FXU && KID <= SCTLGPU_HELMHOLTZDIFF3D_FXDU;

  // The kernel object behind `self`: a GpuKernel pointer (member calls), or the
  // kernel object's bytes as ParticleFMM passes them (fmm-wrapper.txx:618).
  template <class SelfT>
  static const void* ctx_of(const SelfT& self) {
    if constexpr (!kNeedsCtx) {
      return nullptr;
    } else if constexpr (std::is_convertible<SelfT, const void*>::value) {
      const void* p = self;
      return p ? static_cast<const GpuKernel*>(p)->ctx_ptr : nullptr;
    } else {
      return reinterpret_cast<const GpuKernel*>(&self[0])->ctx_ptr;
    }
  }

  template <class V>
  static auto ptr(V& v) -> decltype(&v[0]) {
    return v.Dim() ? &v[0] : nullptr;
  }
  template <class Real>
  static int mode_for() {
    return std::is_same<Real, float>::value ? SCTLGPU_F32 : double_mode();
  }

 public:
  static_assert(KID >= 0 && KID < SCTLGPU_NUM_KERNELS, "unknown sctlgpu kernel id");

  static constexpr long CoordDim() { return 3; }
  static constexpr long NormalDim() { return kDims[KID][0]; }
  static constexpr long SrcDim() { return kDims[KID][1]; }
  static constexpr long TrgDim() { return kDims[KID][2]; }
  static const std::string& Name() {  // the Name() of each micro-kernel, kernel_functions.hpp
    static const std::string names[SCTLGPU_NUM_KERNELS] = {
        "Laplace3D-FxU",    "Laplace3D-DxU",     "Stokes3D-FxU",    "Stokes3D-DxU",
        "Laplace3D-FxdU",   "Laplace3D-Fxd2U",   "Laplace3D-DxdU",  "BiotSavart3D-FxU",
        "BiotSavart3D-FxdU", "Helmholtz3D-FxU",  "Helmholtz3D-DxU", "Helmholtz3D-FxdU",
        "HelmholtzDiff3D-FxdU", "Stokes3D-FxT", "Stokes3D-FSxU",   "Stokes3D-FxUP"};
    return names[KID];
  }

  GpuKernel() : ctx_ptr(nullptr) {}
  void SetCtxPtr(void* ctx) { ctx_ptr = ctx; }
  const void* GetCtxPtr() const { return ctx_ptr; }

  // GenericKernel<uK>::Eval<Real,enable_openmp>(..., digits, self), generic-kernel.hpp:99.
  // `self` is the kernel object; the Helmholtz kernels read their wavenumber through its ctx
  // pointer (SetCtxPtr), a value of type Real.
  template <class Real, bool enable_openmp, class VecT, class SelfT>
  static void Eval(VecT& v_trg, const VecT& r_trg, const VecT& r_src, const VecT& n_src, const VecT& v_src,
                   long digits, SelfT self) {
    static_assert(std::is_same<Real, float>::value || std::is_same<Real, double>::value, "Real must be float or double");
    const long nt = (long)r_trg.Dim() / 3, ns = (long)r_src.Dim() / 3;
    if ((long)r_trg.Dim() != nt * 3 || (long)r_src.Dim() != ns * 3 || (long)v_src.Dim() != ns * SrcDim() ||
        (NormalDim() && (long)n_src.Dim() != ns * NormalDim()))
      SCTLGPU_ON_ERROR(SCTLGPU_ERR_INVALID_SIZE, "GpuKernel::Eval");
    unsigned flags = SCTLGPU_ACCUMULATE;
    if ((long)v_trg.Dim() != nt * TrgDim()) {
      v_trg.ReInit(nt * TrgDim());
      v_trg.SetZero();
      flags = 0;
    }
    const int rc = sctlgpu_eval_ctx(KID, mode_for<Real>(), (int)digits, nt, ptr(r_trg), ns, ptr(r_src),
                                    NormalDim() ? ptr(n_src) : nullptr, ptr(v_src), ptr(v_trg), flags, ctx_of(self),
                                    nullptr);
    if (rc != SCTLGPU_OK) SCTLGPU_ON_ERROR(rc, "GpuKernel::Eval");
  }

  // Member form with compile-time digits, generic-kernel.hpp:112.
  template <class Real, bool enable_openmp = false, long digits = -1, class VecT>
  void Eval(VecT& v_trg, const VecT& r_trg, const VecT& r_src, const VecT& n_src, const VecT& v_src) const {
    Eval<Real, enable_openmp, VecT, const void*>(v_trg, r_trg, r_src, n_src, v_src, digits, this);
  }

  // KernelMatrix<Real,omp,digits>(M, Xt, Xs, Xn), generic-kernel.hpp:124: M[(s*K0+k0)][(t*K1+k1)].
  template <class Real, bool enable_openmp = false, long digits = -1, class MatT, class VecT>
  void KernelMatrix(MatT& M, const VecT& Xt, const VecT& Xs, const VecT& Xn) const {
    const long ns = (long)Xs.Dim() / 3, nt = (long)Xt.Dim() / 3;
    if ((long)M.Dim(0) != ns * SrcDim() || (long)M.Dim(1) != nt * TrgDim()) {
      M.ReInit(ns * SrcDim(), nt * TrgDim());
      M.SetZero();
    }
    if (!ns || !nt) return;
    const int rc = sctlgpu_kernel_matrix_ctx(KID, mode_for<Real>(), (int)digits, nt, ptr(Xt), ns, ptr(Xs),
                                             NormalDim() ? ptr(Xn) : nullptr, &M[0][0], 0, ctx_ptr, nullptr);
    if (rc != SCTLGPU_OK) SCTLGPU_ON_ERROR(rc, "GpuKernel::KernelMatrix");
  }

 private:
  void* ctx_ptr;
};

template <int KID>
constexpr long GpuKernel<KID>::kDims[SCTLGPU_NUM_KERNELS][3];

// The aliases of kernel_functions.hpp:669-684.
using Laplace3D_FxU = GpuKernel<SCTLGPU_LAPLACE3D_FXU>;
using Laplace3D_DxU = GpuKernel<SCTLGPU_LAPLACE3D_DXU>;
using Laplace3D_FxdU = GpuKernel<SCTLGPU_LAPLACE3D_FXDU>;
using Laplace3D_Fxd2U = GpuKernel<SCTLGPU_LAPLACE3D_FXD2U>;
using Laplace3D_DxdU = GpuKernel<SCTLGPU_LAPLACE3D_DXDU>;
using BiotSavart3D_FxU = GpuKernel<SCTLGPU_BIOTSAVART3D_FXU>;
using BiotSavart3D_FxdU = GpuKernel<SCTLGPU_BIOTSAVART3D_FXDU>;
using Helmholtz3D_FxU = GpuKernel<SCTLGPU_HELMHOLTZ3D_FXU>;
using Helmholtz3D_DxU = GpuKernel<SCTLGPU_HELMHOLTZ3D_DXU>;
using Helmholtz3D_FxdU = GpuKernel<SCTLGPU_HELMHOLTZ3D_FXDU>;
using HelmholtzDiff3D_FxdU = GpuKernel<SCTLGPU_HELMHOLTZDIFF3D_FXDU>;
using Stokes3D_FxU = GpuKernel<SCTLGPU_STOKES3D_FXU>;
using Stokes3D_DxU = GpuKernel<SCTLGPU_STOKES3D_DXU>;
using Stokes3D_FxT = GpuKernel<SCTLGPU_STOKES3D_FXT>;
using Stokes3D_FSxU = GpuKernel<SCTLGPU_STOKES3D_FSXU>;
using Stokes3D_FxUP = GpuKernel<SCTLGPU_STOKES3D_FXUP>;

// ParticleFMM's evaluation for one (source, target) pair of names, on the GPU:
// the same setters and Eval / EvalDirect (fmm-wrapper.txx:270-281, 505-623),
// for Real = double and the four hot-path kernels.  Like the reference, Eval
// takes the fast path for 40,000 targets or more (EvalPVFMM, :854-1038, cut-over
// :864-867) -- here the treecode, rebuilt when the coordinates or the accuracy
// changed (the reference's setup_tree flag) -- and EvalDirect otherwise; U is
// re-initialised to Nt * TrgDim and overwritten (:562-563).
template <int KID>
class GpuFarField {
  static_assert(KID >= SCTLGPU_LAPLACE3D_FXU && KID <= SCTLGPU_STOKES3D_DXU, "the four hot-path kernels");

 public:
  static constexpr long kDirectBelow = 40000;

  GpuFarField() = default;
  GpuFarField(const GpuFarField&) = delete;
  GpuFarField& operator=(const GpuFarField&) = delete;
  ~GpuFarField() { Release(); }

  void SetAccuracy(int digits) {  // fmm-wrapper.txx:270-281
    if (digits != digits_) Release();
    digits_ = digits;
  }
  template <class VecT>
  void SetSrcCoord(const VecT& coord, const VecT& normal) {  // :505-519
    Copy(xs_, coord);
    Copy(xn_, normal);
    Release();
  }
  template <class VecT>
  void SetSrcCoord(const VecT& coord) {
    Copy(xs_, coord);
    xn_.clear();
    Release();
  }
  template <class VecT>
  void SetSrcDensity(const VecT& density) {  // :521-524
    Copy(f_, density);
  }
  template <class VecT>
  void SetTrgCoord(const VecT& coord) {  // :526-540
    Copy(xt_, coord);
    Release();
  }

  template <class VecT>
  void Eval(VecT& U) {  // :542-549
    const long nt = (long)xt_.size() / 3;
    if (nt < kDirectBelow) return EvalDirect(U);
    Check();
    Resize(U, nt);
    if (nt == 0) return;
    int rc = SCTLGPU_OK;
    if (!tc_)
      rc = sctlgpu_treecode_create(&tc_, KID, Mode(), digits_, (long)xs_.size() / 3, Ptr(xs_), NDim() ? Ptr(xn_) : nullptr,
                                   nt, Ptr(xt_), nullptr);
    if (rc == SCTLGPU_OK) rc = sctlgpu_treecode_execute(tc_, Ptr(f_), &U[0], 0, nullptr);
    if (rc != SCTLGPU_OK) SCTLGPU_ON_ERROR(rc, "GpuFarField::Eval");
  }
  template <class VecT>
  void EvalDirect(VecT& U) {  // :551-623
    Check();
    const long nt = (long)xt_.size() / 3, ns = (long)xs_.size() / 3;
    Resize(U, nt);
    if (nt == 0) return;
    const int rc = sctlgpu_eval(KID, Mode(), digits_, nt, Ptr(xt_), ns, Ptr(xs_), NDim() ? Ptr(xn_) : nullptr,
                                Ptr(f_), &U[0], 0, nullptr);
    if (rc != SCTLGPU_OK) SCTLGPU_ON_ERROR(rc, "GpuFarField::EvalDirect");
  }

 private:
  static long NDim() { return GpuKernel<KID>::NormalDim(); }
  static int Mode() { return double_mode() == SCTLGPU_F64 ? SCTLGPU_F64 : SCTLGPU_MIXED; }
  static const double* Ptr(const std::vector<double>& v) { return v.empty() ? nullptr : v.data(); }
  template <class VecT>
  static void Copy(std::vector<double>& dst, const VecT& src) {
    dst.resize((size_t)src.Dim());
    for (long i = 0; i < (long)src.Dim(); ++i) dst[(size_t)i] = (double)src[i];
  }
  template <class VecT>
  static void Resize(VecT& U, long nt) {
    if ((long)U.Dim() != nt * GpuKernel<KID>::TrgDim()) U.ReInit(nt * GpuKernel<KID>::TrgDim());
  }
  void Check() const {
    const long ns = (long)xs_.size() / 3;
    if ((long)xs_.size() != ns * 3 || (long)xt_.size() % 3 || (long)f_.size() != ns * GpuKernel<KID>::SrcDim() ||
        (NDim() && (long)xn_.size() != ns * NDim()))
      SCTLGPU_ON_ERROR(SCTLGPU_ERR_INVALID_SIZE, "GpuFarField");
  }
  void Release() {
    if (tc_) sctlgpu_treecode_destroy(tc_);
    tc_ = nullptr;
  }

  std::vector<double> xs_, xn_, xt_, f_;
  int digits_ = 10;  // ParticleFMM's default accuracy (fmm-wrapper.txx:205)
  sctlgpu_treecode tc_ = nullptr;
};

}  // namespace sctlgpu

#endif  // SCTLGPU_HPP_
