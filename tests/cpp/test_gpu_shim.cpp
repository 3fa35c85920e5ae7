// The reference's GenericKernel unit tests (src/test-kernel_functions.cpp:36-132,
// :487-526 and src/test-generic-kernel.cpp:55-103) run through the C++ drop-in
// sctlgpu::GpuKernel on the GPU, with minimal stand-ins for sctl::Vector and
// sctl::Matrix (Dim, operator[], ReInit, SetZero).  Prints "PASS (0 check(s)
// failed)" like the reference's test-utils.hpp.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <initializer_list>
#include <vector>

#include "sctlgpu.hpp"

template <class T>
struct Vec {
  std::vector<T> d;
  Vec() = default;
  Vec(std::initializer_list<T> l) : d(l) {}
  explicit Vec(long n) : d(n, T(0)) {}
  long Dim() const { return (long)d.size(); }
  T& operator[](long i) { return d[i]; }
  const T& operator[](long i) const { return d[i]; }
  void ReInit(long n) { d.assign(n, T(0)); }
  void SetZero() { std::fill(d.begin(), d.end(), T(0)); }
};
template <class T>
struct Mat {
  long r = 0, c = 0;
  std::vector<T> d;
  long Dim(int i) const { return i ? c : r; }
  T* operator[](long i) { return d.data() + i * c; }
  const T* operator[](long i) const { return d.data() + i * c; }
  void ReInit(long a, long b) {
    r = a;
    c = b;
    d.assign(a * b, T(0));
  }
  void SetZero() { std::fill(d.begin(), d.end(), T(0)); }
};

static int failures = 0;
#define CHECK(...)                                                   \
  do {                                                               \
    if (!(__VA_ARGS__)) {                                            \
      std::printf("  FAIL @%d: %s\n", __LINE__, #__VA_ARGS__);       \
      ++failures;                                                    \
    }                                                                \
  } while (0)
template <class T>
static bool approx_eq(T a, T b, T tol) {
  const T diff = std::fabs(a - b), mag = std::max(std::fabs(a), std::fabs(b));
  return diff <= tol || diff <= tol * mag;
}

// ParticleFMM's function-pointer type (fmm-wrapper.txx:153-154) with these stand-ins.
template <class R>
using S2TEval = void (*)(Vec<R>&, const Vec<R>&, const Vec<R>&, const Vec<R>&, const Vec<R>&, long, const char*);

template <class R>
static void known_answers(R tol) {
  const R pi = (R)3.14159265358979323846;
  {
    sctlgpu::Laplace3D_FxU K;
    CHECK(K.CoordDim() == 3 && K.SrcDim() == 1 && K.TrgDim() == 1 && K.NormalDim() == 0);
    CHECK(K.Name() == std::string("Laplace3D-FxU"));
    Vec<R> Xs({0, 0, 0}), Xt({2, 0, 0}), Xn, v_s({3.0}), v_t;
    K.template Eval<R, false>(v_t, Xt, Xs, Xn, v_s);
    CHECK(v_t.Dim() == 1 && approx_eq(v_t[0], R(3.0 / (4 * pi * 2.0)), tol));
  }
  {
    sctlgpu::Laplace3D_DxU K;
    CHECK(K.NormalDim() == 3 && K.Name() == std::string("Laplace3D-DxU"));
    Vec<R> Xs({0, 0, 0}), Xt({2, 0, 0}), Xn({1, 0, 0}), v_s({1.0}), v_t;
    K.template Eval<R, false>(v_t, Xt, Xs, Xn, v_s);
    CHECK(approx_eq(v_t[0], R(1.0 / (16 * pi)), tol));
  }
  {
    sctlgpu::Stokes3D_FxU K;
    CHECK(K.SrcDim() == 3 && K.TrgDim() == 3 && K.NormalDim() == 0);
    Vec<R> Xs({0, 0, 0}), Xn, Xt({2.0, 0.0, 0.0}), v_s({1.0, 0.0, 0.0}), v_t;
    K.template Eval<R, false>(v_t, Xt, Xs, Xn, v_s);
    CHECK(v_t.Dim() == 3 && approx_eq(v_t[0], R(1.0 / (4 * pi * 2.0)), tol));
    CHECK(std::fabs(v_t[1]) < 1e-12 && std::fabs(v_t[2]) < 1e-12);
  }
  {
    sctlgpu::Stokes3D_DxU K;
    CHECK(K.NormalDim() == 3 && K.Name() == std::string("Stokes3D-DxU"));
    Vec<R> Xs({0, 0, 0}), Xt({3, 0, 0}), Xn({0, 1, 0}), v_s({1.0, 0.0, 0.0}), v_t;
    K.template Eval<R, false>(v_t, Xt, Xs, Xn, v_s);
    CHECK(v_t.Dim() == 3);
  }
  {  // test-generic-kernel.cpp:55-103
    sctlgpu::Laplace3D_FxU K;
    const R sf = R(1.0 / (4.0 * pi));
    Vec<R> Xt({1.0, 0.0, 0.0}), Xs({0.0, 0.0, 0.0}), Xn;
    Mat<R> M;
    K.template KernelMatrix<R, false>(M, Xt, Xs, Xn);
    CHECK(M.Dim(0) == 1 && M.Dim(1) == 1 && approx_eq(M[0][0], sf, tol));
    Vec<R> v_s({1.0}), Xt4({1, 0, 0, 2, 0, 0, 3, 0, 0, 5, 0, 0}), v_t;
    K.template Eval<R, false>(v_t, Xt4, Xs, Xn, v_s);
    CHECK(v_t.Dim() == 4 && approx_eq(v_t[0], sf / 1, tol) && approx_eq(v_t[1], sf / 2, tol) &&
          approx_eq(v_t[2], sf / 3, tol) && approx_eq(v_t[3], sf / 5, tol));
    Vec<R> Xs2({0, 0, 0, 4, 0, 0}), v_s2({1.0, 1.0}), Xt1({2, 0, 0}), v_t2;
    K.template Eval<R, false>(v_t2, Xt1, Xs2, Xn, v_s2);
    CHECK(v_t2.Dim() == 1 && approx_eq(v_t2[0], sf, tol));
    // a correctly sized v_trg is accumulated into (generic-kernel.txx:129-132)
    K.template Eval<R, false>(v_t2, Xt1, Xs2, Xn, v_s2);
    CHECK(approx_eq(v_t2[0], 2 * sf, tol));
  }
}

// Eval vs KernelMatrix on the 7 x 5 inputs of test-kernel_functions.cpp:487-526.
template <class K, class R, long DIG = -1>
static void eval_vs_matrix(R tol, R* ctx = nullptr) {
  K ker;
  ker.SetCtxPtr(ctx);
  const long Ns = 7, Nt = 5, K0 = K::SrcDim(), K1 = K::TrgDim(), ND = K::NormalDim();
  Vec<R> Xs(Ns * 3), Xn(Ns * ND), Vs(Ns * K0), Xt(Nt * 3), Vt;
  for (long i = 0; i < Xs.Dim(); i++) Xs[i] = R(0.1 * (i + 1) - 0.35);
  for (long i = 0; i < Vs.Dim(); i++) Vs[i] = R(0.3 * (i % 5) - 0.4);
  for (long i = 0; i < Xt.Dim(); i++) Xt[i] = R(1.7 + 0.2 * i);
  for (long i = 0; i < Ns && ND; i++) {
    Xn[i * 3 + 0] = 0;
    Xn[i * 3 + 1] = 1;
    Xn[i * 3 + 2] = 0;
  }
  ker.template Eval<R, false, DIG>(Vt, Xt, Xs, Xn, Vs);
  Mat<R> M;
  ker.template KernelMatrix<R, false, DIG>(M, Xt, Xs, Xn);
  for (long t = 0; t < Nt; t++)
    for (long k1 = 0; k1 < K1; k1++) {
      R acc = 0;
      for (long s = 0; s < Ns; s++)
        for (long k0 = 0; k0 < K0; k0++) acc += M[s * K0 + k0][t * K1 + k1] * Vs[s * K0 + k0];
      CHECK(approx_eq(Vt[t * K1 + k1], acc, tol));
    }
}

int main() {
  // The static Eval has the type ParticleFMM stores (fmm-wrapper.txx:153-154).
  S2TEval<double> fp = &sctlgpu::Laplace3D_DxU::Eval<double, true, Vec<double>, const char*>;
  S2TEval<float> fp32 = &sctlgpu::Stokes3D_FxU::Eval<float, true, Vec<float>, const char*>;
  {
    Vec<double> Xs({0, 0, 0}), Xt({2, 0, 0}), Xn({1, 0, 0}), v_s({1.0}), v_t;
    fp(v_t, Xt, Xs, Xn, v_s, 10, nullptr);
    CHECK(approx_eq(v_t[0], 1.0 / (16 * 3.14159265358979323846), 1e-12));
    Vec<float> Ys({0, 0, 0}), Yt({2, 0, 0}), Yn, f_s({1, 0, 0}), u_t;
    fp32(u_t, Yt, Ys, Yn, f_s, -1, nullptr);
    CHECK(u_t.Dim() == 3 && approx_eq(u_t[0], float(1.0 / (4 * 3.14159265358979323846 * 2.0)), 1e-6f));
  }
  for (int mode : {SCTLGPU_F64, SCTLGPU_MIXED}) {
    sctlgpu::set_double_mode(mode);
    known_answers<double>(1e-9);
    eval_vs_matrix<sctlgpu::Laplace3D_FxU, double>(1e-10);
    eval_vs_matrix<sctlgpu::Laplace3D_DxU, double>(1e-10);
    eval_vs_matrix<sctlgpu::Stokes3D_FxU, double>(1e-10);
    eval_vs_matrix<sctlgpu::Stokes3D_DxU, double>(1e-10);
    // digits 10: the mixed mode's double-float direct sum and kernel matrix
    eval_vs_matrix<sctlgpu::Laplace3D_FxU, double, 10>(1e-10);
    eval_vs_matrix<sctlgpu::Laplace3D_DxU, double, 10>(1e-10);
    eval_vs_matrix<sctlgpu::Stokes3D_FxU, double, 10>(1e-10);
    eval_vs_matrix<sctlgpu::Stokes3D_DxU, double, 10>(1e-10);
  }
  known_answers<float>(1e-5f);
  eval_vs_matrix<sctlgpu::Stokes3D_DxU, float>(1e-5f);
  // the other micro-kernels (kernel_functions.hpp:81-659), the Helmholtz ones with ctx = wavenumber
  sctlgpu::set_double_mode(SCTLGPU_F64);
  double mu = 2.5;
  float muf = 2.5f;
  eval_vs_matrix<sctlgpu::Laplace3D_FxdU, double>(1e-12);
  eval_vs_matrix<sctlgpu::Laplace3D_Fxd2U, double>(1e-12);
  eval_vs_matrix<sctlgpu::Laplace3D_DxdU, double>(1e-12);
  eval_vs_matrix<sctlgpu::BiotSavart3D_FxU, double>(1e-12);
  eval_vs_matrix<sctlgpu::BiotSavart3D_FxdU, double>(1e-12);
  eval_vs_matrix<sctlgpu::Helmholtz3D_FxU, double>(1e-12, &mu);
  eval_vs_matrix<sctlgpu::Helmholtz3D_DxU, double>(1e-12, &mu);
  eval_vs_matrix<sctlgpu::Helmholtz3D_FxdU, double>(1e-12, &mu);
  eval_vs_matrix<sctlgpu::HelmholtzDiff3D_FxdU, double>(1e-12, &mu);
  eval_vs_matrix<sctlgpu::Stokes3D_FxT, double>(1e-12);
  eval_vs_matrix<sctlgpu::Stokes3D_FSxU, double>(1e-12);
  eval_vs_matrix<sctlgpu::Stokes3D_FxUP, double>(1e-12);
  eval_vs_matrix<sctlgpu::Helmholtz3D_FxdU, float>(1e-5f, &muf);
  {
    // ParticleFMM passes the kernel object's bytes as `self` (fmm-wrapper.txx:618): the
    // static Eval finds the wavenumber through them.
    sctlgpu::Helmholtz3D_FxU H;
    H.SetCtxPtr(&mu);
    S2TEval<double> hp = &sctlgpu::Helmholtz3D_FxU::Eval<double, true, Vec<double>, const char*>;
    Vec<double> Xs({0, 0, 0}), Xt({2, 0, 0}), Xn, v_s({1.0, 0.0}), v_t;
    hp(v_t, Xt, Xs, Xn, v_s, -1, reinterpret_cast<const char*>(&H));
    const double pi = 3.14159265358979323846;
    CHECK(v_t.Dim() == 2 && approx_eq(v_t[0], std::cos(2 * mu) / (4 * pi * 2), 1e-12) &&
          approx_eq(v_t[1], std::sin(2 * mu) / (4 * pi * 2), 1e-12));
  }
  std::printf("\n%s (%d check(s) failed)\n", failures == 0 ? "PASS" : "FAIL", failures);
  return failures == 0 ? 0 : 1;
}
