// The drop-in at the reference's own call sites: SCTL's BoundaryIntegralOp
// and ParticleFMM (compiled from the installed reference headers) run with
// sctlgpu::GpuKernel<KID> in place of sctl::GenericKernel<uK>, and their results
// are compared against the same objects built with the reference's kernels.
//
//  * BoundaryIntegralOp<double, Kernel> (boundary_integral.hpp:250) on a
//    cubed-sphere QuadElemList (experimental/quad_element.hpp), targets
//    outside the near region of every element: ComputePotential
//    (boundary_integral.txx:716-722) -> ComputeFarField (:1248-1309) ->
//    ParticleFMM::Eval -> EvalDirect -> the S2T kernel pointer
//    (fmm-wrapper.txx:450-451, called at :618) = GpuKernel::Eval.  The element
//    list reports MatrixFree() so SetupSelf skips QuadElemList::SelfInterac,
//    which is an asserting stub in the reference (quad_element.cpp:278-281);
//    with far-only targets the near path has no pairs.
//  * ParticleFMM<double,3> directly: SetKernels / AddSrc / AddTrg /
//    SetKernelS2T with the GPU kernel, SetSrcCoord / SetSrcDensity /
//    SetTrgCoord, Eval (fmm-wrapper.hpp:115-190).
//
// Kernels: Laplace3D_DxU, Stokes3D_FxU, Stokes3D_DxU (and Laplace3D_FxU for
// ParticleFMM).  Pass criteria: rel-l2 <= 1e-12 with the FP64 arithmetic
// (sctlgpu::set_double_mode(SCTLGPU_F64), the default) and <= 1e-10 with the
// mixed arithmetic (SCTLGPU_MIXED) at the accuracy the operator asks for
// (SetAccuracy(1e-10) -> digits 11, boundary_integral.txx:592-593).
//
// Build (tests/test_cpp_shim.py does it): g++ -std=c++17 -O2 -fopenmp
//   -I<reference>/include -Iinclude tests/cpp/test_dropin_bio.cpp
//   -Lsctl_gb300 -lsctlgpu
#include <cmath>
#include <cstdio>
#include <random>
#include <string>

#include <sctl.hpp>
#include <sctl/experimental/quad_element.hpp>
#include <sctl/experimental/quad_element.cpp>

#include "sctlgpu.hpp"

namespace {

int g_failed = 0;

void check(bool ok, const char* what, double err, double tol) {
  std::printf("%-64s rel-l2 %.3e (tol %.0e) %s\n", what, err, tol, ok ? "ok" : "FAILED");
  if (!ok) ++g_failed;
}

double rel_l2(const sctl::Vector<double>& a, const sctl::Vector<double>& b) {
  if (a.Dim() != b.Dim()) return 1e300;
  double num = 0, den = 0;
  for (sctl::Long i = 0; i < a.Dim(); ++i) {
    num += (a[i] - b[i]) * (a[i] - b[i]);
    den += b[i] * b[i];
  }
  return std::sqrt(num / (den > 0 ? den : 1));
}

// QuadElemList whose operator setup skips the singular self-interaction (the
// reference's QuadElemList::SelfInterac is a stub that asserts).  Everything
// else -- nodes, far-field rule, far-field distances -- is the reference's.
class FarOnlyQuadElemList : public sctl::QuadElemList<double> {
 public:
  using sctl::QuadElemList<double>::QuadElemList;
  bool MatrixFree() const override { return true; }
};

// Cubed sphere of radius 1: 6 faces x P x P elements of order `order`
// (the geometry of the reference's src/test-quad-elem.cpp).
sctl::Vector<double> cubed_sphere(sctl::Integer order, sctl::Long P) {
  sctl::Vector<double> X;
  const sctl::Vector<double>& nds = sctl::QuadElemList<double>::ParamNodes(order);
  for (int face = 0; face < 6; ++face)
    for (sctl::Long iu = 0; iu < P; ++iu)
      for (sctl::Long iv = 0; iv < P; ++iv)
        for (sctl::Integer i = 0; i < order; ++i)
          for (sctl::Integer j = 0; j < order; ++j) {
            const double a = 2 * (iu + nds[i]) / (double)P - 1, b = 2 * (iv + nds[j]) / (double)P - 1;
            double x = 0, y = 0, z = 0;
            switch (face) {
              case 0: x = 1; y = a; z = b; break;
              case 1: x = -1; y = -a; z = b; break;
              case 2: x = a; y = 1; z = -b; break;
              case 3: x = a; y = -1; z = b; break;
              case 4: x = a; y = b; z = 1; break;
              default: x = -a; y = b; z = -1; break;
            }
            const double r = std::sqrt(x * x + y * y + z * z);
            X.PushBack(x / r);
            X.PushBack(y / r);
            X.PushBack(z / r);
          }
  return X;
}

// Targets at radius 2..3 (every element of the unit sphere is far from them).
sctl::Vector<double> far_targets(sctl::Long n, unsigned seed) {
  std::mt19937_64 g(seed);
  std::normal_distribution<double> N01(0, 1);
  std::uniform_real_distribution<double> U(2.0, 3.0);
  sctl::Vector<double> X(n * 3);
  for (sctl::Long i = 0; i < n; ++i) {
    double v[3] = {N01(g), N01(g), N01(g)};
    const double s = U(g) / std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int k = 0; k < 3; ++k) X[i * 3 + k] = v[k] * s;
  }
  return X;
}

sctl::Vector<double> densities(sctl::Long n, unsigned seed) {
  std::mt19937_64 g(seed);
  std::normal_distribution<double> N01(0, 1);
  sctl::Vector<double> F(n);
  for (auto& f : F) f = N01(g);
  return F;
}

template <class Kernel>
sctl::Vector<double> bio_potential(const FarOnlyQuadElemList& elems, const sctl::Vector<double>& Xt,
                                   const sctl::Vector<double>& F) {
  Kernel ker;
  sctl::BoundaryIntegralOp<double, Kernel> op(ker);
  op.AddElemList(elems);
  op.SetTargetCoord(Xt);
  op.SetAccuracy(1e-10);
  sctl::Vector<double> U;
  op.ComputePotential(U, F);
  return U;
}

template <class RefKernel, class GpuKernelT>
void bio_case(const char* name, const FarOnlyQuadElemList& elems, const sctl::Vector<double>& Xt, sctl::Long nnodes) {
  const sctl::Vector<double> F = densities(nnodes * RefKernel::SrcDim(), 7);
  const sctl::Vector<double> ref = bio_potential<RefKernel>(elems, Xt, F);
  sctlgpu::set_double_mode(SCTLGPU_F64);
  const sctl::Vector<double> g64 = bio_potential<GpuKernelT>(elems, Xt, F);
  sctlgpu::set_double_mode(SCTLGPU_MIXED);
  const sctl::Vector<double> gmx = bio_potential<GpuKernelT>(elems, Xt, F);
  sctlgpu::set_double_mode(SCTLGPU_F64);
  const double e64 = rel_l2(g64, ref), emx = rel_l2(gmx, ref);
  check(e64 <= 1e-12 && ref.Dim() == Xt.Dim() / 3 * RefKernel::TrgDim(),
        (std::string("BoundaryIntegralOp ") + name + " FP64").c_str(), e64, 1e-12);
  check(emx <= 1e-10, (std::string("BoundaryIntegralOp ") + name + " mixed").c_str(), emx, 1e-10);
}

template <class Kernel>
sctl::Vector<double> fmm_potential(const sctl::Vector<double>& Xs, const sctl::Vector<double>& Xn,
                                   const sctl::Vector<double>& F, const sctl::Vector<double>& Xt) {
  Kernel ker;
  sctl::ParticleFMM<double, 3> fmm;
  fmm.SetAccuracy(10);
  fmm.SetKernels(ker, ker, ker);
  fmm.AddSrc("Src", ker, ker);
  fmm.AddTrg("Trg", ker, ker);
  fmm.SetKernelS2T("Src", "Trg", ker);
  fmm.SetSrcCoord("Src", Xs, Kernel::NormalDim() ? Xn : sctl::Vector<double>());
  fmm.SetSrcDensity("Src", F);
  fmm.SetTrgCoord("Trg", Xt);
  sctl::Vector<double> U;
  fmm.Eval(U, "Trg");
  return U;
}

template <class RefKernel, class GpuKernelT>
void fmm_case(const char* name, const sctl::Vector<double>& Xs, const sctl::Vector<double>& Xn,
              const sctl::Vector<double>& Xt) {
  const sctl::Vector<double> F = densities(Xs.Dim() / 3 * RefKernel::SrcDim(), 11);
  const sctl::Vector<double> ref = fmm_potential<RefKernel>(Xs, Xn, F, Xt);
  sctlgpu::set_double_mode(SCTLGPU_F64);
  const sctl::Vector<double> g64 = fmm_potential<GpuKernelT>(Xs, Xn, F, Xt);
  sctlgpu::set_double_mode(SCTLGPU_MIXED);
  const sctl::Vector<double> gmx = fmm_potential<GpuKernelT>(Xs, Xn, F, Xt);
  sctlgpu::set_double_mode(SCTLGPU_F64);
  const double e64 = rel_l2(g64, ref), emx = rel_l2(gmx, ref);
  check(e64 <= 1e-12 && ref.Dim() == Xt.Dim() / 3 * RefKernel::TrgDim(),
        (std::string("ParticleFMM ") + name + " FP64").c_str(), e64, 1e-12);
  check(emx <= 1e-10, (std::string("ParticleFMM ") + name + " mixed").c_str(), emx, 1e-10);
}

}  // namespace

int main(int argc, char** argv) {
  sctl::Comm::MPI_Init(&argc, &argv);
  {
    const sctl::Integer order = 10;
    const sctl::Long P = 4;
    const sctl::Vector<double> X = cubed_sphere(order, P);
    const FarOnlyQuadElemList elems(order, X);
    const sctl::Long nnodes = X.Dim() / 3;
    const sctl::Vector<double> Xt = far_targets(4096, 3);

    bio_case<sctl::Laplace3D_DxU, sctlgpu::Laplace3D_DxU>("Laplace3D_DxU", elems, Xt, nnodes);
    bio_case<sctl::Stokes3D_FxU, sctlgpu::Stokes3D_FxU>("Stokes3D_FxU", elems, Xt, nnodes);
    bio_case<sctl::Stokes3D_DxU, sctlgpu::Stokes3D_DxU>("Stokes3D_DxU", elems, Xt, nnodes);

    sctl::Vector<double> Xs, Xn;
    sctl::Vector<sctl::Long> cnt;
    elems.GetNodeCoord(&Xs, &Xn, &cnt);
    fmm_case<sctl::Laplace3D_FxU, sctlgpu::Laplace3D_FxU>("Laplace3D_FxU", Xs, Xn, Xt);
    fmm_case<sctl::Laplace3D_DxU, sctlgpu::Laplace3D_DxU>("Laplace3D_DxU", Xs, Xn, Xt);
    fmm_case<sctl::Stokes3D_DxU, sctlgpu::Stokes3D_DxU>("Stokes3D_DxU", Xs, Xn, Xt);
  }
  std::printf("%s (%d check(s) failed)\n", g_failed ? "FAIL" : "PASS", g_failed);
  sctl::Comm::MPI_Finalize();
  return g_failed ? 1 : 0;
}
