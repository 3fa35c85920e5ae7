// The REFERENCE's own near-singular boundary quadrature (the legacy
// sctl::Quadrature of boundary_quadrature.hpp) run on the torus panels --
// TEST INFRASTRUCTURE ONLY: it produces the reference values that pin the
// near-singular double-layer quadrature (oracle/panel_oracle.py and the GPU
// panel kernels).  Built by oracle/Makefile (target `legacy`) from the
// installed reference headers into oracle/_ref/legacy_quad.
//
// The legacy quadrature does not compile against the current kernel, FMM and
// tree interfaces for three reasons, all interface gaps, which this file fills
// without touching its algorithm (the third is the bool -> Periodicity
// argument noted at the include below):
//   * it scales results by `kernel.template ScaleFactor<Real>()`
//     (boundary_quadrature.hpp:1635,1664,1671), which today's GenericKernel
//     does not have; today's GenericKernel already applies uKerScaleFactor in
//     Eval and KernelMatrix (generic-kernel.txx:154,206,268,306), so the wrapper
//     kernel below reports 1;
//   * its far part calls a static ParticleFMM<Real,3>::Eval(U, Xt, X, Xn, F,
//     kernel, comm) (boundary_quadrature.hpp:1533) that ParticleFMM no longer
//     has; the specialisation below provides exactly that call as the
//     reference's own direct sum, GenericKernel::Eval<double,true> (the
//     non-PVFMM path of ParticleFMM::Eval, fmm-wrapper.txx:542-549,551-623).
//
// Usage: legacy_quad <in.bin> <out.bin> [green]
//   in.bin : int64 Nt, Np (panels in theta, phi), double Rmajor, Rminor,
//            int64 order_singular, order_direct,
//            double density[Nt*Np*100] (our node order: theta index slow),
//            int64 Ntrg, double Xt[Ntrg*3]
//   out.bin: double U[Ntrg] (Laplace double-layer potential), then, with the
//            third argument, the max error of the legacy test's Green's
//            identity off the surface (boundary_quadrature.hpp:1679-1825) on the
//            same torus and orders (-1 without it).
#include <cstdint>
#include <cstdio>
#include <tuple>
#include <vector>

#include "sctl/common.hpp"
#include "sctl/comm.hpp"
#include "sctl/comm.txx"
#include "sctl/fmm-wrapper.hpp"
#include "sctl/generic-kernel.hpp"
#include "sctl/generic-kernel.txx"
#include "sctl/kernel_functions.hpp"
#include "sctl/vector.hpp"
#include "sctl/vector.txx"

namespace sctl {
// The static direct evaluation the legacy quadrature expects (see above).
template <>
class ParticleFMM<double, 3> {
 public:
  template <class Kernel>
  static void Eval(Vector<double>& U, const Vector<double>& Xt, const Vector<double>& X, const Vector<double>& Xn,
                   const Vector<double>& F, const Kernel& kernel, const Comm&) {
    kernel.template Eval<double, true>(U, Xt, X, Xn, F);
  }
};
}  // namespace sctl

// Everything else of the reference first (its include guard keeps sctl.hpp from
// pulling boundary_quadrature.hpp in yet) ...
#define _SCTL_BOUNDARY_QUADRATURE_HPP_
#include "sctl.hpp"
#undef _SCTL_BOUNDARY_QUADRATURE_HPP_
// ... then the legacy quadrature, whose tree refinement passes a bool where
// Tree::UpdateRefinement now takes a Periodicity (boundary_quadrature.hpp:890,
// tree.hpp:100): mapped for this one header (only non-periodic surfaces here).
#define UpdateRefinement(X, M, B, P) UpdateRefinement(X, M, B, (P) ? sctl::Periodicity::XYZ : sctl::Periodicity::NONE)
#include "sctl/boundary_quadrature.hpp"
#undef UpdateRefinement

namespace {

// A reference kernel with the ScaleFactor the legacy quadrature multiplies by.
template <class K>
struct LegacyKernel : public K {
  template <class Real>
  static constexpr Real ScaleFactor() {
    return 1;
  }
};

constexpr sctl::Integer ORDER = 10;
using Real = double;
using ElemBasis = sctl::Basis<Real, 2, ORDER>;
using ElemListT = sctl::ElemList<3, ElemBasis>;

// Torus panels with the legacy node layout (node k: theta index k % ORDER, phi index k / ORDER).
void build_torus(ElemListT& elements, long Nt, long Np, Real Rmajor, Real Rminor) {
  const auto nodes = ElemListT::CoordBasis::Nodes();
  elements.ReInit(Nt * Np);
  for (long ii = 0; ii < Nt * Np; ii++) {
    const long i = ii / Np, j = ii % Np;
    for (int k = 0; k < nodes.Dim(1); k++) {
      const Real theta = 2 * sctl::const_pi<Real>() * (i + nodes[0][k]) / Nt;
      const Real phi = 2 * sctl::const_pi<Real>() * (j + nodes[1][k]) / Np;
      const Real R = Rmajor + Rminor * sctl::cos<Real>(phi);
      elements(ii, 0)[k] = R * sctl::cos<Real>(theta);
      elements(ii, 1)[k] = R * sctl::sin<Real>(theta);
      elements(ii, 2)[k] = Rminor * sctl::sin<Real>(phi);
    }
  }
}

template <class T>
bool read_vals(FILE* f, T* p, size_t n) {
  return fread(p, sizeof(T), n, f) == n;
}

// Values of fn(U, X, Xn) at the element nodes, with Xn the unit normal of the
// interpolated surface (Xu x Xv / |Xu x Xv|, from Basis::Grad) -- what the
// reference test's DiscretizeSurfaceFn computes (boundary_quadrature.hpp:1848-1890).
void discretize(sctl::Vector<ElemBasis>& U, const ElemListT& el, const std::function<void(Real*, Real*, Real*)>& fn) {
  sctl::Vector<ElemBasis> dX;
  ElemBasis::Grad(dX, el.ElemVector());
  U.ReInit(el.NElem());
  for (long i = 0; i < el.NElem(); i++)
    for (long j = 0; j < ElemBasis::Size(); j++) {
      Real X[3], Xu[3], Xv[3], Xn[3], u;
      for (int k = 0; k < 3; k++) {
        X[k] = el(i, k)[j];
        Xu[k] = dX[(i * 3 + k) * 2 + 0][j];
        Xv[k] = dX[(i * 3 + k) * 2 + 1][j];
      }
      Real dA = 0;
      for (int k = 0; k < 3; k++) {
        Xn[k] = Xu[(k + 1) % 3] * Xv[(k + 2) % 3] - Xv[(k + 1) % 3] * Xu[(k + 2) % 3];
        dA += Xn[k] * Xn[k];
      }
      dA = sctl::sqrt<Real>(dA);
      for (int k = 0; k < 3; k++) Xn[k] /= dA;
      fn(&u, X, Xn);
      U[i][j] = u;
    }
}

// The reference test's Green's identity check, off-surface part
// (boundary_quadrature.hpp:1690-1824) on the given torus: targets at the nodes
// of a coarser concentric torus of minor radius 0.99 * Rminor, point source at
// (3, 2, 1).
double greens_identity_error(long Nt, long Np, Real Rmajor, Real Rminor, int order_singular, int order_direct) {
  using Quad = sctl::Quadrature<Real>;
  const sctl::Comm comm = sctl::Comm::Self();
  ElemListT src, trg;
  build_torus(src, Nt, Np, Rmajor, Rminor);
  build_torus(trg, Nt / 4 + 1, Np / 4 + 1, Rmajor, Rminor * 0.99);
  const Real X0[3] = {3, 2, 1};
  std::function<void(Real*, Real*, Real*)> pot = [X0](Real* U, Real* X, Real*) {
    const Real d[3] = {X[0] - X0[0], X[1] - X0[1], X[2] - X0[2]};
    U[0] = 1 / sctl::sqrt<Real>(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  };
  std::function<void(Real*, Real*, Real*)> dpot = [X0](Real* U, Real* X, Real* Xn) {
    const Real d[3] = {X[0] - X0[0], X[1] - X0[1], X[2] - X0[2]};
    const Real ri = 1 / sctl::sqrt<Real>(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    U[0] = -(d[0] * Xn[0] + d[1] * Xn[1] + d[2] * Xn[2]) * ri * ri * ri;
  };
  sctl::Vector<ElemBasis> dens_sl, dens_dl, U_off;
  discretize(dens_sl, src, dpot);
  discretize(dens_dl, src, pot);
  discretize(U_off, trg, pot);
  sctl::Vector<Real> Xt;
  for (long i = 0; i < trg.NElem(); i++)
    for (long j = 0; j < ElemBasis::Size(); j++)
      for (int k = 0; k < 3; k++) Xt.PushBack(trg(i, k)[j]);
  LegacyKernel<sctl::Laplace3D_FxU> kf;
  LegacyKernel<sctl::Laplace3D_DxU> kd;
  Quad qf, qd;
  qf.Setup<ElemBasis>(src, Xt, kf, order_singular, order_direct, -1.0, comm);
  qd.Setup<ElemBasis>(src, Xt, kd, order_singular, order_direct, -1.0, comm);
  sctl::Vector<Real> U_sl, U_dl;
  qf.Eval(U_sl, src, dens_sl, kf);
  qd.Eval(U_dl, src, dens_dl, kd);
  // Today's Laplace3D_DxU takes r = x_t - y_s (test-kernel_functions.cpp:52-68), the opposite sign
  // of the double layer the legacy test was written for (it adds U_dl), so Green's representation
  // of the harmonic u inside the torus reads SL[du/dn] - DL[u] = u.
  double err = 0;
  for (long i = 0; i < trg.NElem(); i++)
    for (long j = 0; j < ElemBasis::Size(); j++) {
      const long t = i * ElemBasis::Size() + j;
      err = std::max(err, (double)sctl::fabs<Real>(U_off[i][j] - (U_sl[t] - U_dl[t])));
    }
  return err;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 3 && argc != 4) {
    std::fprintf(stderr, "usage: %s in.bin out.bin [green]\n", argv[0]);
    return 2;
  }
  FILE* fi = std::fopen(argv[1], "rb");
  if (!fi) return 3;
  int64_t Nt = 0, Np = 0, os = 0, od = 0, Ntrg = 0;
  double Rmaj = 0, Rmin = 0;
  bool ok = read_vals(fi, &Nt, 1) && read_vals(fi, &Np, 1) && read_vals(fi, &Rmaj, 1) && read_vals(fi, &Rmin, 1) &&
            read_vals(fi, &os, 1) && read_vals(fi, &od, 1);
  std::vector<double> dens(ok ? Nt * Np * ORDER * ORDER : 0);
  ok = ok && read_vals(fi, dens.data(), dens.size()) && read_vals(fi, &Ntrg, 1);
  std::vector<double> xt(ok ? Ntrg * 3 : 0);
  ok = ok && read_vals(fi, xt.data(), xt.size());
  std::fclose(fi);
  if (!ok) return 4;

  const sctl::Comm comm = sctl::Comm::Self();
  ElemListT elements;
  build_torus(elements, Nt, Np, Rmaj, Rmin);
  sctl::Vector<ElemBasis> density(Nt * Np);
  for (long e = 0; e < Nt * Np; e++)
    for (int k = 0; k < ORDER * ORDER; k++) {
      const int a = k % ORDER, b = k / ORDER;  // theta index, phi index
      density[e][k] = dens[e * ORDER * ORDER + a * ORDER + b];
    }
  sctl::Vector<Real> Xt(Ntrg * 3);
  for (long i = 0; i < Ntrg * 3; i++) Xt[i] = xt[i];

  LegacyKernel<sctl::Laplace3D_DxU> kd;
  sctl::Quadrature<Real> q;
  q.Setup<ElemBasis>(elements, Xt, kd, (sctl::Integer)os, (sctl::Integer)od, -1.0, comm);
  sctl::Vector<Real> U;
  q.Eval(U, elements, density, kd);

  const double gerr = argc > 3 ? greens_identity_error(Nt, Np, Rmaj, Rmin, (int)os, (int)od) : -1.0;
  FILE* fo = std::fopen(argv[2], "wb");
  if (!fo) return 5;
  for (long i = 0; i < Ntrg; i++) {
    const double u = U[i];
    std::fwrite(&u, sizeof(double), 1, fo);
  }
  std::fwrite(&gerr, sizeof(double), 1, fo);
  std::fclose(fo);
  std::printf("legacy quadrature: %ld targets, Green's identity error %.3e\n", (long)Ntrg, gerr);
  return 0;
}
