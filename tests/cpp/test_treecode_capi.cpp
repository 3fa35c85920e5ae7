// The treecode's C ABI bound the way a ParticleFMM integration would (host
// coordinates at setup, device or host densities and potentials per
// evaluation), checked against the direct sum of the same library
// (sctlgpu_eval, host arrays): relative l2 within 10^-digits for digits 6 and
// 10, Laplace and Stokes double layers, the accumulate flag, host-array
// execution; and the shim's GpuFarField (ParticleFMM's setters, Eval and
// EvalDirect) on both sides of the 40,000-target cut-over.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "sctlgpu.hpp"

static int failures = 0;
#define CHECK(c, ...)                  \
  do {                                 \
    if (!(c)) {                        \
      std::printf("FAIL: " __VA_ARGS__); \
      std::printf("\n");               \
      ++failures;                      \
    }                                  \
  } while (0)

static double rel_l2(const std::vector<double>& a, const std::vector<double>& b) {
  double n = 0, d = 0;
  for (size_t i = 0; i < a.size(); ++i) {
    n += (a[i] - b[i]) * (a[i] - b[i]);
    d += b[i] * b[i];
  }
  return std::sqrt(n / d);
}

int main() {
  std::mt19937_64 rng(11);
  std::normal_distribution<double> nrm;
  std::uniform_real_distribution<double> uni(0, 1);
  const long ns = 1 << 17, nt = 1 << 15;
  std::vector<double> xs(ns * 3), xn(ns * 3), xt(nt * 3);
  for (long i = 0; i < ns; ++i) {  // unit sphere, outward normals
    double v[3] = {nrm(rng), nrm(rng), nrm(rng)};
    const double r = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int d = 0; d < 3; ++d) xs[i * 3 + d] = xn[i * 3 + d] = v[d] / r;
  }
  for (long i = 0; i < nt; ++i) {  // ball of radius 2
    double v[3] = {nrm(rng), nrm(rng), nrm(rng)};
    const double r = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]), rad = 2.0 * std::cbrt(uni(rng));
    for (int d = 0; d < 3; ++d) xt[i * 3 + d] = v[d] / r * rad;
  }
  const int kernels[2] = {SCTLGPU_LAPLACE3D_DXU, SCTLGPU_STOKES3D_DXU};
  for (int kid : kernels) {
    int nd, sd, td;
    sctlgpu_kernel_dims(kid, nullptr, &nd, &sd, &td);
    std::vector<double> f(ns * sd);
    for (auto& v : f) v = nrm(rng);
    for (int digits : {6, 10}) {
      std::vector<double> ref;  // the direct sum (resized and zeroed by the call)
      ref.assign(nt * td, 0.0);
      int rc = sctlgpu_eval(kid, SCTLGPU_MIXED, digits, nt, xt.data(), ns, xs.data(), xn.data(), f.data(),
                            ref.data(), 0, nullptr);
      CHECK(rc == SCTLGPU_OK, "direct sum rc %d", rc);
      sctlgpu_treecode tc = nullptr;
      rc = sctlgpu_treecode_create(&tc, kid, SCTLGPU_MIXED, digits, ns, xs.data(), xn.data(), nt, xt.data(), nullptr);
      CHECK(rc == SCTLGPU_OK && tc, "create rc %d", rc);
      if (!tc) continue;
      int64_t sizes[10];
      double theta = 0;
      sctlgpu_treecode_info(tc, sizes, &theta);
      CHECK(sizes[5] > 0, "kernel %d digits %d: no proxy interactions", kid, digits);
      double *d_f = nullptr, *d_u = nullptr;
      cudaMalloc(&d_f, f.size() * sizeof(double));
      cudaMalloc(&d_u, nt * td * sizeof(double));
      cudaMemcpy(d_f, f.data(), f.size() * sizeof(double), cudaMemcpyHostToDevice);
      rc = sctlgpu_treecode_execute(tc, d_f, d_u, SCTLGPU_DEVICE_PTRS, nullptr);
      CHECK(rc == SCTLGPU_OK, "execute rc %d", rc);
      std::vector<double> u(nt * td);
      cudaMemcpy(u.data(), d_u, u.size() * sizeof(double), cudaMemcpyDeviceToHost);
      const double err = rel_l2(u, ref);
      std::printf("kernel %d digits %d: order %lld theta %.2f, %lld + %lld of %lld interactions, rel l2 %.2e\n", kid,
                  digits, (long long)sizes[6], theta, (long long)sizes[4], (long long)sizes[5],
                  (long long)ns * nt, err);
      CHECK(err < std::pow(10.0, -digits), "kernel %d digits %d: rel l2 %.3e", kid, digits, err);
      // accumulate: a second execution adds the same potentials
      rc = sctlgpu_treecode_execute(tc, d_f, d_u, SCTLGPU_ACCUMULATE | SCTLGPU_DEVICE_PTRS, nullptr);
      std::vector<double> u2(nt * td);
      cudaMemcpy(u2.data(), d_u, u2.size() * sizeof(double), cudaMemcpyDeviceToHost);
      // host arrays: the same potentials, synchronously
      std::vector<double> uh(nt * td, 0.0);
      CHECK(sctlgpu_treecode_execute(tc, f.data(), uh.data(), 0, nullptr) == SCTLGPU_OK, "host execute");
      CHECK(rel_l2(uh, u) < 1e-14, "host-array execution equals the device one");
      for (auto& v : u) v *= 2;
      CHECK(rc == SCTLGPU_OK && rel_l2(u2, u) < 1e-13, "accumulate");
      CHECK(sctlgpu_treecode_status(tc, nullptr) == SCTLGPU_OK, "status");
      sctlgpu_treecode_destroy(tc);
      cudaFree(d_f);
      cudaFree(d_u);
    }
  }
  // ParticleFMM's calls on the shim's GpuFarField: Eval = treecode for >= 40,000 targets
  {
    struct Vec {  // the members of sctl::Vector the shim uses
      std::vector<double> v;
      long Dim() const { return (long)v.size(); }
      double& operator[](long i) { return v[i]; }
      const double& operator[](long i) const { return v[i]; }
      void ReInit(long n) { v.assign(n, 0.0); }
      void SetZero() { std::fill(v.begin(), v.end(), 0.0); }
    };
    const long nt2 = 1 << 16;  // above the cut-over
    std::vector<double> xt2(nt2 * 3);
    for (long i = 0; i < nt2; ++i) {
      double v[3] = {nrm(rng), nrm(rng), nrm(rng)};
      const double r = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]), rad = 2.0 * std::cbrt(uni(rng));
      for (int d = 0; d < 3; ++d) xt2[i * 3 + d] = v[d] / r * rad;
    }
    Vec Xs{xs}, Xn{xn}, Xt{xt2}, F{std::vector<double>(ns)}, U, Ud;
    for (auto& x : F.v) x = nrm(rng);
    sctlgpu::set_double_mode(SCTLGPU_MIXED);
    sctlgpu::GpuFarField<SCTLGPU_LAPLACE3D_DXU> fmm;
    fmm.SetAccuracy(6);  // the treecode saves most at low digits: this geometry keeps the treecode path
    fmm.SetSrcCoord(Xs, Xn);
    fmm.SetSrcDensity(F);
    fmm.SetTrgCoord(Xt);
    fmm.Eval(U);
    fmm.EvalDirect(Ud);
    const double err = rel_l2(U.v, Ud.v);
    std::printf("GpuFarField Laplace3D_DxU, %ld targets: Eval vs EvalDirect rel l2 %.2e\n", nt2, err);
    CHECK(U.Dim() == nt2 && err < 1e-6 && err > 0, "GpuFarField treecode %.3e", err);
    Vec Xt_small{std::vector<double>(xt.begin(), xt.begin() + 3 * 1000)};
    fmm.SetTrgCoord(Xt_small);
    fmm.Eval(U);
    fmm.EvalDirect(Ud);
    CHECK(U.Dim() == 1000 && U.v == Ud.v, "GpuFarField below 40,000 targets is EvalDirect");
    sctlgpu::set_double_mode(SCTLGPU_F64);
  }
  // argument errors are status codes, before any device work
  sctlgpu_treecode tc = nullptr;
  CHECK(sctlgpu_treecode_create(&tc, SCTLGPU_LAPLACE3D_DXU, SCTLGPU_F32, 10, ns, xs.data(), xn.data(), nt, xt.data(),
                                nullptr) == SCTLGPU_ERR_INVALID_MODE,
        "FP32 mode refused");
  CHECK(sctlgpu_treecode_create(&tc, SCTLGPU_LAPLACE3D_DXU, SCTLGPU_MIXED, 10, ns, xs.data(), nullptr, nt, xt.data(),
                                nullptr) == SCTLGPU_ERR_NULL_POINTER,
        "double layer without normals refused");
  std::printf("%s (%d check(s) failed)\n", failures ? "FAIL" : "PASS", failures);
  return failures ? 1 : 0;
}
