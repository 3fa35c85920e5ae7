// C-ABI dispatcher over the reference's own Eval of the four hot-path kernels
// (ref_hot.cpp, one object per kernel and real type) -- TEST AND BASELINE
// INFRASTRUCTURE ONLY, built into oracle/_ref/libsctlref_hot.so.  bench.py's
// CPU legs time it on the host cores; tests compare against it when present.
#include <cstdint>

#include <omp.h>

#define SCTLREF_DECL(K)                                                                                        \
  extern "C" int ref_hot_eval_##K##_double(int, int64_t, const double*, int64_t, const double*, const double*, \
                                            const double*, double*);                                          \
  extern "C" int ref_hot_eval_##K##_float(int, int64_t, const float*, int64_t, const float*, const float*,     \
                                           const float*, float*);
SCTLREF_DECL(Laplace3D_FxU)
SCTLREF_DECL(Laplace3D_DxU)
SCTLREF_DECL(Stokes3D_FxU)
SCTLREF_DECL(Stokes3D_DxU)

extern "C" {

// kernel: 0 Laplace3D_FxU, 1 Laplace3D_DxU, 2 Stokes3D_FxU, 3 Stokes3D_DxU.
// Adds into v_trg (Nt * TrgDim values), as the reference's Eval does.
int ref_hot_eval(int kernel, int is_double, int digits, int64_t nt, const void* r_trg, int64_t ns, const void* r_src,
                 const void* n_src, const void* v_src, void* v_trg) {
#define SCTLREF_CALL(K)                                                                                          \
  return is_double ? ref_hot_eval_##K##_double(digits, nt, (const double*)r_trg, ns, (const double*)r_src,       \
                                                (const double*)n_src, (const double*)v_src, (double*)v_trg)     \
                   : ref_hot_eval_##K##_float(digits, nt, (const float*)r_trg, ns, (const float*)r_src,         \
                                               (const float*)n_src, (const float*)v_src, (float*)v_trg)
  switch (kernel) {
    case 0: SCTLREF_CALL(Laplace3D_FxU);
    case 1: SCTLREF_CALL(Laplace3D_DxU);
    case 2: SCTLREF_CALL(Stokes3D_FxU);
    case 3: SCTLREF_CALL(Stokes3D_DxU);
    default: return -1;
  }
#undef SCTLREF_CALL
}

// OpenMP threads the reference's Eval<Real,true> uses in this process.
int ref_hot_threads(void) { return omp_get_max_threads(); }

}  // extern "C"
