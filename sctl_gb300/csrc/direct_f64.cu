// FP64 direct sums (SCTLGPU_F64): Newton steps 0..3 after the rsqrt.approx.f64 seed.
#include "launch_direct.cuh"

namespace sctlgpu {

template <int KER>
static cudaError_t eval_f64_k(const EvalCall& c, int newton) {
  switch (newton) {
    case 0: return run_direct<KER, MODE_F64, 0>(c);
    case 1: return run_direct<KER, MODE_F64, 1>(c);
    case 2: return run_direct<KER, MODE_F64, 2>(c);
    default: return run_direct<KER, MODE_F64, 3>(c);
  }
}

cudaError_t eval_f64(const EvalCall& c, int newton) {
  switch (c.kernel) {
    case KER_LFXU: return eval_f64_k<KER_LFXU>(c, newton);
    case KER_LDXU: return eval_f64_k<KER_LDXU>(c, newton);
    case KER_SFXU: return eval_f64_k<KER_SFXU>(c, newton);
    default: return eval_f64_k<KER_SDXU>(c, newton);
  }
}

}  // namespace sctlgpu
