// FP32 direct sums (SCTLGPU_F32): Newton steps 0..2 after the rsqrt.approx.f32 seed.
#include "launch_direct.cuh"

namespace sctlgpu {

template <int KER>
static cudaError_t eval_f32_k(const EvalCall& c, int newton) {
  switch (newton) {
    case 0: return run_direct<KER, MODE_F32, 0>(c);
    case 1: return run_direct<KER, MODE_F32, 1>(c);
    default: return run_direct<KER, MODE_F32, 2>(c);
  }
}

cudaError_t eval_f32(const EvalCall& c, int newton) {
  switch (c.kernel) {
    case KER_LFXU: return eval_f32_k<KER_LFXU>(c, newton);
    case KER_LDXU: return eval_f32_k<KER_LDXU>(c, newton);
    case KER_SFXU: return eval_f32_k<KER_SFXU>(c, newton);
    default: return eval_f32_k<KER_SDXU>(c, newton);
  }
}

}  // namespace sctlgpu
