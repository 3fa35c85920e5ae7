// Kernel ids 4-15 in FP32 (Newton steps 0..1 after the hardware estimate).
#include "ext.cuh"

namespace sctlgpu {
cudaError_t eval_ext_f32(const EvalCall& c, int newton) { return XDispatch<float, 1>::eval_k<4>(c, newton); }
cudaError_t kmat_ext_f32(const KmatCall& c, int newton) { return XDispatch<float, 1>::kmat_k<4>(c, newton); }
}  // namespace sctlgpu
