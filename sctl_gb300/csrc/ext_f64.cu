// Kernel ids 4-15 in FP64 (Newton steps 0..2 after the hardware estimate).
#include "ext.cuh"

namespace sctlgpu {
cudaError_t eval_ext_f64(const EvalCall& c, int newton) { return XDispatch<double, 2>::eval_k<4>(c, newton); }
cudaError_t kmat_ext_f64(const KmatCall& c, int newton) { return XDispatch<double, 2>::kmat_k<4>(c, newton); }
}  // namespace sctlgpu
