// Batched near-field variants in mixed precision (FP32 arithmetic, and
// double-float arithmetic on the packed FP32 pipe with pair records).
#include "near_launch.cuh"

namespace sctlgpu {

NearOps near_ops_mixed(int kernel, int imode, int newton) {
  if (imode == NEAR_MXDF) return near_ops_pk(kernel);  // double-float on the packed FP32 pipe
  return newton <= 0 ? near_ops_for<MODE_MXLO, 0>(kernel) : near_ops_for<MODE_MXLO, 1>(kernel);
}

}  // namespace sctlgpu
