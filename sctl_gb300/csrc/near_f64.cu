// Batched near-field variants in FP64 and FP32.
#include "near_launch.cuh"

namespace sctlgpu {

NearOps near_ops_f64(int kernel, int newton) {
  switch (newton) {
    case 0: return near_ops_for<MODE_F64, 0>(kernel);
    case 1: return near_ops_for<MODE_F64, 1>(kernel);
    default: return near_ops_for<MODE_F64, 2>(kernel);
  }
}

NearOps near_ops_f32(int kernel, int newton) {
  return newton <= 0 ? near_ops_for<MODE_F32, 0>(kernel) : near_ops_for<MODE_F32, 1>(kernel);
}

}  // namespace sctlgpu
