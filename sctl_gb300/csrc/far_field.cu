// ComputeFarField's density weighting (boundary_integral.txx:1266-1285):
// F_far[i*dof + k] = F[i*dof + k] * wts_far[i], on the device, so a far-field
// evaluation (weighting + sctlgpu_eval) launches only this library's kernels.
#include "../../include/sctlgpu.h"
#include "launch.h"

namespace sctlgpu {
namespace {

__global__ void far_densities_kernel(int64_t n, int dof, const double* __restrict__ f, const double* __restrict__ w,
                                     double* __restrict__ out) {
  const int64_t total = n * dof;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = f[i] * w[i / dof];
}

}  // namespace
}  // namespace sctlgpu

using namespace sctlgpu;

extern "C" int sctlgpu_far_densities(int64_t n, int dof, const double* f, const double* w, double* f_far,
                                     void* stream) {
  if (n < 0 || dof < 1 || dof > 64 || n > ((int64_t)1 << 40)) return SCTLGPU_ERR_INVALID_SIZE;
  if (n == 0) return SCTLGPU_OK;
  if (!f || !w || !f_far) return SCTLGPU_ERR_NULL_POINTER;
  int dev = 0, sms = 0;
  unsigned* status = nullptr;
  const int rc = runtime_device(&dev, &status, &sms);
  if (rc != SCTLGPU_OK) return rc;
  const int64_t total = n * dof;
  const int64_t blocks = (total + 255) / 256;
  const unsigned grid = (unsigned)(blocks < (int64_t)sms * 8 ? blocks : (int64_t)sms * 8);
  far_densities_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(n, dof, f, w, f_far);
  g_launches.fetch_add(1, std::memory_order_relaxed);
  return runtime_record(cudaGetLastError());
}
