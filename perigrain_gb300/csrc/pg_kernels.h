// Host-side entry points of the device kernels (pg_kernels.cu, pg_kernels_mixed.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "pg_device.cuh"

namespace pg {

struct LaunchCfg {
  uint32_t force_block = 128;   // threads per block of the fused force kernel (multiple of 32, <= 128)
  uint32_t cells_per_node = 4;  // grid capacity per node of an instance
};

// Per-thread local memory of this process's context at least `bytes` (cudaLimitStackSize), so
// kernels with local frames above the default limit find room for them.
inline cudaError_t ensure_local_bytes(size_t bytes) {
  size_t cur = 0;
  cudaError_t e = cudaDeviceGetLimit(&cur, cudaLimitStackSize);
  if (e != cudaSuccess || cur >= bytes) return e;
  return cudaDeviceSetLimit(cudaLimitStackSize, (bytes + 255) / 256 * 256);
}
// The largest local frame (cudaFuncAttributes::localSizeBytes) among the kernels `fs`.
inline cudaError_t max_local_bytes(const void* const* fs, int n, size_t* out) {
  size_t m = 0;
  for (int k = 0; k < n; ++k) {
    cudaFuncAttributes a;
    const cudaError_t e = cudaFuncGetAttributes(&a, fs[k]);
    if (e != cudaSuccess) return e;
    m = a.localSizeBytes > m ? a.localSizeBytes : m;
  }
  *out = m;
  return cudaSuccess;
}

cudaError_t kernels_init();
// Enqueue one FP64 time step on stream s. Adds the number of kernel launches to *launches. With
// rec the force kernel also records the step's contact and wall masks (Dev::rec_*).
void launch_step(const Dev& P, const LaunchCfg& L, cudaStream_t s, uint64_t* launches, bool rec = false);
// Same as launch_step, with CUDA events e0/e1 recorded around the fused force kernel.
void launch_step_timed(const Dev& P, const LaunchCfg& L, cudaStream_t s, uint64_t* launches,
                       cudaEvent_t e0, cudaEvent_t e1);
const void* force_kernel_ptr(uint32_t dim);
// Blocks of the cooperative grid build (k_grid_coop): every block resident at once (occupancy x
// SMs), no more than the work needs; 0 when the device has no cooperative launch.
uint32_t grid_coop_blocks(const Dev& P, int device);
// out[i] = op(a[i], b[i]) through the integer FP64 routines (pg_ieee64.cuh), op a pg_ieee_op;
// device pointers, n < 2^31 * 256.
cudaError_t launch_ieee64_check(int32_t op, const double* a, const double* b, int64_t n, double* out,
                                cudaStream_t s);

}  // namespace pg
