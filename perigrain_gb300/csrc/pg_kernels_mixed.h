// Host-side entry points of the mixed-precision kernels (pg_kernels_mixed.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "pg_device.cuh"
#include "pg_kernels.h"

namespace pg {

cudaError_t kernels_mixed_init();
// Enqueue one mixed-precision time step; e0/e1 (may be null) bracket the force kernel. With rec
// the force kernel also records the step's contact and wall masks (Dev::rec_*).
void launch_step_mixed(const Dev& P, const LaunchCfg& L, cudaStream_t s, uint64_t* launches,
                       cudaEvent_t e0 = nullptr, cudaEvent_t e1 = nullptr, bool rec = false);
// The same step in three parts (position update; grid build and force kernel; finalize), for
// graphs that run one step's finalize beside the next step's position update.
void launch_mixed_predict(const Dev& P, cudaStream_t s, bool pdl, uint64_t* launches);
void launch_mixed_body(const Dev& P, const LaunchCfg& L, cudaStream_t s, bool pdl, uint64_t* launches,
                       bool rec = false);
void launch_mixed_finalize(const Dev& P, cudaStream_t s, bool pdl, uint64_t* launches);

}  // namespace pg
