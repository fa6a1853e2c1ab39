// Device helpers shared by the frozen-mask replay forward (pg_adjoint.cu) and the reverse step
// (pg_adjoint_rev.cu).
#pragma once
#include <cuda_runtime.h>

#include <cmath>

#include "pg_common.cuh"
#include "pg_device.cuh"

namespace pg {

// A bond is used at step t iff alive at the end of the run or broken at step t or later (the
// force of the step that breaks a bond still includes it, particle2.h:191-232 runs after it).
__device__ __forceinline__ bool bond_used(const uint32_t* end_alive, const uint32_t* break_step, uint32_t word,
                                          uint32_t lane, uint32_t slot, uint32_t t) {
  return ((end_alive[word] >> lane) & 1u) || t <= break_step[slot];
}

// Contact parameters of node p (grain gr) against partner q (grain gq), as the force kernels use
// them: the mean of the two grains' values; self-contact uses R_c' = min(|pos_p - pos_q|, R_c)
// and K_n' = cnot / R_c' (contact.h:709-730).
template <int D>
__device__ __forceinline__ void pair_params(const Dev& P, const InstDev& in, const GrainDev& gr, const GrainDev& gq,
                                            bool same, uint32_t p, uint32_t q, double* Kn, double* Rc, double* zeta,
                                            double* mu) {
  *Rc = in.contact_rad;
  *Kn = (gr.kn + gq.kn) * 0.5;
  *zeta = (gr.zeta + gq.zeta) * 0.5;
  *mu = (gr.mu + gq.mu) * 0.5;
  if (same) {
    double pp[D], pq[D], r[D];
    ldv<D>(P.pos, p, pp);
    ldv<D>(P.pos, q, pq);
    for (int c = 0; c < D; ++c) r[c] = pp[c] - pq[c];
    double r2 = r[0] * r[0];
    for (int c = 1; c < D; ++c) r2 = r2 + r[c] * r[c];
    const double ref = sqrt(r2);
    if (ref < in.contact_rad) {
      *Rc = ref;
      *Kn = gr.cnot / ref;
    } else {
      *Rc = in.contact_rad;
      *Kn = gr.cnot / in.contact_rad;
    }
  }
}

// (side, direction) of the k-th wall side in the reference's call order (timeloop.h:753-769)
template <int D>
__device__ __forceinline__ void wall_side(int k, int* side, int* dir) {
  if constexpr (D == 2) {
    const int s2[4] = {3, 0, 1, 2}, d2[4] = {1, 0, 0, 1};
    *side = s2[k];
    *dir = d2[k];
  } else {
    const int s3[6] = {0, 3, 1, 4, 2, 5}, d3[6] = {0, 0, 1, 1, 2, 2};
    *side = s3[k];
    *dir = d3[k];
  }
}

// Wall bits of side k (call order) in a recorded mask word.
__device__ __forceinline__ bool wb_contact(uint32_t w, int k) { return (w >> (4 * k)) & 1u; }
__device__ __forceinline__ bool wb_fric(uint32_t w, int k) { return (w >> (4 * k + 1)) & 1u; }
__device__ __forceinline__ bool wb_stick(uint32_t w, int k) { return (w >> (4 * k + 2)) & 1u; }
__device__ __forceinline__ bool wb_neg(uint32_t w, int k) { return (w >> (4 * k + 3)) & 1u; }

}  // namespace pg
