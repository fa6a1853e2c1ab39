// Host-side entry points of the gradient kernels (pg_adjoint.cu).
//
// The differentiated map is one PeriDEM time step (reference src/particle/timeloop.h:608-879)
// with its bond-break, contact and friction-branch decisions frozen ("masks"): bond forces
// (particle2.h:102-150), node-node contact with damping and friction (contact.h:668-812), wall
// contact (contact.h:314-431, :16-41) and the velocity-Verlet update (timeloop.h:661-669,
// :834-863). Parameters are per grain: bond stiffness cnot and the contact stiffness, damping
// ratio and friction coefficient (a pair of grains uses the mean of the two grains' values).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "pg_device.cuh"

namespace pg {

constexpr int NPARAM = 4;  // per grain: cnot, normal stiffness, damping ratio, friction coefficient

// One reverse step: maps the cotangent of the state after forward step t to the cotangent of the
// state before it and adds the parameter cotangents of step t to pacc.
struct AdjStep {
  const double* X;         // [N][S] CurrPos of step t (what its forces saw)
  const double* V;         // [N][S] velocity its forces saw
  const double* W;         // [I][2D] wall positions its forces saw
  const uint32_t* tstep;   // step number t
  const uint32_t* off;     // masks of step t (see Dev::rec_*)
  const uint32_t* ent;
  const uint32_t* wall;
  const uint8_t* cnt;
  const uint32_t* end_alive;   // bond used at step t iff alive at the end of the run or t <= break step
  const uint32_t* break_step;
  const double *db, *vb, *ab;        // [N][S] cotangent of disp, vel, acc after step t
  double *db_o, *vb_o, *ab_o;        // [N][S] cotangent before step t
  double* pacc;                      // [N][NPARAM] parameter cotangents, accumulated per node
  const double* rbar;                // [I][2D][D] cotangent of step t's wall reactions, or null
  double* xbb;                       // [N][S] bond share of the position cotangent (scratch)
  double* pcb;                       // [N] bond share of the cnot cotangent (scratch)
  // FP32 bond path (mixed-precision handles; null = FP64 bond path): the step's displacement
  // hi/lo pairs and the FP32 force cotangents (read for step t, rewritten for step t-1)
  const float* df;
  float* fbf;
};

// One FP64 forward step under frozen masks (the map the adjoint differentiates).
struct ReplayStep {
  const uint32_t* off;
  const uint32_t* ent;
  const uint32_t* wall;
  const uint8_t* cnt;
  const uint32_t* end_alive;
  const uint32_t* break_step;
  double* wall_out;  // [N][2D][4] per-node wall terms (normal, tangent 1, tangent 2, damping) or null;
                     // when set, the step's wall reactions are summed into Dev::reaction
};

void launch_replay_step(const Dev& P, const ReplayStep& R, cudaStream_t s, uint64_t* launches);
void launch_adjoint_step(const Dev& P, const AdjStep& A, cudaStream_t s, uint64_t* launches);
// fbf from the seed cotangent (A.ab, A.vb) before the first reverse step of the FP32 bond path
void launch_fb_init(const Dev& P, const AdjStep& A, cudaStream_t s, uint64_t* launches);
// grad[g][k] = sum over the nodes of grain g of pacc[node][k]
void launch_grad_reduce(const Dev& P, const double* pacc, double* grad, cudaStream_t s, uint64_t* launches);

}  // namespace pg
