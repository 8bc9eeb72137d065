// Discrete adjoint step (lbm_adjoint.cu).
#pragma once

#include <cuda_runtime.h>

#include "lbm_device.cuh"

namespace stro {

struct AdjArgs {
    StepArgs a;         // forward arguments of the step; a.f = the stored input state of the step
    float* lam;         // adjoint of the state, 19 planes, plane stride a.plane (FP32)
    double* grad_eps;   // dJ/d eps (N), or null: summed in FP64 (see add_grads)
    float* grad_f;      // dJ/d F_field (3 planes of a.ffield_plane), or null
    float obj_w;        // weight of this step's force in J (odd steps), 0 = none
    float dir[3];       // force direction of the objective
    int box[4];         // x0, x1, y0, y1 (inclusive) of the force box
    int force_terms;    // differentiate the Guo source terms
};

cudaError_t launch_adjoint_step(const AdjArgs& g, int half_storage, int parity, int geo, dim3 block,
                                cudaStream_t st);
// The reverse step split like the forward one over block lists of the
// (block.x, block.y) grid: `bulk` blocks wall-free, `edge` blocks wall-aware.
// At most 128 threads per block.
cudaError_t launch_adjoint_split(const AdjArgs& g, int half_storage, int parity, dim3 block,
                                 const uint32_t* bulk, uint32_t nbulk, const uint32_t* edge,
                                 uint32_t nedge, cudaStream_t st);

// Dissipation objective: lam += w dD/df and grad_f += w dD/dF_field for the
// dissipation sum D (2 nu S:S over fluid cells, as launch_observables) of the
// state g.a.f at an even step count (natural slots). g.lam, g.grad_f and the
// force and cell fields of g.a are used; nu = (1/omega - 1/2) / 3.
cudaError_t launch_adjoint_dissipation(const AdjArgs& g, int half_storage, float nu, float w,
                                       cudaStream_t st);

}  // namespace stro
