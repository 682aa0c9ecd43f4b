// Device-side description of a differentiable 18-DOF rollout (adjoint18.cu) and its launchers.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

#include "../../include/lfdm.h"

namespace lfdm {

struct ClassDev18;

// Caller arrays (controls, reference path, loss and gradients) are [..][n] with row stride n; the
// library's own buffers (states, constants, checkpoints, tape, constant adjoints) use npad.
struct AdjLaunch {
    int n = 0, npad = 0, nsteps = 0, ckpt = 100;
    double dt = 1e-3, weight_u = 1e-3;
    const double* K = nullptr;             // [K18 count][npad]
    const ClassDev18* classes = nullptr;
    int nclasses = 0;
    bool cls_smem = false;                 // classes staged in shared memory (set by the launcher)
    const int32_t* class_of = nullptr;     // [n]
    const double* params = nullptr;        // [n][LFDM_P_COUNT] (device)
    const double* S0 = nullptr;            // [LFDM_S_COUNT][npad] initial states (SoA)
    const double* ctl = nullptr;           // [nsteps][3][n] steering, throttle, braking
    const double* ref = nullptr;           // [nsteps][3][n] x, y, yaw of the reference path
    double* loss = nullptr;                // [n]
    double* ckpts = nullptr;               // [nsteps / ckpt][checkpoint fields][npad]
    double* tape = nullptr;                // [ckpt][tape doubles][npad]
    double* grad_ctl = nullptr;            // [nsteps][3][n]
    double* grad_params = nullptr;         // [5][n]: mass, Jz, a, friction scale, kt
    double* grad_state0 = nullptr;         // [31][n] or nullptr
};

cudaError_t launch_traj18_forward(const AdjLaunch& A, cudaStream_t stream);
cudaError_t launch_traj18_backward(const AdjLaunch& A, cudaStream_t stream);
// Branch signature of the rollout per vehicle (sig [n], device); A.tape holds one step's tape.
cudaError_t launch_traj18_signature(const AdjLaunch& A, uint64_t* sig, cudaStream_t stream);
size_t traj18_tape_doubles_per_step();
size_t traj18_smem(int threads, int nclasses, bool backward, bool* cls_smem);
int traj18_ckpt_fields();
int traj18_state_adjoints();

}  // namespace lfdm
