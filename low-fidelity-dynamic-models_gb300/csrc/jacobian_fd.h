// Batched right-hand-side Jacobians of the 11-, 18- and 24-DOF models by the reference's own
// central-difference scheme (jacobian_fd.cu).
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace lfdm {

struct ClassDev18;

struct JacFdLaunch {
    int model = 18;                        // 11, 18 or 24
    int tire_nr = 0;                       // 1: TMeasyNr tires (no deflection states)
    int n = 0, npad = 0;
    const double* K = nullptr;             // [K count of the model][npad]
    const ClassDev18* classes = nullptr;
    int nclasses = 0;
    bool cls_smem = false;                 // set by the launcher
    const int32_t* class_of = nullptr;     // [n]
    const double* S = nullptr;             // [state count of the model][npad] states (SoA)
    const double* ctl = nullptr;           // [3][n] steering, throttle, braking
    int reference_point = 1;               // 1: PerturbRhsFun's fresh state; 0: the full current state
    double* jac_state = nullptr;           // [ny][ny][n]
    double* jac_ctl = nullptr;             // [ny][2][n]
};

// Packed state count of a model and tire type (the reference's m_num_states).
int jac_fd_ny(int model, bool tire_nr, bool tcbool);

cudaError_t launch_rhs_jacobian_fd(const JacFdLaunch& A, cudaStream_t stream);

}  // namespace lfdm
