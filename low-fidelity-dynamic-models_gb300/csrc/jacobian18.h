// Batched exact Jacobians of the 18-, 11- and 24-DOF right-hand sides (jacobian18.cu, jacobian11.cu,
// jacobian24.cu).
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace lfdm {

struct ClassDev18;

struct JacLaunch {
    int n = 0, npad = 0;
    const double* K = nullptr;             // [K18 count][npad]
    const ClassDev18* classes = nullptr;
    int nclasses = 0;
    bool cls_smem = false;                 // set by the launcher
    const int32_t* class_of = nullptr;     // [n]
    const double* S = nullptr;             // [LFDM_S_COUNT][npad] states (SoA)
    const double* ctl = nullptr;           // [3][n] steering, throttle, braking
    int reference_point = 1;               // 1: PerturbRhsFun's fresh state; 0: the full current state
    int tire_nr = 0;                       // 1: TMeasyNr tires
    double* tape = nullptr;                // [tape doubles][npad] scratch
    double* jac_state = nullptr;           // [ny][ny][n]
    double* jac_ctl = nullptr;             // [ny][2][n]
};

cudaError_t launch_rhs_jacobian18(const JacLaunch& A, cudaStream_t stream);
// The same for the 11-DOF model (jacobian11.cu); S holds [LFDM11_S_COUNT][npad] states.
cudaError_t launch_rhs_jacobian11(const JacLaunch& A, cudaStream_t stream);
// The same for the 24-DOF model with TMeasy tires (jacobian24.cu); S holds [LFDM24_S_COUNT][npad]
// states and the tape needs jac24_tape_doubles() doubles per vehicle.
cudaError_t launch_rhs_jacobian24(const JacLaunch& A, cudaStream_t stream);
size_t jac24_tape_doubles();
// Dynamic shared memory of a Jacobian block (derived constants, their adjoint scratch and, when
// they fit, the class tables; *cls_smem says whether they do).
size_t jac18_smem(int threads, int nclasses, bool* cls_smem);

}  // namespace lfdm
