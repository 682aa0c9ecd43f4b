// The 24-DOF window kernel with TMeasy tires whose tire core runs in FP32 (precision
// LFDM_PREC_MIXED_TIRE; tire_core_tm_f32 in dof18_device.cuh), in its own translation unit so that
// it compiles in parallel with kernels24.cu and kernels24nr.cu.
#include "window24_kernel.cuh"

namespace lfdm {

cudaError_t launch_window24_f32(const Window18& w, cudaStream_t stream) { return launch24_tire<false, true>(w, stream); }

}  // namespace lfdm
