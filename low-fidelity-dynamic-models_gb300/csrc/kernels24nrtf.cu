// The 24-DOF window kernel with TMeasyNr tires whose tire core runs in FP32 (precision
// LFDM_PREC_MIXED_TIRE; tire_core_nr_f32 in dof18_device.cuh), in its own translation unit so that
// it compiles in parallel with the other 24-DOF instantiations.
#include "window24_kernel.cuh"

namespace lfdm {

cudaError_t launch_window24_nr_f32(const Window18& w, cudaStream_t stream) { return launch24_tire<true, true>(w, stream); }

}  // namespace lfdm
