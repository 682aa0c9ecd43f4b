// The 24-DOF window kernel with TMeasyNr tires (24dof-gpu/dof24_gpu.cu:990-1119 for the tire; the
// rest of the step as for TMeasy tires), in its own translation unit so that it compiles in
// parallel with kernels24.cu.
#include "window24_kernel.cuh"

namespace lfdm {

cudaError_t launch_window24_nr(const Window18& w, cudaStream_t stream) { return launch24_tire<true>(w, stream); }

}  // namespace lfdm
