// 24-DOF stepper: derived constants, right-hand side, half-implicit update and window kernel.
//
// Algorithm: rhsFun (24dof-gpu/dof24_halfImplicit_gpu.cu:728-775) and the Integrate update
// (:1016-1081) with the physics of 24dof-gpu/dof24_gpu.cu: strut and unsprung-mass velocities from
// the chassis (vehToSusTransform), contact-patch velocities through pitch and roll
// (vehToTireTransform), TMeasy tires loaded by the integrated tire compression, tire compression
// rate, the 18-DOF powertrain, tire forces into the chassis frame (tireToVehTransform), unsprung
// vertical dynamics and spring rate (computeSusRHS), strut forces, jacking forces and moments
// (computeForcesThroughSus), and the 6-DOF chassis (computeVehicleRHS). The tire curve evaluation,
// tmxy_combined, powertrain, driveTorque and lookups are the 18-DOF device functions
// (dof18_device.cuh). As there, the arithmetic is rearranged only at the rounding level: parameter
// reciprocals once per vehicle, cos/sin of pitch and roll once per step, the loaded-radius and
// Cardan-rate divisions as one reciprocal each.
//
// Carried across steps in registers: the 11 chassis coordinates and rates, the previous step's
// accelerations (read by the next vehToSusTransform), crank speed and gear; per tire xe, ye, their
// rates (stale while the wheel is off the ground, as in the reference), omega, compression xt and
// loaded radius rStat (read by the next vehToTireTransform before it is recomputed); per corner the
// spring compression xs, its rate dxs and the jacking force fzd (both read by the next
// computeSusRHS before they are recomputed) and the unsprung vertical speed wu. Fields that the
// reference computes but never reads back in a later step are written to HBM from the last step of
// a window only (step24 with sink set), so that GetSimState returns the reference's full SimState.
#include <cuda_runtime.h>

#include "window24_kernel.cuh"

namespace lfdm {

int k24_count() { return K24_COUNT; }

__global__ void prepare24_kernel(const double* __restrict__ P, int n, int npad, double* __restrict__ K) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* p = P + (size_t)i * LFDM_P_COUNT;
    auto put = [&](int k, double v) { K[(size_t)k * npad + i] = v; };
    prepare_k24(p, put);
}

cudaError_t launch_prepare24(const double* params_dev, int n, int npad, double* K_dev, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    prepare24_kernel<<<(n + 127) / 128, 128, 0, stream>>>(params_dev, n, npad, K_dev);
    return cudaGetLastError();
}


size_t window24_smem(int threads, int nclasses, bool f32) {
    const size_t cls = nclasses <= kMaxSmemClasses ? (size_t)nclasses * sizeof(ClassDev18) : 0;
    return cls + (size_t)K24_COUNT * threads * (sizeof(double) + (f32 ? sizeof(float) : 0));
}

cudaError_t launch_window24(const Window18& w, cudaStream_t stream) {
    if (w.n <= 0 || w.nsteps <= 0) return cudaSuccess;
    if (w.threads <= 0 || w.threads > 128 || (w.threads & 31)) return cudaErrorInvalidValue;
    if (w.precision == LFDM_PREC_MIXED_TIRE)
        return w.tire_nr ? launch_window24_nr_f32(w, stream) : launch_window24_f32(w, stream);
    if (w.precision != LFDM_PREC_FP64) return cudaErrorInvalidValue;
    return w.tire_nr ? launch_window24_nr(w, stream) : launch24_tire<false>(w, stream);
}

}  // namespace lfdm
