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

#include "dof24_device.cuh"
#include "kernels.h"
#include "window_common.cuh"

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


size_t window24_smem(int threads, int nclasses) {
    const size_t cls = nclasses <= kMaxSmemClasses ? (size_t)nclasses * sizeof(ClassDev18) : 0;
    return cls + (size_t)K24_COUNT * threads * sizeof(double);
}

template <int kCtl, bool kOut>
__global__ void __launch_bounds__(128) window24_kernel(const Window18 w) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int tid = threadIdx.x;
    const bool cls_smem = w.nclasses <= kMaxSmemClasses;
    ClassDev18* cls = reinterpret_cast<ClassDev18*>(smem);
    double* ks = reinterpret_cast<double*>(smem + (cls_smem ? (size_t)w.nclasses * sizeof(ClassDev18) : 0));
    if (cls_smem) {
        const int4* src = reinterpret_cast<const int4*>(w.classes);
        int4* dst = reinterpret_cast<int4*>(smem);
        const int words = (int)(w.nclasses * sizeof(ClassDev18) / 16);
        for (int i = tid; i < words; i += blockDim.x) dst[i] = __ldg(src + i);
    }
    const int vid = blockIdx.x * blockDim.x + tid;
    const bool active = vid < w.n;
    if (active) {
#pragma unroll 4
        for (int k = 0; k < K24_COUNT; ++k) ks[k * blockDim.x + tid] = __ldg(w.K + (size_t)k * w.npad + vid);
    }
    __syncthreads();
    if (!active) return;
    const KView K{ks + tid, (int)blockDim.x};
    const int ci = __ldg(w.class_of + vid);
    const ClassDev18& C = cls_smem ? cls[ci] : w.classes[ci];
    const size_t np = (size_t)w.npad;
    double* S = w.S + vid;

    VehC v;
    Veh24X vx;
    VehAux va;
    TireC ts[4];
    TireAux ta[4];
    Sus24C su[4];
    Corner24K ck[4];
    load_state24(S, np, v, vx, va, ts, ta, su, ck);
    DriverCursor cur;
    double steer = w.steer, thr = w.thr, brk = w.brk;
    if (kCtl == CTL_TABLE) {
        driver_begin(cur, w.rows + 4 * __ldg(w.row_off + vid), __ldg(w.row_len + vid), w.t0);
    } else if (kCtl == CTL_ARRAY) {
        steer = __ldg(w.ctl + vid);
        thr = __ldg(w.ctl + np + vid);
        brk = __ldg(w.ctl + 2 * np + vid);
    }
    int next_k = 0;
    int next_step = (kOut && w.nsamples > 0) ? __ldg(w.sample_steps) : -1;
    double t = w.t0;
    const double dt = w.dt;
    auto controls = [&](int s) {
        if (kCtl == CTL_TABLE) {
            driver_at(cur, t, steer, thr, brk);
        } else if (kCtl == CTL_SCHEDULE) {
            steer = __ldg(w.sched + 3 * s);
            thr = __ldg(w.sched + 3 * s + 1);
            brk = __ldg(w.sched + 3 * s + 2);
        }
    };
    auto sample = [&](int s) {
        if (kOut && s + 1 == next_step) {
            double* r = w.resp + (size_t)next_k * LFDM24_RESP_CHANNELS * w.n + vid;
            const size_t n = (size_t)w.n;
            r[0 * n] = t;
            r[1 * n] = v.x;
            r[2 * n] = v.y;
            r[3 * n] = v.u;
            r[4 * n] = v.v;
            r[5 * n] = v.phi;
            r[6 * n] = v.psi;
            r[7 * n] = vx.theta;
            r[8 * n] = v.wx;
            r[9 * n] = v.wz;
            r[10 * n] = vx.wy;
            r[11 * n] = ts[0].omega;
            r[12 * n] = ts[1].omega;
            r[13 * n] = ts[2].omega;
            r[14 * n] = ts[3].omega;
            ++next_k;
            next_step = next_k < w.nsamples ? __ldg(w.sample_steps + next_k) : -1;
        }
    };
    const int last = w.nsteps - 1;
    for (int s = 0; s <= last; ++s) {
        controls(s);
        // the last step also writes the values the reference leaves in its state structs
        step24(v, vx, va, ts, ta, su, ck, K, C, steer, thr, brk, dt, S, np, s == last);
        t += dt;
        sample(s);
    }

    store_state24(S, np, v, vx, va, ts, ta, su, C.tcbool);
    if (w.status && !state24_finite(v, vx, ts)) w.status[vid] |= 1u;
}

template <int kCtl, bool kOut>
static cudaError_t launch24_t(const Window18& w, cudaStream_t stream) {
    const int threads = w.threads;
    const size_t smem = window24_smem(threads, w.nclasses);
    auto kern = window24_kernel<kCtl, kOut>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<(w.n + threads - 1) / threads, threads, smem, stream>>>(w);
    return cudaGetLastError();
}

template <int kCtl>
static cudaError_t launch24_o(const Window18& w, cudaStream_t s) {
    return (w.resp && w.nsamples > 0) ? launch24_t<kCtl, true>(w, s) : launch24_t<kCtl, false>(w, s);
}

cudaError_t launch_window24(const Window18& w, cudaStream_t stream) {
    if (w.n <= 0 || w.nsteps <= 0) return cudaSuccess;
    if (w.threads <= 0 || w.threads > 128 || (w.threads & 31)) return cudaErrorInvalidValue;
    if (w.tire_nr || w.precision != LFDM_PREC_FP64) return cudaErrorInvalidValue;
    switch (w.ctl_mode) {
        case CTL_TABLE: return launch24_o<CTL_TABLE>(w, stream);
        case CTL_SCALAR: return launch24_o<CTL_SCALAR>(w, stream);
        case CTL_SCHEDULE: return launch24_o<CTL_SCHEDULE>(w, stream);
        default: return launch24_o<CTL_ARRAY>(w, stream);
    }
}

}  // namespace lfdm
