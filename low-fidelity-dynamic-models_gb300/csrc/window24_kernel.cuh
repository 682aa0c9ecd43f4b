// The 24-DOF window kernel and its launch templates, instantiated for TMeasy tires in kernels24.cu,
// for TMeasyNr tires in kernels24nr.cu, and for either tire with the FP32 tire core in kernels24tf.cu
// and kernels24nrtf.cu (four translation units that compile in parallel).
#pragma once

#include <cuda_runtime.h>

#include "../../include/lfdm/device/dof24_device.cuh"
#include "kernels.h"
#include "window_common.cuh"

namespace lfdm {

size_t window24_smem(int threads, int nclasses, bool f32);
cudaError_t launch_window24_nr(const Window18& w, cudaStream_t stream);
cudaError_t launch_window24_f32(const Window18& w, cudaStream_t stream);
cudaError_t launch_window24_nr_f32(const Window18& w, cudaStream_t stream);

// kF32: the TMeasy tire core in FP32 (precision LFDM_PREC_MIXED_TIRE), on FP32 copies of the
// derived constants staged beside the FP64 ones.
template <bool kNr, int kCtl, bool kOut, bool kF32>
__global__ void __launch_bounds__(128) window24_kernel(const Window18 w) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int tid = threadIdx.x;
    const bool cls_smem = w.nclasses <= kMaxSmemClasses;
    ClassDev18* cls = reinterpret_cast<ClassDev18*>(smem);
    double* ks = reinterpret_cast<double*>(smem + (cls_smem ? (size_t)w.nclasses * sizeof(ClassDev18) : 0));
    float* fks = reinterpret_cast<float*>(ks + (size_t)K24_COUNT * blockDim.x);
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
        for (int k = 0; k < K24_COUNT; ++k) {
            const double x = __ldg(w.K + (size_t)k * w.npad + vid);
            ks[k * blockDim.x + tid] = x;
            if (kF32) fks[k * blockDim.x + tid] = (float)x;
        }
    }
    __syncthreads();
    if (!active) return;
    const KView K{ks + tid, (int)blockDim.x, kF32 ? fks + tid : nullptr};
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
        step24<kNr, kF32>(v, vx, va, ts, ta, su, ck, K, C, steer, thr, brk, dt, S, np, s == last);
        t += dt;
        sample(s);
    }

    store_state24(S, np, v, vx, va, ts, ta, su, C.tcbool);
    if (w.status && !state24_finite(v, vx, ts)) w.status[vid] |= 1u;
}

template <bool kNr, int kCtl, bool kOut, bool kF32>
static cudaError_t launch24_t(const Window18& w, cudaStream_t stream) {
    const int threads = w.threads;
    const size_t smem = window24_smem(threads, w.nclasses, kF32);
    auto kern = window24_kernel<kNr, kCtl, kOut, kF32>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<(w.n + threads - 1) / threads, threads, smem, stream>>>(w);
    return cudaGetLastError();
}

template <bool kNr, int kCtl, bool kF32>
static cudaError_t launch24_o(const Window18& w, cudaStream_t s) {
    return (w.resp && w.nsamples > 0) ? launch24_t<kNr, kCtl, true, kF32>(w, s)
                                      : launch24_t<kNr, kCtl, false, kF32>(w, s);
}

// All control modes and output settings of one tire model and tire-core arithmetic.
template <bool kNr, bool kF32 = false>
static cudaError_t launch24_tire(const Window18& w, cudaStream_t stream) {
    switch (w.ctl_mode) {
        case CTL_TABLE: return launch24_o<kNr, CTL_TABLE, kF32>(w, stream);
        case CTL_SCALAR: return launch24_o<kNr, CTL_SCALAR, kF32>(w, stream);
        case CTL_SCHEDULE: return launch24_o<kNr, CTL_SCHEDULE, kF32>(w, stream);
        default: return launch24_o<kNr, CTL_ARRAY, kF32>(w, stream);
    }
}

}  // namespace lfdm
