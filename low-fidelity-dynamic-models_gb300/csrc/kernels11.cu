// 11-DOF (single-track) window kernel; the right-hand side and the half-implicit update are in
// dof11_device.cuh.
#include <cuda_runtime.h>

#include "../../include/lfdm/device/dof11_device.cuh"
#include "kernels.h"
#include "window_common.cuh"

namespace lfdm {

// kF32: the TMeasy tire core in FP32 (precision LFDM_PREC_MIXED_TIRE), on FP32 copies of the
// derived constants staged beside the FP64 ones.
template <bool kNr, int kCtl, bool kOut, bool kF32>
__global__ void __launch_bounds__(128) window11_kernel(const Window18 w) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int tid = threadIdx.x;
    const bool cls_smem = w.nclasses <= kMaxSmemClasses;
    ClassDev18* cls = reinterpret_cast<ClassDev18*>(smem);
    double* ks = reinterpret_cast<double*>(smem + (cls_smem ? (size_t)w.nclasses * sizeof(ClassDev18) : 0));
    float* fks = reinterpret_cast<float*>(ks + (size_t)K18_COUNT * blockDim.x);
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
        for (int k = 0; k < K18_COUNT; ++k) {
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

    Veh11 v;
    Veh11Aux va;
    TireC ts[2];
    TireAux ta[2];
    load_state11(S, np, v, va, ts, ta);
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
    for (int s = 0; s < w.nsteps; ++s) {
        if (kCtl == CTL_TABLE) {
            driver_at(cur, t, steer, thr, brk);
        } else if (kCtl == CTL_SCHEDULE) {
            steer = __ldg(w.sched + 3 * s);
            thr = __ldg(w.sched + 3 * s + 1);
            brk = __ldg(w.sched + 3 * s + 2);
        }
        step11<kNr, kF32>(v, va, ts, ta, K, C, steer, thr, brk, dt);
        t += dt;
        if (kOut && s + 1 == next_step) {
            double* r = w.resp + (size_t)next_k * LFDM11_RESP_CHANNELS * w.n + vid;
            const size_t n = (size_t)w.n;
            r[0 * n] = t;
            r[1 * n] = v.x;
            r[2 * n] = v.y;
            r[3 * n] = v.u;
            r[4 * n] = v.v;
            r[5 * n] = v.psi;
            r[6 * n] = v.wz;
            r[7 * n] = ts[0].omega;
            r[8 * n] = ts[1].omega;
            ++next_k;
            next_step = next_k < w.nsamples ? __ldg(w.sample_steps + next_k) : -1;
        }
    }
    store_state11(S, np, v, va, ts, ta);
    if (w.status && !state11_finite(v, ts)) w.status[vid] |= 1u;
}

template <bool kNr, int kCtl, bool kOut, bool kF32>
static cudaError_t launch11_t(const Window18& w, cudaStream_t stream) {
    const int threads = w.threads;
    const size_t smem = window18_smem(threads, w.nclasses, kF32);
    auto kern = window11_kernel<kNr, kCtl, kOut, kF32>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<(w.n + threads - 1) / threads, threads, smem, stream>>>(w);
    return cudaGetLastError();
}

template <bool kNr, int kCtl, bool kF32>
static cudaError_t launch11_o(const Window18& w, cudaStream_t s) {
    return (w.resp && w.nsamples > 0) ? launch11_t<kNr, kCtl, true, kF32>(w, s)
                                      : launch11_t<kNr, kCtl, false, kF32>(w, s);
}
template <bool kNr, bool kF32 = false>
static cudaError_t launch11_c(const Window18& w, cudaStream_t stream) {
    switch (w.ctl_mode) {
        case CTL_TABLE: return launch11_o<kNr, CTL_TABLE, kF32>(w, stream);
        case CTL_SCALAR: return launch11_o<kNr, CTL_SCALAR, kF32>(w, stream);
        case CTL_SCHEDULE: return launch11_o<kNr, CTL_SCHEDULE, kF32>(w, stream);
        default: return launch11_o<kNr, CTL_ARRAY, kF32>(w, stream);
    }
}

// ---------------------------------------------------------------------------------------------
// Split-warp window kernel for small fleets. On GB300 an SM sub-partition accepts one warp-wide FP64
// instruction every 64 cycles whatever the number of active lanes, so a fleet of a few thousand
// vehicles (one warp per 32 vehicles, on a few dozen of the 608 sub-partitions) is bound by the
// FP64 instruction count of ONE vehicle's step. Here two warps carry the same 32 vehicles, each
// holding their full state: per step, warp 0 computes the front wheel's angle and tire and the yaw
// sine/cosine while warp 1 computes the rear tire and the powertrain (which only needs the front
// wheel's speed, zero when that wheel is off the ground, known from the loads), they exchange those
// results through shared memory (double-buffered by step parity, so one barrier per step suffices),
// and both run the wheel accelerations, chassis and update. The phases are the functions rhs11 and
// update11 are composed of, so every vehicle steps bit for bit as in window11_kernel.
constexpr int kSplit11Fields = 33;  // exchanged doubles per vehicle and step: 16 from warp 0, 17 from warp 1

size_t window11_split_smem(int nclasses, bool f32) {
    const size_t cls = nclasses <= kMaxSmemClasses ? (size_t)nclasses * sizeof(ClassDev18) : 0;
    return cls + (size_t)K18_COUNT * 32 * sizeof(double) + 2 * (size_t)kSplit11Fields * 32 * sizeof(double) +
           (f32 ? (size_t)K18_COUNT * 32 * sizeof(float) : 0);
}

template <bool kNr, int kCtl, bool kOut, bool kF32>
__global__ void __launch_bounds__(64) window11_split_kernel(const Window18 w) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int tid = threadIdx.x, lane = tid & 31, role = tid >> 5;
    const bool cls_smem = w.nclasses <= kMaxSmemClasses;
    ClassDev18* cls = reinterpret_cast<ClassDev18*>(smem);
    double* ks = reinterpret_cast<double*>(smem + (cls_smem ? (size_t)w.nclasses * sizeof(ClassDev18) : 0));
    double* xbuf = ks + (size_t)K18_COUNT * 32;
    float* fks = reinterpret_cast<float*>(xbuf + 2 * (size_t)kSplit11Fields * 32);
    if (cls_smem) {
        const int4* src = reinterpret_cast<const int4*>(w.classes);
        int4* dst = reinterpret_cast<int4*>(smem);
        const int words = (int)(w.nclasses * sizeof(ClassDev18) / 16);
        for (int i = tid; i < words; i += blockDim.x) dst[i] = __ldg(src + i);
    }
    const int vid_raw = blockIdx.x * 32 + lane;
    const bool active = vid_raw < w.n;
    // lanes past the fleet run a copy of the last vehicle (so that both warps reach every barrier)
    // and store nothing
    const int vid = active ? vid_raw : w.n - 1;
    for (int k = role; k < K18_COUNT; k += 2) {
        const double x = __ldg(w.K + (size_t)k * w.npad + vid);
        ks[k * 32 + lane] = x;
        if (kF32) fks[k * 32 + lane] = (float)x;
    }
    __syncthreads();
    const KView K{ks + lane, 32, kF32 ? fks + lane : nullptr};
    const int ci = __ldg(w.class_of + vid);
    const ClassDev18& C = cls_smem ? cls[ci] : w.classes[ci];
    const size_t np = (size_t)w.npad;
    double* S = w.S + vid;

    Veh11 v;
    Veh11Aux va;
    TireC ts[2];
    TireAux ta[2];
    load_state11(S, np, v, va, ts, ta);
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
    for (int s = 0; s < w.nsteps; ++s) {
        if (kCtl == CTL_TABLE) {
            driver_at(cur, t, steer, thr, brk);
        } else if (kCtl == CTL_SCHEDULE) {
            steer = __ldg(w.sched + 3 * s);
            thr = __ldg(w.sched + 3 * s + 1);
            brk = __ldg(w.sched + 3 * s + 2);
        }
        loads11(v, ta, K);
        double* X = xbuf + (size_t)(s & 1) * kSplit11Fields * 32 + lane;
        double cd, sd, sp, cp;
        if (role == 0) {
            front_kinematics11(v, ta[0], K, C, steer, cd, sd);
            tire11<kNr, true, kF32>(ts[0], ta[0], K, cd, sd);
            sincos(v.psi, &sp, &cp);
            const double out[16] = {ts[0].xe, ts[0].ye, ts[0].xedot, ts[0].yedot, ts[0].omega, ta[0].xt, ta[0].rStat,
                                    ta[0].fx, ta[0].fy, ta[0].My, ta[0].vsx, ta[0].vsy, cd, sd, sp, cp};
#pragma unroll
            for (int f = 0; f < 16; ++f) X[f * 32] = out[f];
        } else {
            rear_kinematics11(v, ta[1], K);
            tire11<kNr, false, kF32>(ts[1], ta[1], K, 1.0, 0.0);
            const double w0 = gt0(ta[0].fz) ? ts[0].omega : 0.0;  // the front tire zeroes it off the ground
            powertrain11(v, va, w0, ts[1].omega, ta[0].engTor, ta[1].engTor, K, C, thr);
            const double out[17] = {ts[1].xe, ts[1].ye, ts[1].xedot, ts[1].yedot, ts[1].omega, ta[1].xt, ta[1].rStat,
                                    ta[1].fx, ta[1].fy, ta[1].My, ta[1].vsx, ta[1].vsy, (double)v.gear, v.crank,
                                    va.dOmega_crank, ta[0].engTor, ta[1].engTor};
#pragma unroll
            for (int f = 0; f < 17; ++f) X[(16 + f) * 32] = out[f];
        }
        __syncthreads();
        if (role == 0) {
            ts[1].xe = X[16 * 32];
            ts[1].ye = X[17 * 32];
            ts[1].xedot = X[18 * 32];
            ts[1].yedot = X[19 * 32];
            ts[1].omega = X[20 * 32];
            ta[1].xt = X[21 * 32];
            ta[1].rStat = X[22 * 32];
            ta[1].fx = X[23 * 32];
            ta[1].fy = X[24 * 32];
            ta[1].My = X[25 * 32];
            ta[1].vsx = X[26 * 32];
            ta[1].vsy = X[27 * 32];
            v.gear = (int)X[28 * 32];
            v.crank = X[29 * 32];
            va.dOmega_crank = X[30 * 32];
            ta[0].engTor = X[31 * 32];
            ta[1].engTor = X[32 * 32];
        } else {
            ts[0].xe = X[0];
            ts[0].ye = X[1 * 32];
            ts[0].xedot = X[2 * 32];
            ts[0].yedot = X[3 * 32];
            ts[0].omega = X[4 * 32];
            ta[0].xt = X[5 * 32];
            ta[0].rStat = X[6 * 32];
            ta[0].fx = X[7 * 32];
            ta[0].fy = X[8 * 32];
            ta[0].My = X[9 * 32];
            ta[0].vsx = X[10 * 32];
            ta[0].vsy = X[11 * 32];
            cd = X[12 * 32];
            sd = X[13 * 32];
            sp = X[14 * 32];
            cp = X[15 * 32];
        }
        chassis11(v, va, ts, ta, K, brk, cd, sd);
        update11_sc<kNr>(v, va, ts, ta, C, dt, sp, cp);
        t += dt;
        if (kOut && s + 1 == next_step) {
            if (role == 0 && active) {
                double* r = w.resp + (size_t)next_k * LFDM11_RESP_CHANNELS * w.n + vid;
                const size_t n = (size_t)w.n;
                r[0 * n] = t;
                r[1 * n] = v.x;
                r[2 * n] = v.y;
                r[3 * n] = v.u;
                r[4 * n] = v.v;
                r[5 * n] = v.psi;
                r[6 * n] = v.wz;
                r[7 * n] = ts[0].omega;
                r[8 * n] = ts[1].omega;
            }
            ++next_k;
            next_step = next_k < w.nsamples ? __ldg(w.sample_steps + next_k) : -1;
        }
    }
    if (role == 0 && active) {
        store_state11(S, np, v, va, ts, ta);
        if (w.status && !state11_finite(v, ts)) w.status[vid] |= 1u;
    }
}

template <bool kNr, int kCtl, bool kOut, bool kF32>
static cudaError_t launch11_split_t(const Window18& w, cudaStream_t stream) {
    const size_t smem = window11_split_smem(w.nclasses, kF32);
    auto kern = window11_split_kernel<kNr, kCtl, kOut, kF32>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<(w.n + 31) / 32, 64, smem, stream>>>(w);
    return cudaGetLastError();
}
template <bool kNr, int kCtl, bool kF32>
static cudaError_t launch11_split_o(const Window18& w, cudaStream_t s) {
    return (w.resp && w.nsamples > 0) ? launch11_split_t<kNr, kCtl, true, kF32>(w, s)
                                      : launch11_split_t<kNr, kCtl, false, kF32>(w, s);
}
template <bool kNr, bool kF32 = false>
static cudaError_t launch11_split_c(const Window18& w, cudaStream_t stream) {
    switch (w.ctl_mode) {
        case CTL_TABLE: return launch11_split_o<kNr, CTL_TABLE, kF32>(w, stream);
        case CTL_SCALAR: return launch11_split_o<kNr, CTL_SCALAR, kF32>(w, stream);
        case CTL_SCHEDULE: return launch11_split_o<kNr, CTL_SCHEDULE, kF32>(w, stream);
        default: return launch11_split_o<kNr, CTL_ARRAY, kF32>(w, stream);
    }
}

// Fleets this small run the split-warp kernel: its 2 warps per 32 vehicles still fit one warp per SM
// sub-partition (2 blocks of 64 threads per SM).
static bool use_split11(const Window18& w) {
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            sms = 1;
    }
    return w.split != 0 && (w.split > 0 || (w.n + 31) / 32 <= 2 * sms);
}

cudaError_t launch_window11(const Window18& w, cudaStream_t stream) {
    if (w.n <= 0 || w.nsteps <= 0) return cudaSuccess;
    if (w.threads <= 0 || w.threads > 128 || (w.threads & 31)) return cudaErrorInvalidValue;
    if (w.precision == LFDM_PREC_MIXED_TIRE) {
        if (use_split11(w))
            return w.tire_nr ? launch11_split_c<true, true>(w, stream) : launch11_split_c<false, true>(w, stream);
        return w.tire_nr ? launch11_c<true, true>(w, stream) : launch11_c<false, true>(w, stream);
    }
    if (w.precision != LFDM_PREC_FP64) return cudaErrorInvalidValue;
    if (use_split11(w)) return w.tire_nr ? launch11_split_c<true>(w, stream) : launch11_split_c<false>(w, stream);
    return w.tire_nr ? launch11_c<true>(w, stream) : launch11_c<false>(w, stream);
}

}  // namespace lfdm
