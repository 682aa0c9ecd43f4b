// 11-DOF (single-track) window kernel; the right-hand side and the half-implicit update are in
// dof11_device.cuh.
#include <cuda_runtime.h>

#include "dof11_device.cuh"
#include "kernels.h"
#include "window_common.cuh"

namespace lfdm {

template <bool kNr, int kCtl, bool kOut>
__global__ void __launch_bounds__(128) window11_kernel(const Window18 w) {
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
        for (int k = 0; k < K18_COUNT; ++k) ks[k * blockDim.x + tid] = __ldg(w.K + (size_t)k * w.npad + vid);
    }
    __syncthreads();
    if (!active) return;
    const KView K{ks + tid, (int)blockDim.x};
    const int ci = __ldg(w.class_of + vid);
    const ClassDev18& C = cls_smem ? cls[ci] : w.classes[ci];
    const size_t np = (size_t)w.npad;
    double* S = w.S + vid;

    Veh11 v;
    Veh11Aux va;
    TireC ts[2];
    TireAux ta[2];
    v.x = S[LFDM11_S_X * np];
    v.y = S[LFDM11_S_Y * np];
    v.u = S[LFDM11_S_U * np];
    v.v = S[LFDM11_S_V * np];
    v.psi = S[LFDM11_S_PSI * np];
    v.wz = S[LFDM11_S_WZ * np];
    v.udot = S[LFDM11_S_UDOT * np];
    v.vdot = S[LFDM11_S_VDOT * np];
    v.crank = S[LFDM11_S_CRANKOMEGA * np];
    v.gear = (int)S[LFDM11_S_CURRENT_GR * np];
    va.wzdot = S[LFDM11_S_WZDOT * np];
    va.dOmega_crank = S[LFDM11_S_DOMEGA_CRANK * np];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const size_t b = (size_t)(LFDM11_S_TIRE0 + k * LFDM_S_TIRE_STRIDE) * np;
        ts[k].xe = S[b + LFDM_T_XE * np];
        ts[k].ye = S[b + LFDM_T_YE * np];
        ts[k].xedot = S[b + LFDM_T_XEDOT * np];
        ts[k].yedot = S[b + LFDM_T_YEDOT * np];
        ts[k].omega = S[b + LFDM_T_OMEGA * np];
        ta[k].dOmega = S[b + LFDM_T_DOMEGA * np];
        ta[k].xt = S[b + LFDM_T_XT * np];
        ta[k].rStat = S[b + LFDM_T_RSTAT * np];
        ta[k].fx = S[b + LFDM_T_FX * np];
        ta[k].fy = S[b + LFDM_T_FY * np];
        ta[k].fz = S[b + LFDM_T_FZ * np];
        ta[k].vsx = S[b + LFDM_T_VSX * np];
        ta[k].vsy = S[b + LFDM_T_VSY * np];
        ta[k].My = S[b + LFDM_T_MY * np];
        ta[k].engTor = S[b + LFDM_T_ENGTOR * np];
    }
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
        step11<kNr>(v, va, ts, ta, K, C, steer, thr, brk, dt);
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
    S[LFDM11_S_X * np] = v.x;
    S[LFDM11_S_Y * np] = v.y;
    S[LFDM11_S_U * np] = v.u;
    S[LFDM11_S_V * np] = v.v;
    S[LFDM11_S_PSI * np] = v.psi;
    S[LFDM11_S_WZ * np] = v.wz;
    S[LFDM11_S_UDOT * np] = v.udot;
    S[LFDM11_S_VDOT * np] = v.vdot;
    S[LFDM11_S_WZDOT * np] = va.wzdot;
    S[LFDM11_S_CRANKOMEGA * np] = v.crank;
    S[LFDM11_S_DOMEGA_CRANK * np] = va.dOmega_crank;
    S[LFDM11_S_CURRENT_GR * np] = (double)v.gear;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const size_t b = (size_t)(LFDM11_S_TIRE0 + k * LFDM_S_TIRE_STRIDE) * np;
        S[b + LFDM_T_XE * np] = ts[k].xe;
        S[b + LFDM_T_YE * np] = ts[k].ye;
        S[b + LFDM_T_XEDOT * np] = ts[k].xedot;
        S[b + LFDM_T_YEDOT * np] = ts[k].yedot;
        S[b + LFDM_T_OMEGA * np] = ts[k].omega;
        S[b + LFDM_T_DOMEGA * np] = ta[k].dOmega;
        S[b + LFDM_T_XT * np] = ta[k].xt;
        S[b + LFDM_T_RSTAT * np] = ta[k].rStat;
        S[b + LFDM_T_FX * np] = ta[k].fx;
        S[b + LFDM_T_FY * np] = ta[k].fy;
        S[b + LFDM_T_FZ * np] = ta[k].fz;
        S[b + LFDM_T_VSX * np] = ta[k].vsx;
        S[b + LFDM_T_VSY * np] = ta[k].vsy;
        S[b + LFDM_T_MY * np] = ta[k].My;
        S[b + LFDM_T_ENGTOR * np] = ta[k].engTor;
    }
    if (w.status) {
        const bool bad = !(isfinite(v.x) && isfinite(v.y) && isfinite(v.u) && isfinite(v.v) && isfinite(v.psi) &&
                           isfinite(v.wz) && isfinite(ts[0].omega) && isfinite(ts[1].omega));
        if (bad) w.status[vid] |= 1u;
    }
}

template <bool kNr, int kCtl, bool kOut>
static cudaError_t launch11_t(const Window18& w, cudaStream_t stream) {
    const int threads = w.threads;
    const size_t smem = window18_smem(threads, w.nclasses);
    auto kern = window11_kernel<kNr, kCtl, kOut>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<(w.n + threads - 1) / threads, threads, smem, stream>>>(w);
    return cudaGetLastError();
}

template <bool kNr, int kCtl>
static cudaError_t launch11_o(const Window18& w, cudaStream_t s) {
    return (w.resp && w.nsamples > 0) ? launch11_t<kNr, kCtl, true>(w, s) : launch11_t<kNr, kCtl, false>(w, s);
}
template <bool kNr>
static cudaError_t launch11_c(const Window18& w, cudaStream_t stream) {
    switch (w.ctl_mode) {
        case CTL_TABLE: return launch11_o<kNr, CTL_TABLE>(w, stream);
        case CTL_SCALAR: return launch11_o<kNr, CTL_SCALAR>(w, stream);
        case CTL_SCHEDULE: return launch11_o<kNr, CTL_SCHEDULE>(w, stream);
        default: return launch11_o<kNr, CTL_ARRAY>(w, stream);
    }
}

cudaError_t launch_window11(const Window18& w, cudaStream_t stream) {
    if (w.n <= 0 || w.nsteps <= 0) return cudaSuccess;
    if (w.threads <= 0 || w.threads > 128 || (w.threads & 31)) return cudaErrorInvalidValue;
    if (w.precision != LFDM_PREC_FP64) return cudaErrorInvalidValue;
    return w.tire_nr ? launch11_c<true>(w, stream) : launch11_c<false>(w, stream);
}

}  // namespace lfdm
