// Right-hand-side Jacobians of the 11-, 18- and 24-DOF models with either tire, batched over
// vehicles, by the scheme of the reference's CPU solvers: IntegrateStepWithJacobian
// (11dof/dof11_halfImplicit.cpp:335-429, 18dof/dof18_halfImplicit.cpp:356-449,
// 24dof/dof24_halfImplicit.cpp:402-494) perturbs every packed state by +-|1e-3 y_i| (1e-3 where that
// is below 1e-8) and steering and throttle by +-1e-3 (braking 0), evaluates PerturbRhsFun at each
// perturbed point and takes central differences. Here one thread does that for one vehicle: 2 ny + 4
// right-hand-side evaluations (the model's rhs11 / rhs18 / rhs24, the arithmetic of the window
// kernels) with the same perturbations, quotients and packed orders, so the result is the reference's
// Jacobian up to the last-bit differences of the right-hand side (libm, fused multiply-adds), which
// the quotients magnify by 1 / (2 h).
//
// Packed orders (packY / packYDOT): 11-DOF {xe, ye} x 2, omega x 2, crank, x, y, u, v, psi, wz
// (11dof/dof11_halfImplicit.cpp:769-929); 18-DOF {xe, ye} x 4, omega x 4, crank, x, y, u, v, psi, wz,
// phi, wx (18dof/dof18_halfImplicit.cpp:879-1101); 24-DOF {xe, ye, xt} x 4, omega x 4, {wu, xs} x 4,
// crank, x, y, u, v, w, wz, wx, wy, psi, phi, theta (24dof/dof24_halfImplicit.cpp:1015-1386). The crank
// speed is a state only with a torque converter; TMeasyNr tires carry no deflection states.
//
// Evaluation point: PerturbRhsFun unpacks into freshly constructed states (every other field 0,
// first gear); reference_point selects that, otherwise the packed states are unpacked on top of the
// vehicle's full current state. The reference's 24-DOF TMeasyNr PerturbRhsFun skips the unpacking
// (its state Jacobian is zero); here every model and tire unpacks.
#include <cuda_runtime.h>

#include "../../include/lfdm/device/dof11_device.cuh"
#include "../../include/lfdm/device/dof24_device.cuh"
#include "jacobian_fd.h"
#include "window_common.cuh"

namespace lfdm {

namespace {

constexpr int kMaxNy = 36;

// x and y rates of computeVehRHS / computeVehicleRHS (11dof/dof11.cpp:904-905,
// 18dof/dof18.cpp:1075-1077, 24dof/dof24.cpp:1729-1731), from the unupdated u, v, psi.
__device__ __forceinline__ void xy_rates(double u, double v, double psi, double& dx, double& dy) {
    double sp, cp;
    sincos(psi, &sp, &cp);
    dx = u * cp - v * sp;
    dy = u * sp + v * cp;
}

template <int kModel, bool kNr>
struct Fd;

template <bool kNr>
struct Fd<11, kNr> {
    static constexpr int kCount = K18_COUNT;
    struct State {
        Veh11 v;
        Veh11Aux va;
        TireC ts[2];
        TireAux ta[2];
    };
    __device__ static void load(const double* S, size_t np, State& s) { load_state11(S, np, s.v, s.va, s.ts, s.ta); }
    __device__ static int pack(const State& s, bool tc, double* y) {
        int i = 0;
        if (!kNr)
            for (int k = 0; k < 2; ++k) {
                y[i++] = s.ts[k].xe;
                y[i++] = s.ts[k].ye;
            }
        for (int k = 0; k < 2; ++k) y[i++] = s.ts[k].omega;
        if (tc) y[i++] = s.v.crank;
        y[i++] = s.v.x;
        y[i++] = s.v.y;
        y[i++] = s.v.u;
        y[i++] = s.v.v;
        y[i++] = s.v.psi;
        y[i++] = s.v.wz;
        return i;
    }
    __device__ static void unpack(const double* y, bool tc, State& s) {
        int i = 0;
        if (!kNr)
            for (int k = 0; k < 2; ++k) {
                s.ts[k].xe = y[i++];
                s.ts[k].ye = y[i++];
            }
        for (int k = 0; k < 2; ++k) s.ts[k].omega = y[i++];
        if (tc) s.v.crank = y[i++];
        s.v.x = y[i++];
        s.v.y = y[i++];
        s.v.u = y[i++];
        s.v.v = y[i++];
        s.v.psi = y[i++];
        s.v.wz = y[i++];
    }
    __device__ static void rhs(State& s, const KView& K, const ClassDev18& C, double st, double th, double br, bool tc,
                               double* yd) {
        double dx, dy;
        xy_rates(s.v.u, s.v.v, s.v.psi, dx, dy);
        rhs11<kNr>(s.v, s.va, s.ts, s.ta, K, C, st, th, br);
        int i = 0;
        if (!kNr)
            for (int k = 0; k < 2; ++k) {
                yd[i++] = s.ts[k].xedot;
                yd[i++] = s.ts[k].yedot;
            }
        for (int k = 0; k < 2; ++k) yd[i++] = s.ta[k].dOmega;
        if (tc) yd[i++] = s.va.dOmega_crank;
        yd[i++] = dx;
        yd[i++] = dy;
        yd[i++] = s.v.udot;
        yd[i++] = s.v.vdot;
        yd[i++] = s.v.wz;
        yd[i++] = s.va.wzdot;
    }
};

template <bool kNr>
struct Fd<18, kNr> {
    static constexpr int kCount = K18_COUNT;
    struct State {
        VehC v;
        VehAux va;
        TireC ts[4];
        TireAux ta[4];
    };
    __device__ static void load(const double* S, size_t np, State& s) { load_state18(S, np, s.v, s.va, s.ts, s.ta); }
    __device__ static int pack(const State& s, bool tc, double* y) {
        int i = 0;
        if (!kNr)
            for (int k = 0; k < 4; ++k) {
                y[i++] = s.ts[k].xe;
                y[i++] = s.ts[k].ye;
            }
        for (int k = 0; k < 4; ++k) y[i++] = s.ts[k].omega;
        if (tc) y[i++] = s.v.crank;
        y[i++] = s.v.x;
        y[i++] = s.v.y;
        y[i++] = s.v.u;
        y[i++] = s.v.v;
        y[i++] = s.v.psi;
        y[i++] = s.v.wz;
        y[i++] = s.v.phi;
        y[i++] = s.v.wx;
        return i;
    }
    __device__ static void unpack(const double* y, bool tc, State& s) {
        int i = 0;
        if (!kNr)
            for (int k = 0; k < 4; ++k) {
                s.ts[k].xe = y[i++];
                s.ts[k].ye = y[i++];
            }
        for (int k = 0; k < 4; ++k) s.ts[k].omega = y[i++];
        if (tc) s.v.crank = y[i++];
        s.v.x = y[i++];
        s.v.y = y[i++];
        s.v.u = y[i++];
        s.v.v = y[i++];
        s.v.psi = y[i++];
        s.v.wz = y[i++];
        s.v.phi = y[i++];
        s.v.wx = y[i++];
    }
    __device__ static void rhs(State& s, const KView& K, const ClassDev18& C, double st, double th, double br, bool tc,
                               double* yd) {
        double dx, dy;
        xy_rates(s.v.u, s.v.v, s.v.psi, dx, dy);
        rhs18<kNr>(s.v, s.va, s.ts, s.ta, K, C, st, th, br);
        int i = 0;
        if (!kNr)
            for (int k = 0; k < 4; ++k) {
                yd[i++] = s.ts[k].xedot;
                yd[i++] = s.ts[k].yedot;
            }
        for (int k = 0; k < 4; ++k) yd[i++] = s.ta[k].dOmega;
        if (tc) yd[i++] = s.va.dOmega_crank;
        yd[i++] = dx;
        yd[i++] = dy;
        yd[i++] = s.v.udot;
        yd[i++] = s.v.vdot;
        yd[i++] = s.v.wz;
        yd[i++] = s.va.wzdot;
        yd[i++] = s.v.wx;
        yd[i++] = s.va.wxdot;
    }
};

template <bool kNr>
struct Fd<24, kNr> {
    static constexpr int kCount = K24_COUNT;
    struct State {
        VehC v;
        Veh24X vx;
        VehAux va;
        TireC ts[4];
        TireAux ta[4];
        Sus24C su[4];
        Corner24K ck[4];
    };
    __device__ static void load(const double* S, size_t np, State& s) {
        load_state24(S, np, s.v, s.vx, s.va, s.ts, s.ta, s.su, s.ck);
    }
    __device__ static int pack(const State& s, bool tc, double* y) {
        int i = 0;
        for (int c = 0; c < 4; ++c) {
            if (!kNr) {
                y[i++] = s.ts[c].xe;
                y[i++] = s.ts[c].ye;
            }
            y[i++] = s.ta[c].xt;
        }
        for (int c = 0; c < 4; ++c) y[i++] = s.ts[c].omega;
        for (int c = 0; c < 4; ++c) {
            y[i++] = s.su[c].wu;
            y[i++] = s.su[c].xs;
        }
        if (tc) y[i++] = s.v.crank;
        y[i++] = s.v.x;
        y[i++] = s.v.y;
        y[i++] = s.v.u;
        y[i++] = s.v.v;
        y[i++] = s.vx.w;
        y[i++] = s.v.wz;
        y[i++] = s.v.wx;
        y[i++] = s.vx.wy;
        y[i++] = s.v.psi;
        y[i++] = s.v.phi;
        y[i++] = s.vx.theta;
        return i;
    }
    __device__ static void unpack(const double* y, bool tc, State& s) {
        int i = 0;
        for (int c = 0; c < 4; ++c) {
            if (!kNr) {
                s.ts[c].xe = y[i++];
                s.ts[c].ye = y[i++];
            }
            s.ta[c].xt = y[i++];
        }
        for (int c = 0; c < 4; ++c) s.ts[c].omega = y[i++];
        for (int c = 0; c < 4; ++c) {
            s.su[c].wu = y[i++];
            s.su[c].xs = y[i++];
        }
        if (tc) s.v.crank = y[i++];
        s.v.x = y[i++];
        s.v.y = y[i++];
        s.v.u = y[i++];
        s.v.v = y[i++];
        s.vx.w = y[i++];
        s.v.wz = y[i++];
        s.v.wx = y[i++];
        s.vx.wy = y[i++];
        s.v.psi = y[i++];
        s.v.phi = y[i++];
        s.vx.theta = y[i++];
    }
    __device__ static void rhs(State& s, const KView& K, const ClassDev18& C, double st, double th, double br, bool tc,
                               double* yd) {
        double dx, dy;
        xy_rates(s.v.u, s.v.v, s.v.psi, dx, dy);
        // Cardan angle rates of computeVehicleRHS (24dof/dof24.cpp:1722-1726) at the unupdated rates
        const double sph = sin(s.v.phi), cph = cos(s.v.phi), cth = cos(s.vx.theta), tth = tan(s.vx.theta);
        const double wx = s.v.wx, wy = s.vx.wy, wz = s.v.wz;
        const double dtheta = wy * cph - wz * sph;
        const double dpsi = (wy * sph / cth) + (wz * cph / cth);
        const double dphi = wx + wy * sph * tth + wz * cph * tth;
        Rhs24 R;
        rhs24<kNr>(s.v, s.vx, s.va, s.ts, s.ta, s.su, s.ck, K, C, st, th, br, R, nullptr, 0, false);
        int i = 0;
        for (int c = 0; c < 4; ++c) {
            if (!kNr) {
                yd[i++] = s.ts[c].xedot;
                yd[i++] = s.ts[c].yedot;
            }
            yd[i++] = R.dxt[c];
        }
        for (int c = 0; c < 4; ++c) yd[i++] = s.ta[c].dOmega;
        for (int c = 0; c < 4; ++c) {
            yd[i++] = R.dwu[c];
            yd[i++] = s.su[c].dxs;
        }
        if (tc) yd[i++] = s.va.dOmega_crank;
        yd[i++] = dx;
        yd[i++] = dy;
        yd[i++] = s.v.udot;
        yd[i++] = s.v.vdot;
        yd[i++] = R.wdot;
        yd[i++] = s.vx.wzdot;
        yd[i++] = s.vx.wxdot;
        yd[i++] = s.vx.wydot;
        yd[i++] = dpsi;
        yd[i++] = dphi;
        yd[i++] = dtheta;
    }
};

}  // namespace

int jac_fd_ny(int model, bool tire_nr, bool tcbool) {
    const int t = tcbool ? 1 : 0;
    if (model == 11) return (tire_nr ? 8 : 12) + t;
    if (model == 18) return (tire_nr ? 12 : 20) + t;
    return (tire_nr ? 27 : 35) + t;
}

template <int kModel, bool kNr>
__global__ void __launch_bounds__(128) rhs_jacobian_fd_kernel(const JacFdLaunch A) {
    using M = Fd<kModel, kNr>;
    extern __shared__ __align__(16) unsigned char smem[];
    const int tid = threadIdx.x;
    const ClassDev18* cls = A.cls_smem ? reinterpret_cast<const ClassDev18*>(smem) : A.classes;
    double* ks = reinterpret_cast<double*>(smem + (A.cls_smem ? (size_t)A.nclasses * sizeof(ClassDev18) : 0));
    if (A.cls_smem) {
        const int4* src = reinterpret_cast<const int4*>(A.classes);
        int4* dst = reinterpret_cast<int4*>(smem);
        const int words = (int)(A.nclasses * sizeof(ClassDev18) / 16);
        for (int i = tid; i < words; i += blockDim.x) dst[i] = __ldg(src + i);
    }
    const int vid = blockIdx.x * blockDim.x + tid;
    if (vid < A.n) {
#pragma unroll 4
        for (int k = 0; k < M::kCount; ++k) ks[k * blockDim.x + tid] = __ldg(A.K + (size_t)k * A.npad + vid);
    }
    __syncthreads();
    if (vid >= A.n) return;
    const size_t np = (size_t)A.npad, nu = (size_t)A.n;
    const KView K{ks + tid, (int)blockDim.x};
    const ClassDev18& C = cls[__ldg(A.class_of + vid)];
    const bool tc = C.tcbool != 0;
    const bool full = A.reference_point == 0;
    const double* S = A.S + vid;
    const double steer = __ldg(A.ctl + vid), thr = __ldg(A.ctl + nu + vid), brk = __ldg(A.ctl + 2 * nu + vid);

    double y[kMaxNy], dp[kMaxNy], dm[kMaxNy];
    int ny;
    {
        typename M::State s;
        M::load(S, np, s);
        ny = M::pack(s, tc, y);
    }
    // PerturbRhsFun: the packed states unpacked into a fresh state (or the full state), one RHS
    auto eval = [&](double st, double th, double br, double* yd) {
        typename M::State s = {};
        if (full) M::load(S, np, s);
        M::unpack(y, tc, s);
        M::rhs(s, K, C, st, th, br, tc, yd);
    };
    for (int c = 0; c < ny; ++c) {
        const double y0 = y[c];
        double del = fabs(y0 * 1e-3);
        if (del < 1e-8) del = 1e-3;
        y[c] = y0 + del;
        eval(steer, thr, brk, dp);
        y[c] = y0 - del;
        eval(steer, thr, brk, dm);
        y[c] = y0;
        for (int r = 0; r < ny; ++r) A.jac_state[((size_t)r * ny + c) * nu + vid] = (dp[r] - dm[r]) / (2 * del);
    }
    for (int c = 0; c < 2; ++c) {
        const double sp = c == 0 ? steer + 1e-3 : steer, tp = c == 1 ? thr + 1e-3 : thr;
        const double sm = c == 0 ? steer - 1e-3 : steer, tm = c == 1 ? thr - 1e-3 : thr;
        eval(sp, tp, 0.0, dp);
        eval(sm, tm, 0.0, dm);
        for (int r = 0; r < ny; ++r) A.jac_ctl[((size_t)r * 2 + c) * nu + vid] = (dp[r] - dm[r]) / (2 * 1e-3);
    }
}

template <int kModel, bool kNr>
static cudaError_t launch_t(const JacFdLaunch& A, cudaStream_t stream) {
    constexpr int threads = 128;
    JacFdLaunch L = A;
    const size_t base = (size_t)Fd<kModel, kNr>::kCount * threads * sizeof(double);
    const size_t cls = (size_t)A.nclasses * sizeof(ClassDev18);
    L.cls_smem = A.nclasses <= kMaxSmemClasses;
    const size_t smem = base + (L.cls_smem ? cls : 0);
    auto kern = rhs_jacobian_fd_kernel<kModel, kNr>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<(A.n + threads - 1) / threads, threads, smem, stream>>>(L);
    return cudaGetLastError();
}

cudaError_t launch_rhs_jacobian_fd(const JacFdLaunch& A, cudaStream_t stream) {
    if (A.n <= 0) return cudaSuccess;
    switch (A.model) {
        case 11: return A.tire_nr ? launch_t<11, true>(A, stream) : launch_t<11, false>(A, stream);
        case 18: return A.tire_nr ? launch_t<18, true>(A, stream) : launch_t<18, false>(A, stream);
        case 24: return A.tire_nr ? launch_t<24, true>(A, stream) : launch_t<24, false>(A, stream);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace lfdm
