// Exact Jacobians of the 18-DOF right-hand side, batched over vehicles.
//
// The reference's CPU solver offers them by central differences (IntegrateStepWithJacobian,
// 18dof/dof18_halfImplicit.cpp:356-520: every state perturbed by 1e-3 of its value, PerturbRhsFun
// :679-745 evaluated twice per column, results in GetJacobianState / GetJacobianControls); its GPU
// solver has none. Here the Jacobian is exact: one right-hand-side evaluation with its tape
// (fwd18_tape) per vehicle, then one reverse sweep of the right-hand side (rev18_rhs) per dynamic
// row; the four kinematic rows (dx, dy, dpsi = wz, dphi = wx) are written from their closed forms.
//
// Packed order (packY / packYDOT, 18dof/dof18_halfImplicit.cpp:879-1018): states
// {xe, ye} of LF, RF, LR, RR (TMeasy tires only); omega of LF, RF, LR, RR; crank speed (torque
// converter only); x, y, u, v, psi, wz, phi, wx. Right-hand side in the same order: {xedot, yedot}
// x 4, domega x 4, dcrank, dx, dy, udot, vdot, wz, wzdot, wx, wxdot. Controls: steering, throttle
// (braking enters the right-hand side additively through the brake torque, so no derivative
// depends on it). The TMeasyNr tire is reversed by tire_rev_nr (dof18_adjoint.cuh).
//
// Evaluation point: PerturbRhsFun unpacks the packed states into a freshly constructed vehicle
// state, so the reference differentiates with the previous accelerations (read by the load
// transfer) at 0 and the first gear engaged; reference_point selects that point, otherwise the
// vehicle's full current state (its accelerations and gear) is used.
#include <cuda_runtime.h>

#include "dof18_adjoint.cuh"
#include "jacobian18.h"
#include "window_common.cuh"

namespace lfdm {

size_t jac18_smem(int threads, int nclasses, bool* cls_smem) {
    const size_t base = (size_t)(K18_COUNT + KB_COUNT) * threads * sizeof(double);
    const size_t cls = (size_t)nclasses * sizeof(ClassDev18);
    const bool in = nclasses <= kMaxSmemClasses && 2 * (base + cls + 1024) <= 228 * 1024;
    if (cls_smem) *cls_smem = in;
    return base + (in ? cls : 0);
}

template <bool kNr>
__global__ void __launch_bounds__(128) rhs_jacobian18_kernel(const JacLaunch A) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int tid = threadIdx.x;
    const ClassDev18* cls = A.cls_smem ? reinterpret_cast<const ClassDev18*>(smem) : A.classes;
    double* ks = reinterpret_cast<double*>(smem + (A.cls_smem ? (size_t)A.nclasses * sizeof(ClassDev18) : 0));
    double* kbs = ks + (size_t)K18_COUNT * blockDim.x;
    if (A.cls_smem) {
        const int4* src = reinterpret_cast<const int4*>(A.classes);
        int4* dst = reinterpret_cast<int4*>(smem);
        const int words = (int)(A.nclasses * sizeof(ClassDev18) / 16);
        for (int i = tid; i < words; i += blockDim.x) dst[i] = __ldg(src + i);
    }
    const int vid = blockIdx.x * blockDim.x + tid;
    if (vid < A.n) {
#pragma unroll 4
        for (int k = 0; k < K18_COUNT; ++k) ks[k * blockDim.x + tid] = __ldg(A.K + (size_t)k * A.npad + vid);
    }
    __syncthreads();
    if (vid >= A.n) return;
    const size_t np = (size_t)A.npad, nu = (size_t)A.n;
    const KView K{ks + tid, (int)blockDim.x};
    const KBar kb{kbs + tid, (int)blockDim.x};  // parameter-constant adjoints: scratch, not reported
    const ClassDev18& C = cls[__ldg(A.class_of + vid)];

    VehC v;
    VehAux va;
    TireC ts[4];
    TireAux ta[4];
    load_state18(A.S + vid, np, v, va, ts, ta);
    if (A.reference_point) {  // a freshly constructed VehicleState / TMeasyState holding the packed states
        v.udot = 0.0;
        v.vdot = 0.0;
        v.gear = 0;
        if (!C.tcbool) v.crank = 0.0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            ts[k].xedot = 0.0;
            ts[k].yedot = 0.0;
        }
    }
    const double psi = v.psi, u = v.u, vv = v.v;
    const double steer = __ldg(A.ctl + vid), thr = __ldg(A.ctl + nu + vid), brk = __ldg(A.ctl + 2 * nu + vid);
    const TapeRef T{A.tape + vid, np};
    fwd18_tape<kNr>(v, va, ts, ta, T, K, C, steer, thr, brk, 1e-3);

    const bool tc = C.tcbool != 0;
    // TMeasy: {xe, ye} x 4, omega x 4, crank, x...; TMeasyNr: omega x 4, crank, x...
    const int nt = kNr ? 0 : 8;                     // deflection states before the wheel speeds
    const int ny = nt + (tc ? 13 : 12), o = nt + (tc ? 5 : 4);  // o: index of x in the packed vector
    auto J = [&](int r, int c) -> double& { return A.jac_state[((size_t)r * ny + c) * nu + vid]; };
    auto Ju = [&](int r, int c) -> double& { return A.jac_ctl[((size_t)r * 2 + c) * nu + vid]; };
    for (int r = 0; r < ny; ++r) {
        const bool kinematic = r == o || r == o + 1 || r == o + 4 || r == o + 6;
        if (kinematic) {
            for (int c = 0; c < ny; ++c) J(r, c) = 0.0;
            Ju(r, 0) = 0.0;
            Ju(r, 1) = 0.0;
            double sp, cp;
            sincos(psi, &sp, &cp);
            if (r == o) {  // dx = u cos(psi) - v sin(psi)
                J(r, o + 2) = cp;
                J(r, o + 3) = -sp;
                J(r, o + 4) = fma(-u, sp, -vv * cp);
            } else if (r == o + 1) {  // dy = u sin(psi) + v cos(psi)
                J(r, o + 2) = sp;
                J(r, o + 3) = cp;
                J(r, o + 4) = fma(u, cp, -vv * sp);
            } else if (r == o + 4) {  // dpsi = wz
                J(r, o + 5) = 1.0;
            } else {  // dphi = wx
                J(r, o + 7) = 1.0;
            }
            continue;
        }
        // seed the adjoint of right-hand-side output r
        double udotb = 0, vdotb = 0, wxdotb = 0, wzdotb = 0, dOcb = 0;
        double dOmb[4] = {0, 0, 0, 0}, xedotb[4] = {0, 0, 0, 0}, yedotb[4] = {0, 0, 0, 0};
        if (r < nt) (r & 1 ? yedotb : xedotb)[r >> 1] = 1.0;
        else if (r < nt + 4) dOmb[r - nt] = 1.0;
        else if (tc && r == nt + 4) dOcb = 1.0;
        else if (r == o + 2) udotb = 1.0;
        else if (r == o + 3) vdotb = 1.0;
        else if (r == o + 5) wzdotb = 1.0;
        else wxdotb = 1.0;  // r == o + 7
        double ub = 0, vb = 0, wxb = 0, wzb = 0, phib = 0, crankb = 0, om_midb[4] = {0, 0, 0, 0};
        double steerb = 0, thrb = 0, brkb = 0;
        Adj18 L = {};
        rev18_rhs<kNr>(T, K, C, kb, udotb, vdotb, wxdotb, wzdotb, dOcb, 0.0, dOmb, xedotb, yedotb, ub, vb, wxb, wzb,
                       phib, crankb, om_midb, L, steerb, thrb, brkb);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (!kNr) {
                J(r, 2 * k) = L.xe[k];
                J(r, 2 * k + 1) = L.ye[k];
            }
            J(r, nt + k) = L.om[k];
        }
        if (tc) J(r, nt + 4) = crankb;
        J(r, o) = 0.0;      // x
        J(r, o + 1) = 0.0;  // y
        J(r, o + 2) = ub;
        J(r, o + 3) = vb;
        J(r, o + 4) = 0.0;  // psi enters only dx and dy
        J(r, o + 5) = wzb;
        J(r, o + 6) = phib;
        J(r, o + 7) = wxb;
        Ju(r, 0) = steerb;
        Ju(r, 1) = thrb;
    }
}

cudaError_t launch_rhs_jacobian18(const JacLaunch& A, cudaStream_t stream) {
    if (A.n <= 0) return cudaSuccess;
    constexpr int threads = 128;
    JacLaunch L = A;
    const size_t smem = jac18_smem(threads, A.nclasses, &L.cls_smem);
    auto kern = A.tire_nr ? rhs_jacobian18_kernel<true> : rhs_jacobian18_kernel<false>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<(A.n + threads - 1) / threads, threads, smem, stream>>>(L);
    return cudaGetLastError();
}

}  // namespace lfdm
