// Exact Jacobians of the 11-DOF right-hand side, batched over vehicles.
//
// The reference's CPU solver offers them by central differences (IntegrateStepWithJacobian,
// 11dof/dof11_halfImplicit.cpp:335-429: every packed state perturbed by 1e-3 of its value,
// PerturbRhsFun twice per column, results in GetJacobianState / GetJacobianControls); its GPU
// solver has none. As for the 18-DOF model (jacobian18.cu), one right-hand-side evaluation is
// recorded on a tape per vehicle and reversed once per dynamic row; the tires are the 18-DOF
// model's (tire_fwd_tape / tire_rev and their TMeasyNr forms, dof18_adjoint.cuh, on the first two
// tire slots of the step tape), the vehicle level is the single-track model's: axle loads
// (computeTireLoads, 11dof-gpu/dof11_gpu.cu:234-252), contact-patch velocities (vehToTireTransform,
// :41-68), the powertrain with the front/rear differential (computePowertrainRHS, :601-745,
// differentialSplit, :276-315), the wheel accelerations, the rotation of the front forces
// (11dof/dof11.cpp:100-124) and computeVehRHS (11dof-gpu/dof11_gpu.cu:893-909).
//
// Packed order (packY / packYDOT, 11dof/dof11_halfImplicit.cpp:769-929): states {xe, ye} of the
// front and rear tire (TMeasy only), omega front and rear, crank speed (torque converter only), x, y,
// u, v, psi, wz; right-hand side {xedot, yedot} x 2, domega x 2, dcrank, dx, dy, udot, vdot, wz,
// wzdot; controls steering, throttle. The kinematic rows (dx, dy, dpsi = wz) have closed forms.
#include <cuda_runtime.h>

#include "../../include/lfdm/device/dof11_device.cuh"
#include "dof18_adjoint.cuh"
#include "jacobian18.h"
#include "window_common.cuh"

namespace lfdm {

namespace {

// rhs11 with its tape (the arithmetic of loads11, front/rear_kinematics11, tire11, powertrain11 and
// chassis11); the step tape's 18-DOF fields are reused where they mean the same quantity, tires in
// slots 0 (front) and 1 (rear).
template <bool kNr>
__device__ __forceinline__ void fwd11_tape(Veh11& v, Veh11Aux& va, TireC* ts, TireAux* ta, const TapeRef& T,
                                           const KView& K, const ClassDev18& C, double steering, double throttle,
                                           double braking) {
    T.at(TS_(u)) = v.u;
    T.at(TS_(v)) = v.v;
    T.at(TS_(wz)) = v.wz;
    T.at(TS_(psi)) = v.psi;
    T.at(TS_(steer)) = steering;
    T.at(TS_(thr)) = throttle;
    T.at(TS_(brk)) = braking;
    // axle loads
    {
        const double lon = fma(-v.wz, v.v, v.udot);
        const double Z2 = K(K_Z4) * lon;
        T.at(TS_(lon)) = lon;
        T.at(TS_(fzarg) + 0) = K(K_Z1F) - Z2;
        T.at(TS_(fzarg) + 1) = K(K_Z1R) + Z2;
        ta[0].fz = pos_part(K(K_Z1F) - Z2);
        ta[1].fz = pos_part(K(K_Z1R) + Z2);
    }
    // wheel angle and contact-patch velocities
    double delta;
    if (C.nonLinearSteer) {
        delta = map_y(C.steer, steering);
        T.at(TS_(dslope)) = map_slope(C.steer, steering);
    } else {
        delta = steering * K(K_MAXSTEER);
        T.at(TS_(dslope)) = K(K_MAXSTEER);
    }
    double cd = 1.0, sd = 0.0;
    if (!is_zero(delta)) sincos(delta, &sd, &cd);
    T.at(TS_(delta)) = delta;
    T.at(TS_(cd)) = cd;
    T.at(TS_(sd)) = sd;
    const double vsyf = fma(v.wz, K(K_A), v.v);
    T.at(TS_(vsyf)) = vsyf;
    ta[0].vsy = vsyf;
    ta[0].vsx = fma(v.u, cd, vsyf * sd);
    ta[1].vsy = fma(-v.wz, K(K_B), v.v);
    ta[1].vsx = v.u;
    if (kNr) {
        tire_fwd_tape_nr<true>(ts[0], ta[0], tire_ref(T, 0), K, cd, sd);
        tire_fwd_tape_nr<false>(ts[1], ta[1], tire_ref(T, 1), K, 1.0, 0.0);
    } else {
        tire_fwd_tape<true>(ts[0], ta[0], tire_ref(T, 0), K, cd, sd);
        tire_fwd_tape<false>(ts[1], ta[1], tire_ref(T, 1), K, 1.0, 0.0);
    }
    // powertrain (the wheel speeds the tires leave: zero for a wheel off the ground)
    const double w0 = ts[0].omega, w1 = ts[1].omega;
    const int g = v.gear;
    double torque_t;
    T.at(TS_(rev)) = 0;
    T.at(TS_(tclip)) = 0;
    if (C.tcbool) {
        bool reverse = false;
        const double omega_out = 0.5 * (w0 + w1) / C.gear[g];
        const double omega_in = v.crank;
        T.at(TS_(omega_out)) = omega_out;
        T.at(TS_(omega_in)) = omega_in;
        double sr = 0;
        T.at(TS_(srmode)) = 0;
        if (!(lt_(omega_out, 1e-9) || lt_(omega_in, 1e-9))) {
            sr = omega_out / omega_in;
            T.at(TS_(srmode)) = 1;
            if (gt_nn(sr, 1.)) {
                sr = 1. - (sr - 1.);
                reverse = true;
            }
            if (lt_(sr, 0.0)) {
                sr = 0;
                T.at(TS_(srmode)) = 0;
            }
        }
        T.at(TS_(rev)) = reverse ? 1.0 : 0.0;
        const double cf = map_y(C.cf, sr), tr = map_y(C.tr, sr);
        T.at(TS_(cf)) = cf;
        T.at(TS_(tr)) = tr;
        T.at(TS_(cfs)) = map_slope(C.cf, sr);
        T.at(TS_(trs)) = map_slope(C.tr, sr);
        const double r = omega_in / cf;
        T.at(TS_(r)) = r;
        double torque_in = -(r * r);
        if (reverse) torque_in = -torque_in;
        T.at(TS_(torque_in)) = torque_in;
        const double torque_out = reverse ? -torque_in : -tr * torque_in;
        torque_t = torque_out * C.invgear[g];
        if (lt_(v.u, 1e-9) && lt_(torque_t, 0.0)) {
            torque_t = 0;
            T.at(TS_(tclip)) = 1;
        }
        va.dOmega_crank = K(K_INVCI) * (drive_torque(C, throttle, v.crank) + torque_in);
        T.at(TS_(dt_map)) = map_y(C.pt, v.crank);
        T.at(TS_(dt_slope)) = fma(map_slope(C.pt, v.crank), throttle, map_slope(C.loss, v.crank));
    } else {
        v.crank = 0.5 * (w0 + w1) / C.gear[g];
        torque_t = drive_torque(C, throttle, v.crank) * C.invgear[g];
        T.at(TS_(dt_map)) = map_y(C.pt, v.crank);
        T.at(TS_(dt_slope)) = fma(map_slope(C.pt, v.crank), throttle, map_slope(C.loss, v.crank));
        if (lt_(v.u, 1e-9) && lt_(torque_t, 0.0)) {
            torque_t = 0;
            T.at(TS_(tclip)) = 1;
        }
    }
    T.at(TS_(torque_t)) = torque_t;
    // differentialSplit between the rear (slow side when |w1| < |w0|) and the front axle
    double alpha = 0.5, dal = 0.0, rear_slow = 0.0;
    if (C.driveType) {
        const double diff = fabs(w1 - w0);
        if (diff > 0.5) {
            alpha = 2.0 / 3.0;
        } else if (diff > 0.25) {
            const double bias = 4 * (2.0 - 1) * diff + (2 - 2.0);
            alpha = bias / (1 + bias);
            dal = 4.0 / ((1 + bias) * (1 + bias));
        }
        const double slow = alpha * torque_t, fast = torque_t - slow;
        rear_slow = fabs(w1) < fabs(w0) ? 1.0 : 0.0;
        ta[1].engTor = rear_slow != 0.0 ? slow : fast;
        ta[0].engTor = rear_slow != 0.0 ? fast : slow;
    } else if (C.whichWheels) {
        ta[1].engTor = torque_t;
        ta[0].engTor = 0;
    } else {
        ta[1].engTor = 0;
        ta[0].engTor = torque_t;
    }
    T.at(TS_(alf)) = alpha;
    T.at(TS_(dalf)) = dal;
    T.at(TS_(slowf)) = rear_slow;
    // wheel accelerations, front forces into the vehicle frame, chassis
    const double brake = K(K_MAXBRAKE) * braking, ijw = K(K_INVJW);
#pragma unroll
    for (int k = 0; k < 2; ++k)
        ta[k].dOmega = ijw * (fma(-sgnd(ts[k].omega), brake, ta[k].engTor + ta[k].My) - ta[k].fx * ta[k].rStat);
    {
        const double fx = ta[0].fx, fy = ta[0].fy;
        ta[0].fx = fma(fx, cd, -fy * sd);
        ta[0].fy = fma(fx, sd, fy * cd);
    }
    const double im = K(K_INVMT);
    v.vdot = fma(-v.u, v.wz, (ta[0].fy + ta[1].fy) * im);
    v.udot = fma(v.v, v.wz, (ta[0].fx + ta[1].fx) * im);
    va.wzdot = fma(K(K_A), ta[0].fy, -K(K_B) * ta[1].fy) * K(K_INVJZ);
}

// Reverse of fwd11_tape: from the adjoints of the right-hand-side outputs to those of the packed
// states and the controls. Lifted wheels (xe, ye, omega zeroed by the tire) pass nothing back.
template <bool kNr>
__device__ __forceinline__ void rev11_rhs(const TapeRef& T, const KView& K, const ClassDev18& C, const KBar& kb,
                                          double udotb, double vdotb, double wzdotb, double dOcb, const double* dOmb,
                                          const double* xedotb, const double* yedotb, double& ub, double& vb,
                                          double& wzb, double& crankb, double* xeb, double* yeb, double* omb,
                                          double& steerb, double& thrb) {
    const int g = (int)T.at(TS_(gear));
    const double u = T.at(TS_(u)), vv = T.at(TS_(v)), wz = T.at(TS_(wz));
    const double cd = T.at(TS_(cd)), sd = T.at(TS_(sd));
    const double im = K(K_INVMT), ijz = K(K_INVJZ);
    // computeVehRHS
    vb = fma(wz, udotb, vb);
    wzb = fma(vv, udotb, fma(-u, vdotb, wzb));
    ub = fma(-wz, vdotb, ub);
    double fxrb[2] = {im * udotb, im * udotb};
    double fyrb[2] = {fma(K(K_A) * ijz, wzdotb, im * vdotb), fma(-K(K_B) * ijz, wzdotb, im * vdotb)};
    // front forces rotated into the vehicle frame
    double fxb[2], fyb[2], cdb = 0, sdb = 0;
    {
        const double fx = tire_ref(T, 0).at(TT_(fx)), fy = tire_ref(T, 0).at(TT_(fy));
        fxb[0] = fma(cd, fxrb[0], sd * fyrb[0]);
        fyb[0] = fma(-sd, fxrb[0], cd * fyrb[0]);
        cdb = fma(fx, fxrb[0], fy * fyrb[0]);
        sdb = fma(-fy, fxrb[0], fx * fyrb[0]);
        fxb[1] = fxrb[1];
        fyb[1] = fyrb[1];
    }
    // wheel accelerations
    double Myb[2], rStatb[2], engb[2], om_mid[2], om_midb[2] = {0, 0};
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        om_mid[k] = tire_ref(T, k).at(TT_(on)) != 0.0 ? tire_ref(T, k).at(TT_(om)) : 0.0;
        const double gk = K(K_INVJW) * dOmb[k];
        engb[k] = gk;
        Myb[k] = gk;
        fxb[k] = fma(-tire_ref(T, k).at(TT_(rStat)), gk, fxb[k]);
        rStatb[k] = -tire_ref(T, k).at(TT_(fx)) * gk;
    }
    // differential
    double torque_tb;
    if (C.driveType) {
        const bool rear_slow = T.at(TS_(slowf)) != 0.0;
        const double alpha = T.at(TS_(alf)), dal = T.at(TS_(dalf));
        const double slowb = rear_slow ? engb[1] : engb[0];
        const double fastb = rear_slow ? engb[0] : engb[1];
        const double diffb = dal * T.at(TS_(torque_t)) * (slowb - fastb);
        if (diffb != 0.0) {  // diff = |w1 - w0|
            const double sg = (om_mid[1] - om_mid[0]) >= 0 ? 1.0 : -1.0;
            om_midb[1] = fma(sg, diffb, om_midb[1]);
            om_midb[0] -= sg * diffb;
        }
        torque_tb = fma(alpha, slowb, (1.0 - alpha) * fastb);
    } else {
        torque_tb = C.whichWheels ? engb[1] : engb[0];
    }
    if (T.at(TS_(tclip)) != 0.0) torque_tb = 0;
    // powertrain
    if (C.tcbool) {
        const double torque_outb = C.invgear[g] * torque_tb;
        double torque_inb = 0, trb = 0;
        if (T.at(TS_(rev)) != 0.0) {
            torque_inb = -torque_outb;
        } else {
            trb = -T.at(TS_(torque_in)) * torque_outb;
            torque_inb = -T.at(TS_(tr)) * torque_outb;
        }
        const double dtqb = K(K_INVCI) * dOcb;
        torque_inb = fma(K(K_INVCI), dOcb, torque_inb);
        thrb = fma(T.at(TS_(dt_map)), dtqb, thrb);
        crankb = fma(T.at(TS_(dt_slope)), dtqb, crankb);
        const double rb = (T.at(TS_(rev)) != 0.0 ? 2.0 * T.at(TS_(r)) : -2.0 * T.at(TS_(r))) * torque_inb;
        const double icf = 1.0 / T.at(TS_(cf));
        double omega_inb = rb * icf;
        const double cfb = -T.at(TS_(r)) * icf * rb;
        const double srb = fma(T.at(TS_(cfs)), cfb, T.at(TS_(trs)) * trb);
        double omega_outb = 0;
        if (T.at(TS_(srmode)) != 0.0) {
            const double sr0b = T.at(TS_(rev)) != 0.0 ? -srb : srb;
            const double iin = 1.0 / T.at(TS_(omega_in));
            omega_outb = sr0b * iin;
            omega_inb = fma(-T.at(TS_(omega_out)) * iin * iin, sr0b, omega_inb);
        }
        const double wb = 0.5 * omega_outb / C.gear[g];
        om_midb[0] += wb;
        om_midb[1] += wb;
        crankb += omega_inb;
    } else {
        const double dtqb = C.invgear[g] * torque_tb;
        thrb = fma(T.at(TS_(dt_map)), dtqb, thrb);
        const double wb = 0.5 * T.at(TS_(dt_slope)) * dtqb / C.gear[g];
        om_midb[0] += wb;
        om_midb[1] += wb;
    }
    // tires
    double vsxinb[2] = {0, 0}, vsyb[2] = {0, 0}, fzb[2] = {0, 0};
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        xeb[k] = yeb[k] = omb[k] = 0;
        if (tire_ref(T, k).at(TT_(on)) == 0.0) continue;
        double xk = 0, yk = 0, ok = om_midb[k];
        if (kNr) {
            if (k == 0)
                tire_rev_nr<true>(tire_ref(T, 0), K, kb, fxb[0], fyb[0], Myb[0], rStatb[0], ok, vsxinb[0], vsyb[0],
                                  fzb[0], cdb, sdb, cd, sd);
            else {
                double cdum = 0, sdum = 0;
                tire_rev_nr<false>(tire_ref(T, 1), K, kb, fxb[1], fyb[1], Myb[1], rStatb[1], ok, vsxinb[1], vsyb[1],
                                   fzb[1], cdum, sdum, 1.0, 0.0);
            }
        } else if (k == 0) {
            tire_rev<true>(tire_ref(T, 0), K, kb, xedotb[0], yedotb[0], fxb[0], fyb[0], Myb[0], rStatb[0], xk, yk, ok,
                           vsxinb[0], vsyb[0], fzb[0], cdb, sdb, cd, sd);
        } else {
            double cdum = 0, sdum = 0;
            tire_rev<false>(tire_ref(T, 1), K, kb, xedotb[1], yedotb[1], fxb[1], fyb[1], Myb[1], rStatb[1], xk, yk, ok,
                            vsxinb[1], vsyb[1], fzb[1], cdum, sdum, 1.0, 0.0);
        }
        xeb[k] = xk;
        yeb[k] = yk;
        omb[k] = ok;
    }
    // contact-patch velocities: vsx0 = u cd + vsyf sd, vsy0 = vsyf = v + wz a; vsx1 = u, vsy1 = v - wz b
    {
        const double vsyfb = fma(sd, vsxinb[0], vsyb[0]);
        sdb = fma(T.at(TS_(vsyf)), vsxinb[0], sdb);
        cdb = fma(u, vsxinb[0], cdb);
        ub += fma(cd, vsxinb[0], vsxinb[1]);
        wzb = fma(K(K_A), vsyfb, fma(-K(K_B), vsyb[1], wzb));
        vb += vsyfb + vsyb[1];
    }
    // wheel angle
    steerb = fma(T.at(TS_(dslope)), fma(cd, sdb, -sd * cdb), steerb);
    // axle loads: fz0 = max(Z1F - Z4 lon, 0), fz1 = max(Z1R + Z4 lon, 0), lon = udot - wz v
    {
        const double g0 = T.at(TS_(fzarg) + 0) > 0 ? 1.0 : 0.0, g1 = T.at(TS_(fzarg) + 1) > 0 ? 1.0 : 0.0;
        const double lonb = K(K_Z4) * fma(-fzb[0], g0, fzb[1] * g1);
        wzb = fma(-vv, lonb, wzb);
        vb = fma(-wz, lonb, vb);
    }
}

template <bool kNr>
__global__ void __launch_bounds__(128) rhs_jacobian11_kernel(const JacLaunch A) {
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

    Veh11 v;
    Veh11Aux va;
    TireC ts[2];
    TireAux ta[2];
    load_state11(A.S + vid, np, v, va, ts, ta);
    if (A.reference_point) {  // PerturbRhsFun's freshly constructed states holding the packed ones
        v.udot = 0.0;
        v.vdot = 0.0;
        v.gear = 0;
        if (!C.tcbool) v.crank = 0.0;
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            ts[k].xedot = 0.0;
            ts[k].yedot = 0.0;
        }
    }
    const double psi = v.psi, u = v.u, vv = v.v;
    const double steer = __ldg(A.ctl + vid), thr = __ldg(A.ctl + nu + vid), brk = __ldg(A.ctl + 2 * nu + vid);
    const TapeRef T{A.tape + vid, np};
    T.at(TS_(gear)) = (double)v.gear;
    fwd11_tape<kNr>(v, va, ts, ta, T, K, C, steer, thr, brk);

    const bool tc = C.tcbool != 0;
    const int nt = kNr ? 0 : 4;                                  // deflection states before the wheel speeds
    const int ny = nt + (tc ? 9 : 8), o = nt + (tc ? 3 : 2);     // o: index of x in the packed vector
    auto J = [&](int r, int c) -> double& { return A.jac_state[((size_t)r * ny + c) * nu + vid]; };
    auto Ju = [&](int r, int c) -> double& { return A.jac_ctl[((size_t)r * 2 + c) * nu + vid]; };
    for (int r = 0; r < ny; ++r) {
        if (r == o || r == o + 1 || r == o + 4) {  // dx, dy, dpsi
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
            } else {  // dpsi = wz
                J(r, o + 5) = 1.0;
            }
            continue;
        }
        double udotb = 0, vdotb = 0, wzdotb = 0, dOcb = 0;
        double dOmb[2] = {0, 0}, xedotb[2] = {0, 0}, yedotb[2] = {0, 0};
        if (r < nt) (r & 1 ? yedotb : xedotb)[r >> 1] = 1.0;
        else if (r < nt + 2) dOmb[r - nt] = 1.0;
        else if (tc && r == nt + 2) dOcb = 1.0;
        else if (r == o + 2) udotb = 1.0;
        else if (r == o + 3) vdotb = 1.0;
        else wzdotb = 1.0;  // r == o + 5
        double ub = 0, vb = 0, wzb = 0, crankb = 0, steerb = 0, thrb = 0;
        double xeb[2], yeb[2], omb[2];
        rev11_rhs<kNr>(T, K, C, kb, udotb, vdotb, wzdotb, dOcb, dOmb, xedotb, yedotb, ub, vb, wzb, crankb, xeb, yeb,
                       omb, steerb, thrb);
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            if (!kNr) {
                J(r, 2 * k) = xeb[k];
                J(r, 2 * k + 1) = yeb[k];
            }
            J(r, nt + k) = omb[k];
        }
        if (tc) J(r, nt + 2) = crankb;
        J(r, o) = 0.0;      // x
        J(r, o + 1) = 0.0;  // y
        J(r, o + 2) = ub;
        J(r, o + 3) = vb;
        J(r, o + 4) = 0.0;  // psi enters only dx and dy
        J(r, o + 5) = wzb;
        Ju(r, 0) = steerb;
        Ju(r, 1) = thrb;
    }
}

}  // namespace

cudaError_t launch_rhs_jacobian11(const JacLaunch& A, cudaStream_t stream) {
    if (A.n <= 0) return cudaSuccess;
    constexpr int threads = 128;
    JacLaunch L = A;
    const size_t smem = jac18_smem(threads, A.nclasses, &L.cls_smem);
    auto kern = A.tire_nr ? rhs_jacobian11_kernel<true> : rhs_jacobian11_kernel<false>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<(A.n + threads - 1) / threads, threads, smem, stream>>>(L);
    return cudaGetLastError();
}

}  // namespace lfdm
