// 11-DOF (single-track) model: right-hand side and half-implicit update of one vehicle.
//
// Algorithm: rhsFun (11dof-gpu/dof11_halfImplicit_gpu.cu:663-700) and the Integrate update
// (:855-880) with the physics of 11dof-gpu/dof11_gpu.cu, whose tire model, tmxy_combined, driveTorque
// and lookups are the 18-DOF ones (shared here through dof18_device.cuh). The front lateral force
// is rotated into the vehicle frame (11dof/dof11.cpp:100-124, 11dof-gpu/dof11_gpu.cu:98-123).
// Derived constants come from the same prepare kernel
// as the 18-DOF model (K_Z1F, K_Z4 and K_Z1R are exactly the 11-DOF axle-load terms).
#pragma once

#include "dof18_device.cuh"

namespace lfdm {

struct Veh11 {
    double x, y, u, v, psi, wz, udot, vdot, crank;
    int gear;
};
struct Veh11Aux {
    double wzdot, dOmega_crank;
};

// differentialSplit (11dof-gpu/dof11_gpu.cu:276-315), max_bias = 2
__device__ __forceinline__ void diff_split11(double torque, double w_rear, double w_front, double& t_rear,
                                             double& t_front, int split, int whichWheels) {
    if (split) {
        const double diff = fabs(w_rear - w_front);
        double alpha;
        if (diff > 0.5) alpha = 2.0 / 3.0;
        else if (diff > 0.25) {
            const double bias = 4 * (2.0 - 1) * diff + (2 - 2.0);
            alpha = bias / (1 + bias);
        } else alpha = 0.5;
        const double slow = alpha * torque;
        const double fast = torque - slow;
        if (fabs(w_rear) < fabs(w_front)) {
            t_rear = slow;
            t_front = fast;
        } else {
            t_rear = fast;
            t_front = slow;
        }
    } else if (whichWheels) {
        t_rear = torque;
        t_front = 0;
    } else {
        t_rear = 0;
        t_front = torque;
    }
}

// The right-hand side in the phases a step can be split into (the split-warp kernel runs the tire
// phases of one vehicle on two warps): loads and contact-patch velocities, the tires, the
// powertrain (which reads the wheel speeds the tires leave: zero for a wheel off the ground),
// wheel accelerations and the chassis.

// computeTireLoads (dof11_gpu.cu:234-252)
__device__ __forceinline__ void loads11(const Veh11& v, TireAux* ta, const KView& K) {
    const double Z2 = K(K_Z4) * fma(-v.wz, v.v, v.udot);
    ta[0].fz = pos_part(K(K_Z1F) - Z2);
    ta[1].fz = pos_part(K(K_Z1R) + Z2);
}
// vehToTireTransform (dof11_gpu.cu:41-68), front tire: wheel angle, its cosine and sine
__device__ __forceinline__ void front_kinematics11(const Veh11& v, TireAux& ta, const KView& K, const ClassDev18& C,
                                                   double steering, double& cd, double& sd) {
    const double delta = C.nonLinearSteer ? map_y(C.steer, steering) : steering * K(K_MAXSTEER);
    cd = 1.0;
    sd = 0.0;
    if (!is_zero(delta)) sincos(delta, &sd, &cd);
    const double vsyf = fma(v.wz, K(K_A), v.v);
    ta.vsy = vsyf;
    ta.vsx = fma(v.u, cd, vsyf * sd);
}
__device__ __forceinline__ void rear_kinematics11(const Veh11& v, TireAux& ta, const KView& K) {
    ta.vsy = fma(-v.wz, K(K_B), v.v);
    ta.vsx = v.u;
}
template <bool kNr, bool kSteered, bool kF32 = false>
__device__ __forceinline__ void tire11(TireC& ts, TireAux& ta, const KView& K, double cd, double sd) {
    if (kNr) tire_rhs_nr<kSteered, kF32>(ts, ta, K, cd, sd);  // computeTireRHS, TMeasyNr (dof11_gpu.cu:470-599)
    else tire_rhs_tm<kSteered, kF32>(ts, ta, K, cd, sd);
}
// computePowertrainRHS (dof11_gpu.cu:601-745) up to the wheel torques: converter, engine, gear,
// differential. w0, w1: the front and rear wheel speeds after the tires.
__device__ __forceinline__ void powertrain11(Veh11& v, Veh11Aux& va, double w0, double w1, double& eng0, double& eng1,
                                             const KView& K, const ClassDev18& C, double throttle) {
    double torque_t;
    const int g = v.gear;
    if (C.tcbool) {
        bool reverse = false;
        const double omega_out = 0.5 * (w0 + w1) / C.gear[g];
        const double omega_in = v.crank;
        double sr = 0;
        if (!(lt_(omega_out, 1e-9) || lt_(omega_in, 1e-9))) {
            sr = omega_out / omega_in;
            if (gt_nn(sr, 1.)) {
                sr = 1. - (sr - 1.);
                reverse = true;
            }
            if (lt_(sr, 0.0)) sr = 0;
        }
        const double cf = map_y(C.cf, sr), tr = map_y(C.tr, sr);
        const double r = omega_in / cf;
        double torque_in = -(r * r);
        if (reverse) torque_in = -torque_in;
        const double torque_out = reverse ? -torque_in : -tr * torque_in;
        torque_t = torque_out * C.invgear[g];
        if (lt_(v.u, 1e-9) && lt_(torque_t, 0.0)) torque_t = 0;
        va.dOmega_crank = K(K_INVCI) * (drive_torque(C, throttle, v.crank) + torque_in);
        if (lt_(C.up[g], omega_out)) {
            if (g < C.noGears - 1) v.gear = g + 1;
        } else if (lt_(omega_out, C.down[g])) {
            if (g > 0) v.gear = g - 1;
        }
    } else {
        v.crank = 0.5 * (w0 + w1) / C.gear[g];
        torque_t = drive_torque(C, throttle, v.crank) * C.invgear[g];
        if (lt_(v.u, 1e-9) && lt_(torque_t, 0.0)) torque_t = 0;
        if (lt_(C.up[g], v.crank)) {
            if (g < C.noGears - 1) v.gear = g + 1;
        } else if (lt_(v.crank, C.down[g])) {
            if (g > 0) v.gear = g - 1;
        }
    }
    diff_split11(torque_t, w1, w0, eng1, eng0, C.driveType, C.whichWheels);
}
// wheel accelerations, tireToVehTransform (11dof/dof11.cpp:100-124: both front forces rotated) and
// computeVehRHS (dof11_gpu.cu:893-909)
__device__ __forceinline__ void chassis11(Veh11& v, Veh11Aux& va, const TireC* ts, TireAux* ta, const KView& K,
                                          double braking, double cd, double sd) {
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

// One right-hand-side evaluation (rhsFun, 11dof-gpu/dof11_halfImplicit_gpu.cu:663-700).
template <bool kNr, bool kF32 = false>
__device__ __forceinline__ void rhs11(Veh11& v, Veh11Aux& va, TireC* ts, TireAux* ta, const KView& K,
                                      const ClassDev18& C, double steering, double throttle, double braking) {
    loads11(v, ta, K);
    double cd, sd;
    front_kinematics11(v, ta[0], K, C, steering, cd, sd);
    rear_kinematics11(v, ta[1], K);
    tire11<kNr, true, kF32>(ts[0], ta[0], K, cd, sd);
    tire11<kNr, false, kF32>(ts[1], ta[1], K, 1.0, 0.0);
    powertrain11(v, va, ts[0].omega, ts[1].omega, ta[0].engTor, ta[1].engTor, K, C, throttle);
    chassis11(v, va, ts, ta, K, braking, cd, sd);
}

// The half-implicit update (dof11_halfImplicit_gpu.cu:863-880) with the rates of rhs11, given the
// sine and cosine of the yaw angle before the step.
template <bool kNr>
__device__ __forceinline__ void update11_sc(Veh11& v, const Veh11Aux& va, TireC* ts, const TireAux* ta,
                                            const ClassDev18& C, double dt, double sp, double cp) {
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        if (!kNr) {  // the TMeasyNr tire has no deflection states
            ts[k].xe = fma(ts[k].xedot, dt, ts[k].xe);
            ts[k].ye = fma(ts[k].yedot, dt, ts[k].ye);
        }
        ts[k].omega = fma(ta[k].dOmega, dt, ts[k].omega);
    }
    if (C.tcbool) v.crank = fma(va.dOmega_crank, dt, v.crank);
    v.u = fma(v.udot, dt, v.u);
    v.v = fma(v.vdot, dt, v.v);
    v.wz = fma(va.wzdot, dt, v.wz);
    v.x = fma(fma(v.u, cp, -v.v * sp), dt, v.x);
    v.y = fma(fma(v.u, sp, v.v * cp), dt, v.y);
    v.psi = fma(v.wz, dt, v.psi);
}
template <bool kNr>
__device__ __forceinline__ void update11(Veh11& v, const Veh11Aux& va, TireC* ts, const TireAux* ta,
                                         const ClassDev18& C, double dt) {
    double sp, cp;
    sincos(v.psi, &sp, &cp);
    update11_sc<kNr>(v, va, ts, ta, C, dt, sp, cp);
}

// One step: rhs11 followed by update11.
template <bool kNr, bool kF32 = false>
__device__ __forceinline__ void step11(Veh11& v, Veh11Aux& va, TireC* ts, TireAux* ta, const KView& K,
                                       const ClassDev18& C, double steering, double throttle, double braking,
                                       double dt) {
    rhs11<kNr, kF32>(v, va, ts, ta, K, C, steering, throttle, braking);
    update11<kNr>(v, va, ts, ta, C, dt);
}

// The 11-DOF state of one vehicle from its SoA column S (S[field * np]).
__device__ __forceinline__ void load_state11(const double* S, size_t np, Veh11& v, Veh11Aux& va, TireC* ts,
                                             TireAux* ta) {
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
}

__device__ __forceinline__ void store_state11(double* S, size_t np, const Veh11& v, const Veh11Aux& va,
                                              const TireC* ts, const TireAux* ta) {
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
}
__device__ __forceinline__ bool state11_finite(const Veh11& v, const TireC* ts) {
    return isfinite(v.x) && isfinite(v.y) && isfinite(v.u) && isfinite(v.v) && isfinite(v.psi) && isfinite(v.wz) &&
           isfinite(ts[0].omega) && isfinite(ts[1].omega);
}

}  // namespace lfdm
