// 24-DOF vehicle model: device-side constants, carried state and the right-hand side +
// half-implicit update (used by the window kernel in kernels24.cu and the fleet kernel in fleet.cu).
//
// Algorithm: rhsFun (24dof-gpu/dof24_halfImplicit_gpu.cu:728-775) and the Integrate update
// (:1016-1081) with the physics of 24dof-gpu/dof24_gpu.cu; see kernels24.cu for the data layout
// and what is carried across steps.
#pragma once

#include "dof18_device.cuh"

namespace lfdm {

// Derived per-vehicle constants of the 24-DOF model: the shared tire/powertrain prefix of K18
// followed by these.
enum K24 : int {
    K24_A = KT_COUNT, K24_B, K24_CF2, K24_CR2, K24_KT,
    K24_MUF, K24_MUR, K24_INVMUF, K24_INVMUR, K24_MUFG, K24_MURG,
    K24_KS, K24_BS, K24_HRCF, K24_HRCR, K24_INVCF, K24_INVCR,
    K24_INVM, K24_INVJX, K24_INVJY, K24_INVJZ,
    K24_COUNT
};

// Derived constants of one vehicle from its flat parameter vector p (shared prefix + K24).
template <typename Put>
__device__ __forceinline__ void prepare_k24(const double* p, Put& put) {
    prepare_shared_k(p, put);
    put(K24_A, p[LFDM_P_A]);
    put(K24_B, p[LFDM_P_B]);
    put(K24_CF2, p[LFDM_P_CF] / 2.);
    put(K24_CR2, p[LFDM_P_CR] / 2.);
    put(K24_KT, p[LFDM_P_KT]);
    put(K24_MUF, p[LFDM_P_MUF]);
    put(K24_MUR, p[LFDM_P_MUR]);
    put(K24_INVMUF, 1 / p[LFDM_P_MUF]);
    put(K24_INVMUR, 1 / p[LFDM_P_MUR]);
    put(K24_MUFG, p[LFDM_P_MUF] * kG);
    put(K24_MURG, p[LFDM_P_MUR] * kG);
    put(K24_KS, p[LFDM_P_KS]);
    put(K24_BS, p[LFDM_P_BS]);
    put(K24_HRCF, p[LFDM_P_HRCF]);
    put(K24_HRCR, p[LFDM_P_HRCR]);
    put(K24_INVCF, 1 / p[LFDM_P_CF]);
    put(K24_INVCR, 1 / p[LFDM_P_CR]);
    put(K24_INVM, 1 / p[LFDM_P_M]);
    put(K24_INVJX, 1 / p[LFDM_P_JX]);
    put(K24_INVJY, 1 / p[LFDM_P_JY]);
    put(K24_INVJZ, 1 / p[LFDM_P_JZ]);
}

// Chassis coordinates the 18-DOF VehC does not hold.
struct Veh24X {
    double w, theta, wy, wxdot, wydot, wzdot;
};
// Carried suspension state of one corner.
struct Sus24C {
    double xs, dxs, wu, fzd;
};
// Per-corner constants of the state (initial spring compression and strut length, road vertical
// speed), read once per window.
struct Corner24K {
    double xsi, lsi, vsz;
};

#define SINK(field, value)                           \
    do {                                             \
        if (sink) S[(size_t)(field) * np] = (value); \
    } while (0)

// Rates of one right-hand-side evaluation that are not held in the carried state, with the pitch
// and roll sines and cosines the update reuses.
struct Rhs24 {
    double dxt[4], dwu[4], wdot, sth, cth, sph, cph;
};

// One right-hand-side evaluation (rhsFun, 24dof-gpu/dof24_halfImplicit_gpu.cu:728-775). sink: also
// write the step's non-carried values to S. The flag is a run-time value on purpose: every step runs
// the same compiled arithmetic (a separate instantiation for storing steps could fuse multiplies
// and adds differently and round differently).
template <bool kNr, bool kF32 = false>
__device__ __forceinline__ void rhs24(VehC& v, Veh24X& vx, VehAux& va, TireC* ts, TireAux* ta, Sus24C* su,
                                      const Corner24K* ck, const KView& K, const ClassDev18& C, double steering,
                                      double throttle, double braking, Rhs24& R, double* S, size_t np, bool sink) {
    const double cf2 = K(K24_CF2), cr2 = K(K24_CR2), a = K(K24_A), b = K(K24_B);
    double sth, cth, sph, cph;
    sincos(vx.theta, &sth, &cth);
    sincos(v.phi, &sph, &cph);
    // vehToSusTransform (dof24_gpu.cu; CPU 24dof/dof24.cpp:148-229): corner offsets (x, y) =
    // LF (a, cf/2), RF (a, -cf/2), LR (-b, cr/2), RR (-b, -cr/2) as lateral sign terms below.
    double uu[4], vu[4], ws[4], ls[4], duu[4], dvu[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const double lat = c == 0 ? -cf2 : c == 1 ? cf2 : c == 2 ? -cr2 : cr2;  // x-velocity term * wz
        const double lon = c < 2 ? a : -b;
        const double us = fma(lat, v.wz, v.u);
        const double vs = fma(lon, v.wz, v.v);
        ws[c] = fma(-lat, v.wx, fma(-lon, vx.wy, vx.w));
        ls[c] = ck[c].lsi - (su[c].xs - ck[c].xsi);
        uu[c] = fma(-ls[c], vx.wy, us);
        vu[c] = fma(ls[c], v.wx, vs);
        const double dus = fma(lat, vx.wzdot, v.udot);
        const double dvs = fma(lon, vx.wzdot, v.vdot);
        duu[c] = dus - fma(-su[c].dxs, vx.wy, ls[c] * vx.wydot);
        dvu[c] = dvs + fma(-su[c].dxs, v.wx, ls[c] * vx.wxdot);
        const int sb = LFDM24_S_SUS0 + c * LFDM24_SUS_COUNT;
        SINK(sb + LFDM24_SUS_LS, ls[c]);
        SINK(sb + LFDM24_SUS_US, us);
        SINK(sb + LFDM24_SUS_VS, vs);
        SINK(sb + LFDM24_SUS_WS, ws[c]);
        SINK(sb + LFDM24_SUS_DUS, dus);
        SINK(sb + LFDM24_SUS_DVS, dvs);
        SINK(sb + LFDM24_SUS_UU, uu[c]);
        SINK(sb + LFDM24_SUS_VU, vu[c]);
        SINK(sb + LFDM24_SUS_DUU, duu[c]);
        SINK(sb + LFDM24_SUS_DVU, dvu[c]);
    }
    // vehToTireTransform: contact-patch velocities through pitch and roll (uses the previous rStat)
    double delta;
    if (C.nonLinearSteer) delta = map_y(C.steer, steering);
    else delta = steering * K(K_MAXSTEER);
    double cd = 1.0, sd = 0.0;
    if (!is_zero(delta)) sincos(delta, &sd, &cd);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const double r = ta[c].rStat;
        const double vgx = fma(cth, fma(-vx.wy, r, uu[c]), sth * fma(su[c].wu, cph, sph * fma(v.wx, r, vu[c])));
        const double vgy = fma(cph, fma(v.wx, r, vu[c]), -su[c].wu * sph);
        ta[c].vsy = vgy;
        ta[c].vsx = c < 2 ? fma(vgx, cd, vgy * sd) : vgx;
        const int tb = LFDM24_S_TIRE0 + c * LFDM24_T_COUNT;
        SINK(tb + LFDM24_T_VGX, vgx);
        SINK(tb + LFDM24_T_VGY, vgy);
    }
    // computeTireRHS (TMeasy): load from the compression, loaded radius through pitch and roll
    const double icc = 1.0 / (cth * cph);
    const double r0 = K(K_R0), kt = K(K24_KT);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const double xt = ta[c].xt;
        const double fz = xt * kt;
        ta[c].fz = fz;
        ta[c].rStat = (r0 - xt) * icc;
        if (!gt0(fz)) {
            if (!kNr) {
                ts[c].xe = 0;
                ts[c].ye = 0;
            }
            ts[c].omega = 0;
            ta[c].xt = 0;
            ta[c].rStat = r0;
            ta[c].fz = 0;
            ta[c].fx = 0;
            ta[c].fy = 0;
            ta[c].My = 0;
        } else {
            const double rs = ta[c].rStat;
            const double rdynco =
                !gt_nn(fz, K(K_FZRD)) ? fma(K(K_DRD), fma(fz, K(K_INVPN), -1.0), K(K_RDPN)) : K(K_RDCRIT);
            const double r_eff = fma(rdynco, r0 - rs, rs);
            if (kNr) {  // computeTireRHS, TMeasyNr (24dof-gpu/dof24_gpu.cu:990-1119)
                if (c < 2) tire_core_nr_p<true, kF32>(ts[c], ta[c], K, cd, sd, fz, r_eff);
                else tire_core_nr_p<false, kF32>(ts[c], ta[c], K, 1.0, 0.0, fz, r_eff);
            } else {
                if (c < 2) tire_core_tm_p<true, kF32>(ts[c], ta[c], K, cd, sd, fz, r_eff);
                else tire_core_tm_p<false, kF32>(ts[c], ta[c], K, 1.0, 0.0, fz, r_eff);
            }
        }
    }
    // computeTireCompressionVelocity
    double dxt[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        dxt[c] = ck[c].vsz - fma(cth, fma(su[c].wu, cph, vu[c] * sph), -uu[c] * sth);
        SINK(LFDM24_S_TIRE0 + c * LFDM24_T_COUNT + LFDM24_T_DXT, dxt[c]);
    }
    // computePowertrainRHS (the 18-DOF powertrain; reads the unrotated fx)
    powertrain_rhs<false>(v, va, ts, ta, K, C, throttle, braking);
    // tireToVehTransform: front forces rotated by the wheel angle and stored, then all four into the
    // chassis frame
    double fxg[4], fyg[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        if (c < 2) {
            const double fx = ta[c].fx, fy = ta[c].fy;
            ta[c].fx = fma(fx, cd, -fy * sd);
            ta[c].fy = fma(fx, sd, fy * cd);
        }
        const double fx = ta[c].fx, fy = ta[c].fy, fz = ta[c].fz;
        fxg[c] = fma(fx, cth, -fz * sth);
        fyg[c] = fma(fx * sph, sth, fma(fy, cph, fz * sph * cth));
        const int tb = LFDM24_S_TIRE0 + c * LFDM24_T_COUNT;
        SINK(tb + LFDM24_T_FXG, fxg[c]);
        SINK(tb + LFDM24_T_FYG, fyg[c]);
        SINK(tb + LFDM24_T_FZG, fma(fx * sth, cph, fma(-fy, sph, fz * cph * cth)));
    }
    // computeSusRHS: unsprung vertical acceleration with the previous fzd and dxs, then the new dxs
    const double ks = K(K24_KS), bs = K(K24_BS);
    double dwu[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const double mu = c < 2 ? K(K24_MUF) : K(K24_MUR);
        const double imu = c < 2 ? K(K24_INVMUF) : K(K24_INVMUR);
        const double muG = c < 2 ? K(K24_MUFG) : K(K24_MURG);
        const double inner = fma(cph, fma(cth, ta[c].fz - muG, sth * ta[c].fx), -sph * ta[c].fy);
        const double rest = fma(su[c].xs, ks, su[c].dxs * bs) + su[c].fzd;
        dwu[c] = imu * (inner - rest - mu * fma(vu[c], v.wx, -uu[c] * vx.wy));
        su[c].dxs = su[c].wu - ws[c];
        SINK(LFDM24_S_SUS0 + c * LFDM24_SUS_COUNT + LFDM24_SUS_DWU, dwu[c]);
    }
    // computeForcesThroughSus (the rear-right lateral force without cos(theta), as in the reference)
    double fxs[4], fys[4], fzs[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const double mu = c < 2 ? K(K24_MUF) : K(K24_MUR);
        const double muG = c < 2 ? K(K24_MUFG) : K(K24_MURG);
        fxs[c] = fma(muG, sth, fxg[c]) + mu * (fma(v.wz, vu[c], -duu[c]) - vx.wy * su[c].wu);
        const double gl = c < 3 ? muG * sph * cth : muG * sph;
        fys[c] = (fyg[c] - gl) + mu * (fma(v.wx, su[c].wu, -dvu[c]) - v.wz * uu[c]);
        fzs[c] = fma(su[c].xs, ks, su[c].dxs * bs);
    }
    const double hrcf = K(K24_HRCF), hrcr = K(K24_HRCR);
    const double fzd_f = (fma(fyg[1], ta[1].rStat, fys[1] * ls[1]) + fma(fyg[0], ta[0].rStat, fys[0] * ls[0]) -
                          (fys[1] + fys[0]) * hrcf) * K(K24_INVCF);
    const double fzd_r = (fma(fyg[3], ta[3].rStat, fys[3] * ls[3]) + fma(fyg[2], ta[2].rStat, fys[2] * ls[2]) -
                          (fys[3] + fys[2]) * hrcr) * K(K24_INVCR);
    su[0].fzd = -fzd_f;
    su[1].fzd = fzd_f;
    su[2].fzd = -fzd_r;
    su[3].fzd = fzd_r;
    double mx[4], my[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        mx[c] = fys[c] * (c < 2 ? hrcf : hrcr);
        my[c] = -fma(fxg[c], ta[c].rStat, fxs[c] * ls[c]);
        const int sb = LFDM24_S_SUS0 + c * LFDM24_SUS_COUNT;
        SINK(sb + LFDM24_SUS_FXS, fxs[c]);
        SINK(sb + LFDM24_SUS_FYS, fys[c]);
        SINK(sb + LFDM24_SUS_FZS, fzs[c]);
        SINK(sb + LFDM24_SUS_MX, mx[c]);
        SINK(sb + LFDM24_SUS_MY, my[c]);
        SINK(sb + LFDM24_SUS_MZ, 0.0);
    }
    // computeVehicleRHS: 6-DOF chassis
    const double im = K(K24_INVM);
    const double sfx = ((fxs[0] + fxs[1]) + fxs[2]) + fxs[3];
    const double sfy = ((fys[0] + fys[1]) + fys[2]) + fys[3];
    const double sfz = ((((((fzs[0] + fzs[1]) + fzs[2]) + fzs[3]) + su[0].fzd) + su[1].fzd) + su[2].fzd) + su[3].fzd;
    v.udot = fma(v.wz, v.v, -vx.wy * vx.w) + fma(im, sfx, kG * sth);
    v.vdot = fma(v.wx, vx.w, -v.wz * v.u) + fma(im, sfy, -kG * sph * cth);
    const double wdot = fma(vx.wy, v.u, -v.wx * v.v) + fma(im, sfz, -kG * cph * cth);
    vx.wxdot = K(K24_INVJX) * ((((mx[0] + mx[1]) + mx[2]) + mx[3]) + fma(fzs[0] - fzs[1], cf2, (fzs[2] - fzs[3]) * cr2));
    vx.wydot = K(K24_INVJY) * ((((my[0] + my[1]) + my[2]) + my[3]) + fma(fzs[2] + fzs[3], b, -(fzs[0] + fzs[1]) * a));
    vx.wzdot = K(K24_INVJZ) * fma(fys[0] + fys[1], a, fma(-(fys[2] + fys[3]), b,
                                                        fma(fxs[1] - fxs[0], cf2, (fxs[3] - fxs[2]) * cr2)));
    SINK(LFDM24_S_WDOT, wdot);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        R.dxt[c] = dxt[c];
        R.dwu[c] = dwu[c];
    }
    R.wdot = wdot;
    R.sth = sth;
    R.cth = cth;
    R.sph = sph;
    R.cph = cph;
}

// The half-implicit update (dof24_halfImplicit_gpu.cu:1016-1081) with the rates of rhs24.
template <bool kNr>
__device__ __forceinline__ void update24(VehC& v, Veh24X& vx, const VehAux& va, TireC* ts, TireAux* ta, Sus24C* su,
                                         const ClassDev18& C, const Rhs24& R, double dt, double* S, size_t np,
                                         bool sink) {
    const double* dxt = R.dxt;
    const double* dwu = R.dwu;
    const double wdot = R.wdot, sth = R.sth, cth = R.cth, sph = R.sph, cph = R.cph;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        if (!kNr) {  // the TMeasyNr tire has no deflection states
            ts[c].xe = fma(ts[c].xedot, dt, ts[c].xe);
            ts[c].ye = fma(ts[c].yedot, dt, ts[c].ye);
        }
        ta[c].xt = fma(dxt[c], dt, ta[c].xt);
        ts[c].omega = fma(ta[c].dOmega, dt, ts[c].omega);
        su[c].wu = fma(dwu[c], dt, su[c].wu);
        su[c].xs = fma(su[c].dxs, dt, su[c].xs);
    }
    if (C.tcbool) v.crank = fma(va.dOmega_crank, dt, v.crank);
    v.u = fma(v.udot, dt, v.u);
    v.v = fma(v.vdot, dt, v.v);
    vx.w = fma(wdot, dt, vx.w);
    v.wx = fma(vx.wxdot, dt, v.wx);
    vx.wy = fma(vx.wydot, dt, vx.wy);
    v.wz = fma(vx.wzdot, dt, v.wz);
    // Cardan angle rates with the updated body rates and the pre-update pitch and roll
    const double icth = 1.0 / cth;
    const double q = fma(vx.wy, sph, v.wz * cph);
    const double dtheta = fma(vx.wy, cph, -v.wz * sph);
    const double dpsi = q * icth;
    const double dphi = fma(q, sth * icth, v.wx);
    vx.theta = fma(dtheta, dt, vx.theta);
    v.psi = fma(dpsi, dt, v.psi);
    v.phi = fma(dphi, dt, v.phi);
    SINK(LFDM24_S_DTHETA, dtheta);
    SINK(LFDM24_S_DPSI, dpsi);
    SINK(LFDM24_S_DPHI, dphi);
    double sp, cp;
    sincos(v.psi, &sp, &cp);
    v.x = fma(fma(v.u, cp, -v.v * sp), dt, v.x);
    v.y = fma(fma(v.u, sp, v.v * cp), dt, v.y);
}
#undef SINK

// One step: rhs24 followed by update24 (kF32: the FP32 tire core).
template <bool kNr, bool kF32 = false>
__device__ __forceinline__ void step24(VehC& v, Veh24X& vx, VehAux& va, TireC* ts, TireAux* ta, Sus24C* su,
                                       const Corner24K* ck, const KView& K, const ClassDev18& C, double steering,
                                       double throttle, double braking, double dt, double* S, size_t np, bool sink) {
    Rhs24 R;
    rhs24<kNr, kF32>(v, vx, va, ts, ta, su, ck, K, C, steering, throttle, braking, R, S, np, sink);
    update24<kNr>(v, vx, va, ts, ta, su, C, R, dt, S, np, sink);
}

// The carried 24-DOF state of one vehicle from / to its SoA column S (S[field * np]); the fields a
// step writes only from a window's last step are written by step24 with sink set.
__device__ __forceinline__ void load_state24(const double* S, size_t np, VehC& v, Veh24X& vx, VehAux& va,
                                             TireC* ts, TireAux* ta, Sus24C* su, Corner24K* ck) {
    v.x = S[LFDM24_S_X * np];
    v.y = S[LFDM24_S_Y * np];
    v.u = S[LFDM24_S_U * np];
    v.v = S[LFDM24_S_V * np];
    v.psi = S[LFDM24_S_PSI * np];
    v.wz = S[LFDM24_S_WZ * np];
    v.phi = S[LFDM24_S_PHI * np];
    v.wx = S[LFDM24_S_WX * np];
    v.udot = S[LFDM24_S_UDOT * np];
    v.vdot = S[LFDM24_S_VDOT * np];
    v.crank = S[LFDM24_S_CRANKOMEGA * np];
    v.gear = (int)S[LFDM24_S_CURRENT_GR * np];
    vx.w = S[LFDM24_S_W * np];
    vx.theta = S[LFDM24_S_THETA * np];
    vx.wy = S[LFDM24_S_WY * np];
    vx.wxdot = S[LFDM24_S_WXDOT * np];
    vx.wydot = S[LFDM24_S_WYDOT * np];
    vx.wzdot = S[LFDM24_S_WZDOT * np];
    va.dOmega_crank = S[LFDM24_S_DOMEGA_CRANK * np];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const size_t tb = (size_t)(LFDM24_S_TIRE0 + c * LFDM24_T_COUNT) * np;
        ts[c].xe = S[tb + LFDM24_T_XE * np];
        ts[c].ye = S[tb + LFDM24_T_YE * np];
        ts[c].xedot = S[tb + LFDM24_T_XEDOT * np];
        ts[c].yedot = S[tb + LFDM24_T_YEDOT * np];
        ts[c].omega = S[tb + LFDM24_T_OMEGA * np];
        ta[c].xt = S[tb + LFDM24_T_XT * np];
        ta[c].rStat = S[tb + LFDM24_T_RSTAT * np];
        ck[c].vsz = S[tb + LFDM24_T_VSZ * np];
        const size_t sb = (size_t)(LFDM24_S_SUS0 + c * LFDM24_SUS_COUNT) * np;
        su[c].xs = S[sb + LFDM24_SUS_XS * np];
        su[c].dxs = S[sb + LFDM24_SUS_DXS * np];
        su[c].wu = S[sb + LFDM24_SUS_WU * np];
        su[c].fzd = S[sb + LFDM24_SUS_FZD * np];
        ck[c].xsi = S[sb + LFDM24_SUS_XSI * np];
        ck[c].lsi = S[sb + LFDM24_SUS_LSI * np];
    }
}
__device__ __forceinline__ void store_state24(double* S, size_t np, const VehC& v, const Veh24X& vx, const VehAux& va,
                                              const TireC* ts, const TireAux* ta, const Sus24C* su, bool tcbool) {
    S[LFDM24_S_X * np] = v.x;
    S[LFDM24_S_Y * np] = v.y;
    S[LFDM24_S_U * np] = v.u;
    S[LFDM24_S_V * np] = v.v;
    S[LFDM24_S_PSI * np] = v.psi;
    S[LFDM24_S_WZ * np] = v.wz;
    S[LFDM24_S_PHI * np] = v.phi;
    S[LFDM24_S_WX * np] = v.wx;
    S[LFDM24_S_UDOT * np] = v.udot;
    S[LFDM24_S_VDOT * np] = v.vdot;
    S[LFDM24_S_CRANKOMEGA * np] = v.crank;
    S[LFDM24_S_CURRENT_GR * np] = (double)v.gear;
    S[LFDM24_S_W * np] = vx.w;
    S[LFDM24_S_THETA * np] = vx.theta;
    S[LFDM24_S_WY * np] = vx.wy;
    S[LFDM24_S_WXDOT * np] = vx.wxdot;
    S[LFDM24_S_WYDOT * np] = vx.wydot;
    S[LFDM24_S_WZDOT * np] = vx.wzdot;
    if (tcbool) S[LFDM24_S_DOMEGA_CRANK * np] = va.dOmega_crank;  // not written without a converter
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const size_t tb = (size_t)(LFDM24_S_TIRE0 + c * LFDM24_T_COUNT) * np;
        S[tb + LFDM24_T_XE * np] = ts[c].xe;
        S[tb + LFDM24_T_YE * np] = ts[c].ye;
        S[tb + LFDM24_T_XEDOT * np] = ts[c].xedot;
        S[tb + LFDM24_T_YEDOT * np] = ts[c].yedot;
        S[tb + LFDM24_T_OMEGA * np] = ts[c].omega;
        S[tb + LFDM24_T_DOMEGA * np] = ta[c].dOmega;
        S[tb + LFDM24_T_XT * np] = ta[c].xt;
        S[tb + LFDM24_T_RSTAT * np] = ta[c].rStat;
        S[tb + LFDM24_T_FX * np] = ta[c].fx;
        S[tb + LFDM24_T_FY * np] = ta[c].fy;
        S[tb + LFDM24_T_FZ * np] = ta[c].fz;
        S[tb + LFDM24_T_VSX * np] = ta[c].vsx;
        S[tb + LFDM24_T_VSY * np] = ta[c].vsy;
        S[tb + LFDM24_T_MY * np] = ta[c].My;
        S[tb + LFDM24_T_ENGTOR * np] = ta[c].engTor;
        const size_t sb = (size_t)(LFDM24_S_SUS0 + c * LFDM24_SUS_COUNT) * np;
        S[sb + LFDM24_SUS_XS * np] = su[c].xs;
        S[sb + LFDM24_SUS_DXS * np] = su[c].dxs;
        S[sb + LFDM24_SUS_WU * np] = su[c].wu;
        S[sb + LFDM24_SUS_FZD * np] = su[c].fzd;
    }
}
__device__ __forceinline__ bool state24_finite(const VehC& v, const Veh24X& vx, const TireC* ts) {
    return isfinite(v.x) && isfinite(v.y) && isfinite(v.u) && isfinite(v.v) && isfinite(v.psi) && isfinite(v.wz) &&
           isfinite(vx.w) && isfinite(vx.theta) && isfinite(ts[0].omega) && isfinite(ts[1].omega) &&
           isfinite(ts[2].omega) && isfinite(ts[3].omega);
}

}  // namespace lfdm
