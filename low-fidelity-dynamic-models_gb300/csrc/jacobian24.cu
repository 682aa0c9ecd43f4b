// Exact Jacobians of the 24-DOF right-hand side (TMeasy tires), batched over vehicles.
//
// The reference's CPU solver offers them by central differences (IntegrateStepWithJacobian,
// 24dof/dof24_halfImplicit.cpp:402-494: every packed state perturbed by 1e-3 of its value,
// PerturbRhsFun twice per column, results in GetJacobianState / GetJacobianControls); its GPU solver
// has none. As for the 18- and 11-DOF models (jacobian18.cu, jacobian11.cu), one right-hand-side
// evaluation (rhs24's arithmetic, dof24_device.cuh) is recorded on a tape per vehicle and reversed
// once per dynamic row. The tires are the 18-DOF model's taped core (tire_fwd_tape_core /
// tire_rev_core, dof18_adjoint.cuh) with the 24-DOF load and radii around it: the load from the
// integrated compression (fz = xt kt), the loaded radius through pitch and roll
// (rStat = (r0 - xt) / (cos theta cos phi)) and the effective radius fma(rdynco, r0 - rStat, rStat).
// The vehicle level reverses vehToSusTransform, vehToTireTransform, the 18-DOF powertrain and
// differential, tireToVehTransform, computeSusRHS, computeForcesThroughSus and the 6-DOF chassis
// (24dof-gpu/dof24_gpu.cu; CPU twins in 24dof/dof24.cpp).
//
// Packed order (packY / packYDOT, 24dof/dof24_halfImplicit.cpp:1015-1386): states {xe, ye, xt} of
// LF, RF, LR, RR; omega x 4; {wu, xs} x 4; crank speed (torque converter only); x, y, u, v, w, wz,
// wx, wy, psi, phi, theta. Right-hand side {xedot, yedot, dxt} x 4, domega x 4, {dwu, dxs} x 4,
// dcrank, dx, dy, udot, vdot, wdot, wzdot, wxdot, wydot, dpsi, dphi, dtheta. Controls steering,
// throttle. The kinematic rows (dx, dy, dxs = wu - ws, and the Cardan rates dpsi, dphi, dtheta at
// the unupdated angular rates, 24dof/dof24.cpp:1722-1731) have closed forms.
#include <cuda_runtime.h>

#include "../../include/lfdm/device/dof24_device.cuh"
#include "dof18_adjoint.cuh"
#include "jacobian18.h"
#include "window_common.cuh"

namespace lfdm {

namespace {

// The 24-DOF quantities of one evaluation, after the 18-DOF step tape (whose powertrain, wheel
// angle, control, force-rotation and tire fields are reused with the same meaning).
struct Tape24X {
    double w, wy, wx, theta, sth, cth, sph, cph, icc;
    double ls[4], uu[4], vu[4], wu[4], xs[4];
    double dxsp[4], rprev[4];         // the previous step's strut rate and loaded radius (constants here)
    double wxdotp, wydotp;            // the previous step's roll and pitch accelerations (constants here)
    double vgx[4], vgy[4];
    double xt[4], rs[4], rdynco[4], fzrd[4], fz[4];
    double fxg[4], fyg[4], fxs[4], fys[4];
};
struct Tape24 {
    StepTape s;
    Tape24X x;
};
#define TX_(f) ((int)((offsetof(Tape24, x) + offsetof(Tape24X, f)) / sizeof(double)))

// rhs24<false>'s arithmetic (TMeasy) with its tape.
__device__ __forceinline__ void fwd24_tape(VehC& v, Veh24X& vx, VehAux& va, TireC* ts, TireAux* ta, Sus24C* su,
                                           const Corner24K* ck, const TapeRef& T, const KView& K, const ClassDev18& C,
                                           double steering, double throttle, double braking) {
    const double cf2 = K(K24_CF2), cr2 = K(K24_CR2), a = K(K24_A), b = K(K24_B);
    T.at(TS_(u)) = v.u;
    T.at(TS_(v)) = v.v;
    T.at(TS_(wz)) = v.wz;
    T.at(TS_(phi)) = v.phi;
    T.at(TS_(crank)) = v.crank;
    T.at(TS_(gear)) = (double)v.gear;
    T.at(TS_(steer)) = steering;
    T.at(TS_(thr)) = throttle;
    T.at(TS_(brk)) = braking;
    T.at(TX_(w)) = vx.w;
    T.at(TX_(wy)) = vx.wy;
    T.at(TX_(wx)) = v.wx;
    T.at(TX_(theta)) = vx.theta;
    T.at(TX_(wxdotp)) = vx.wxdot;
    T.at(TX_(wydotp)) = vx.wydot;
    double sth, cth, sph, cph;
    sincos(vx.theta, &sth, &cth);
    sincos(v.phi, &sph, &cph);
    T.at(TX_(sth)) = sth;
    T.at(TX_(cth)) = cth;
    T.at(TX_(sph)) = sph;
    T.at(TX_(cph)) = cph;
    double uu[4], vu[4], ls[4], duu[4], dvu[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const double lat = c == 0 ? -cf2 : c == 1 ? cf2 : c == 2 ? -cr2 : cr2;
        const double lon = c < 2 ? a : -b;
        const double us = fma(lat, v.wz, v.u);
        const double vs = fma(lon, v.wz, v.v);
        ls[c] = ck[c].lsi - (su[c].xs - ck[c].xsi);
        uu[c] = fma(-ls[c], vx.wy, us);
        vu[c] = fma(ls[c], v.wx, vs);
        const double dus = fma(lat, vx.wzdot, v.udot);
        const double dvs = fma(lon, vx.wzdot, v.vdot);
        duu[c] = dus - fma(-su[c].dxs, vx.wy, ls[c] * vx.wydot);
        dvu[c] = dvs + fma(-su[c].dxs, v.wx, ls[c] * vx.wxdot);
        T.at(TX_(ls) + c) = ls[c];
        T.at(TX_(uu) + c) = uu[c];
        T.at(TX_(vu) + c) = vu[c];
        T.at(TX_(wu) + c) = su[c].wu;
        T.at(TX_(xs) + c) = su[c].xs;
        T.at(TX_(dxsp) + c) = su[c].dxs;
    }
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
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const double r = ta[c].rStat;
        const double vgx = fma(cth, fma(-vx.wy, r, uu[c]), sth * fma(su[c].wu, cph, sph * fma(v.wx, r, vu[c])));
        const double vgy = fma(cph, fma(v.wx, r, vu[c]), -su[c].wu * sph);
        ta[c].vsy = vgy;
        ta[c].vsx = c < 2 ? fma(vgx, cd, vgy * sd) : vgx;
        T.at(TX_(rprev) + c) = r;
        T.at(TX_(vgx) + c) = vgx;
        T.at(TX_(vgy) + c) = vgy;
    }
    const double icc = 1.0 / (cth * cph);
    T.at(TX_(icc)) = icc;
    const double r0 = K(K_R0), kt = K(K24_KT);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const TapeRef R = tire_ref(T, c);
        const double xt = ta[c].xt;
        const double fz = xt * kt;
        T.at(TX_(xt) + c) = xt;
        R.at(TT_(fz)) = fz;
        R.at(TT_(om)) = ts[c].omega;
        R.at(TT_(xe)) = ts[c].xe;
        R.at(TT_(ye)) = ts[c].ye;
        R.at(TT_(vsy)) = ta[c].vsy;
        R.at(TT_(on)) = gt0(fz) ? 1.0 : 0.0;
        if (!gt0(fz)) {
            ts[c].xe = 0;
            ts[c].ye = 0;
            ts[c].omega = 0;
            ta[c].xt = 0;
            ta[c].rStat = r0;
            ta[c].fz = 0;
            ta[c].fx = 0;
            ta[c].fy = 0;
            ta[c].My = 0;
            R.at(TT_(rStat)) = r0;
            R.at(TT_(fx)) = R.at(TT_(fy)) = R.at(TT_(My)) = 0;
            T.at(TX_(rs) + c) = r0;
            T.at(TX_(fz) + c) = 0;
            T.at(TX_(fzrd) + c) = 0;
            T.at(TX_(rdynco) + c) = 0;
        } else {
            const double rs = (r0 - xt) * icc;
            ta[c].fz = fz;
            ta[c].rStat = rs;
            const bool band = !gt_nn(fz, K(K_FZRD));
            const double rdynco = band ? fma(K(K_DRD), fma(fz, K(K_INVPN), -1.0), K(K_RDPN)) : K(K_RDCRIT);
            const double r_eff = fma(rdynco, r0 - rs, rs);
            R.at(TT_(rStat)) = rs;
            T.at(TX_(rs) + c) = rs;
            T.at(TX_(fz) + c) = fz;
            T.at(TX_(fzrd) + c) = band ? 1.0 : 0.0;
            T.at(TX_(rdynco) + c) = rdynco;
            if (c < 2) tire_fwd_tape_core<true>(ts[c], ta[c], R, K, cd, sd, fz, r_eff);
            else tire_fwd_tape_core<false>(ts[c], ta[c], R, K, 1.0, 0.0, fz, r_eff);
        }
    }
    // powertrain (powertrain_rhs<false>, as taped by fwd18_tape)
    {
        double torque_t;
        const int g = v.gear;
        T.at(TS_(rev)) = 0;
        T.at(TS_(tclip)) = 0;
        if (C.tcbool) {
            bool reverse = false;
            const double omega_t = 0.25 * (((ts[0].omega + ts[1].omega) + ts[2].omega) + ts[3].omega);
            const double omega_out = omega_t / C.gear[g];
            const double omega_in = v.crank;
            T.at(TS_(omega_t)) = omega_t;
            T.at(TS_(omega_out)) = omega_out;
            T.at(TS_(omega_in)) = omega_in;
            double sr;
            if ((omega_out < 1e-9) || (omega_in < 1e-9)) {
                sr = 0;
                T.at(TS_(srmode)) = 0;
            } else {
                sr = omega_out / omega_in;
                T.at(TS_(srmode)) = 1;
                if (sr > 1.) {
                    sr = 1. - (sr - 1.);
                    reverse = true;
                }
                if (sr < 0) {
                    sr = 0;
                    T.at(TS_(srmode)) = 0;
                }
            }
            T.at(TS_(sr)) = sr;
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
            if (v.u < 1e-9 && torque_t < 0) {
                torque_t = 0;
                T.at(TS_(tclip)) = 1;
            }
            T.at(TS_(dt_map)) = map_y(C.pt, v.crank);
            T.at(TS_(dt_slope)) = fma(map_slope(C.pt, v.crank), throttle, map_slope(C.loss, v.crank));
            va.dOmega_crank = K(K_INVCI) * (drive_torque(C, throttle, v.crank) + torque_in);
        } else {
            v.crank = 0.25 * (((ts[0].omega + ts[1].omega) + ts[2].omega) + ts[3].omega) / C.gear[g];
            T.at(TS_(omega_in)) = v.crank;
            torque_t = drive_torque(C, throttle, v.crank) * C.invgear[g];
            T.at(TS_(dt_map)) = map_y(C.pt, v.crank);
            T.at(TS_(dt_slope)) = fma(map_slope(C.pt, v.crank), throttle, map_slope(C.loss, v.crank));
            if (v.u < 1e-9 && torque_t < 0) {
                torque_t = 0;
                T.at(TS_(tclip)) = 1;
            }
        }
        T.at(TS_(torque_t)) = torque_t;
        double tf, trr;
        if (C.driveType) {
            tf = torque_t * 0.5;
            trr = torque_t * 0.5;
        } else if (C.whichWheels) {
            tf = 0;
            trr = torque_t;
        } else {
            tf = torque_t;
            trr = 0;
        }
        T.at(TS_(tf)) = tf;
        T.at(TS_(trr)) = trr;
        auto split = [&](double torque, double wl, double wr, double& alpha, double& dal, double& slowleft) {
            const double diff = fabs(wl - wr);
            if (diff > 0.5) {
                alpha = 2.0 / 3.0;
                dal = 0;
            } else if (diff > 0.25) {
                const double bias = 4 * (2.0 - 1) * diff + (2 - 2.0);
                alpha = bias / (1 + bias);
                dal = 4.0 / ((1 + bias) * (1 + bias));
            } else {
                alpha = 0.5;
                dal = 0;
            }
            slowleft = fabs(wl) < fabs(wr) ? 1 : 0;
            (void)torque;
        };
        split(tf, ts[0].omega, ts[1].omega, T.at(TS_(alf)), T.at(TS_(dalf)), T.at(TS_(slowf)));
        split(trr, ts[2].omega, ts[3].omega, T.at(TS_(alr)), T.at(TS_(dalr)), T.at(TS_(slowr)));
    }
    // tireToVehTransform
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        double fxr = ta[c].fx, fyr = ta[c].fy;
        if (c < 2) {
            fxr = fma(ta[c].fx, cd, -ta[c].fy * sd);
            fyr = fma(ta[c].fx, sd, ta[c].fy * cd);
        }
        const double fz = ta[c].fz;
        T.at(TS_(fxr) + c) = fxr;
        T.at(TS_(fyr) + c) = fyr;
        T.at(TX_(fxg) + c) = fma(fxr, cth, -fz * sth);
        T.at(TX_(fyg) + c) = fma(fxr * sph, sth, fma(fyr, cph, fz * sph * cth));
    }
    // computeForcesThroughSus (the values the reverse reads)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const double mu = c < 2 ? K(K24_MUF) : K(K24_MUR);
        const double muG = c < 2 ? K(K24_MUFG) : K(K24_MURG);
        const double fxg = T.at(TX_(fxg) + c), fyg = T.at(TX_(fyg) + c);
        T.at(TX_(fxs) + c) = fma(muG, sth, fxg) + mu * (fma(v.wz, vu[c], -duu[c]) - vx.wy * su[c].wu);
        const double gl = c < 3 ? muG * sph * cth : muG * sph;
        T.at(TX_(fys) + c) = (fyg - gl) + mu * (fma(v.wx, su[c].wu, -dvu[c]) - v.wz * uu[c]);
    }
}

// Adjoints of the packed states and controls of one dynamic row (seeded output adjoints).
struct Rev24In {
    double xedotb[4], yedotb[4], dxtb[4], dOmb[4], dwub[4];
    double dOcb, udotb, vdotb, wdotb, wzdotb, wxdotb, wydotb;
};
struct Rev24Out {
    double xeb[4], yeb[4], xtb[4], omb[4], wub[4], xsb[4];
    double crankb, ub, vb, wb, wzb, wxb, wyb, phib, thetab, steerb, thrb;
};

__device__ __forceinline__ void rev24_rhs(const TapeRef& T, const KView& K, const ClassDev18& C, const KBar& kb,
                                          const Rev24In& in, Rev24Out& o) {
    const int g = (int)T.at(TS_(gear));
    const double cf2 = K(K24_CF2), cr2 = K(K24_CR2), a = K(K24_A), b = K(K24_B);
    const double u = T.at(TS_(u)), vv = T.at(TS_(v)), wz = T.at(TS_(wz));
    const double w = T.at(TX_(w)), wy = T.at(TX_(wy)), wx = T.at(TX_(wx));
    const double sth = T.at(TX_(sth)), cth = T.at(TX_(cth)), sph = T.at(TX_(sph)), cph = T.at(TX_(cph));
    const double cd = T.at(TS_(cd)), sd = T.at(TS_(sd));
    const double ks = K(K24_KS), bs = K(K24_BS), im = K(K24_INVM);
    const double hrcf = K(K24_HRCF), hrcr = K(K24_HRCR);
    double ub = 0, vb = 0, wb = 0, wzb = 0, wxb = 0, wyb = 0, sthb = 0, cthb = 0, sphb = 0, cphb = 0;
    double sdb = 0, cdb = 0, iccb = 0, steerb = 0, thrb = 0, crankb = 0;
    double uub[4], vub[4], lsb[4], wub[4], xsb[4], wsb[4], duub[4], dvub[4];
    double fxsb[4], fysb[4], fzsb[4], fxgb[4], fygb[4], rsb[4], fxrb[4], fyrb[4], fzb[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        uub[c] = vub[c] = lsb[c] = wub[c] = xsb[c] = wsb[c] = duub[c] = dvub[c] = 0;
        fxsb[c] = fysb[c] = fzsb[c] = fxgb[c] = fygb[c] = rsb[c] = fxrb[c] = fyrb[c] = fzb[c] = 0;
    }
    // computeVehicleRHS: 6-DOF chassis
    {
        wzb = fma(vv, in.udotb, wzb);
        vb = fma(wz, in.udotb, vb);
        wyb = fma(-w, in.udotb, wyb);
        wb = fma(-wy, in.udotb, wb);
        const double sfxb = im * in.udotb;
        sthb = fma(kG, in.udotb, sthb);
        wxb = fma(w, in.vdotb, wxb);
        wb = fma(wx, in.vdotb, wb);
        wzb = fma(-u, in.vdotb, wzb);
        ub = fma(-wz, in.vdotb, ub);
        const double sfyb = im * in.vdotb;
        sphb = fma(-kG * cth, in.vdotb, sphb);
        cthb = fma(-kG * sph, in.vdotb, cthb);
        wyb = fma(u, in.wdotb, wyb);
        ub = fma(wy, in.wdotb, ub);
        wxb = fma(-vv, in.wdotb, wxb);
        vb = fma(-wx, in.wdotb, vb);
        const double sfzb = im * in.wdotb;
        cphb = fma(-kG * cth, in.wdotb, cphb);
        cthb = fma(-kG * cph, in.wdotb, cthb);
        const double tx = K(K24_INVJX) * in.wxdotb, ty = K(K24_INVJY) * in.wydotb, tz = K(K24_INVJZ) * in.wzdotb;
        fzsb[0] += fma(cf2, tx, -a * ty);
        fzsb[1] += fma(-cf2, tx, -a * ty);
        fzsb[2] += fma(cr2, tx, b * ty);
        fzsb[3] += fma(-cr2, tx, b * ty);
        fysb[0] += a * tz;
        fysb[1] += a * tz;
        fysb[2] -= b * tz;
        fysb[3] -= b * tz;
        fxsb[0] -= cf2 * tz;
        fxsb[1] += cf2 * tz;
        fxsb[2] -= cr2 * tz;
        fxsb[3] += cr2 * tz;
        double fzdb[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            fxsb[c] += sfxb;
            fysb[c] += sfyb;
            fzsb[c] += sfzb;
            fzdb[c] = sfzb;
            // mx = fys h, my = -(fxg rs + fxs ls)
            fysb[c] = fma(c < 2 ? hrcf : hrcr, tx, fysb[c]);
            fxgb[c] = fma(-T.at(TX_(rs) + c), ty, fxgb[c]);
            rsb[c] = fma(-T.at(TX_(fxg) + c), ty, rsb[c]);
            fxsb[c] = fma(-T.at(TX_(ls) + c), ty, fxsb[c]);
            lsb[c] = fma(-T.at(TX_(fxs) + c), ty, lsb[c]);
        }
        // fzd: front -fzd_f, fzd_f; rear -fzd_r, fzd_r
        const double ff = K(K24_INVCF) * (fzdb[1] - fzdb[0]), fr = K(K24_INVCR) * (fzdb[3] - fzdb[2]);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const double t = c < 2 ? ff : fr;
            const double h = c < 2 ? hrcf : hrcr;
            fygb[c] = fma(T.at(TX_(rs) + c), t, fygb[c]);
            rsb[c] = fma(T.at(TX_(fyg) + c), t, rsb[c]);
            fysb[c] = fma(T.at(TX_(ls) + c) - h, t, fysb[c]);
            lsb[c] = fma(T.at(TX_(fys) + c), t, lsb[c]);
        }
    }
    // computeForcesThroughSus and computeSusRHS
    double dxsnb[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const double mu = c < 2 ? K(K24_MUF) : K(K24_MUR);
        const double muG = c < 2 ? K(K24_MUFG) : K(K24_MURG);
        const double imu = c < 2 ? K(K24_INVMUF) : K(K24_INVMUR);
        const double wu = T.at(TX_(wu) + c), uu = T.at(TX_(uu) + c), vu = T.at(TX_(vu) + c);
        // fzs = xs ks + dxs_new bs
        xsb[c] = fma(ks, fzsb[c], xsb[c]);
        dxsnb[c] = bs * fzsb[c];
        // fys = (fyg - gl) + mu ((wx wu - dvu) - wz uu)
        fygb[c] += fysb[c];
        if (c < 3) {
            sphb = fma(-muG * cth, fysb[c], sphb);
            cthb = fma(-muG * sph, fysb[c], cthb);
        } else {
            sphb = fma(-muG, fysb[c], sphb);
        }
        {
            const double m = mu * fysb[c];
            wxb = fma(wu, m, wxb);
            wub[c] = fma(wx, m, wub[c]);
            dvub[c] -= m;
            wzb = fma(-uu, m, wzb);
            uub[c] = fma(-wz, m, uub[c]);
        }
        // fxs = (muG sth + fxg) + mu ((wz vu - duu) - wy wu)
        sthb = fma(muG, fxsb[c], sthb);
        fxgb[c] += fxsb[c];
        {
            const double m = mu * fxsb[c];
            wzb = fma(vu, m, wzb);
            vub[c] = fma(wz, m, vub[c]);
            duub[c] -= m;
            wyb = fma(-wu, m, wyb);
            wub[c] = fma(-wy, m, wub[c]);
        }
        // dxs_new = wu - ws
        wub[c] += dxsnb[c];
        wsb[c] -= dxsnb[c];
        // dwu = imu (inner - rest - mu (vu wx - uu wy)), inner = cph (cth (fz - muG) + sth fxr) - sph fyr
        const double gg = imu * in.dwub[c];
        {
            const double m = -mu * gg;
            vub[c] = fma(wx, m, vub[c]);
            wxb = fma(vu, m, wxb);
            uub[c] = fma(-wy, m, uub[c]);
            wyb = fma(-uu, m, wyb);
            xsb[c] = fma(-ks, gg, xsb[c]);  // rest = xs ks + dxs_prev bs + fzd_prev
            const double fz = T.at(TX_(fz) + c), fxr = T.at(TS_(fxr) + c), fyr = T.at(TS_(fyr) + c);
            const double A = fma(cth, fz - muG, sth * fxr);
            cphb = fma(A, gg, cphb);
            const double Ab = cph * gg;
            cthb = fma(fz - muG, Ab, cthb);
            fzb[c] = fma(cth, Ab, fzb[c]);
            sthb = fma(fxr, Ab, sthb);
            fxrb[c] = fma(sth, Ab, fxrb[c]);
            sphb = fma(-fyr, gg, sphb);
            fyrb[c] = fma(-sph, gg, fyrb[c]);
        }
        // fxg = fxr cth - fz sth; fyg = fxr sph sth + fyr cph + fz sph cth
        {
            const double fz = T.at(TX_(fz) + c), fxr = T.at(TS_(fxr) + c), fyr = T.at(TS_(fyr) + c);
            fxrb[c] = fma(cth, fxgb[c], fxrb[c]);
            cthb = fma(fxr, fxgb[c], cthb);
            fzb[c] = fma(-sth, fxgb[c], fzb[c]);
            sthb = fma(-fz, fxgb[c], sthb);
            fxrb[c] = fma(sph * sth, fygb[c], fxrb[c]);
            sphb = fma(fma(fxr, sth, fz * cth), fygb[c], sphb);
            sthb = fma(fxr * sph, fygb[c], sthb);
            fyrb[c] = fma(cph, fygb[c], fyrb[c]);
            cphb = fma(fyr, fygb[c], cphb);
            fzb[c] = fma(sph * cth, fygb[c], fzb[c]);
            cthb = fma(fz * sph, fygb[c], cthb);
        }
        // dxt = vsz - (cth (wu cph + vu sph) - uu sth)
        {
            const double Bq = fma(wu, cph, vu * sph);
            const double db = in.dxtb[c];
            cthb = fma(-Bq, db, cthb);
            const double Bb = -cth * db;
            wub[c] = fma(cph, Bb, wub[c]);
            cphb = fma(wu, Bb, cphb);
            vub[c] = fma(sph, Bb, vub[c]);
            sphb = fma(vu, Bb, sphb);
            uub[c] = fma(sth, db, uub[c]);
            sthb = fma(uu, db, sthb);
        }
    }
    // the front forces rotated by the wheel angle (fx, fy as the tires returned them)
    double fxb[4], fyb[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        if (c < 2) {
            const double fx = tire_ref(T, c).at(TT_(fx)), fy = tire_ref(T, c).at(TT_(fy));
            fxb[c] = fma(cd, fxrb[c], sd * fyrb[c]);
            fyb[c] = fma(-sd, fxrb[c], cd * fyrb[c]);
            cdb += fma(fx, fxrb[c], fy * fyrb[c]);
            sdb += fma(-fy, fxrb[c], fx * fyrb[c]);
        } else {
            fxb[c] = fxrb[c];
            fyb[c] = fyrb[c];
        }
    }
    // powertrain: wheel accelerations, differential, converter and engine (as rev18_rhs)
    double Myb[4], engb[4], om_mid[4], om_midb[4] = {0, 0, 0, 0};
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        om_mid[c] = tire_ref(T, c).at(TT_(on)) != 0.0 ? tire_ref(T, c).at(TT_(om)) : 0.0;
        const double gk = K(K_INVJW) * in.dOmb[c];
        engb[c] = gk;
        Myb[c] = gk;
        fxb[c] = fma(-T.at(TX_(rs) + c), gk, fxb[c]);
        rsb[c] = fma(-tire_ref(T, c).at(TT_(fx)), gk, rsb[c]);
    }
    auto split_rev = [](double torque, double alpha, double dal, double slowleft, double tlb, double trb, double wl,
                        double wr, double& wlb, double& wrb) {
        const double slowb = slowleft != 0.0 ? tlb : trb;
        const double fastb = slowleft != 0.0 ? trb : tlb;
        const double alphab = torque * (slowb - fastb);
        const double diffb = dal * alphab;
        if (diffb != 0.0) {
            const double sg = (wl - wr) >= 0 ? 1.0 : -1.0;
            wlb = fma(sg, diffb, wlb);
            wrb -= sg * diffb;
        }
        return alpha * slowb + (1.0 - alpha) * fastb;
    };
    const double tfb = split_rev(T.at(TS_(tf)), T.at(TS_(alf)), T.at(TS_(dalf)), T.at(TS_(slowf)), engb[0], engb[1],
                                 om_mid[0], om_mid[1], om_midb[0], om_midb[1]);
    const double trrb = split_rev(T.at(TS_(trr)), T.at(TS_(alr)), T.at(TS_(dalr)), T.at(TS_(slowr)), engb[2], engb[3],
                                  om_mid[2], om_mid[3], om_midb[2], om_midb[3]);
    double torque_tb = C.driveType ? 0.5 * (tfb + trrb) : (C.whichWheels ? trrb : tfb);
    if (T.at(TS_(tclip)) != 0.0) torque_tb = 0;
    if (C.tcbool) {
        const double torque_outb = C.invgear[g] * torque_tb;
        double torque_inb = 0, trb = 0;
        if (T.at(TS_(rev)) != 0.0) {
            torque_inb = -torque_outb;
        } else {
            trb = -T.at(TS_(torque_in)) * torque_outb;
            torque_inb = -T.at(TS_(tr)) * torque_outb;
        }
        const double dtqb = K(K_INVCI) * in.dOcb;
        torque_inb = fma(K(K_INVCI), in.dOcb, torque_inb);
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
        const double omega_tb = omega_outb * C.invgear[g];
#pragma unroll
        for (int c = 0; c < 4; ++c) om_midb[c] += 0.25 * omega_tb;
        crankb += omega_inb;
    } else {
        const double dtqb = C.invgear[g] * torque_tb;
        thrb = fma(T.at(TS_(dt_map)), dtqb, thrb);
        const double crank_outb = T.at(TS_(dt_slope)) * dtqb;
#pragma unroll
        for (int c = 0; c < 4; ++c) om_midb[c] += 0.25 * crank_outb * C.invgear[g];
    }
    // tires, with the 24-DOF load and radii: fz = xt kt, rs = (r0 - xt) icc, r_eff = fma(rdynco, r0 - rs, rs)
    double vsxinb[4], vsyb[4];
    const double r0 = K(K_R0), kt = K(K24_KT);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        vsxinb[c] = vsyb[c] = 0;
        o.xeb[c] = o.yeb[c] = o.omb[c] = o.xtb[c] = 0;
        const TapeRef R = tire_ref(T, c);
        if (R.at(TT_(on)) == 0.0) continue;  // lifted: the outputs do not depend on the states
        double xeb = 0, yeb = 0, omb = om_midb[c], fzbt = fzb[c], reffb = 0, rsbt = rsb[c];
        const bool any = in.xedotb[c] != 0.0 || in.yedotb[c] != 0.0 || fxb[c] != 0.0 || fyb[c] != 0.0 ||
                         Myb[c] != 0.0 || rsbt != 0.0 || omb != 0.0;
        if (any) {
            if (c < 2)
                tire_rev_core<true>(R, K, kb, in.xedotb[c], in.yedotb[c], fxb[c], fyb[c], Myb[c], rsbt, xeb, yeb, omb,
                                    vsxinb[c], vsyb[c], fzbt, reffb, cdb, sdb, cd, sd);
            else {
                double cdum = 0, sdum = 0;
                tire_rev_core<false>(R, K, kb, in.xedotb[c], in.yedotb[c], fxb[c], fyb[c], Myb[c], rsbt, xeb, yeb,
                                     omb, vsxinb[c], vsyb[c], fzbt, reffb, cdum, sdum, 1.0, 0.0);
            }
        }
        const double rs = T.at(TX_(rs) + c), rdynco = T.at(TX_(rdynco) + c), xt = T.at(TX_(xt) + c);
        // r_eff = rdynco (r0 - rs) + rs
        rsbt = fma(1.0 - rdynco, reffb, rsbt);
        if (T.at(TX_(fzrd) + c) != 0.0) fzbt = fma(K(K_DRD) * K(K_INVPN) * (r0 - rs), reffb, fzbt);
        // rs = (r0 - xt) icc, fz = xt kt
        double xtb = -T.at(TX_(icc)) * rsbt;
        iccb = fma(r0 - xt, rsbt, iccb);
        xtb = fma(kt, fzbt, xtb);
        o.xeb[c] = xeb;
        o.yeb[c] = yeb;
        o.omb[c] = omb;
        o.xtb[c] = xtb;
    }
    // icc = 1 / (cth cph)
    {
        const double icc = T.at(TX_(icc));
        cthb = fma(-icc * icc * cph, iccb, cthb);
        cphb = fma(-icc * icc * cth, iccb, cphb);
    }
    // vehToTireTransform: vsx (front rotated by the wheel angle), vsy from vgx, vgy
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        double vgxb, vgyb;
        if (c < 2) {
            vgxb = cd * vsxinb[c];
            vgyb = fma(sd, vsxinb[c], vsyb[c]);
            cdb = fma(T.at(TX_(vgx) + c), vsxinb[c], cdb);
            sdb = fma(T.at(TX_(vgy) + c), vsxinb[c], sdb);
        } else {
            vgxb = vsxinb[c];
            vgyb = vsyb[c];
        }
        const double r = T.at(TX_(rprev) + c), wu = T.at(TX_(wu) + c), uu = T.at(TX_(uu) + c), vu = T.at(TX_(vu) + c);
        const double vr = fma(wx, r, vu);
        // vgy = cph vr - wu sph
        cphb = fma(vr, vgyb, cphb);
        vub[c] = fma(cph, vgyb, vub[c]);
        wxb = fma(cph * r, vgyb, wxb);
        wub[c] = fma(-sph, vgyb, wub[c]);
        sphb = fma(-wu, vgyb, sphb);
        // vgx = cth (uu - wy r) + sth (wu cph + sph vr)
        cthb = fma(fma(-wy, r, uu), vgxb, cthb);
        uub[c] = fma(cth, vgxb, uub[c]);
        wyb = fma(-cth * r, vgxb, wyb);
        sthb = fma(fma(wu, cph, sph * vr), vgxb, sthb);
        const double Qb = sth * vgxb;
        wub[c] = fma(cph, Qb, wub[c]);
        cphb = fma(wu, Qb, cphb);
        sphb = fma(vr, Qb, sphb);
        vub[c] = fma(sph, Qb, vub[c]);
        wxb = fma(sph * r, Qb, wxb);
    }
    // wheel angle
    steerb = fma(T.at(TS_(dslope)), fma(cd, sdb, -sd * cdb), steerb);
    // vehToSusTransform
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const double lat = c == 0 ? -cf2 : c == 1 ? cf2 : c == 2 ? -cr2 : cr2;
        const double lon = c < 2 ? a : -b;
        const double ls = T.at(TX_(ls) + c), dxsp = T.at(TX_(dxsp) + c);
        // uu = us - ls wy, vu = vs + ls wx
        const double usb = uub[c], vsb = vub[c];
        lsb[c] = fma(-wy, uub[c], lsb[c]);
        wyb = fma(-ls, uub[c], wyb);
        lsb[c] = fma(wx, vub[c], lsb[c]);
        wxb = fma(ls, vub[c], wxb);
        // duu = dus + dxs_prev wy - ls wydot_prev, dvu = dvs - dxs_prev wx + ls wxdot_prev (the
        // previous accelerations and strut rate are not states)
        wyb = fma(dxsp, duub[c], wyb);
        wxb = fma(-dxsp, dvub[c], wxb);
        lsb[c] = fma(-T.at(TX_(wydotp)), duub[c], fma(T.at(TX_(wxdotp)), dvub[c], lsb[c]));
        // ws = w - lat wx - lon wy
        wb += wsb[c];
        wxb = fma(-lat, wsb[c], wxb);
        wyb = fma(-lon, wsb[c], wyb);
        // us = u + lat wz, vs = v + lon wz
        ub += usb;
        wzb = fma(lat, usb, wzb);
        vb += vsb;
        wzb = fma(lon, vsb, wzb);
        // ls = lsi - (xs - xsi)
        xsb[c] -= lsb[c];
    }
    o.ub = ub;
    o.vb = vb;
    o.wb = wb;
    o.wzb = wzb;
    o.wxb = wxb;
    o.wyb = wyb;
    o.thetab = fma(cth, sthb, -sth * cthb);
    o.phib = fma(cph, sphb, -sph * cphb);
    o.crankb = crankb;
    o.steerb = steerb;
    o.thrb = thrb;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        o.wub[c] = wub[c];
        o.xsb[c] = xsb[c];
    }
}

__global__ void __launch_bounds__(128) rhs_jacobian24_kernel(const JacLaunch A) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int tid = threadIdx.x;
    const ClassDev18* cls = A.cls_smem ? reinterpret_cast<const ClassDev18*>(smem) : A.classes;
    double* ks = reinterpret_cast<double*>(smem + (A.cls_smem ? (size_t)A.nclasses * sizeof(ClassDev18) : 0));
    double* kbs = ks + (size_t)K24_COUNT * blockDim.x;
    if (A.cls_smem) {
        const int4* src = reinterpret_cast<const int4*>(A.classes);
        int4* dst = reinterpret_cast<int4*>(smem);
        const int words = (int)(A.nclasses * sizeof(ClassDev18) / 16);
        for (int i = tid; i < words; i += blockDim.x) dst[i] = __ldg(src + i);
    }
    const int vid = blockIdx.x * blockDim.x + tid;
    if (vid < A.n) {
#pragma unroll 4
        for (int k = 0; k < K24_COUNT; ++k) ks[k * blockDim.x + tid] = __ldg(A.K + (size_t)k * A.npad + vid);
    }
    __syncthreads();
    if (vid >= A.n) return;
    const size_t np = (size_t)A.npad, nu = (size_t)A.n;
    const KView K{ks + tid, (int)blockDim.x};
    const KBar kb{kbs + tid, (int)blockDim.x};  // parameter-constant adjoints: scratch, not reported
    const ClassDev18& C = cls[__ldg(A.class_of + vid)];

    VehC v;
    Veh24X vx;
    VehAux va;
    TireC ts[4];
    TireAux ta[4];
    Sus24C su[4];
    Corner24K ck[4];
    load_state24(A.S + vid, np, v, vx, va, ts, ta, su, ck);
    if (A.reference_point) {
        // PerturbRhsFun: the packed states in freshly constructed structs, every other field zero
        v.udot = v.vdot = 0.0;
        v.gear = 0;
        if (!C.tcbool) v.crank = 0.0;
        vx.wxdot = vx.wydot = vx.wzdot = 0.0;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            ts[c].xedot = ts[c].yedot = 0.0;
            ta[c].rStat = 0.0;
            su[c].dxs = su[c].fzd = 0.0;
            ck[c].xsi = ck[c].lsi = ck[c].vsz = 0.0;
        }
    }
    const double psi = v.psi, u = v.u, vv = v.v, phi = v.phi, theta = vx.theta;
    const double wys = vx.wy, wzs = v.wz;
    const double steer = __ldg(A.ctl + vid), thr = __ldg(A.ctl + nu + vid), brk = __ldg(A.ctl + 2 * nu + vid);
    const TapeRef T{A.tape + vid, np};
    fwd24_tape(v, vx, va, ts, ta, su, ck, T, K, C, steer, thr, brk);

    const bool tc = C.tcbool != 0;
    const int ny = 35 + (tc ? 1 : 0), o = 24 + (tc ? 1 : 0);  // o: index of x in the packed vector
    auto J = [&](int r, int c) -> double& { return A.jac_state[((size_t)r * ny + c) * nu + vid]; };
    auto Ju = [&](int r, int c) -> double& { return A.jac_ctl[((size_t)r * 2 + c) * nu + vid]; };
    const double cf2 = K(K24_CF2), cr2 = K(K24_CR2), a = K(K24_A), b = K(K24_B);
    double sp, cp, sph, cph, sth, cth;
    sincos(psi, &sp, &cp);
    sincos(phi, &sph, &cph);
    sincos(theta, &sth, &cth);
    for (int r = 0; r < ny; ++r) {
        const bool dxs_row = r >= 16 && r < 24 && ((r - 16) & 1);
        const bool kin = r == o || r == o + 1 || r >= o + 8 || dxs_row;
        if (kin) {
            for (int c = 0; c < ny; ++c) J(r, c) = 0.0;
            Ju(r, 0) = 0.0;
            Ju(r, 1) = 0.0;
            if (r == o) {  // dx = u cos(psi) - v sin(psi)
                J(r, o + 2) = cp;
                J(r, o + 3) = -sp;
                J(r, o + 8) = fma(-u, sp, -vv * cp);
            } else if (r == o + 1) {  // dy = u sin(psi) + v cos(psi)
                J(r, o + 2) = sp;
                J(r, o + 3) = cp;
                J(r, o + 8) = fma(u, cp, -vv * sp);
            } else if (dxs_row) {  // dxs = wu - ws, ws = w - lat wx - lon wy
                const int c = (r - 16) >> 1;
                const double lat = c == 0 ? -cf2 : c == 1 ? cf2 : c == 2 ? -cr2 : cr2;
                const double lon = c < 2 ? a : -b;
                J(r, 16 + 2 * c) = 1.0;
                J(r, o + 4) = -1.0;
                J(r, o + 6) = lat;
                J(r, o + 7) = lon;
            } else {
                const double ic = 1.0 / cth, tth = sth * ic;
                const double P = fma(wys, sph, wzs * cph), Pp = fma(wys, cph, -wzs * sph);
                if (r == o + 8) {  // dpsi = (wy sph + wz cph) / cth
                    J(r, o + 7) = sph * ic;
                    J(r, o + 5) = cph * ic;
                    J(r, o + 9) = Pp * ic;
                    J(r, o + 10) = P * sth * ic * ic;
                } else if (r == o + 9) {  // dphi = wx + (wy sph + wz cph) tan(theta)
                    J(r, o + 6) = 1.0;
                    J(r, o + 7) = sph * tth;
                    J(r, o + 5) = cph * tth;
                    J(r, o + 9) = Pp * tth;
                    J(r, o + 10) = P * ic * ic;
                } else {  // dtheta = wy cph - wz sph
                    J(r, o + 7) = cph;
                    J(r, o + 5) = -sph;
                    J(r, o + 9) = -P;
                }
            }
            continue;
        }
        Rev24In in = {};
        if (r < 12) {
            const int c = r / 3, k = r % 3;
            (k == 0 ? in.xedotb : k == 1 ? in.yedotb : in.dxtb)[c] = 1.0;
        } else if (r < 16) {
            in.dOmb[r - 12] = 1.0;
        } else if (r < 24) {
            in.dwub[(r - 16) >> 1] = 1.0;
        } else if (tc && r == 24) {
            in.dOcb = 1.0;
        } else if (r == o + 2) {
            in.udotb = 1.0;
        } else if (r == o + 3) {
            in.vdotb = 1.0;
        } else if (r == o + 4) {
            in.wdotb = 1.0;
        } else if (r == o + 5) {
            in.wzdotb = 1.0;
        } else if (r == o + 6) {
            in.wxdotb = 1.0;
        } else {
            in.wydotb = 1.0;  // r == o + 7
        }
        Rev24Out ob;
        rev24_rhs(T, K, C, kb, in, ob);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            J(r, 3 * c) = ob.xeb[c];
            J(r, 3 * c + 1) = ob.yeb[c];
            J(r, 3 * c + 2) = ob.xtb[c];
            J(r, 12 + c) = ob.omb[c];
            J(r, 16 + 2 * c) = ob.wub[c];
            J(r, 17 + 2 * c) = ob.xsb[c];
        }
        if (tc) J(r, 24) = ob.crankb;
        J(r, o) = 0.0;
        J(r, o + 1) = 0.0;
        J(r, o + 2) = ob.ub;
        J(r, o + 3) = ob.vb;
        J(r, o + 4) = ob.wb;
        J(r, o + 5) = ob.wzb;
        J(r, o + 6) = ob.wxb;
        J(r, o + 7) = ob.wyb;
        J(r, o + 8) = 0.0;  // psi enters only dx and dy
        J(r, o + 9) = ob.phib;
        J(r, o + 10) = ob.thetab;
        Ju(r, 0) = ob.steerb;
        Ju(r, 1) = ob.thrb;
    }
}

}  // namespace

size_t jac24_tape_doubles() { return sizeof(Tape24) / sizeof(double); }

cudaError_t launch_rhs_jacobian24(const JacLaunch& A, cudaStream_t stream) {
    if (A.n <= 0) return cudaSuccess;
    if (A.tire_nr) return cudaErrorInvalidValue;
    constexpr int threads = 128;
    JacLaunch L = A;
    const size_t base = (size_t)(K24_COUNT + KB_COUNT) * threads * sizeof(double);
    const size_t cls = (size_t)A.nclasses * sizeof(ClassDev18);
    L.cls_smem = A.nclasses <= kMaxSmemClasses && 2 * (base + cls + 1024) <= 228 * 1024;
    const size_t smem = base + (L.cls_smem ? cls : 0);
    cudaError_t e = cudaFuncSetAttribute(rhs_jacobian24_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    rhs_jacobian24_kernel<<<(A.n + threads - 1) / threads, threads, smem, stream>>>(L);
    return cudaGetLastError();
}

}  // namespace lfdm
