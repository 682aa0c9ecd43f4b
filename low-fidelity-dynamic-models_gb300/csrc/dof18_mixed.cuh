// 18-DOF model, mixed precision: the right-hand side (loads, transforms, TMeasy tire, powertrain,
// vehicle dynamics) in FP32; FP64 kept where accuracy or stability needs it:
//   * the integrated states and the half-implicit update (u, v, wx, wz, crank and wheel speeds,
//     tire deflections) — increments of ~1e-3 relative would otherwise drift in FP32;
//   * the global X/Y/yaw accumulation, with the yaw angle reduced to [-pi, pi] in FP64 before
//     its FP32 sine/cosine;
//   * the TMeasy slip velocity vsx - omega*r_eff (a cancellation of two large numbers at speed) and
//     the transport velocity vta = r_eff*|omega| + 0.01 (dof18_gpu.cu:424-431), rounded to FP32
//     before the slips are formed.
// Same algorithm and branch structure as dof18_device.cuh (the FP64 form), which is its oracle.
#pragma once

#include "../../include/lfdm/device/dof18_device.cuh"

namespace lfdm {

// FP32 per-class tables (maps with segment widths), built on the host from the FP64 ones.
struct MapF {
    int n;
    int pad_[3];
    float x[LFDM_MAX_MAP];
    float y[LFDM_MAX_MAP];
    float dx[LFDM_MAX_MAP];
    float dy[LFDM_MAX_MAP];
};
struct ClassDev18F {
    int nonLinearSteer, tcbool, throttleMod, driveType, whichWheels, noGears;
    int pad_[2];
    float gear[LFDM_MAX_GEARS];
    float down[LFDM_MAX_GEARS];
    float up[LFDM_MAX_GEARS];
    MapF steer, pt, loss, cf, tr;
};

__device__ __forceinline__ float map_yf(const MapF& m, float x) {
    if (x <= m.x[0]) return m.y[0];
    if (x >= m.x[m.n - 1]) return m.y[m.n - 1];
    int l = 0, h = m.n;
    while (l < h) {
        int mid = (l + h) >> 1;
        if (x <= m.x[mid]) h = mid;
        else l = mid + 1;
    }
    const int lf = l - 1;
    const float mbar = (x == m.x[l]) ? 1.0f : __fdividef(x - m.x[lf], m.dx[lf]);
    return fmaf(mbar, m.dy[lf], m.y[lf]);
}

__device__ __forceinline__ float map_yf_scaled(const MapF& m, float x, float s) {
    const int n = m.n;
    if (x <= m.x[0] * s) return m.y[0] * s;
    if (x >= m.x[n - 1] * s) return m.y[n - 1] * s;
    int l = 0, h = n;
    while (l < h) {
        int mid = (l + h) >> 1;
        if (x <= m.x[mid] * s) h = mid;
        else l = mid + 1;
    }
    const int lf = l - 1;
    const float xl = m.x[lf] * s, xr = m.x[l] * s;
    const float mbar = (x - xl) / (xr - xl);
    return fmaf(mbar, m.y[l] * s - m.y[lf] * s, m.y[lf] * s);
}

__device__ __forceinline__ float sgnf_(float v) { return (float)((0.f < v) - (v < 0.f)); }
// Sign of a double as a float (-1, 0, +1) from its bit pattern: integer-pipe instructions in place of
// two FP64 comparisons.
__device__ __forceinline__ float sgnf_of_d(double v) {
    const long long b = __double_as_longlong(v);
    return (b << 1) == 0 ? 0.f : (b < 0 ? -1.f : 1.f);
}

// FP32 view of the derived constants: KF(i).
struct KViewF {
    const float* base;
    int stride;
    __device__ __forceinline__ float operator()(int i) const { return base[i * stride]; }
};

// Mixed-precision carried state: FP64 for the accumulated kinematic states, FP32 for the tire
// deflections (a contractive first-order relaxation: rounding errors decay instead of drifting).
struct TireM {
    double omega;
    float xe, ye, xedot, yedot;  // xedot/yedot persist across steps (stale when the wheel lifts off)
};
struct VehM {
    double x, y, u, v, psi, wz, phi, wx, crank;
    float udot, vdot;
    int gear;
};
struct TireAuxF {
    float dOmega, xt, rStat, fx, fy, fz, vsx, vsy, My, engTor;
};

// computeTireRHS, TMeasy (dof18_gpu.cu:379-530): FP32 except the slip and transport velocities.
template <bool kSteered>
__device__ __forceinline__ void tire_rhs_tm_mixed(TireM& ts, TireAuxF& ta, const KViewF& K, float c, float s) {
    float fz = ta.fz;
    const float vsy = ta.vsy;
    if (fz <= 0.f) {
        ts.xe = 0;
        ts.ye = 0;
        ts.omega = 0;
        ta.xt = 0;
        ta.rStat = K(K_R0);
        ta.fx = 0;
        ta.fy = 0;
        ta.My = 0;
        return;  // xedot/yedot stay stale, as in the reference
    }
    const double omega = ts.omega;
    ta.xt = fz * K(K_INVKT);
    ta.rStat = K(K_R0) - ta.xt;
    float r_eff;
    if (fz <= K(K_FZRD)) {
        const float rdynco = fmaf(K(K_DRD), fmaf(fz, K(K_INVPN), -1.0f), K(K_RDPN));
        r_eff = fmaf(rdynco, ta.xt, ta.rStat);
    } else {
        r_eff = fmaf(K(K_RDCRIT), ta.xt, ta.rStat);
    }
    // FP64 island: the slip velocity (a difference of nearly equal terms near rolling without slip)
    // and the transport velocity
    const double r_d = (double)r_eff;
    const double vsx_d = fma(-omega, r_d, (double)ta.vsx);
    const double vta_d = fma(r_d, fabs(omega), 0.01);
    const float vsx = (float)vsx_d;
    const float vta = (float)vta_d;
    const float sx = -vsx / vta;
    const float rw = vta - 0.01f;
    float sy;
    if (kSteered) {
        // -tan(atan2(vsy, vta) - delta): infinite where the steered wheel's slip angle passes 90 degrees
        // (vta c + vsy s = 0), a denominator FP32 can round to exactly 0; the slip is held to +-1e6,
        // where the force curve is saturated and the force direction is the FP64 one to FP32 rounding.
        sy = -(vsy * c - vta * s) / (vta * c + vsy * s);
        sy = fminf(fmaxf(sy, -1e6f), 1e6f);
    } else {
        sy = -vsy / vta;
    }
    fz = fminf(fz, K(K_PNMAX));
    const float fzn = fz * K(K_INVPN);
    const float dfx0 = fzn * fmaf(-K(K_Q2DFX0), fzn, K(K_Q1DFX0));
    const float dfy0 = fzn * fmaf(-K(K_Q2DFY0), fzn, K(K_Q1DFY0));
    const float fxm = fzn * fmaf(-K(K_Q2FXM), fzn, K(K_Q1FXM));
    const float fym = fzn * fmaf(-K(K_Q2FYM), fzn, K(K_Q1FYM));
    const float fxs = fzn * fmaf(-K(K_Q2FXS), fzn, K(K_Q1FXS));
    const float fys = fzn * fmaf(-K(K_Q2FYS), fzn, K(K_Q1FYS));
    const float fzn1 = fzn - 1.0f;
    const float sxm = fmaf(K(K_DSXM), fzn1, K(K_LSXM));
    const float sym = fmaf(K(K_DSYM), fzn1, K(K_LSYM));
    const float sxs = fmaf(K(K_DSXS), fzn1, K(K_LSXS));
    const float sys = fmaf(K(K_DSYS), fzn1, K(K_LSYS));
    const float fxd = fxm * dfy0, fyd = fym * dfx0;
    const float issum = 1.0f / (sxm + sym), ifsum = 1.0f / (fxd + fyd);
    const float hsxn = fmaf(sxm, issum, fxd * ifsum);
    const float hsyn = fmaf(sym, issum, fyd * ifsum);
    const float ihx = 1.0f / hsxn, ihy = 1.0f / hsyn;
    const float sxn = sx * ihx, syn = sy * ihy;
    const float q = fmaf(sxn, sxn, syn * syn);
    float sc, calpha, salpha;
    if (q > 0.f) {
        const float isc = rsqrtf(q);
        sc = q * isc;
        calpha = sxn * isc;
        salpha = syn * isc;
    } else {
        sc = 0.f;
        calpha = 0.70710678f;
        salpha = 0.70710678f;
    }
    auto hyp = [](float a, float b) { return sqrtf(fmaf(a, a, b * b)); };
    const float df0 = hyp(dfx0 * calpha * hsxn, dfy0 * salpha * hsyn);
    const float fm = hyp(fxm * calpha, fym * salpha);
    const float cax = calpha * ihx, say = salpha * ihy;
    const float sm = hyp(sxm * cax, sym * say);
    const float fs = hyp(fxs * calpha, fys * salpha);
    const float ss = hyp(sxs * cax, sys * say);
    float f, fos;
    tmxyf(f, fos, sc, df0, sm, fm, ss, fs);
    ta.My = -K(K_RR) * fz * ta.rStat * sgnf_of_d(omega);
    const float vtxs = fmaf(rw, hsxn, 0.01f);
    const float vtys = fmaf(rw, hsyn, 0.01f);
    const float cx = K(K_CX), cy = K(K_CY), dx = K(K_DX), dy = K(K_DY);
    const float xe = ts.xe, ye = ts.ye;
    const float numx = fmaf(-vtxs * cx, xe, -fos * vsx);
    const float numy = fmaf(-vtys * cy, ye, fos * (sy * vta));
    const float xedot = numx / fmaf(vtxs, dx, fos);
    const float yedot = numy / fmaf(vtys, dy, fos);
    ts.xedot = xedot;
    ts.yedot = yedot;
    const float fxdyn = fmaf(dx, xedot, cx * xe);
    const float fydyn = fmaf(dy, yedot, cy * ye);
    const float fxstr = fminf(fmaxf(fmaf(xe, cx, xedot * dx), -K(K_FXMP2N)), K(K_FXMP2N));
    const float fystr = fminf(fmaxf(fmaf(ye, cy, yedot * dy), -K(K_FYMP2N)), K(K_FYMP2N));
    const float wx = sine_stepf(fabsf(vsx), 1.f, 1.f, 1.5f, 0.f);
    const float wy = sine_stepf(fabsf(sy * vta), 1.f, 1.f, 1.5f, 0.f);
    ta.fx = (wx == 0.f) ? fxdyn : fmaf(wx, fxstr, (1.f - wx) * fxdyn);
    ta.fy = (wy == 0.f) ? fydyn : fmaf(wy, fystr, (1.f - wy) * fydyn);
}

__device__ __forceinline__ void diff_splitf(float torque, float wl, float wr, float& tl, float& tr) {
    const float diff = fabsf(wl - wr);
    float alpha;
    if (diff > 0.5f) alpha = 2.0f / 3.0f;
    else if (diff > 0.25f) {
        const float bias = 4.f * diff;
        alpha = bias / (1.f + bias);
    } else alpha = 0.5f;
    const float slow = alpha * torque;
    const float fast = torque - slow;
    if (fabsf(wl) < fabsf(wr)) {
        tl = slow;
        tr = fast;
    } else {
        tl = fast;
        tr = slow;
    }
}

__device__ __forceinline__ float drive_torquef(const ClassDev18F& C, float throttle, float w) {
    if (C.throttleMod) return map_yf_scaled(C.pt, w, throttle) + map_yf(C.loss, w);
    return fmaf(map_yf(C.pt, w), throttle, map_yf(C.loss, w));
}

// One mixed-precision step: RHS then the half-implicit update (FP64 states).
__device__ __forceinline__ void step18_mixed(VehM& v, VehAux& va, TireM* ts, TireAuxF* ta, const KViewF& K,
                                             const ClassDev18F& C, float steering, float throttle, float braking,
                                             double dt) {
    const float u = (float)v.u, vv = (float)v.v, wz = (float)v.wz, wx = (float)v.wx, phi = (float)v.phi;
    {
        const float lat = fmaf(wz, u, v.vdot);
        const float lon = fmaf(-wz, vv, v.udot);
        const float Z4 = K(K_Z4) * lon;
        const float Z2f = K(K_Z2F) * lat, Z3f = fmaf(K(K_Z3FK), phi, K(K_Z3FB) * wx);
        const float Z2r = K(K_Z2R) * lat, Z3r = fmaf(K(K_Z3RK), phi, K(K_Z3RB) * wx);
        const float Af = K(K_Z1F) - Z4, Bf = Z2f + Z3f, Ar = K(K_Z1R) + Z4, Br = Z2r + Z3r;
        ta[0].fz = fmaxf(Af - Bf, 0.f);
        ta[1].fz = fmaxf(Af + Bf, 0.f);
        ta[2].fz = fmaxf(Ar - Br, 0.f);
        ta[3].fz = fmaxf(Ar + Br, 0.f);
    }
    const float delta = C.nonLinearSteer ? map_yf(C.steer, steering) : steering * K(K_MAXSTEER);
    float cd = 1.f, sd = 0.f;
    if (delta != 0.f) __sincosf(delta, &sd, &cd);
    {
        const float vsyf = fmaf(wz, K(K_A), vv), vsyr = fmaf(-wz, K(K_B), vv);
        const float wcf = wz * K(K_CF2), wcr = wz * K(K_CR2);
        ta[0].vsy = vsyf;
        ta[1].vsy = vsyf;
        ta[0].vsx = fmaf(u - wcf, cd, vsyf * sd);
        ta[1].vsx = fmaf(u + wcf, cd, vsyf * sd);
        ta[2].vsy = vsyr;
        ta[3].vsy = vsyr;
        ta[2].vsx = u - wcr;
        ta[3].vsx = u + wcr;
    }
    tire_rhs_tm_mixed<true>(ts[0], ta[0], K, cd, sd);
    tire_rhs_tm_mixed<true>(ts[1], ta[1], K, cd, sd);
    tire_rhs_tm_mixed<false>(ts[2], ta[2], K, 1.f, 0.f);
    tire_rhs_tm_mixed<false>(ts[3], ta[3], K, 1.f, 0.f);
    // powertrain (dof18_gpu.cu:664-839)
    const float w0 = (float)ts[0].omega, w1 = (float)ts[1].omega, w2 = (float)ts[2].omega, w3 = (float)ts[3].omega;
    float torque_t;
    float dcrank = 0.f;
    const int g = v.gear;
    if (C.tcbool) {
        bool reverse = false;
        const float omega_out = 0.25f * (((w0 + w1) + w2) + w3) / C.gear[g];
        const float omega_in = (float)v.crank;
        float sr = 0.f;
        if (!((omega_out < 1e-9f) || (omega_in < 1e-9f))) {
            sr = omega_out / omega_in;
            if (sr > 1.f) {
                sr = 1.f - (sr - 1.f);
                reverse = true;
            }
            if (sr < 0.f) sr = 0.f;
        }
        const float cf = map_yf(C.cf, sr), tr = map_yf(C.tr, sr);
        const float r = omega_in / cf;
        float torque_in = -(r * r);
        if (reverse) torque_in = -torque_in;
        const float torque_out = reverse ? -torque_in : -tr * torque_in;
        torque_t = torque_out / C.gear[g];
        if (u < 1e-9f && torque_t < 0.f) torque_t = 0.f;
        dcrank = K(K_INVCI) * (drive_torquef(C, throttle, omega_in) + torque_in);
        if (omega_out > C.up[g]) {
            if (g < C.noGears - 1) v.gear = g + 1;
        } else if (omega_out < C.down[g]) {
            if (g > 0) v.gear = g - 1;
        }
    } else {
        const float crank = 0.25f * (((w0 + w1) + w2) + w3) / C.gear[g];
        v.crank = crank;
        torque_t = drive_torquef(C, throttle, crank) / C.gear[g];
        if (u < 1e-9f && torque_t < 0.f) torque_t = 0.f;
        if (crank > C.up[g]) {
            if (g < C.noGears - 1) v.gear = g + 1;
        } else if (crank < C.down[g]) {
            if (g > 0) v.gear = g - 1;
        }
    }
    float tf, trr;
    if (C.driveType) {
        tf = torque_t * 0.5f;
        trr = torque_t * 0.5f;
    } else if (C.whichWheels) {
        tf = 0.f;
        trr = torque_t;
    } else {
        tf = torque_t;
        trr = 0.f;
    }
    diff_splitf(tf, w0, w1, ta[0].engTor, ta[1].engTor);
    diff_splitf(trr, w2, w3, ta[2].engTor, ta[3].engTor);
    const float brake = K(K_MAXBRAKE) * braking, ijw = K(K_INVJW);
    const float wk[4] = {w0, w1, w2, w3};
#pragma unroll
    for (int k = 0; k < 4; ++k)
        ta[k].dOmega = ijw * (fmaf(-sgnf_(wk[k]), brake, ta[k].engTor + ta[k].My) - ta[k].fx * ta[k].rStat);
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const float fx = ta[k].fx, fy = ta[k].fy;
        ta[k].fx = fmaf(fx, cd, -fy * sd);
        ta[k].fy = fmaf(fx, sd, fy * cd);
    }
    float udot, vdot, wxdot, wzdot;
    {
        const float fx0 = ta[0].fx, fx1 = ta[1].fx, fx2 = ta[2].fx, fx3 = ta[3].fx;
        const float fy0 = ta[0].fy, fy1 = ta[1].fy, fy2 = ta[2].fy, fy3 = ta[3].fy;
        const float wu = wz * u, fyf = fy0 + fy1, fyr = fy2 + fy3;
        const float E1 = fmaf(-K(K_MT), wu, fyf + fyr);
        const float E2 = fmaf(K(K_E2WU), wu,
                              fmaf(fx3 - fx2, K(K_CR2), fmaf(fx1 - fx0, K(K_CF2), fmaf(fyf, K(K_A), -fyr * K(K_B)))));
        const float E3 = fmaf(K(K_E3WU), wu, fmaf(K(K_E3PHI), phi, K(K_E3WX) * wx));
        const float sfx = ((fx0 + fx1) + fx2) + fx3;
        udot = fmaf(K(K_INVMT), fmaf(K(K_UWZ2), wz * wz, fmaf(-K(K_UWZWX), wz * wx, sfx)), wz * vv);
        vdot = fmaf(K(K_CV1), E1, fmaf(K(K_CV2), E2, K(K_CV3) * E3));
        wxdot = fmaf(K(K_CV3), E1, fmaf(K(K_CX2), E2, K(K_CX3) * E3));
        wzdot = fmaf(K(K_CV2), E1, fmaf(K(K_CZ2), E2, K(K_CX2) * E3));
    }
    // half-implicit update in FP64 (dof18_halfImplicit_gpu.cu:913-946)
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        ts[k].xe = fmaf(ts[k].xedot, (float)dt, ts[k].xe);
        ts[k].ye = fmaf(ts[k].yedot, (float)dt, ts[k].ye);
        ts[k].omega = fma((double)ta[k].dOmega, dt, ts[k].omega);
    }
    va.dOmega_crank = dcrank;
    if (C.tcbool) v.crank = fma((double)dcrank, dt, v.crank);
    v.udot = udot;
    v.vdot = vdot;
    va.wxdot = wxdot;
    va.wzdot = wzdot;
    v.u = fma((double)udot, dt, v.u);
    v.v = fma((double)vdot, dt, v.v);
    v.wx = fma((double)wxdot, dt, v.wx);
    v.wz = fma((double)wzdot, dt, v.wz);
    // yaw reduced to [-pi, pi] in FP64, then FP32 sine/cosine; X/Y accumulated in FP64
    const double pr = v.psi - 6.283185307179586 * rint(v.psi * 0.15915494309189535);
    float sp, cp;
    sincosf((float)pr, &sp, &cp);
    const float uu = (float)v.u, vn = (float)v.v;
    v.x = fma((double)fmaf(uu, cp, -vn * sp), dt, v.x);
    v.y = fma((double)fmaf(uu, sp, vn * cp), dt, v.y);
    v.psi = fma(v.wz, dt, v.psi);
    v.phi = fma(v.wx, dt, v.phi);
}

}  // namespace lfdm
