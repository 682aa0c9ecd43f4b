// 18-DOF vehicle model: device-side data layouts and the right-hand side + half-implicit update.
//
// Algorithm: the reference's rhsFun (18dof-gpu/dof18_halfImplicit_gpu.cu:685-729) and Integrate
// update (:913-946) with the physics of 18dof-gpu/dof18_gpu.cu. The arithmetic is rearranged for
// a GPU whose FP64 issue rate is the bottleneck (every rearrangement is exact in real arithmetic
// and changes results only at the rounding level):
//   * parameter-only subexpressions are evaluated once per vehicle (prepare_constants18);
//   * pow(x, 2) -> x*x; hypot(x, y) -> sqrt(x*x + y*y);
//   * -tan(atan2(vsy, vta) - delta) -> -(vsy*cos d - vta*sin d) / (vta*cos d + vsy*sin d)
//     (tangent difference identity; vta > 0);
//   * sin/cos of the wheel angle once per step instead of once per use;
//   * divisions sharing a step are merged into one reciprocal where the operands allow.
// Branch structure (wheel lift-off, tmxy_combined regimes, gear shifts, torque-converter flow
// direction, sineStep bands) is kept exactly, so the branch taken matches the reference whenever
// the compared quantities agree.
#pragma once

#include <cstdint>

#include "../../lfdm.h"
#include "fp_order.cuh"

namespace lfdm {

constexpr double kG = 9.81;                                       // utils/utils_gpu.cuh:12
constexpr double k2Pi = 6.283185307179586476925286766559;         // utils/utils_gpu.cuh:11
constexpr double kSqrt2Over2 = 0.70710678118654757;               // sqrt(2.)/2. rounded to double

// ---------------------------------------------------------------------------------------------
// Per-vehicle derived constants (FP64), SoA [K18_COUNT][n_pad] in HBM, staged per block.
enum K18 : int {
    // Shared prefix [0, KT_COUNT), also the head of the 24-DOF constants (K24 in dof24_device.cuh):
    // computeTireRHS (dof18_gpu.cu:379-530)
    K_R0 = 0, K_INVKT, K_INVPN, K_PNMAX, K_FZRD, K_RDPN, K_DRD, K_RDCRIT,
    K_Q1DFX0, K_Q2DFX0, K_Q1DFY0, K_Q2DFY0, K_Q1FXM, K_Q2FXM, K_Q1FYM, K_Q2FYM, K_Q1FXS, K_Q2FXS, K_Q1FYS,
    K_Q2FYS,
    K_LSXM, K_DSXM, K_LSYM, K_DSYM, K_LSXS, K_DSXS, K_LSYS, K_DSYS,
    K_CX, K_CY, K_DX, K_DY, K_FXMP2N, K_FYMP2N, K_RR,
    // TMeasyNr extras (dof18_gpu.cu:532-662)
    K_MU, K_VCOUL, K_FRB0, K_FRB1,
    // powertrain and steering
    K_INVCI, K_MAXBRAKE, K_INVJW, K_MAXSTEER,
    KT_COUNT,
    // 18-DOF (and 11-DOF) only
    K_A = KT_COUNT, K_B, K_CF2, K_CR2,
    // computeTireLoads (dof18_gpu.cu:305-340)
    K_Z1F, K_Z2F, K_Z3FK, K_Z3FB, K_Z4, K_Z1R, K_Z2R, K_Z3RK, K_Z3RB,
    // computeVehRHS (dof18_gpu.cu:1017-1068)
    K_MT, K_INVMT, K_E2WU, K_E3PHI, K_E3WX, K_E3WU, K_UWZ2, K_UWZWX,
    K_CV1, K_CV2, K_CV3, K_CX2, K_CX3, K_CZ2,
    // 11-DOF yaw (11dof-gpu/dof11_gpu.cu:893-909)
    K_INVJZ,
    K18_COUNT
};

// ---------------------------------------------------------------------------------------------
// Per-class tables (flags, gears, maps) with precomputed segment reciprocals, staged in smem.
struct MapDev {
    int n;
    int pad_;
    double x[LFDM_MAX_MAP];
    double y[LFDM_MAX_MAP];
    double dx[LFDM_MAX_MAP];     // x[k+1] - x[k]
    double dy[LFDM_MAX_MAP];     // y[k+1] - y[k]
    double idx[LFDM_MAX_MAP];    // 1 / dx[k]
    long long kx[LFDM_MAX_MAP];  // order keys of x[k] (okey)
};
struct ClassDev18 {
    int nonLinearSteer, tcbool, throttleMod, driveType, whichWheels, noGears;
    double gear[LFDM_MAX_GEARS];
    double invgear[LFDM_MAX_GEARS];
    double down[LFDM_MAX_GEARS];
    double up[LFDM_MAX_GEARS];
    MapDev steer, pt, loss, cf, tr;
};

// lower_bound over the order keys of a sorted array: first k with x <= a[k]
// (utils/utils_gpu.cu:109-121), with integer compares.
__device__ __forceinline__ int lower_bound_key(const long long* a, int n, long long k) {
    int l = 0, h = n;
    while (l < h) {
        int mid = (l + h) >> 1;
        if (k <= a[mid]) h = mid;
        else l = mid + 1;
    }
    return l;
}

// lower_bound over a sorted key array: first k with x <= a[k] (utils/utils_gpu.cu:109-121).
__device__ __forceinline__ int lower_bound_x(const double* a, int n, double x) {
    int l = 0, h = n;
    while (l < h) {
        int mid = (l + h) >> 1;
        if (x <= a[mid]) h = mid;
        else l = mid + 1;
    }
    return l;
}

// getMapY (utils/utils_gpu.cu:60-75): clamp outside, linear interpolation inside. The quotient
// (x - x[l]) / dx[l] is a product with the segment's stored reciprocal, except at the segment's
// right grid point, where it is exactly 1 as the reference's division gives: a map evaluated at a
// grid point returns the tabulated value (an engine at rest sees exactly the loss torque at
// 0 rad/s and stays at rest, as in the reference).
__device__ __forceinline__ double map_y(const MapDev& m, double x) {
    const long long k = okey(x);
    if (k <= m.kx[0]) return m.y[0];
    if (k >= m.kx[m.n - 1]) return m.y[m.n - 1];
    const int r = lower_bound_key(m.kx, m.n, k);
    const int l = r - 1;
    const double mbar = (k == m.kx[r]) ? 1.0 : (x - m.x[l]) * m.idx[l];
    return fma(mbar, m.dy[l], m.y[l]);
}

// getMapY on the map with both coordinates scaled by s (driveTorque with throttleMod,
// dof18_gpu.cu:18-31; the scaled copy is private to the call as in 18dof/dof18.cpp:23-29).
__device__ __forceinline__ double map_y_scaled(const MapDev& m, double x, double s) {
    const int n = m.n;
    if (x <= m.x[0] * s) return m.y[0] * s;
    if (x >= m.x[n - 1] * s) return m.y[n - 1] * s;
    int l = 0, h = n;
    while (l < h) {
        int mid = (l + h) >> 1;
        if (x <= m.x[mid] * s) h = mid;
        else l = mid + 1;
    }
    const int r = l, lf = r - 1;
    const double xl = m.x[lf] * s, xr = m.x[r] * s, yl = m.y[lf] * s, yr = m.y[r] * s;
    double mbar = (x - xl) / (xr - xl);
    return yl + mbar * (yr - yl);
}

// sineStep (utils/utils_gpu.cu:78-88). sin(2 pi u) for u in (0, 1) is taken as sinpi(2 u): the same
// function, with an exact argument reduction instead of the reduction of the rounded 2 pi u.
__device__ __forceinline__ double sine_step(double x, double x1, double y1, double x2, double y2) {
    if (x <= x1) return y1;
    if (x >= x2) return y2;
    double dx = x2 - x1;
    double dy = y2 - y1;
    double u = (x - x1) / dx;
    return y1 + dy * u - (dy / k2Pi) * sinpi(2.0 * u);
}

// sgn (utils/utils_gpu.cuh): -1, 0 or 1 (0 for both zeros)
__device__ __forceinline__ double sgnd(double v) {
    const unsigned long long u = static_cast<unsigned long long>(dbits(v));
    return (u << 1) == 0 ? 0.0 : ((u >> 63) ? -1.0 : 1.0);
}

// sineStep for x >= 0 and 0 <= x1 < x2 (the tire blends): the same value, integer bound tests
__device__ __forceinline__ double sine_step_nn(double x, double x1, double y1, double x2, double y2) {
    if (!gt_nn(x, x1)) return y1;
    if (!gt_nn(x2, x)) return y2;
    const double dx = x2 - x1;
    const double dy = y2 - y1;
    const double u = (x - x1) / dx;
    return y1 + dy * u - (dy / k2Pi) * sinpi(2.0 * u);
}

// The structural/dynamic blend weights of one tire, sineStep(a, 1, 1, 1.5, 0) of its longitudinal
// and lateral slip speeds (computeTireRHS, 18dof-gpu/dof18_gpu.cu:509-529), for the lanes of a warp
// together. Outside the band 1 < a < 1.5 the weight is 1 or 0; inside it takes a division by a
// constant and a sine. Evaluated lane by lane, a warp runs the band code once for the x blend and
// once for the y blend whenever any of its lanes is in that band, so it pays two band evaluations
// on nearly every step. Here the warp's in-band arguments (x blends first, then y blends) are dealt
// to its lanes, each lane evaluates one (with sine_step_nn itself, so each weight is the value it
// had lane by lane, bit for bit) and the weights are returned to their lanes: one band evaluation
// per 32 in-band arguments. The lanes that reach this point together (__activemask) take part, so
// lanes that left earlier (a lifted wheel, a finished vehicle) are not waited for.
__device__ __forceinline__ void blend_weights(double ax, double ay, double& wx, double& wy) {
    const bool bx = gt_nn(ax, 1.0) && gt_nn(1.5, ax);
    const bool by = gt_nn(ay, 1.0) && gt_nn(1.5, ay);
    wx = gt_nn(ax, 1.0) ? 0.0 : 1.0;  // the band's lanes are filled in below
    wy = gt_nn(ay, 1.0) ? 0.0 : 1.0;
    const unsigned act = __activemask();
    const unsigned mx = __ballot_sync(act, bx), my = __ballot_sync(act, by);
    const int nx = __popc(mx), total = nx + __popc(my);
    if (total == 0) return;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned below = (1u << lane) - 1u;
    const int nact = __popc(act), rank = __popc(act & below);
    const int ex = __popc(mx & below), ey = nx + __popc(my & below);  // this lane's entries
    for (int base = 0; base < total; base += nact) {
        const int e = base + rank;  // the entry this lane evaluates
        const bool isx = e < nx;
        const unsigned src = e < total ? __fns(isx ? mx : my, 0, (isx ? e : e - nx) + 1) : lane;
        const double vx = __shfl_sync(act, ax, src), vy = __shfl_sync(act, ay, src);
        const double a = e < total ? (isx ? vx : vy) : 1.25;  // idle lanes evaluate an in-band dummy
        const double w = sine_step_nn(a, 1., 1., 1.5, 0.);
        const int ox = ex - base, oy = ey - base;
        const bool gx = bx && ox >= 0 && ox < nact, gy = by && oy >= 0 && oy < nact;
        const double rx = __shfl_sync(act, w, gx ? __fns(act, 0, ox + 1) : lane);
        const double ry = __shfl_sync(act, w, gy ? __fns(act, 0, oy + 1) : lane);
        if (gx) wx = rx;
        if (gy) wy = ry;
    }
}

// The shared prefix [0, KT_COUNT) of the derived constants from one flat parameter vector p:
// tire curve coefficients (InterpQ(fz,w1,w2,pn) = fzn*(Q1 - Q2*fzn), InterpL(fz,w1,w2,pn) =
// w1 + (w2-w1)*(fzn-1) with fzn = fz/pn, utils_gpu.cuh:86-93), powertrain and steering constants.
template <typename Put>
__device__ __forceinline__ void prepare_shared_k(const double* p, Put& put) {
    put(K_MAXSTEER, p[LFDM_P_MAXSTEER]);
    put(K_INVCI, 1. / p[LFDM_P_CRANKINERTIA]);
    put(K_MAXBRAKE, p[LFDM_P_MAXBRAKETORQUE]);
    put(K_INVJW, 1 / p[LFDM_P_JW]);
    put(K_R0, p[LFDM_P_R0]);
    put(K_INVKT, 1. / p[LFDM_P_KT]);
    put(K_INVPN, 1. / p[LFDM_P_PN]);
    put(K_PNMAX, p[LFDM_P_PNMAX]);
    put(K_FZRD, p[LFDM_P_FZRDYNCO]);
    put(K_RDPN, p[LFDM_P_RDYNCOPN]);
    put(K_DRD, p[LFDM_P_RDYNCOP2N] - p[LFDM_P_RDYNCOPN]);
    put(K_RDCRIT, p[LFDM_P_RDYNCOCRIT]);
    auto q = [&](int k1, int k2, double w1, double w2) {
        put(k1, 2. * w1 - 0.5 * w2);
        put(k2, w1 - 0.5 * w2);
    };
    q(K_Q1DFX0, K_Q2DFX0, p[LFDM_P_DFX0PN], p[LFDM_P_DFX0P2N]);
    q(K_Q1DFY0, K_Q2DFY0, p[LFDM_P_DFY0PN], p[LFDM_P_DFY0P2N]);
    q(K_Q1FXM, K_Q2FXM, p[LFDM_P_FXMPN], p[LFDM_P_FXMP2N]);
    q(K_Q1FYM, K_Q2FYM, p[LFDM_P_FYMPN], p[LFDM_P_FYMP2N]);
    q(K_Q1FXS, K_Q2FXS, p[LFDM_P_FXSPN], p[LFDM_P_FXSP2N]);
    q(K_Q1FYS, K_Q2FYS, p[LFDM_P_FYSPN], p[LFDM_P_FYSP2N]);
    auto l = [&](int k1, int k2, double w1, double w2) {
        put(k1, w1);
        put(k2, w2 - w1);
    };
    l(K_LSXM, K_DSXM, p[LFDM_P_SXMPN], p[LFDM_P_SXMP2N]);
    l(K_LSYM, K_DSYM, p[LFDM_P_SYMPN], p[LFDM_P_SYMP2N]);
    l(K_LSXS, K_DSXS, p[LFDM_P_SXSPN], p[LFDM_P_SXSP2N]);
    l(K_LSYS, K_DSYS, p[LFDM_P_SYSPN], p[LFDM_P_SYSP2N]);
    put(K_CX, p[LFDM_P_CX]);
    put(K_CY, p[LFDM_P_CY]);
    put(K_DX, p[LFDM_P_DX]);
    put(K_DY, p[LFDM_P_DY]);
    put(K_FXMP2N, p[LFDM_P_FXMP2N]);
    put(K_FYMP2N, p[LFDM_P_FYMP2N]);
    put(K_RR, p[LFDM_P_RR]);
    put(K_MU, p[LFDM_P_MU]);
    put(K_VCOUL, p[LFDM_P_VCOULOMB]);
    put(K_FRB0, p[LFDM_P_FRBLEND_BEGIN]);
    put(K_FRB1, p[LFDM_P_FRBLEND_END]);
}

// ---------------------------------------------------------------------------------------------
// Carried state of one vehicle (registers).
struct TireC {
    double xe, ye, xedot, yedot, omega;
};
struct VehC {
    double x, y, u, v, psi, wz, phi, wx, udot, vdot, crank;
    int gear;
};
// Values of the last RHS evaluation (written back with the state at the end of a window so that
// GetSimState returns the reference's full SimState).
struct TireAux {
    double dOmega, xt, rStat, fx, fy, fz, vsx, vsy, My, engTor;
};
struct VehAux {
    double wxdot, wzdot, dOmega_crank;
};

// The 18-DOF state of one vehicle from / to its SoA column S (S[field * np]).
__device__ __forceinline__ void load_state18(const double* S, size_t np, VehC& v, VehAux& va, TireC* ts,
                                             TireAux* ta) {
    v.x = S[LFDM_S_X * np];
    v.y = S[LFDM_S_Y * np];
    v.u = S[LFDM_S_U * np];
    v.v = S[LFDM_S_V * np];
    v.psi = S[LFDM_S_PSI * np];
    v.wz = S[LFDM_S_WZ * np];
    v.phi = S[LFDM_S_PHI * np];
    v.wx = S[LFDM_S_WX * np];
    v.udot = S[LFDM_S_UDOT * np];
    v.vdot = S[LFDM_S_VDOT * np];
    v.crank = S[LFDM_S_CRANKOMEGA * np];
    v.gear = (int)S[LFDM_S_CURRENT_GR * np];
    va.wxdot = S[LFDM_S_WXDOT * np];
    va.wzdot = S[LFDM_S_WZDOT * np];
    va.dOmega_crank = S[LFDM_S_DOMEGA_CRANK * np];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const size_t b = (size_t)(LFDM_S_TIRE0 + k * LFDM_S_TIRE_STRIDE) * np;
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
__device__ __forceinline__ void store_state18(double* S, size_t np, const VehC& v, const VehAux& va, const TireC* ts,
                                              const TireAux* ta) {
    S[LFDM_S_X * np] = v.x;
    S[LFDM_S_Y * np] = v.y;
    S[LFDM_S_U * np] = v.u;
    S[LFDM_S_V * np] = v.v;
    S[LFDM_S_PSI * np] = v.psi;
    S[LFDM_S_WZ * np] = v.wz;
    S[LFDM_S_PHI * np] = v.phi;
    S[LFDM_S_WX * np] = v.wx;
    S[LFDM_S_UDOT * np] = v.udot;
    S[LFDM_S_VDOT * np] = v.vdot;
    S[LFDM_S_WXDOT * np] = va.wxdot;
    S[LFDM_S_WZDOT * np] = va.wzdot;
    S[LFDM_S_CRANKOMEGA * np] = v.crank;
    S[LFDM_S_DOMEGA_CRANK * np] = va.dOmega_crank;
    S[LFDM_S_CURRENT_GR * np] = (double)v.gear;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const size_t b = (size_t)(LFDM_S_TIRE0 + k * LFDM_S_TIRE_STRIDE) * np;
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
__device__ __forceinline__ bool state18_finite(const VehC& v, const TireC* ts) {
    return isfinite(v.x) && isfinite(v.y) && isfinite(v.u) && isfinite(v.v) && isfinite(v.psi) && isfinite(v.wz) &&
           isfinite(ts[0].omega) && isfinite(ts[1].omega) && isfinite(ts[2].omega) && isfinite(ts[3].omega);
}

// Constant accessor: K(i) reads derived constant i of this thread's vehicle.
struct KView {
    const double* base;  // base + i*stride
    int stride;
    const float* fbase = nullptr;  // FP32 copies of the same constants (kernels with an FP32 tire core)
    __device__ __forceinline__ double operator()(int i) const { return base[i * stride]; }
    __device__ __forceinline__ float f(int i) const { return fbase[i * stride]; }
};

// The transition regime of tmxy_combined (sm <= s <= ss; dof18_gpu.cu:262-276) without a division.
// With q = fm / sm, D = df0loc sm, dss = ss - sm, E = q^2 dss and H = (fm - fs) D, the first
// parabola's coefficient is a = q^2 / D and the parabolas' joint is sstar = sm + H / E; as D and E
// are positive here, sstar <= ss reads H <= dss E and s <= sstar reads (s - sm) E <= H. Returns 0
// (first parabola), 1 (second parabola) or 2 (the cubic, where the joint lies beyond ss).
__device__ __forceinline__ int tmxy_joint(double s, double fm, double ism, double df0loc, double sm, double ss,
                                          double fs, double& q2, double& D, double& E, double& H) {
    const double q = fm * ism;
    q2 = q * q;
    D = df0loc * sm;
    E = q2 * (ss - sm);
    H = (fm - fs) * D;
    if (H <= (ss - sm) * E) return (s - sm) * E <= H ? 0 : 1;
    return 2;
}

// The force of the transition regime as f = num / den over the denominator of its piece.
__device__ __forceinline__ void tmxy_transition(double& num, double& den, double s, double df0loc, double sm,
                                                double ism, double fm, double ss, double fs) {
    double q2, D, E, H;
    const int piece = tmxy_joint(s, fm, ism, df0loc, sm, ss, fs, q2, D, E, H);
    const double ds = s - sm, dss = ss - sm;
    if (piece == 0) {  // f = fm - a ds^2, a = q^2 / D
        num = fma(-q2 * ds, ds, fm * D);
        den = D;
    } else if (piece == 1) {  // f = fs + b (ss - s)^2, b = a (sstar - sm) / (ss - sstar) = q^2 (fm - fs) / G
        const double G = fma(dss, E, -H);
        const double r = ss - s;
        num = fma(q2 * (fm - fs) * r, r, fs * G);
        den = G;
    } else {  // f = fm - (fm - fs) sn^2 (3 - 2 sn), sn = ds / dss
        const double d3 = dss * dss * dss;
        num = fma(-(fm - fs) * ds * ds, fma(-2.0, ds, 3.0 * dss), fm * d3);
        den = d3;
    }
}

// tmxy_combined (dof18_gpu.cu:243-285) given the reciprocals of s, sm and fm (is, ism, ifm; the
// TMeasy tire has them from the rsqrt of the squared norms it takes anyway). Returns the ratio of
// the combined force to the combined slip, fos = f / s, as a fraction fn / fd that the caller folds
// into its own division: in the adhesion regime, which nearly every step is in, fos = df0 / dn; in
// the transition regime fd is the denominator of its piece (tmxy_transition); in full sliding
// fd = 1. No regime divides (is = 1/s).
__device__ __forceinline__ void tmxy_frac(double& fn, double& fd, double s, double is, double df0, double sm,
                                          double ism, double fm, double ifm, double ss, double fs) {
    fd = 1.0;
    double df0loc = 0.0;
    if (gt0(sm)) df0loc = max_nn(2.0 * fm * ism, df0);
    if (gt0(s) && gt0(df0loc)) {
        if (gt_nn(s, ss)) {
            fn = fs * is;
        } else if (gt_nn(sm, s)) {  // adhesion: f = df0 sm sn / dn, s = sm sn
            const double p = df0loc * sm * ifm - 2.0;
            const double sn = s * ism;
            fd = fma(sn + p, sn, 1.0);
            fn = df0loc;
        } else {  // transition: fos = num / (den s)
            tmxy_transition(fn, fd, s, df0loc, sm, ism, fm, ss, fs);
            fn *= is;
        }
    } else {
        fn = 0.0;
    }
}

// sqrt(a^2 + b^2) and its reciprocal from one rsqrt (0 and 0 for a zero vector)
__device__ __forceinline__ void hyp_rcp(double a, double b, double& h, double& ih) {
    const double q = fma(a, a, b * b);
    if (gt0(q)) {
        ih = rsqrt(q);
        h = q * ih;
    } else {
        h = 0.0;
        ih = 0.0;
    }
}

// tmxy_combined (dof18_gpu.cu:243-285)
__device__ __forceinline__ void tmxy(double& f, double& fos, double s, double df0, double sm, double fm,
                                     double ss, double fs) {
    double df0loc = 0.0;
    double ism = 0.0;
    if (sm > 0.0) {
        ism = 1.0 / sm;
        df0loc = fmax(2.0 * fm * ism, df0);
    }
    if (s > 0.0 && df0loc > 0.0) {
        if (s > ss) {
            f = fs;
            fos = fs / s;
        } else if (s < sm) {  // adhesion
            double p = df0loc * sm / fm - 2.0;
            double sn = s * ism;
            double dn = fma(sn + p, sn, 1.0);
            double idn = 1.0 / dn;
            f = df0loc * sm * sn * idn;
            fos = df0loc * idn;
        } else {  // the piece and its force as tmxy_frac takes them, with one division
            double num, den;
            tmxy_transition(num, den, s, df0loc, sm, ism, fm, ss, fs);
            f = num / den;
            fos = f / s;
        }
    } else {
        f = 0.0;
        fos = 0.0;
    }
}

// The part of computeTireRHS, TMeasy (dof18_gpu.cu:379-530; 24dof-gpu/dof24_gpu.cu), that follows
// the loaded and effective radii: slips, curve parameters, combined force, rolling resistance,
// relaxation rates and the structural/dynamic blend. fz > 0 is the unclamped load, ta.rStat the
// loaded radius. (c, s) = (cos, sin) of this tire's wheel angle; steered says whether the angle
// may be nonzero.
template <bool kSteered>
__device__ __forceinline__ void tire_core_tm(TireC& ts, TireAux& ta, const KView& K, double c, double s, double fz,
                                             double r_eff) {
    const double omega = ts.omega;
    const double vsy = ta.vsy;
    const double vsx = fma(-omega, r_eff, ta.vsx);
    const double rw = r_eff * fabs(omega);
    const double vta = rw + 0.01;
    fz = min_nn(fz, K(K_PNMAX));
    const double fzn = fz * K(K_INVPN);
    const double dfx0 = fzn * fma(-K(K_Q2DFX0), fzn, K(K_Q1DFX0));
    const double dfy0 = fzn * fma(-K(K_Q2DFY0), fzn, K(K_Q1DFY0));
    const double fxm = fzn * fma(-K(K_Q2FXM), fzn, K(K_Q1FXM));
    const double fym = fzn * fma(-K(K_Q2FYM), fzn, K(K_Q1FYM));
    const double fxs = fzn * fma(-K(K_Q2FXS), fzn, K(K_Q1FXS));
    const double fys = fzn * fma(-K(K_Q2FYS), fzn, K(K_Q1FYS));
    const double fzn1 = fzn - 1.0;
    const double sxm = fma(K(K_DSXM), fzn1, K(K_LSXM));
    const double sym = fma(K(K_DSYM), fzn1, K(K_LSYM));
    const double sxs = fma(K(K_DSXS), fzn1, K(K_LSXS));
    const double sys = fma(K(K_DSYS), fzn1, K(K_LSYS));
    // hsxn = sxm/(sxm+sym) + (fxm/dfx0)/(fxm/dfx0 + fym/dfy0). One division gives 1/(ssum fsum) for
    // both quotients, 1/vta for the slips and, on a steered wheel, 1/(vta c + vsy s) for the
    // lateral slip -(vsy c - vta s)/(vta c + vsy s) (sy = -tan(atan2(vsy, vta) - delta)).
    const double ssum = sxm + sym;
    const double fxd = fxm * dfy0, fyd = fym * dfx0;
    const double fsum = fxd + fyd;
    const double p12 = ssum * fsum;
    double r12, ivta, sy;
    if (kSteered) {
        const double den = fma(vta, c, vsy * s);
        const double pv = vta * den;
        const double r = 1.0 / (p12 * pv);
        r12 = pv * r;
        const double ipv = p12 * r;
        ivta = den * ipv;
        sy = -fma(vsy, c, -vta * s) * (vta * ipv);
    } else {
        const double r = 1.0 / (p12 * vta);
        r12 = vta * r;
        ivta = p12 * r;
        sy = -vsy * ivta;
    }
    const double sx = -vsx * ivta;
    const double issum = fsum * r12, ifsum = ssum * r12;
    const double hsxn = fma(sxm, issum, fxd * ifsum);
    const double hsyn = fma(sym, issum, fyd * ifsum);
    const double rh = 1.0 / (hsxn * hsyn);
    const double ihx = hsyn * rh, ihy = hsxn * rh;
    const double sxn = sx * ihx;
    const double syn = sy * ihy;
    const double q = fma(sxn, sxn, syn * syn);
    double sc, calpha, salpha, isc = 0.0;
    if (gt0(q)) {
        isc = rsqrt(q);
        sc = q * isc;
        calpha = sxn * isc;
        salpha = syn * isc;
    } else {
        sc = 0;
        calpha = kSqrt2Over2;
        salpha = kSqrt2Over2;
    }
    auto hyp = [](double a, double b) { return sqrt(fma(a, a, b * b)); };
    const double df0 = hyp(dfx0 * calpha * hsxn, dfy0 * salpha * hsyn);
    double fm, ifm, sm, ism;
    hyp_rcp(fxm * calpha, fym * salpha, fm, ifm);
    const double cax = calpha * ihx, say = salpha * ihy;
    hyp_rcp(sxm * cax, sym * say, sm, ism);
    const double fs = hyp(fxs * calpha, fys * salpha);
    const double ss = hyp(sxs * cax, sys * say);
    double fn, fd;
    tmxy_frac(fn, fd, sc, isc, df0, sm, ism, fm, ifm, ss, fs);
    // rolling resistance: sineStep(vta, 0, 0, 0, 1) == 1 for vta >= 0.01
    ta.My = -K(K_RR) * fz * ta.rStat * sgnd(omega);
    const double vtxs = fma(rw, hsxn, 0.01);
    const double vtys = fma(rw, hsyn, 0.01);
    const double cx = K(K_CX), cy = K(K_CY), dx = K(K_DX), dy = K(K_DY);
    // xedot = (-vtxs cx xe - fos vsx) / (vtxs dx + fos) with fos = fn / fd, numerator and denominator
    // scaled by fd (likewise yedot); one division for both rates
    const double numx = fma(-vtxs * cx, ts.xe * fd, -fn * vsx);
    const double numy = fma(-vtys * cy, ts.ye * fd, fn * (sy * vta));
    const double denx = fma(vtxs * dx, fd, fn), deny = fma(vtys * dy, fd, fn);
    const double rd = 1.0 / (denx * deny);
    ts.xedot = numx * (deny * rd);
    ts.yedot = numy * (denx * rd);
    const double fxdyn = fma(dx, ts.xedot, cx * ts.xe);
    const double fydyn = fma(dy, ts.yedot, cy * ts.ye);
    const double fxstr = clamp_sym(fma(ts.xe, cx, ts.xedot * dx), K(K_FXMP2N));
    const double fystr = clamp_sym(fma(ts.ye, cy, ts.yedot * dy), K(K_FYMP2N));
    double wx, wy;
    blend_weights(fabs(vsx), fabs(sy * vta), wx, wy);
    ta.fx = is_zero(wx) ? fxdyn : fma(wx, fxstr, (1. - wx) * fxdyn);
    ta.fy = is_zero(wy) ? fydyn : fma(wy, fystr, (1. - wy) * fydyn);
}

// ---------------------------------------------------------------------------------------------
// FP32 tire core (precision LFDM_PREC_MIXED_TIRE): the part of computeTireRHS, TMeasy, that dominates
// a step's FP64 instructions — load interpolation of the curve parameters, slips, combined-slip
// normalisation, the tmxy_combined curve, the relaxation rates and the structural/dynamic blend —
// in FP32, on FP32 copies of the derived constants (K.f). Kept in FP64: the slip velocity
// vsx - omega r_eff and the transport velocity r_eff |omega| + 0.01 (a cancellation of nearly equal
// terms at rolling without slip), rounded to FP32 before the slips are formed, and the rolling
// resistance; the wheel speed and the deflections stay FP64 states. The branch structure is that of
// tire_core_tm.

__device__ __forceinline__ float sine_stepf(float x, float x1, float y1, float x2, float y2) {
    if (x <= x1) return y1;
    if (x >= x2) return y2;
    const float dx = x2 - x1, dy = y2 - y1;
    const float u = (x - x1) / dx;
    return y1 + dy * u - (dy * (1.0f / 6.2831853071795865f)) * __sinf(6.2831853071795865f * u);
}

// tmxy_combined (dof18_gpu.cu:243-285) in FP32: the combined force f and f / s
__device__ __forceinline__ void tmxyf(float& f, float& fos, float s, float df0, float sm, float fm, float ss,
                                      float fs) {
    float df0loc = 0.0f;
    if (sm > 0.0f) df0loc = fmaxf(2.0f * fm / sm, df0);
    if (s > 0.0f && df0loc > 0.0f) {
        if (s > ss) {
            f = fs;
            fos = fs / s;
        } else if (s < sm) {
            const float p = df0loc * sm / fm - 2.0f;
            const float sn = s / sm;
            const float dn = fmaf(sn + p, sn, 1.0f);
            const float idn = 1.0f / dn;
            f = df0loc * sm * sn * idn;
            fos = df0loc * idn;
        } else {
            const float q = fm / sm;
            const float a = q * q / (df0loc * sm);
            const float sstar = sm + (fm - fs) / (a * (ss - sm));
            if (sstar <= ss) {
                if (s <= sstar) {
                    f = fm - a * (s - sm) * (s - sm);
                } else {
                    const float b = a * (sstar - sm) / (ss - sstar);
                    f = fs + b * (ss - s) * (ss - s);
                }
            } else {
                const float sn = (s - sm) / (ss - sm);
                f = fm - (fm - fs) * sn * sn * (3.0f - 2.0f * sn);
            }
            fos = f / s;
        }
    } else {
        f = 0.0f;
        fos = 0.0f;
    }
}

template <bool kSteered>
__device__ __forceinline__ void tire_core_tm_f32(TireC& ts, TireAux& ta, const KView& K, double c_d, double s_d,
                                                 double fz_d, double r_eff_d) {
    const double omega = ts.omega;
    const double vsx_d = fma(-omega, r_eff_d, ta.vsx);
    const double rw_d = r_eff_d * fabs(omega);
    const float vsx = (float)vsx_d;
    const float vta = (float)(rw_d + 0.01);
    const float rw = (float)rw_d;
    const float vsy = (float)ta.vsy;
    const float sx = -vsx / vta;
    float sy;
    if (kSteered) {
        const float c = (float)c_d, s = (float)s_d;
        // -tan(atan2(vsy, vta) - delta) is infinite where the steered wheel's slip angle passes 90
        // degrees (vta c + vsy s = 0), a denominator FP32 can round to exactly 0: held to +-1e6,
        // where the force curve is saturated and the direction is the FP64 one to FP32 rounding
        sy = -(vsy * c - vta * s) / (vta * c + vsy * s);
        sy = fminf(fmaxf(sy, -1e6f), 1e6f);
    } else {
        sy = -vsy / vta;
    }
    const float fz = fminf((float)fz_d, K.f(K_PNMAX));
    const float fzn = fz * K.f(K_INVPN);
    const float dfx0 = fzn * fmaf(-K.f(K_Q2DFX0), fzn, K.f(K_Q1DFX0));
    const float dfy0 = fzn * fmaf(-K.f(K_Q2DFY0), fzn, K.f(K_Q1DFY0));
    const float fxm = fzn * fmaf(-K.f(K_Q2FXM), fzn, K.f(K_Q1FXM));
    const float fym = fzn * fmaf(-K.f(K_Q2FYM), fzn, K.f(K_Q1FYM));
    const float fxs = fzn * fmaf(-K.f(K_Q2FXS), fzn, K.f(K_Q1FXS));
    const float fys = fzn * fmaf(-K.f(K_Q2FYS), fzn, K.f(K_Q1FYS));
    const float fzn1 = fzn - 1.0f;
    const float sxm = fmaf(K.f(K_DSXM), fzn1, K.f(K_LSXM));
    const float sym = fmaf(K.f(K_DSYM), fzn1, K.f(K_LSYM));
    const float sxs = fmaf(K.f(K_DSXS), fzn1, K.f(K_LSXS));
    const float sys = fmaf(K.f(K_DSYS), fzn1, K.f(K_LSYS));
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
    ta.My = -K(K_RR) * min_nn(fz_d, K(K_PNMAX)) * ta.rStat * sgnd(omega);
    const float vtxs = fmaf(rw, hsxn, 0.01f);
    const float vtys = fmaf(rw, hsyn, 0.01f);
    const float cx = K.f(K_CX), cy = K.f(K_CY), dx = K.f(K_DX), dy = K.f(K_DY);
    const float xe = (float)ts.xe, ye = (float)ts.ye;
    const float numx = fmaf(-vtxs * cx, xe, -fos * vsx);
    const float numy = fmaf(-vtys * cy, ye, fos * (sy * vta));
    const float xedot = numx / fmaf(vtxs, dx, fos);
    const float yedot = numy / fmaf(vtys, dy, fos);
    ts.xedot = xedot;
    ts.yedot = yedot;
    const float fxdyn = fmaf(dx, xedot, cx * xe);
    const float fydyn = fmaf(dy, yedot, cy * ye);
    const float fxstr = fminf(fmaxf(fmaf(xe, cx, xedot * dx), -K.f(K_FXMP2N)), K.f(K_FXMP2N));
    const float fystr = fminf(fmaxf(fmaf(ye, cy, yedot * dy), -K.f(K_FYMP2N)), K.f(K_FYMP2N));
    const float wx = sine_stepf(fabsf(vsx), 1.f, 1.f, 1.5f, 0.f);
    const float wy = sine_stepf(fabsf(sy * vta), 1.f, 1.f, 1.5f, 0.f);
    ta.fx = (wx == 0.f) ? fxdyn : fmaf(wx, fxstr, (1.f - wx) * fxdyn);
    ta.fy = (wy == 0.f) ? fydyn : fmaf(wy, fystr, (1.f - wy) * fydyn);
}

// The TMeasy tire core in the arithmetic a kernel runs: FP64 (tire_core_tm) or FP32 (kF32).
template <bool kSteered, bool kF32>
__device__ __forceinline__ void tire_core_tm_p(TireC& ts, TireAux& ta, const KView& K, double c, double s, double fz,
                                               double r_eff) {
    if constexpr (kF32) tire_core_tm_f32<kSteered>(ts, ta, K, c, s, fz, r_eff);
    else tire_core_tm<kSteered>(ts, ta, K, c, s, fz, r_eff);
}

// computeTireRHS, TMeasy (dof18_gpu.cu:379-530). (c, s) = (cos, sin) of this tire's wheel angle;
// steered says whether the angle may be nonzero. Writes xedot/yedot (left stale when the wheel is
// off the ground, as in the reference) and the aux values.
template <bool kSteered, bool kF32 = false>
__device__ __forceinline__ void tire_rhs_tm(TireC& ts, TireAux& ta, const KView& K, double c, double s) {
    const double fz = ta.fz;
    if (!gt0(fz)) {
        ts.xe = 0;
        ts.ye = 0;
        ts.omega = 0;
        ta.xt = 0;
        ta.rStat = K(K_R0);
        ta.fx = 0;
        ta.fy = 0;
        ta.My = 0;
        return;
    }
    ta.xt = fz * K(K_INVKT);
    ta.rStat = K(K_R0) - ta.xt;
    double r_eff;
    if (!gt_nn(fz, K(K_FZRD))) {
        double rdynco = fma(K(K_DRD), fma(fz, K(K_INVPN), -1.0), K(K_RDPN));
        r_eff = fma(rdynco, ta.xt, ta.rStat);
    } else {
        r_eff = fma(K(K_RDCRIT), ta.xt, ta.rStat);
    }
    tire_core_tm_p<kSteered, kF32>(ts, ta, K, c, s, fz, r_eff);
}

// computeCombinedCoulombForce (dof18_gpu.cu:287-303)
__device__ __forceinline__ void coulomb(double& fx, double& fy, double mu, double vsx, double vsy, double fz,
                                        double vcoul) {
    fx = tanh(-2.0 * vsx / vcoul) * fz * mu;
    fy = tanh(-2.0 * vsy / vcoul) * fz * mu;
    const double h = sqrt(fma(fx, fx, fy * fy));
    if (h > fz * mu) {
        double f = fz * mu / h;
        fx *= f;
        fy *= f;
    }
}

// The part of computeTireRHS, TMeasyNr (dof18_gpu.cu:532-662; 24dof-gpu/dof24_gpu.cu:990-1119),
// that follows the loaded and effective radii: Coulomb force, slips, curve parameters, combined
// force, blend and rolling resistance. fz > 0 is the unclamped load, ta.rStat the loaded radius.
template <bool kSteered>
__device__ __forceinline__ void tire_core_nr(TireC& ts, TireAux& ta, const KView& K, double c, double s, double fz,
                                             double r_eff) {
    const double vsy = ta.vsy;
    const double omega = ts.omega;
    const double mu = K(K_MU);
    const double vsx = fma(-omega, r_eff, ta.vsx);
    const double vta = r_eff * fabs(omega) + 0.01;
    double Fx0, Fy0;
    coulomb(Fx0, Fy0, mu, vsx, vsy, fz, K(K_VCOUL));
    const double sx = -vsx / vta;
    double sy;
    if (kSteered) sy = -(vsy * c - vta * s) / (vta * c + vsy * s);
    else sy = -vsy / vta;
    fz = fmin(fz, K(K_PNMAX));
    const double fzn = fz * K(K_INVPN);
    const double dfx0 = fzn * fma(-K(K_Q2DFX0), fzn, K(K_Q1DFX0));
    const double dfy0 = fzn * fma(-K(K_Q2DFY0), fzn, K(K_Q1DFY0));
    const double fxm = fzn * fma(-K(K_Q2FXM), fzn, K(K_Q1FXM));
    const double fym = fzn * fma(-K(K_Q2FYM), fzn, K(K_Q1FYM));
    const double fxs = fzn * fma(-K(K_Q2FXS), fzn, K(K_Q1FXS));
    const double fys = fzn * fma(-K(K_Q2FYS), fzn, K(K_Q1FYS));
    const double fzn1 = fzn - 1.0;
    const double sxm = fma(K(K_DSXM), fzn1, K(K_LSXM));
    const double sym = fma(K(K_DSYM), fzn1, K(K_LSYM));
    const double sxs = fma(K(K_DSXS), fzn1, K(K_LSXS));
    const double sys = fma(K(K_DSYS), fzn1, K(K_LSYS));
    const double frblend = sine_step(fabs(ta.vsx), K(K_FRB0), 0., K(K_FRB1), 1.);
    const double q = fma(sx, sx, sy * sy);
    double sc, calpha, salpha, isc = 0;
    if (q > 0) {
        isc = rsqrt(q);
        sc = q * isc;
        calpha = sx * isc;
        salpha = sy * isc;
    } else {
        sc = 0;
        calpha = kSqrt2Over2;
        salpha = kSqrt2Over2;
    }
    auto hyp = [](double a, double b) { return sqrt(fma(a, a, b * b)); };
    const double df0 = hyp(dfx0 * calpha, dfy0 * salpha);
    const double fm = mu * hyp(fxm * calpha, fym * salpha);
    const double sm = mu * hyp(sxm * calpha, sym * salpha);
    const double fs = mu * hyp(fxs * calpha, fys * salpha);
    const double ss = mu * hyp(sxs * calpha, sys * salpha);
    double f, fos;
    tmxy(f, fos, sc, df0, sm, fm, ss, fs);
    double Fx = 0., Fy = 0.;
    if (sc > 0.) {
        Fx = f * sx * isc;
        Fy = f * sy * isc;
    }
    ta.fx = fma(1.0 - frblend, Fx0, frblend * Fx);
    ta.fy = fma(1.0 - frblend, Fy0, frblend * Fy);
    ta.My = -K(K_RR) * fz * ta.rStat * tanh(omega);
}

// tire_core_nr with its Coulomb force, slips, curve parameters, combined force and blend in FP32 (on
// the FP32 copies of the derived constants, precision LFDM_PREC_MIXED_TIRE). As in tire_core_tm_f32,
// the slip velocity vsx - omega r_eff and the transport velocity r_eff |omega| + 0.01 are formed in
// FP64 and rounded once, the steered lateral slip is held to +-1e6 and the rolling resistance stays
// FP64.
template <bool kSteered>
__device__ __forceinline__ void tire_core_nr_f32(TireC& ts, TireAux& ta, const KView& K, double c_d, double s_d,
                                                 double fz_d, double r_eff_d) {
    const double omega = ts.omega;
    const float vsx = (float)fma(-omega, r_eff_d, ta.vsx);
    const float vta = (float)(r_eff_d * fabs(omega) + 0.01);
    const float vsy = (float)ta.vsy;
    const float mu = K.f(K_MU);
    const float fzf = (float)fz_d;
    // computeCombinedCoulombForce
    float Fx0 = tanhf(-2.0f * vsx / K.f(K_VCOUL)) * fzf * mu;
    float Fy0 = tanhf(-2.0f * vsy / K.f(K_VCOUL)) * fzf * mu;
    {
        const float h = sqrtf(fmaf(Fx0, Fx0, Fy0 * Fy0));
        if (h > fzf * mu) {
            const float r = fzf * mu / h;
            Fx0 *= r;
            Fy0 *= r;
        }
    }
    const float sx = -vsx / vta;
    float sy;
    if (kSteered) {
        const float c = (float)c_d, s = (float)s_d;
        sy = -(vsy * c - vta * s) / (vta * c + vsy * s);
        sy = fminf(fmaxf(sy, -1e6f), 1e6f);
    } else {
        sy = -vsy / vta;
    }
    const float fz = fminf(fzf, K.f(K_PNMAX));
    const float fzn = fz * K.f(K_INVPN);
    const float dfx0 = fzn * fmaf(-K.f(K_Q2DFX0), fzn, K.f(K_Q1DFX0));
    const float dfy0 = fzn * fmaf(-K.f(K_Q2DFY0), fzn, K.f(K_Q1DFY0));
    const float fxm = fzn * fmaf(-K.f(K_Q2FXM), fzn, K.f(K_Q1FXM));
    const float fym = fzn * fmaf(-K.f(K_Q2FYM), fzn, K.f(K_Q1FYM));
    const float fxs = fzn * fmaf(-K.f(K_Q2FXS), fzn, K.f(K_Q1FXS));
    const float fys = fzn * fmaf(-K.f(K_Q2FYS), fzn, K.f(K_Q1FYS));
    const float fzn1 = fzn - 1.0f;
    const float sxm = fmaf(K.f(K_DSXM), fzn1, K.f(K_LSXM));
    const float sym = fmaf(K.f(K_DSYM), fzn1, K.f(K_LSYM));
    const float sxs = fmaf(K.f(K_DSXS), fzn1, K.f(K_LSXS));
    const float sys = fmaf(K.f(K_DSYS), fzn1, K.f(K_LSYS));
    const float frblend = sine_stepf(fabsf((float)ta.vsx), K.f(K_FRB0), 0.f, K.f(K_FRB1), 1.f);
    const float q = fmaf(sx, sx, sy * sy);
    float sc, calpha, salpha, isc = 0.f;
    if (q > 0.f) {
        isc = rsqrtf(q);
        sc = q * isc;
        calpha = sx * isc;
        salpha = sy * isc;
    } else {
        sc = 0.f;
        calpha = 0.70710678f;
        salpha = 0.70710678f;
    }
    auto hyp = [](float a, float b) { return sqrtf(fmaf(a, a, b * b)); };
    const float df0 = hyp(dfx0 * calpha, dfy0 * salpha);
    const float fm = mu * hyp(fxm * calpha, fym * salpha);
    const float sm = mu * hyp(sxm * calpha, sym * salpha);
    const float fs = mu * hyp(fxs * calpha, fys * salpha);
    const float ss = mu * hyp(sxs * calpha, sys * salpha);
    float f, fos;
    tmxyf(f, fos, sc, df0, sm, fm, ss, fs);
    float Fx = 0.f, Fy = 0.f;
    if (sc > 0.f) {
        Fx = f * sx * isc;
        Fy = f * sy * isc;
    }
    ta.fx = fmaf(1.0f - frblend, Fx0, frblend * Fx);
    ta.fy = fmaf(1.0f - frblend, Fy0, frblend * Fy);
    ta.My = -K(K_RR) * fmin(fz_d, K(K_PNMAX)) * ta.rStat * tanh(omega);
}

// The TMeasyNr tire core in the arithmetic a kernel runs: FP64 (tire_core_nr) or FP32 (kF32).
template <bool kSteered, bool kF32>
__device__ __forceinline__ void tire_core_nr_p(TireC& ts, TireAux& ta, const KView& K, double c, double s, double fz,
                                               double r_eff) {
    if constexpr (kF32) tire_core_nr_f32<kSteered>(ts, ta, K, c, s, fz, r_eff);
    else tire_core_nr<kSteered>(ts, ta, K, c, s, fz, r_eff);
}

// computeTireRHS, TMeasyNr (dof18_gpu.cu:532-662)
template <bool kSteered, bool kF32 = false>
__device__ __forceinline__ void tire_rhs_nr(TireC& ts, TireAux& ta, const KView& K, double c, double s) {
    const double fz = ta.fz;
    if (!gt0(fz)) {
        ts.omega = 0;
        ta.xt = 0;
        ta.rStat = K(K_R0);
        ta.fx = 0;
        ta.fy = 0;
        ta.My = 0;
        return;
    }
    ta.xt = fz * K(K_INVKT);
    ta.rStat = K(K_R0) - ta.xt;
    double r_eff;
    if (!gt_nn(fz, K(K_FZRD))) {
        double rdynco = fma(K(K_DRD), fma(fz, K(K_INVPN), -1.0), K(K_RDPN));
        r_eff = fma(rdynco, ta.xt, ta.rStat);
    } else {
        r_eff = fma(K(K_RDCRIT), ta.xt, ta.rStat);
    }
    tire_core_nr_p<kSteered, kF32>(ts, ta, K, c, s, fz, r_eff);
}

// differentialSplit (dof18_gpu.cu:42-69) with max_bias = 2.
__device__ __forceinline__ void diff_split(double torque, double wl, double wr, double& tl, double& tr) {
    double diff = fabs(wl - wr);
    double alpha;
    if (gt_nn(diff, 0.5)) alpha = 2.0 / 3.0;    // bias = max_bias = 2
    else if (gt_nn(diff, 0.25)) {
        double bias = 4 * (2.0 - 1) * diff + (2 - 2.0);
        alpha = bias / (1 + bias);
    } else alpha = 0.5;                          // bias = 1
    double slow = alpha * torque;
    double fast = torque - slow;
    if (gt_nn(fabs(wr), fabs(wl))) {
        tl = slow;
        tr = fast;
    } else {
        tl = fast;
        tr = slow;
    }
}

// driveTorque (dof18_gpu.cu:15-38)
__device__ __forceinline__ double drive_torque(const ClassDev18& C, double throttle, double w) {
    if (C.throttleMod) {
        double t = map_y_scaled(C.pt, w, throttle);
        return t + map_y(C.loss, w);
    }
    return fma(map_y(C.pt, w), throttle, map_y(C.loss, w));
}

// computePowertrainRHS (dof18_gpu.cu:664-839). Mutates crank (no converter) and gear.
template <bool kNr>
__device__ __forceinline__ void powertrain_rhs(VehC& v, VehAux& va, TireC* ts, TireAux* ta, const KView& K,
                                               const ClassDev18& C, double throttle, double braking) {
    double torque_t;
    const int g = v.gear;
    if (C.tcbool) {
        bool reverse = false;
        const double omega_t = 0.25 * (((ts[0].omega + ts[1].omega) + ts[2].omega) + ts[3].omega);
        // division as in the reference: a converter started locked (crank = wheel speed / ratio)
        // must see a speed ratio of exactly 1, not 1 + ulp (which would select reverse flow)
        const double omega_out = omega_t / C.gear[g];
        const double omega_in = v.crank;
        double sr, cf, tr;
        if (lt_(omega_out, 1e-9) || lt_(omega_in, 1e-9)) {
            sr = 0;
        } else {
            sr = omega_out / omega_in;
            if (gt_nn(sr, 1.)) {
                sr = 1. - (sr - 1.);
                reverse = true;
            }
            if (lt_(sr, 0.0)) sr = 0;
        }
        cf = map_y(C.cf, sr);
        tr = map_y(C.tr, sr);
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
        v.crank = 0.25 * (((ts[0].omega + ts[1].omega) + ts[2].omega) + ts[3].omega) / C.gear[g];
        torque_t = drive_torque(C, throttle, v.crank) * C.invgear[g];
        if (lt_(v.u, 1e-9) && lt_(torque_t, 0.0)) torque_t = 0;
        if (lt_(C.up[g], v.crank)) {
            if (g < C.noGears - 1) v.gear = g + 1;
        } else if (lt_(v.crank, C.down[g])) {
            if (g > 0) v.gear = g - 1;
        }
    }
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
    diff_split(tf, ts[0].omega, ts[1].omega, ta[0].engTor, ta[1].engTor);
    diff_split(trr, ts[2].omega, ts[3].omega, ta[2].engTor, ta[3].engTor);
    const double brake = K(K_MAXBRAKE) * braking;
    const double ijw = K(K_INVJW);
#pragma unroll
    for (int k = 0; k < 4; ++k)
        ta[k].dOmega = ijw * (fma(-sgnd(ts[k].omega), brake, ta[k].engTor + ta[k].My) - ta[k].fx * ta[k].rStat);
}

// One right-hand-side evaluation (rhsFun, dof18_halfImplicit_gpu.cu:685-729): tire loads, tire
// forces and deflection rates, powertrain (wheel and crank accelerations, gear), chassis
// accelerations. steering/throttle/braking are the driver inputs.
template <bool kNr, bool kF32 = false>
__device__ __forceinline__ void rhs18(VehC& v, VehAux& va, TireC* ts, TireAux* ta, const KView& K,
                                      const ClassDev18& C, double steering, double throttle, double braking) {
    // computeTireLoads (dof18_gpu.cu:305-340); udot/vdot are the previous step's accelerations.
    {
        const double lat = fma(v.wz, v.u, v.vdot);
        const double lon = fma(-v.wz, v.v, v.udot);
        const double Z4 = K(K_Z4) * lon;
        const double Z2f = K(K_Z2F) * lat;
        const double Z3f = fma(K(K_Z3FK), v.phi, K(K_Z3FB) * v.wx);
        const double Z2r = K(K_Z2R) * lat;
        const double Z3r = fma(K(K_Z3RK), v.phi, K(K_Z3RB) * v.wx);
        const double Af = K(K_Z1F) - Z4, Bf = Z2f + Z3f;
        const double Ar = K(K_Z1R) + Z4, Br = Z2r + Z3r;
        ta[0].fz = pos_part(Af - Bf);
        ta[1].fz = pos_part(Af + Bf);
        ta[2].fz = pos_part(Ar - Br);
        ta[3].fz = pos_part(Ar + Br);
    }
    // vehToTireTransform (dof18_gpu.cu:71-109)
    double delta;
    if (C.nonLinearSteer) delta = map_y(C.steer, steering);
    else delta = steering * K(K_MAXSTEER);
    double cd = 1.0, sd = 0.0;
    if (!is_zero(delta)) sincos(delta, &sd, &cd);
    {
        const double vsyf = fma(v.wz, K(K_A), v.v);
        const double vsyr = fma(-v.wz, K(K_B), v.v);
        const double wcf = v.wz * K(K_CF2), wcr = v.wz * K(K_CR2);
        ta[0].vsy = vsyf;
        ta[1].vsy = vsyf;
        ta[0].vsx = fma(v.u - wcf, cd, vsyf * sd);
        ta[1].vsx = fma(v.u + wcf, cd, vsyf * sd);
        ta[2].vsy = vsyr;
        ta[3].vsy = vsyr;
        ta[2].vsx = v.u - wcr;
        ta[3].vsx = v.u + wcr;
    }
    if (kNr) {
        tire_rhs_nr<true, kF32>(ts[0], ta[0], K, cd, sd);
        tire_rhs_nr<true, kF32>(ts[1], ta[1], K, cd, sd);
        tire_rhs_nr<false, kF32>(ts[2], ta[2], K, 1.0, 0.0);
        tire_rhs_nr<false, kF32>(ts[3], ta[3], K, 1.0, 0.0);
    } else {
        tire_rhs_tm<true, kF32>(ts[0], ta[0], K, cd, sd);
        tire_rhs_tm<true, kF32>(ts[1], ta[1], K, cd, sd);
        tire_rhs_tm<false, kF32>(ts[2], ta[2], K, 1.0, 0.0);
        tire_rhs_tm<false, kF32>(ts[3], ta[3], K, 1.0, 0.0);
    }
    powertrain_rhs<kNr>(v, va, ts, ta, K, C, throttle, braking);
    // tireToVehTransform (dof18_gpu.cu:152-185): front forces into the vehicle frame
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const double fx = ta[k].fx, fy = ta[k].fy;
        ta[k].fx = fma(fx, cd, -fy * sd);
        ta[k].fy = fma(fx, sd, fy * cd);
    }
    // computeVehRHS (dof18_gpu.cu:1017-1068)
    {
        const double fx0 = ta[0].fx, fx1 = ta[1].fx, fx2 = ta[2].fx, fx3 = ta[3].fx;
        const double fy0 = ta[0].fy, fy1 = ta[1].fy, fy2 = ta[2].fy, fy3 = ta[3].fy;
        const double wu = v.wz * v.u;
        const double fyf = fy0 + fy1, fyr = fy2 + fy3;
        const double E1 = fma(-K(K_MT), wu, fyf + fyr);
        const double E2 = fma(K(K_E2WU), wu,
                              fma(fx3 - fx2, K(K_CR2), fma(fx1 - fx0, K(K_CF2), fma(fyf, K(K_A), -fyr * K(K_B)))));
        const double E3 = fma(K(K_E3WU), wu, fma(K(K_E3PHI), v.phi, K(K_E3WX) * v.wx));
        const double sfx = ((fx0 + fx1) + fx2) + fx3;
        v.udot = fma(K(K_INVMT), fma(K(K_UWZ2), v.wz * v.wz, fma(-K(K_UWZWX), v.wz * v.wx, sfx)), v.wz * v.v);
        v.vdot = fma(K(K_CV1), E1, fma(K(K_CV2), E2, K(K_CV3) * E3));
        va.wxdot = fma(K(K_CV3), E1, fma(K(K_CX2), E2, K(K_CX3) * E3));
        va.wzdot = fma(K(K_CV2), E1, fma(K(K_CZ2), E2, K(K_CX2) * E3));
    }
}

// The half-implicit update (dof18_halfImplicit_gpu.cu:913-946) with the rates of rhs18.
template <bool kNr>
__device__ __forceinline__ void update18(VehC& v, const VehAux& va, TireC* ts, const TireAux* ta, const ClassDev18& C,
                                         double dt) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (!kNr) {
            ts[k].xe = fma(ts[k].xedot, dt, ts[k].xe);
            ts[k].ye = fma(ts[k].yedot, dt, ts[k].ye);
        }
        ts[k].omega = fma(ta[k].dOmega, dt, ts[k].omega);
    }
    if (C.tcbool) v.crank = fma(va.dOmega_crank, dt, v.crank);
    v.u = fma(v.udot, dt, v.u);
    v.v = fma(v.vdot, dt, v.v);
    v.wx = fma(va.wxdot, dt, v.wx);
    v.wz = fma(va.wzdot, dt, v.wz);
    double sp, cp;
    sincos(v.psi, &sp, &cp);
    v.x = fma(fma(v.u, cp, -v.v * sp), dt, v.x);
    v.y = fma(fma(v.u, sp, v.v * cp), dt, v.y);
    v.psi = fma(v.wz, dt, v.psi);
    v.phi = fma(v.wx, dt, v.phi);
}

// One step: rhs18 followed by update18 (kF32: the FP32 tire core).
template <bool kNr, bool kF32 = false>
__device__ __forceinline__ void step18(VehC& v, VehAux& va, TireC* ts, TireAux* ta, const KView& K,
                                       const ClassDev18& C, double steering, double throttle, double braking,
                                       double dt) {
    rhs18<kNr, kF32>(v, va, ts, ta, K, C, steering, throttle, braking);
    update18<kNr>(v, va, ts, ta, C, dt);
}

}  // namespace lfdm
