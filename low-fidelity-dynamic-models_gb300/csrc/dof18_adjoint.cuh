// Hand-written adjoint (reverse mode) of one 18-DOF TMeasy half-implicit step.
//
// fwd18_tape() runs the same arithmetic as step18<false> (dof18_device.cuh; reference rhsFun
// 18dof-gpu/dof18_halfImplicit_gpu.cu:685-729 and the update :913-946) and records on a tape
// the intermediates the reverse sweep needs; rev18() propagates the adjoint of the state after the
// step back to the state before it, to the step's controls and to the derived constants that
// depend on the differentiable parameters (mass, Jz, CG-to-front distance a, tire peak/sliding
// friction scale, tire vertical stiffness). The tape is written to HBM by a segment's forward
// recomputation and read back by its reverse sweep, so each step's forward arithmetic runs twice
// in total (rollout and recomputation) and the reverse sweep does not recompute it.
//
// Branches (wheel lift-off, tmxy_combined regimes, clamps, sineStep bands, converter flow
// direction, differential bias band, gear shifts, map segments) are differentiated on the branch
// the forward step took; the gear is piecewise constant and carries no adjoint.
//
// The library is compiled without implicit multiply-add contraction (so that every kernel that runs
// a forward step rounds it alike); the reverse sweep, which no other kernel has to match, writes
// its sums of products as explicit fma() instead, halving the FP64 instructions of those updates. Supported: TMeasy
// tires (and, for the right-hand-side Jacobian, TMeasyNr tires: tire_fwd_tape_nr / tire_rev_nr),
// linear or mapped steering, with or without torque converter, throttleMod off.
#pragma once

#include <cstddef>

#include "../../include/lfdm/device/dof18_device.cuh"

namespace lfdm {

// Derived constants that depend on the differentiable parameters; their adjoints are accumulated
// per vehicle and contracted with dK/dp at the end of the backward pass.
enum KB : int {
    KB_Z1F = 0, KB_Z2F, KB_Z4, KB_Z1R, KB_Z2R, KB_MT, KB_INVMT, KB_E2WU, KB_E3PHI, KB_E3WU, KB_UWZ2, KB_UWZWX,
    KB_CV1, KB_CV2, KB_CV3, KB_CX2, KB_CX3, KB_CZ2, KB_A,
    KB_Q1FXM, KB_Q2FXM, KB_Q1FYM, KB_Q2FYM, KB_Q1FXS, KB_Q2FXS, KB_Q1FYS, KB_Q2FYS, KB_FXMP2N, KB_FYMP2N,
    KB_INVKT,
    KB_COUNT
};
// The K18 index of each KB entry.
__device__ __forceinline__ int kb_to_k(int i) {
    switch (i) {
        case KB_Z1F: return K_Z1F;
        case KB_Z2F: return K_Z2F;
        case KB_Z4: return K_Z4;
        case KB_Z1R: return K_Z1R;
        case KB_Z2R: return K_Z2R;
        case KB_MT: return K_MT;
        case KB_INVMT: return K_INVMT;
        case KB_E2WU: return K_E2WU;
        case KB_E3PHI: return K_E3PHI;
        case KB_E3WU: return K_E3WU;
        case KB_UWZ2: return K_UWZ2;
        case KB_UWZWX: return K_UWZWX;
        case KB_CV1: return K_CV1;
        case KB_CV2: return K_CV2;
        case KB_CV3: return K_CV3;
        case KB_CX2: return K_CX2;
        case KB_CX3: return K_CX3;
        case KB_CZ2: return K_CZ2;
        case KB_A: return K_A;
        case KB_Q1FXM: return K_Q1FXM;
        case KB_Q2FXM: return K_Q2FXM;
        case KB_Q1FYM: return K_Q1FYM;
        case KB_Q2FYM: return K_Q2FYM;
        case KB_Q1FXS: return K_Q1FXS;
        case KB_Q2FXS: return K_Q2FXS;
        case KB_Q1FYS: return K_Q1FYS;
        case KB_Q2FYS: return K_Q2FYS;
        case KB_FXMP2N: return K_FXMP2N;
        case KB_FYMP2N: return K_FYMP2N;
        default: return K_INVKT;
    }
}

// Accumulator of the constant adjoints (strided per-vehicle column).
struct KBar {
    double* base;
    int stride;
    __device__ __forceinline__ void add(int i, double v) const { base[i * stride] += v; }
    __device__ __forceinline__ double& at(int i) const { return base[i * stride]; }
};

// The differentiable state of one vehicle (the carried state of step18 minus the gear).
struct Adj18 {
    double x, y, u, v, psi, wz, phi, wx, udot, vdot, crank;
    double xe[4], ye[4], xedot[4], yedot[4], om[4];
};
constexpr int kAdj18Count = 31;

// Per-tire tape of one step.
struct TireTape {
    double on;                       // 1: wheel on the ground (fz > 0)
    double fz, xt, rStat, r_eff, rdynco, fzrd;  // fzrd: 1 when fz <= fzRdynco (rdynco interpolated)
    double om, xe, ye, vsx, vsy, rw, vta, sx, sy, N, D;  // N, D: the steered sy = -N / D
    double fzc, fzcl, fzn;           // fzcl: 1 when fz was limited to pnmax
    double dfx0, dfy0, fxm, fym, fxs, fys, sxm, sym, sxs, sys;
    double ssum, fsum, fxd, fyd, hsxn, hsyn, ihx, ihy, sxn, syn, sc, isc, calpha, salpha, qpos;
    double df0, fm, sm, fs, ss, fos;
    double vtxs, vtys, numx, numy, denx, deny, xedot, yedot, idenx, ideny, issum, ifsum, ivta;
    double Fx, Fy, fxstr, fystr, clx, cly, wxw, wyw, dwx, dwy;  // clx/cly: -1/0/+1 clamp side
    double fx, fy, My, sgn;
    double reg;  // tmxy_combined regime (0 no force, 1 sliding, 2 adhesion, 3/4 the two parabolas, 5 cubic)
};
// Per-tire tape of a TMeasyNr tire, in the slots of TireTape: the fields the vehicle-level sweep
// reads (on, om, rStat, fx, fy, My) sit at the same offsets as in TireTape, the rest of the head in
// slots the TMeasy tire uses for its own intermediates.
struct TireTapeNrHead {
    double on, fz, xt, rStat, r_eff, rdynco, fzrd, om;  // as TireTape
    double vsxin, vsx, vsy, vta, sx, sy, N, D;
    double tx, ty, a0, b0, h0, clamp, Fx0, Fy0;          // Coulomb force: tanh terms, before/after the clamp
    double fzc, fzcl, fzn, dfx0, dfy0, fxm, fym, fxs, fys, sxm, sym, sxs, sys;
    double w, dw;                                        // slip blend (frblend) and its slope in |vsx|
    double qpos, q, isc, sc, calpha, salpha;
    double df0, hfm, hsm, hfs, hss, fm, sm, fs, ss, f, fos, Fx, Fy, th;  // th = tanh(omega)
};
struct TireTapeNr {
    TireTapeNrHead h;
    double pad[(offsetof(TireTape, fx) - sizeof(TireTapeNrHead)) / sizeof(double)];
    double fx, fy, My;
};
static_assert(offsetof(TireTapeNr, h) == 0, "the head starts the tire tape");
static_assert(offsetof(TireTapeNrHead, on) == offsetof(TireTape, on) &&
                  offsetof(TireTapeNrHead, rStat) == offsetof(TireTape, rStat) &&
                  offsetof(TireTapeNrHead, om) == offsetof(TireTape, om),
              "shared tire tape fields");
static_assert(offsetof(TireTapeNr, fx) == offsetof(TireTape, fx) && offsetof(TireTapeNr, fy) == offsetof(TireTape, fy) &&
                  offsetof(TireTapeNr, My) == offsetof(TireTape, My) && sizeof(TireTapeNr) <= sizeof(TireTape),
              "the TMeasyNr tape fits the TMeasy slots");

// Step tape: inputs, tire tapes and the vehicle-level intermediates.
struct StepTape {
    double u, v, psi, wz, phi, wx, udot, vdot, crank, gear;
    double lat, lon, fzarg[4];
    double delta, cd, sd, dslope;   // dslope: d delta / d steering
    double vsyf, vsyr, wcf, wcr;
    // powertrain
    double omega_t, omega_out, omega_in, sr, srmode, cf, tr, cfs, trs, r, torque_in, torque_out, torque_t,
        tclip, rev, dt_map, dt_slope, tf, trr, alf, alr, dalf, dalr, slowf, slowr, dOc;
    double thr, brk, steer;
    double fxr[4], fyr[4];          // forces after the front rotation
    double wu, E1, E2, E3, inner;
    double u1, v1, wx1, wz1;        // updated speeds
    double sp, cp;
    double x1, y1, psi1;            // position and yaw after the step (the loss reads them)
    TireTape t[4];
};
constexpr int kStepTapeDoubles = (int)(sizeof(StepTape) / sizeof(double));
static_assert(sizeof(StepTape) % sizeof(double) == 0, "the step tape is a flat array of doubles");
constexpr int kTireTapeDoubles = (int)(sizeof(TireTape) / sizeof(double));

// A vehicle's column of the step tape in HBM ([tape doubles][npad]): field i lives at p[i * s]. The
// forward recomputation writes each field once, where it is computed, and the reverse sweep reads
// it where it is used, so no tape is held in registers or on the stack.
struct TapeRef {
    double* p;
    size_t s;
    __device__ __forceinline__ double& at(int i) const { return p[i * s]; }
};
#define TS_(f) ((int)(offsetof(StepTape, f) / sizeof(double)))
#define TT_(f) ((int)(offsetof(TireTape, f) / sizeof(double)))
#define TN_(f) ((int)(offsetof(TireTapeNrHead, f) / sizeof(double)))
__device__ __forceinline__ TapeRef tire_ref(const TapeRef& T, int k) {
    return {T.p + (size_t)(TS_(t) + k * kTireTapeDoubles) * T.s, T.s};
}

// map slope of the segment getMapY uses at x (0 where the map clamps)
__device__ __forceinline__ double map_slope(const MapDev& m, double x) {
    if (x <= m.x[0] || x >= m.x[m.n - 1]) return 0.0;
    const int r = lower_bound_x(m.x, m.n, x);
    return m.dy[r - 1] / m.dx[r - 1];
}
// sineStep(x, 1, 1, 1.5, 0) and its derivative
__device__ __forceinline__ void sine_step_w(double x, double& y, double& dy) {
    if (x <= 1.0) {
        y = 1.0;
        dy = 0.0;
        return;
    }
    if (x >= 1.5) {
        y = 0.0;
        dy = 0.0;
        return;
    }
    y = sine_step(x, 1., 1., 1.5, 0.);
    const double u = (x - 1.0) / 0.5;
    dy = -2.0 + 2.0 * cospi(2.0 * u);
}

// ---------------------------------------------------------------------------------------------
// forward with tape (the arithmetic of tire_rhs_tm / tire_core_tm / powertrain_rhs / step18)

// The regime tmxy_frac takes for these arguments, by its own comparisons (the quantities they
// compare are computed by the same expressions, so they round alike): 0 no force, 1 full sliding,
// 2 adhesion, 3 and 4 the two parabolas, 5 the cubic fallback; plus 8 where the initial slope is
// 2 fm / sm rather than df0 (the max of the two is a kink of the curve in every regime that reads it).
__device__ __forceinline__ double tmxy_regime(double s, double df0, double sm, double ism, double fm, double ss,
                                              double fs) {
    double df0loc = 0.0, side = 0.0;
    if (gt0(sm)) {
        const double c2 = 2.0 * fm * ism;
        df0loc = max_nn(c2, df0);
        side = gt_nn(c2, df0) ? 8.0 : 0.0;
    }
    if (!(gt0(s) && gt0(df0loc))) return 0.0;
    if (gt_nn(s, ss)) return 1.0;
    if (gt_nn(sm, s)) return 2.0 + side;
    double q2, D, E, H;
    return 3.0 + tmxy_joint(s, fm, ism, df0loc, sm, ss, fs, q2, D, E, H) + side;
}

template <bool kSteered>
__device__ __forceinline__ void tire_fwd_tape_core(TireC& ts, TireAux& ta, const TapeRef& T, const KView& K, double c,
                                                   double s, double fz, double r_eff);

template <bool kSteered>
__device__ __forceinline__ void tire_fwd_tape(TireC& ts, TireAux& ta, const TapeRef& T, const KView& K, double c, double s) {
    const double fz = ta.fz;
    T.at(TT_(fz)) = fz;
    T.at(TT_(om)) = ts.omega;
    T.at(TT_(xe)) = ts.xe;
    T.at(TT_(ye)) = ts.ye;
    T.at(TT_(vsy)) = ta.vsy;
    T.at(TT_(on)) = fz > 0 ? 1.0 : 0.0;
    if (fz <= 0) {
        ts.xe = 0;
        ts.ye = 0;
        ts.omega = 0;
        ta.xt = 0;
        ta.rStat = K(K_R0);
        ta.fx = 0;
        ta.fy = 0;
        ta.My = 0;
        T.at(TT_(rStat)) = ta.rStat;
        T.at(TT_(fx)) = T.at(TT_(fy)) = T.at(TT_(My)) = 0;
        return;
    }
    ta.xt = fz * K(K_INVKT);
    ta.rStat = K(K_R0) - ta.xt;
    T.at(TT_(xt)) = ta.xt;
    T.at(TT_(rStat)) = ta.rStat;
    if (fz <= K(K_FZRD)) {
        T.at(TT_(fzrd)) = 1.0;
        T.at(TT_(rdynco)) = fma(K(K_DRD), fma(fz, K(K_INVPN), -1.0), K(K_RDPN));
    } else {
        T.at(TT_(fzrd)) = 0.0;
        T.at(TT_(rdynco)) = K(K_RDCRIT);
    }
    const double r_eff = fma(T.at(TT_(rdynco)), ta.xt, ta.rStat);
    tire_fwd_tape_core<kSteered>(ts, ta, T, K, c, s, fz, r_eff);
}

// The part of tire_fwd_tape that follows the load and the radii (tire_core_tm's arithmetic): the
// caller has set ta.vsx, ta.vsy, ta.rStat, the tape's fz, om, xe, ye, vsy and on fields, and
// passes the load fz > 0 and the effective radius r_eff.
template <bool kSteered>
__device__ __forceinline__ void tire_fwd_tape_core(TireC& ts, TireAux& ta, const TapeRef& T, const KView& K, double c,
                                                   double s, double fz, double r_eff) {
    T.at(TT_(r_eff)) = r_eff;
    const double omega = ts.omega;
    const double vsy = ta.vsy;
    const double vsx = fma(-omega, r_eff, ta.vsx);
    T.at(TT_(vsx)) = vsx;
    const double rw = r_eff * fabs(omega);
    const double vta = rw + 0.01;
    T.at(TT_(rw)) = rw;
    T.at(TT_(vta)) = vta;
    const double fzc = fmin(fz, K(K_PNMAX));
    T.at(TT_(fzc)) = fzc;
    T.at(TT_(fzcl)) = fz > K(K_PNMAX) ? 1.0 : 0.0;
    const double fzn = fzc * K(K_INVPN);
    T.at(TT_(fzn)) = fzn;
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
    T.at(TT_(dfx0)) = dfx0; T.at(TT_(dfy0)) = dfy0; T.at(TT_(fxm)) = fxm; T.at(TT_(fym)) = fym; T.at(TT_(fxs)) = fxs; T.at(TT_(fys)) = fys;
    T.at(TT_(sxm)) = sxm; T.at(TT_(sym)) = sym; T.at(TT_(sxs)) = sxs; T.at(TT_(sys)) = sys;
    const double ssum = sxm + sym;
    const double fxd = fxm * dfy0, fyd = fym * dfx0;
    const double fsum = fxd + fyd;
    // one division for 1/(ssum fsum), 1/vta and the steered wheel's 1/D, as in tire_core_tm
    const double p12 = ssum * fsum;
    double r12, ivta, sy;
    if (kSteered) {
        const double den = fma(vta, c, vsy * s);
        const double num = fma(vsy, c, -vta * s);
        T.at(TT_(N)) = num;
        T.at(TT_(D)) = den;
        const double pv = vta * den;
        const double r = 1.0 / (p12 * pv);
        r12 = pv * r;
        const double ipv = p12 * r;
        ivta = den * ipv;
        sy = -num * (vta * ipv);
    } else {
        const double r = 1.0 / (p12 * vta);
        r12 = vta * r;
        ivta = p12 * r;
        sy = -vsy * ivta;
    }
    const double sx = -vsx * ivta;
    T.at(TT_(ivta)) = ivta;
    T.at(TT_(sx)) = sx;
    T.at(TT_(sy)) = sy;
    const double issum = fsum * r12, ifsum = ssum * r12;
    const double hsxn = fma(sxm, issum, fxd * ifsum);
    const double hsyn = fma(sym, issum, fyd * ifsum);
    const double rh = 1.0 / (hsxn * hsyn);
    const double ihx = hsyn * rh, ihy = hsxn * rh;
    T.at(TT_(ssum)) = ssum; T.at(TT_(fsum)) = fsum; T.at(TT_(issum)) = issum; T.at(TT_(ifsum)) = ifsum; T.at(TT_(fxd)) = fxd; T.at(TT_(fyd)) = fyd; T.at(TT_(hsxn)) = hsxn; T.at(TT_(hsyn)) = hsyn; T.at(TT_(ihx)) = ihx; T.at(TT_(ihy)) = ihy;
    const double sxn = sx * ihx;
    const double syn = sy * ihy;
    const double q = fma(sxn, sxn, syn * syn);
    double sc, calpha, salpha, isc = 0;
    if (q > 0) {
        isc = rsqrt(q);
        sc = q * isc;
        calpha = sxn * isc;
        salpha = syn * isc;
    } else {
        sc = 0;
        calpha = kSqrt2Over2;
        salpha = kSqrt2Over2;
    }
    T.at(TT_(sxn)) = sxn; T.at(TT_(syn)) = syn; T.at(TT_(sc)) = sc; T.at(TT_(isc)) = isc; T.at(TT_(calpha)) = calpha; T.at(TT_(salpha)) = salpha;
    T.at(TT_(qpos)) = q > 0 ? 1.0 : 0.0;
    auto hyp = [](double a, double b) { return sqrt(fma(a, a, b * b)); };
    const double df0 = hyp(dfx0 * calpha * hsxn, dfy0 * salpha * hsyn);
    double fm, ifm, sm, ism;
    hyp_rcp(fxm * calpha, fym * salpha, fm, ifm);
    const double cax = calpha * ihx, say = salpha * ihy;
    hyp_rcp(sxm * cax, sym * say, sm, ism);
    const double fs = hyp(fxs * calpha, fys * salpha);
    const double ss = hyp(sxs * cax, sys * say);
    T.at(TT_(df0)) = df0; T.at(TT_(fm)) = fm; T.at(TT_(sm)) = sm; T.at(TT_(fs)) = fs; T.at(TT_(ss)) = ss;
    double fn, fd;
    tmxy_frac(fn, fd, sc, isc, df0, sm, ism, fm, ifm, ss, fs);
    T.at(TT_(fos)) = fn / fd;  // the ratio itself, for the reverse
    T.at(TT_(reg)) = tmxy_regime(sc, df0, sm, ism, fm, ss, fs);
    T.at(TT_(sgn)) = sgnd(omega);
    ta.My = -K(K_RR) * fzc * ta.rStat * T.at(TT_(sgn));
    const double vtxs = fma(rw, hsxn, 0.01);
    const double vtys = fma(rw, hsyn, 0.01);
    const double cx = K(K_CX), cy = K(K_CY), dx = K(K_DX), dy = K(K_DY);
    const double numx = fma(-vtxs * cx, ts.xe * fd, -fn * vsx);
    const double numy = fma(-vtys * cy, ts.ye * fd, fn * (sy * vta));
    const double denx = fma(vtxs * dx, fd, fn), deny = fma(vtys * dy, fd, fn);
    const double rd = 1.0 / (denx * deny);
    ts.xedot = numx * (deny * rd);
    ts.yedot = numy * (denx * rd);
    T.at(TT_(idenx)) = fd * (deny * rd);  // 1 / (vtxs dx + fos)
    T.at(TT_(ideny)) = fd * (denx * rd);
    T.at(TT_(vtxs)) = vtxs; T.at(TT_(vtys)) = vtys; T.at(TT_(numx)) = numx; T.at(TT_(numy)) = numy; T.at(TT_(denx)) = denx; T.at(TT_(deny)) = deny;
    T.at(TT_(xedot)) = ts.xedot; T.at(TT_(yedot)) = ts.yedot;
    const double fxdyn = fma(dx, ts.xedot, cx * ts.xe);
    const double fydyn = fma(dy, ts.yedot, cy * ts.ye);
    const double Gx = fma(ts.xe, cx, ts.xedot * dx);
    const double Gy = fma(ts.ye, cy, ts.yedot * dy);
    const double fxstr = fmin(fmax(Gx, -K(K_FXMP2N)), K(K_FXMP2N));
    const double fystr = fmin(fmax(Gy, -K(K_FYMP2N)), K(K_FYMP2N));
    T.at(TT_(Fx)) = fxdyn; T.at(TT_(Fy)) = fydyn; T.at(TT_(fxstr)) = fxstr; T.at(TT_(fystr)) = fystr;
    T.at(TT_(clx)) = Gx > K(K_FXMP2N) ? 1.0 : (Gx < -K(K_FXMP2N) ? -1.0 : 0.0);
    T.at(TT_(cly)) = Gy > K(K_FYMP2N) ? 1.0 : (Gy < -K(K_FYMP2N) ? -1.0 : 0.0);
    double wx, wy, dwx, dwy;
    sine_step_w(fabs(vsx), wx, dwx);
    sine_step_w(fabs(sy * vta), wy, dwy);
    T.at(TT_(wxw)) = wx; T.at(TT_(wyw)) = wy; T.at(TT_(dwx)) = dwx; T.at(TT_(dwy)) = dwy;
    ta.fx = (wx == 0.0) ? fxdyn : fma(wx, fxstr, (1. - wx) * fxdyn);
    ta.fy = (wy == 0.0) ? fydyn : fma(wy, fystr, (1. - wy) * fydyn);
    T.at(TT_(fx)) = ta.fx;
    T.at(TT_(fy)) = ta.fy;
    T.at(TT_(My)) = ta.My;
}

// sineStep(x, x1, 0, x2, 1) (the TMeasyNr slip blend) and its slope
__device__ __forceinline__ void sine_step01(double x, double x1, double x2, double& y, double& dy) {
    y = sine_step(x, x1, 0., x2, 1.);
    if (x <= x1 || x >= x2) {
        dy = 0.0;
        return;
    }
    const double u = (x - x1) / (x2 - x1);
    dy = (1.0 - cospi(2.0 * u)) / (x2 - x1);
}

// The arithmetic of tire_rhs_nr / tire_core_nr (dof18_device.cuh) with its tape.
template <bool kSteered>
__device__ __forceinline__ void tire_fwd_tape_nr(TireC& ts, TireAux& ta, const TapeRef& T, const KView& K, double c,
                                                 double s) {
    const double fz = ta.fz;
    T.at(TN_(fz)) = fz;
    T.at(TN_(om)) = ts.omega;
    T.at(TN_(vsy)) = ta.vsy;
    T.at(TN_(vsxin)) = ta.vsx;
    T.at(TN_(on)) = gt0(fz) ? 1.0 : 0.0;
    if (!gt0(fz)) {
        ts.omega = 0;
        ta.xt = 0;
        ta.rStat = K(K_R0);
        ta.fx = 0;
        ta.fy = 0;
        ta.My = 0;
        T.at(TN_(rStat)) = ta.rStat;
        T.at(TT_(fx)) = T.at(TT_(fy)) = T.at(TT_(My)) = 0;
        return;
    }
    ta.xt = fz * K(K_INVKT);
    ta.rStat = K(K_R0) - ta.xt;
    T.at(TN_(xt)) = ta.xt;
    T.at(TN_(rStat)) = ta.rStat;
    double rdynco;
    if (!gt_nn(fz, K(K_FZRD))) {
        T.at(TN_(fzrd)) = 1.0;
        rdynco = fma(K(K_DRD), fma(fz, K(K_INVPN), -1.0), K(K_RDPN));
    } else {
        T.at(TN_(fzrd)) = 0.0;
        rdynco = K(K_RDCRIT);
    }
    T.at(TN_(rdynco)) = rdynco;
    const double r_eff = fma(rdynco, ta.xt, ta.rStat);
    T.at(TN_(r_eff)) = r_eff;
    const double vsy = ta.vsy;
    const double omega = ts.omega;
    const double mu = K(K_MU);
    const double vsx = fma(-omega, r_eff, ta.vsx);
    const double vta = r_eff * fabs(omega) + 0.01;
    T.at(TN_(vsx)) = vsx;
    T.at(TN_(vta)) = vta;
    // computeCombinedCoulombForce
    const double vcoul = K(K_VCOUL);
    const double tx = tanh(-2.0 * vsx / vcoul), ty = tanh(-2.0 * vsy / vcoul);
    double Fx0 = tx * fz * mu, Fy0 = ty * fz * mu;
    T.at(TN_(tx)) = tx; T.at(TN_(ty)) = ty; T.at(TN_(a0)) = Fx0; T.at(TN_(b0)) = Fy0;
    const double h0 = sqrt(fma(Fx0, Fx0, Fy0 * Fy0));
    T.at(TN_(h0)) = h0;
    T.at(TN_(clamp)) = 0.0;
    if (h0 > fz * mu) {
        const double g = fz * mu / h0;
        Fx0 *= g;
        Fy0 *= g;
        T.at(TN_(clamp)) = 1.0;
    }
    T.at(TN_(Fx0)) = Fx0; T.at(TN_(Fy0)) = Fy0;
    const double sx = -vsx / vta;
    double sy;
    if (kSteered) {
        const double N = vsy * c - vta * s, D = vta * c + vsy * s;
        T.at(TN_(N)) = N;
        T.at(TN_(D)) = D;
        sy = -N / D;
    } else {
        sy = -vsy / vta;
    }
    T.at(TN_(sx)) = sx; T.at(TN_(sy)) = sy;
    const double fzc = fmin(fz, K(K_PNMAX));
    T.at(TN_(fzc)) = fzc;
    T.at(TN_(fzcl)) = fz > K(K_PNMAX) ? 1.0 : 0.0;
    const double fzn = fzc * K(K_INVPN);
    T.at(TN_(fzn)) = fzn;
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
    T.at(TN_(dfx0)) = dfx0; T.at(TN_(dfy0)) = dfy0; T.at(TN_(fxm)) = fxm; T.at(TN_(fym)) = fym; T.at(TN_(fxs)) = fxs; T.at(TN_(fys)) = fys;
    T.at(TN_(sxm)) = sxm; T.at(TN_(sym)) = sym; T.at(TN_(sxs)) = sxs; T.at(TN_(sys)) = sys;
    double w, dw;
    sine_step01(fabs(ta.vsx), K(K_FRB0), K(K_FRB1), w, dw);
    T.at(TN_(w)) = w; T.at(TN_(dw)) = dw;
    const double q = fma(sx, sx, sy * sy);
    double sc, calpha, salpha, isc = 0;
    if (q > 0) {
        isc = rsqrt(q);
        sc = q * isc;
        calpha = sx * isc;
        salpha = sy * isc;
        T.at(TN_(qpos)) = 1.0;
    } else {
        sc = 0;
        calpha = kSqrt2Over2;
        salpha = kSqrt2Over2;
        T.at(TN_(qpos)) = 0.0;
    }
    T.at(TN_(q)) = q; T.at(TN_(isc)) = isc; T.at(TN_(sc)) = sc; T.at(TN_(calpha)) = calpha; T.at(TN_(salpha)) = salpha;
    auto hyp = [](double a, double b) { return sqrt(fma(a, a, b * b)); };
    const double df0 = hyp(dfx0 * calpha, dfy0 * salpha);
    const double hfm = hyp(fxm * calpha, fym * salpha), hsm = hyp(sxm * calpha, sym * salpha);
    const double hfs = hyp(fxs * calpha, fys * salpha), hss = hyp(sxs * calpha, sys * salpha);
    const double fm = mu * hfm, sm = mu * hsm, fs = mu * hfs, ss = mu * hss;
    T.at(TN_(df0)) = df0; T.at(TN_(hfm)) = hfm; T.at(TN_(hsm)) = hsm; T.at(TN_(hfs)) = hfs; T.at(TN_(hss)) = hss;
    T.at(TN_(fm)) = fm; T.at(TN_(sm)) = sm; T.at(TN_(fs)) = fs; T.at(TN_(ss)) = ss;
    double f, fos;
    tmxy(f, fos, sc, df0, sm, fm, ss, fs);
    T.at(TN_(f)) = f; T.at(TN_(fos)) = fos;
    double Fx = 0., Fy = 0.;
    if (sc > 0.) {
        Fx = f * sx * isc;
        Fy = f * sy * isc;
    }
    T.at(TN_(Fx)) = Fx; T.at(TN_(Fy)) = Fy;
    ta.fx = fma(1.0 - w, Fx0, w * Fx);
    ta.fy = fma(1.0 - w, Fy0, w * Fy);
    const double th = tanh(omega);
    T.at(TN_(th)) = th;
    ta.My = -K(K_RR) * fzc * ta.rStat * th;
    T.at(TT_(fx)) = ta.fx;
    T.at(TT_(fy)) = ta.fy;
    T.at(TT_(My)) = ta.My;
}

// One step18<kNr> with its tape; v/va/ts/ta as in step18.
template <bool kNr = false>
__device__ __forceinline__ void fwd18_tape(VehC& v, VehAux& va, TireC* ts, TireAux* ta, const TapeRef& T, const KView& K,
                                           const ClassDev18& C, double steering, double throttle, double braking,
                                           double dt) {
    T.at(TS_(u)) = v.u; T.at(TS_(v)) = v.v; T.at(TS_(psi)) = v.psi; T.at(TS_(wz)) = v.wz; T.at(TS_(phi)) = v.phi; T.at(TS_(wx)) = v.wx;
    T.at(TS_(udot)) = v.udot; T.at(TS_(vdot)) = v.vdot; T.at(TS_(crank)) = v.crank; T.at(TS_(gear)) = (double)v.gear;
    T.at(TS_(steer)) = steering; T.at(TS_(thr)) = throttle; T.at(TS_(brk)) = braking;
    {
        const double lat = fma(v.wz, v.u, v.vdot);
        const double lon = fma(-v.wz, v.v, v.udot);
        T.at(TS_(lat)) = lat;
        T.at(TS_(lon)) = lon;
        const double Z4 = K(K_Z4) * lon;
        const double Z2f = K(K_Z2F) * lat;
        const double Z3f = fma(K(K_Z3FK), v.phi, K(K_Z3FB) * v.wx);
        const double Z2r = K(K_Z2R) * lat;
        const double Z3r = fma(K(K_Z3RK), v.phi, K(K_Z3RB) * v.wx);
        const double Af = K(K_Z1F) - Z4, Bf = Z2f + Z3f;
        const double Ar = K(K_Z1R) + Z4, Br = Z2r + Z3r;
        T.at(TS_(fzarg) + 0) = Af - Bf;
        T.at(TS_(fzarg) + 1) = Af + Bf;
        T.at(TS_(fzarg) + 2) = Ar - Br;
        T.at(TS_(fzarg) + 3) = Ar + Br;
        ta[0].fz = fmax(Af - Bf, 0.0);
        ta[1].fz = fmax(Af + Bf, 0.0);
        ta[2].fz = fmax(Ar - Br, 0.0);
        ta[3].fz = fmax(Ar + Br, 0.0);
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
    if (delta != 0.0) sincos(delta, &sd, &cd);
    T.at(TS_(delta)) = delta;
    T.at(TS_(cd)) = cd;
    T.at(TS_(sd)) = sd;
    {
        const double vsyf = fma(v.wz, K(K_A), v.v);
        const double vsyr = fma(-v.wz, K(K_B), v.v);
        const double wcf = v.wz * K(K_CF2), wcr = v.wz * K(K_CR2);
        T.at(TS_(vsyf)) = vsyf; T.at(TS_(vsyr)) = vsyr; T.at(TS_(wcf)) = wcf; T.at(TS_(wcr)) = wcr;
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
        tire_fwd_tape_nr<true>(ts[0], ta[0], tire_ref(T, 0), K, cd, sd);
        tire_fwd_tape_nr<true>(ts[1], ta[1], tire_ref(T, 1), K, cd, sd);
        tire_fwd_tape_nr<false>(ts[2], ta[2], tire_ref(T, 2), K, 1.0, 0.0);
        tire_fwd_tape_nr<false>(ts[3], ta[3], tire_ref(T, 3), K, 1.0, 0.0);
    } else {
        tire_fwd_tape<true>(ts[0], ta[0], tire_ref(T, 0), K, cd, sd);
        tire_fwd_tape<true>(ts[1], ta[1], tire_ref(T, 1), K, cd, sd);
        tire_fwd_tape<false>(ts[2], ta[2], tire_ref(T, 2), K, 1.0, 0.0);
        tire_fwd_tape<false>(ts[3], ta[3], tire_ref(T, 3), K, 1.0, 0.0);
    }
    // powertrain (powertrain_rhs<false>) with its tape
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
                T.at(TS_(srmode)) = 0;  // constant
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
            T.at(TS_(torque_out)) = torque_out;
            torque_t = torque_out * C.invgear[g];
            if (v.u < 1e-9 && torque_t < 0) {
                torque_t = 0;
                T.at(TS_(tclip)) = 1;
            }
            const double dtq = drive_torque(C, throttle, v.crank);
            T.at(TS_(dt_map)) = map_y(C.pt, v.crank);
            T.at(TS_(dt_slope)) = fma(map_slope(C.pt, v.crank), throttle, map_slope(C.loss, v.crank));
            va.dOmega_crank = K(K_INVCI) * (dtq + torque_in);
            if (omega_out > C.up[g]) {
                if (g < C.noGears - 1) v.gear = g + 1;
            } else if (omega_out < C.down[g]) {
                if (g > 0) v.gear = g - 1;
            }
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
            if (v.crank > C.up[g]) {
                if (g < C.noGears - 1) v.gear = g + 1;
            } else if (v.crank < C.down[g]) {
                if (g > 0) v.gear = g - 1;
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
        // differential split with the bias and its slope recorded
        auto split = [&](double torque, double wl, double wr, double& tl, double& tR, double& alpha, double& dal,
                         double& slowleft) {
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
            const double slow = alpha * torque;
            const double fast = torque - slow;
            if (fabs(wl) < fabs(wr)) {
                tl = slow;
                tR = fast;
                slowleft = 1;
            } else {
                tl = fast;
                tR = slow;
                slowleft = 0;
            }
        };
        split(tf, ts[0].omega, ts[1].omega, ta[0].engTor, ta[1].engTor, T.at(TS_(alf)), T.at(TS_(dalf)), T.at(TS_(slowf)));
        split(trr, ts[2].omega, ts[3].omega, ta[2].engTor, ta[3].engTor, T.at(TS_(alr)), T.at(TS_(dalr)), T.at(TS_(slowr)));
        const double brake = K(K_MAXBRAKE) * braking;
        const double ijw = K(K_INVJW);
#pragma unroll
        for (int k = 0; k < 4; ++k)
            ta[k].dOmega =
                ijw * (fma(-sgnd(ts[k].omega), brake, ta[k].engTor + ta[k].My) - ta[k].fx * ta[k].rStat);
        T.at(TS_(dOc)) = va.dOmega_crank;
    }
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const double fx = ta[k].fx, fy = ta[k].fy;
        ta[k].fx = fma(fx, cd, -fy * sd);
        ta[k].fy = fma(fx, sd, fy * cd);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        T.at(TS_(fxr) + k) = ta[k].fx;
        T.at(TS_(fyr) + k) = ta[k].fy;
    }
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
        const double inner = fma(K(K_UWZ2), v.wz * v.wz, fma(-K(K_UWZWX), v.wz * v.wx, sfx));
        T.at(TS_(wu)) = wu; T.at(TS_(E1)) = E1; T.at(TS_(E2)) = E2; T.at(TS_(E3)) = E3; T.at(TS_(inner)) = inner;
        v.udot = fma(K(K_INVMT), inner, v.wz * v.v);
        v.vdot = fma(K(K_CV1), E1, fma(K(K_CV2), E2, K(K_CV3) * E3));
        va.wxdot = fma(K(K_CV3), E1, fma(K(K_CX2), E2, K(K_CX3) * E3));
        va.wzdot = fma(K(K_CV2), E1, fma(K(K_CZ2), E2, K(K_CX2) * E3));
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (!kNr) {  // the TMeasyNr tire has no deflection states
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
    T.at(TS_(u1)) = v.u; T.at(TS_(v1)) = v.v; T.at(TS_(wx1)) = v.wx; T.at(TS_(wz1)) = v.wz;
    double sp, cp;
    sincos(v.psi, &sp, &cp);
    T.at(TS_(sp)) = sp;
    T.at(TS_(cp)) = cp;
    v.x = fma(fma(v.u, cp, -v.v * sp), dt, v.x);
    v.y = fma(fma(v.u, sp, v.v * cp), dt, v.y);
    v.psi = fma(v.wz, dt, v.psi);
    v.phi = fma(v.wx, dt, v.phi);
    T.at(TS_(x1)) = v.x;
    T.at(TS_(y1)) = v.y;
    T.at(TS_(psi1)) = v.psi;
}

// ---------------------------------------------------------------------------------------------
// reverse sweep

// tmxy_combined (dof18_gpu.cu:243-285): adjoints of (s, df0, sm, fm, ss, fs) from that of fos, on
// the regime the forward took (the intermediates are recomputed; they are cheap).
__device__ __forceinline__ void tmxy_rev(double s, double df0, double sm, double fm, double ss, double fs, double fosb,
                                         double& sb, double& df0b, double& smb, double& fmb, double& ssb,
                                         double& fsb) {
    double df0loc = 0.0, ism = 0.0;
    bool dsel = false;
    if (sm > 0.0) {
        ism = 1.0 / sm;
        const double c2 = 2.0 * fm * ism;
        df0loc = fmax(c2, df0);
        dsel = c2 >= df0;
    }
    if (!(s > 0.0 && df0loc > 0.0) || fosb == 0.0) return;
    double df0locb = 0.0;
    const double is = 1.0 / s;
    if (s > ss) {  // full sliding: fos = fs / s
        fsb = fma(fosb, is, fsb);
        sb = fma(-fs * is * is, fosb, sb);
        return;
    }
    if (s < sm) {  // adhesion: fos = df0loc / dn
        const double ifm = 1.0 / fm;
        const double p = fma(df0loc * sm, ifm, -2.0);
        const double sn = s * ism;
        const double dn = fma(sn + p, sn, 1.0);
        const double idn = 1.0 / dn;
        const double dnb = -df0loc * idn * idn * fosb;
        df0locb = fma(fosb, idn, df0locb);
        const double snb = (fma(2.0, sn, p)) * dnb;
        const double pb = sn * dnb;
        df0locb = fma(sm * ifm, pb, df0locb);
        smb = fma(df0loc * ifm, pb, smb);
        fmb = fma(-df0loc * sm * ifm * ifm, pb, fmb);
        sb = fma(snb, ism, sb);
        smb = fma(-s * ism * ism, snb, smb);
    } else {
        double q2, D, E, H;  // the piece the forward step took, by its comparisons
        const int piece = tmxy_joint(s, fm, ism, df0loc, sm, ss, fs, q2, D, E, H);
        const double q = fm * ism;
        const double idsm = 1.0 / (df0loc * sm);
        const double a = q * q * idsm;
        const double ida = 1.0 / (a * (ss - sm));
        const double sstar = fma((fm - fs), ida, sm);
        double f, ab = 0.0, sstarb = 0.0;
        double b = 0.0, sn3 = 0.0;
        if (piece != 2) {
            if (piece == 0) {
                f = fm - a * (s - sm) * (s - sm);
            } else {
                b = a * (sstar - sm) / (ss - sstar);
                f = fs + b * (ss - s) * (ss - s);
            }
        } else {
            sn3 = (s - sm) / (ss - sm);
            f = fm - (fm - fs) * sn3 * sn3 * (3.0 - 2.0 * sn3);
        }
        const double fb = fosb * is;  // fos = f / s
        sb = fma(-f * is * is, fosb, sb);
        if (piece != 2) {
            if (piece == 0) {
                fmb += fb;
                ab = fma(-(s - sm) * (s - sm), fb, ab);
                sb = fma(-2.0 * a * (s - sm), fb, sb);
                smb = fma(2.0 * a * (s - sm), fb, smb);
            } else {
                fsb += fb;
                const double bb = (ss - s) * (ss - s) * fb;
                ssb = fma(2.0 * b * (ss - s), fb, ssb);
                sb = fma(-2.0 * b * (ss - s), fb, sb);
                const double id = 1.0 / (ss - sstar);
                ab = fma((sstar - sm) * id, bb, ab);
                sstarb = fma((fma(a, id, a * (sstar - sm) * id * id)), bb, sstarb);
                smb = fma(-a * id, bb, smb);
                ssb = fma(-a * (sstar - sm) * id * id, bb, ssb);
            }
        } else {
            const double g = sn3 * sn3 * (fma(-2.0, sn3, 3.0));
            fmb = fma(fb, (1.0 - g), fmb);
            fsb = fma(fb, g, fsb);
            const double snb = -(fm - fs) * (fma(6.0, sn3, -(6.0 * sn3) * sn3)) * fb;
            const double id = 1.0 / (ss - sm);
            sb = fma(snb, id, sb);
            smb = fma(snb, (fma((s - sm) * id, id, -id)), smb);
            ssb = fma(-snb * (s - sm) * id, id, ssb);
        }
        if (sstarb != 0.0) {  // sstar = sm + (fm - fs) / (a (ss - sm))
            smb += sstarb;
            fmb = fma(sstarb, ida, fmb);
            fsb = fma(-sstarb, ida, fsb);
            const double denb = -(fm - fs) * ida * ida * sstarb;
            ab = fma((ss - sm), denb, ab);
            ssb = fma(a, denb, ssb);
            smb = fma(-a, denb, smb);
        }
        if (ab != 0.0) {  // a = q^2 / (df0loc sm), q = fm / sm
            const double qb = 2.0 * q * idsm * ab;
            df0locb += -a / df0loc * ab;
            smb = fma(-a * ism, ab, smb);
            fmb = fma(qb, ism, fmb);
            smb = fma(-fm * ism * ism, qb, smb);
        }
    }
    if (dsel) {  // df0loc = max(2 fm / sm, df0)
        fmb = fma(2.0 * ism, df0locb, fmb);
        smb = fma(-2.0 * fm * ism * ism, df0locb, smb);
    } else {
        df0b += df0locb;
    }
}

// Tire adjoint (on-ground tire): from the adjoints of the core outputs (xedot, yedot, fx, fy, My as
// the tire model returns them, before any frame rotation) and of rStat, to those of the inputs
// (xe, ye, omega, vsx before the slip correction, vsy, fz, cos/sin of the wheel angle).
// tire_rev_core is the part that ends at the effective radius: its adjoint is returned in reffb,
// the load's (through the curve parameters) is added to fzb and rStatb is taken as it comes (the
// rolling resistance adds to it inside); the caller maps r_eff and rStat to its own states.
template <bool kSteered>
__device__ __forceinline__ void tire_rev_core(const TapeRef& T, const KView& K, const KBar& kb, double xedotb,
                                              double yedotb, double fxb, double fyb, double Myb, double& rStatb,
                                              double& xeb, double& yeb, double& omb, double& vsxinb, double& vsyb,
                                              double& fzb, double& reffb, double& cb, double& sb_, double c, double s) {
    const double cx = K(K_CX), cy = K(K_CY), dx = K(K_DX), dy = K(K_DY);
    double vsxb = 0, syb = 0, vtab = 0, fosb = 0, rwb = 0, hsxnb = 0, hsynb = 0, fzcb = 0, sxb = 0;
    // blend of structural and dynamic forces
    const double wxb = (T.at(TT_(fxstr)) - T.at(TT_(Fx))) * fxb, wyb = (T.at(TT_(fystr)) - T.at(TT_(Fy))) * fyb;
    const double fxstrb = T.at(TT_(wxw)) * fxb, fystrb = T.at(TT_(wyw)) * fyb;
    const double Fxb = (1.0 - T.at(TT_(wxw))) * fxb, Fyb = (1.0 - T.at(TT_(wyw))) * fyb;
    vsxb = fma(T.at(TT_(dwx)) * (T.at(TT_(vsx)) >= 0 ? 1.0 : -1.0), wxb, vsxb);
    {
        const double arg = T.at(TT_(sy)) * T.at(TT_(vta));
        const double argb = T.at(TT_(dwy)) * (arg >= 0 ? 1.0 : -1.0) * wyb;
        syb = fma(T.at(TT_(vta)), argb, syb);
        vtab = fma(T.at(TT_(sy)), argb, vtab);
    }
    double Gxb = 0, Gyb = 0;
    if (T.at(TT_(clx)) == 0.0) Gxb = fxstrb;
    else kb.at(KB_FXMP2N) = fma(T.at(TT_(clx)), fxstrb, kb.at(KB_FXMP2N));
    if (T.at(TT_(cly)) == 0.0) Gyb = fystrb;
    else kb.at(KB_FYMP2N) = fma(T.at(TT_(cly)), fystrb, kb.at(KB_FYMP2N));
    xeb = fma(cx, (Gxb + Fxb), xeb);
    xedotb = fma(dx, (Gxb + Fxb), xedotb);
    yeb = fma(cy, (Gyb + Fyb), yeb);
    yedotb = fma(dy, (Gyb + Fyb), yedotb);
    // relaxation rates
    const double idenx = T.at(TT_(idenx)), ideny = T.at(TT_(ideny));
    const double numxb = xedotb * idenx, denxb = -T.at(TT_(xedot)) * idenx * xedotb;
    const double numyb = yedotb * ideny, denyb = -T.at(TT_(yedot)) * ideny * yedotb;
    double vtxsb = fma(-cx * T.at(TT_(xe)), numxb, dx * denxb);
    xeb = fma(-T.at(TT_(vtxs)) * cx, numxb, xeb);
    fosb = fma(-T.at(TT_(vsx)), numxb, fosb + denxb);
    vsxb = fma(-T.at(TT_(fos)), numxb, vsxb);
    double vtysb = fma(-cy * T.at(TT_(ye)), numyb, dy * denyb);
    yeb = fma(-T.at(TT_(vtys)) * cy, numyb, yeb);
    fosb = fma(T.at(TT_(sy)) * T.at(TT_(vta)), numyb, fosb + denyb);
    syb = fma(T.at(TT_(fos)) * T.at(TT_(vta)), numyb, syb);
    vtab = fma(T.at(TT_(fos)) * T.at(TT_(sy)), numyb, vtab);
    rwb = fma(T.at(TT_(hsxn)), vtxsb, fma(T.at(TT_(hsyn)), vtysb, rwb));
    hsxnb = fma(T.at(TT_(rw)), vtxsb, hsxnb);
    hsynb = fma(T.at(TT_(rw)), vtysb, hsynb);
    // rolling resistance (no adjoint through sgn)
    fzcb = fma(-K(K_RR) * T.at(TT_(rStat)) * T.at(TT_(sgn)), Myb, fzcb);
    rStatb = fma(-K(K_RR) * T.at(TT_(fzc)) * T.at(TT_(sgn)), Myb, rStatb);
    // combined-slip force curve
    double scb = 0, df0b = 0, smb = 0, fmb = 0, ssb = 0, fsb = 0;
    tmxy_rev(T.at(TT_(sc)), T.at(TT_(df0)), T.at(TT_(sm)), T.at(TT_(fm)), T.at(TT_(ss)), T.at(TT_(fs)), fosb, scb, df0b, smb, fmb, ssb, fsb);
    double calphab = 0, salphab = 0, caxb = 0, sayb = 0, ihxb = 0, ihyb = 0;
    double dfx0b = 0, dfy0b = 0, fxmb = 0, fymb = 0, fxsb = 0, fysb = 0, sxmb = 0, symb = 0, sxsb = 0, sysb = 0;
    const double cax = T.at(TT_(calpha)) * T.at(TT_(ihx)), say = T.at(TT_(salpha)) * T.at(TT_(ihy));
    auto hyp_rev = [](double a, double b, double h, double hb, double& ab, double& bb) {
        if (h > 0 && hb != 0.0) {
            const double t = hb / h;
            ab = fma(a, t, ab);
            bb = fma(b, t, bb);
        }
    };
    {
        double Pb = 0, Qb = 0;
        hyp_rev(T.at(TT_(sxs)) * cax, T.at(TT_(sys)) * say, T.at(TT_(ss)), ssb, Pb, Qb);
        sxsb = fma(cax, Pb, sxsb);
        caxb = fma(T.at(TT_(sxs)), Pb, caxb);
        sysb = fma(say, Qb, sysb);
        sayb = fma(T.at(TT_(sys)), Qb, sayb);
    }
    {
        double Pb = 0, Qb = 0;
        hyp_rev(T.at(TT_(fxs)) * T.at(TT_(calpha)), T.at(TT_(fys)) * T.at(TT_(salpha)), T.at(TT_(fs)), fsb, Pb, Qb);
        fxsb = fma(T.at(TT_(calpha)), Pb, fxsb);
        calphab = fma(T.at(TT_(fxs)), Pb, calphab);
        fysb = fma(T.at(TT_(salpha)), Qb, fysb);
        salphab = fma(T.at(TT_(fys)), Qb, salphab);
    }
    {
        double Pb = 0, Qb = 0;
        hyp_rev(T.at(TT_(sxm)) * cax, T.at(TT_(sym)) * say, T.at(TT_(sm)), smb, Pb, Qb);
        sxmb = fma(cax, Pb, sxmb);
        caxb = fma(T.at(TT_(sxm)), Pb, caxb);
        symb = fma(say, Qb, symb);
        sayb = fma(T.at(TT_(sym)), Qb, sayb);
    }
    calphab = fma(T.at(TT_(ihx)), caxb, calphab);
    ihxb = fma(T.at(TT_(calpha)), caxb, ihxb);
    salphab = fma(T.at(TT_(ihy)), sayb, salphab);
    ihyb = fma(T.at(TT_(salpha)), sayb, ihyb);
    {
        double Pb = 0, Qb = 0;
        hyp_rev(T.at(TT_(fxm)) * T.at(TT_(calpha)), T.at(TT_(fym)) * T.at(TT_(salpha)), T.at(TT_(fm)), fmb, Pb, Qb);
        fxmb = fma(T.at(TT_(calpha)), Pb, fxmb);
        calphab = fma(T.at(TT_(fxm)), Pb, calphab);
        fymb = fma(T.at(TT_(salpha)), Qb, fymb);
        salphab = fma(T.at(TT_(fym)), Qb, salphab);
    }
    {
        double Pb = 0, Qb = 0;
        hyp_rev(T.at(TT_(dfx0)) * T.at(TT_(calpha)) * T.at(TT_(hsxn)), T.at(TT_(dfy0)) * T.at(TT_(salpha)) * T.at(TT_(hsyn)), T.at(TT_(df0)), df0b, Pb, Qb);
        dfx0b = fma(T.at(TT_(calpha)) * T.at(TT_(hsxn)), Pb, dfx0b);
        calphab = fma(T.at(TT_(dfx0)) * T.at(TT_(hsxn)), Pb, calphab);
        hsxnb = fma(T.at(TT_(dfx0)) * T.at(TT_(calpha)), Pb, hsxnb);
        dfy0b = fma(T.at(TT_(salpha)) * T.at(TT_(hsyn)), Qb, dfy0b);
        salphab = fma(T.at(TT_(dfy0)) * T.at(TT_(hsyn)), Qb, salphab);
        hsynb = fma(T.at(TT_(dfy0)) * T.at(TT_(salpha)), Qb, hsynb);
    }
    double sxnb = 0, synb = 0;
    if (T.at(TT_(qpos)) != 0.0) {
        const double iscb = fma(T.at(TT_(sxn)), calphab, T.at(TT_(syn)) * salphab);
        sxnb = fma(T.at(TT_(isc)), calphab, sxnb);
        synb = fma(T.at(TT_(isc)), salphab, synb);
        const double sct = fma(-(iscb * T.at(TT_(isc))), T.at(TT_(isc)), scb);
        sxnb = fma(T.at(TT_(sxn)) * T.at(TT_(isc)), sct, sxnb);
        synb = fma(T.at(TT_(syn)) * T.at(TT_(isc)), sct, synb);
    }
    sxb = fma(T.at(TT_(ihx)), sxnb, sxb);
    ihxb = fma(T.at(TT_(sx)), sxnb, ihxb);
    syb = fma(T.at(TT_(ihy)), synb, syb);
    ihyb = fma(T.at(TT_(sy)), synb, ihyb);
    hsxnb = fma(-T.at(TT_(ihx)) * T.at(TT_(ihx)), ihxb, hsxnb);
    hsynb = fma(-T.at(TT_(ihy)) * T.at(TT_(ihy)), ihyb, hsynb);
    {
        const double issum = T.at(TT_(issum)), ifsum = T.at(TT_(ifsum));
        const double ssumb = -(T.at(TT_(sxm)) * hsxnb + T.at(TT_(sym)) * hsynb) * (issum * issum);
        const double fsumb = -(T.at(TT_(fxd)) * hsxnb + T.at(TT_(fyd)) * hsynb) * (ifsum * ifsum);
        sxmb = fma(hsxnb, issum, sxmb + ssumb);
        symb = fma(hsynb, issum, symb + ssumb);
        const double fxdb = fma(hsxnb, ifsum, fsumb);
        const double fydb = fma(hsynb, ifsum, fsumb);
        fxmb = fma(T.at(TT_(dfy0)), fxdb, fxmb);
        dfy0b = fma(T.at(TT_(fxm)), fxdb, dfy0b);
        fymb = fma(T.at(TT_(dfx0)), fydb, fymb);
        dfx0b = fma(T.at(TT_(fym)), fydb, dfx0b);
    }
    // curve parameters from the normalised load
    const double fzn = T.at(TT_(fzn));
    double fznb = 0;
    fznb = fma(fma(-2.0 * K(K_Q2DFX0), fzn, K(K_Q1DFX0)), dfx0b, fznb);
    fznb = fma(fma(-2.0 * K(K_Q2DFY0), fzn, K(K_Q1DFY0)), dfy0b, fznb);
    fznb = fma(fma(-2.0 * K(K_Q2FXM), fzn, K(K_Q1FXM)), fxmb, fznb);
    fznb = fma(fma(-2.0 * K(K_Q2FYM), fzn, K(K_Q1FYM)), fymb, fznb);
    fznb = fma(fma(-2.0 * K(K_Q2FXS), fzn, K(K_Q1FXS)), fxsb, fznb);
    fznb = fma(fma(-2.0 * K(K_Q2FYS), fzn, K(K_Q1FYS)), fysb, fznb);
    kb.at(KB_Q1FXM) = fma(fzn, fxmb, kb.at(KB_Q1FXM));
    kb.at(KB_Q2FXM) = fma(-fzn * fzn, fxmb, kb.at(KB_Q2FXM));
    kb.at(KB_Q1FYM) = fma(fzn, fymb, kb.at(KB_Q1FYM));
    kb.at(KB_Q2FYM) = fma(-fzn * fzn, fymb, kb.at(KB_Q2FYM));
    kb.at(KB_Q1FXS) = fma(fzn, fxsb, kb.at(KB_Q1FXS));
    kb.at(KB_Q2FXS) = fma(-fzn * fzn, fxsb, kb.at(KB_Q2FXS));
    kb.at(KB_Q1FYS) = fma(fzn, fysb, kb.at(KB_Q1FYS));
    kb.at(KB_Q2FYS) = fma(-fzn * fzn, fysb, kb.at(KB_Q2FYS));
    fznb = fma(K(K_DSXM), sxmb, fma(K(K_DSYM), symb, fma(K(K_DSXS), sxsb, fma(K(K_DSYS), sysb, fznb))));
    fzcb = fma(K(K_INVPN), fznb, fzcb);
    if (T.at(TT_(fzcl)) == 0.0) fzb += fzcb;
    // slips
    const double ivta = T.at(TT_(ivta));
    vsxb = fma(-ivta, sxb, vsxb);
    vtab = fma(T.at(TT_(vsx)) * ivta * ivta, sxb, vtab);
    if (kSteered) {
        const double iD = 1.0 / T.at(TT_(D));
        const double Nb = -syb * iD, Db = T.at(TT_(N)) * (iD * iD) * syb;
        vsyb = fma(c, Nb, fma(s, Db, vsyb));
        vtab = fma(-s, Nb, fma(c, Db, vtab));
        cb = fma(T.at(TT_(vsy)), Nb, fma(T.at(TT_(vta)), Db, cb));
        sb_ = fma(-T.at(TT_(vta)), Nb, fma(T.at(TT_(vsy)), Db, sb_));
    } else {
        vsyb = fma(-ivta, syb, vsyb);
        vtab = fma(T.at(TT_(vsy)) * ivta * ivta, syb, vtab);
    }
    rwb += vtab;
    reffb = fabs(T.at(TT_(om))) * rwb;
    omb = fma(T.at(TT_(r_eff)) * T.at(TT_(sgn)), rwb, omb);
    vsxinb += vsxb;
    omb = fma(-T.at(TT_(r_eff)), vsxb, omb);
    reffb = fma(-T.at(TT_(om)), vsxb, reffb);
}

template <bool kSteered>
__device__ __forceinline__ void tire_rev(const TapeRef& T, const KView& K, const KBar& kb, double xedotb,
                                         double yedotb, double fxb, double fyb, double Myb, double rStatb, double& xeb,
                                         double& yeb, double& omb, double& vsxinb, double& vsyb, double& fzb,
                                         double& cb, double& sb_, double c, double s) {
    double reffb = 0.0;
    tire_rev_core<kSteered>(T, K, kb, xedotb, yedotb, fxb, fyb, Myb, rStatb, xeb, yeb, omb, vsxinb, vsyb, fzb, reffb,
                            cb, sb_, c, s);
    // r_eff = rdynco xt + rStat, rStat = r0 - xt, xt = fz / kt
    double xtb = T.at(TT_(rdynco)) * reffb;
    rStatb += reffb;
    if (T.at(TT_(fzrd)) != 0.0) fzb += K(K_DRD) * K(K_INVPN) * (T.at(TT_(xt)) * reffb);  // rdynco interpolated in fz
    xtb += -rStatb;
    fzb = fma(K(K_INVKT), xtb, fzb);
    kb.at(KB_INVKT) = fma(T.at(TT_(fz)), xtb, kb.at(KB_INVKT));
}

// TMeasyNr tire adjoint (on-ground tire): from the adjoints of fx, fy, My (before any frame rotation)
// and of rStat to those of omega, vsx before the slip correction, vsy, fz and cos/sin of the wheel
// angle; branches (Coulomb clamp, blend band, curve regime, load clamp) as the forward took them.
template <bool kSteered>
__device__ __forceinline__ void tire_rev_nr(const TapeRef& T, const KView& K, const KBar& kb, double fxb, double fyb,
                                            double Myb, double rStatb, double& omb, double& vsxinb, double& vsyb,
                                            double& fzb, double& cb, double& sb_, double c, double s) {
    const double mu = K(K_MU);
    // rolling resistance My = -rr fzc rStat tanh(omega)
    const double th = T.at(TN_(th)), fzc = T.at(TN_(fzc)), rStat = T.at(TN_(rStat));
    double fzcb = -K(K_RR) * rStat * th * Myb;
    rStatb = fma(-K(K_RR) * fzc * th, Myb, rStatb);
    omb = fma(-K(K_RR) * fzc * rStat * fma(-th, th, 1.0), Myb, omb);
    // blend of the Coulomb and the slip forces
    const double w = T.at(TN_(w));
    const double Fx0b = (1.0 - w) * fxb, Fy0b = (1.0 - w) * fyb;
    const double Fxb = w * fxb, Fyb = w * fyb;
    const double wb = fma(T.at(TN_(Fx)) - T.at(TN_(Fx0)), fxb, (T.at(TN_(Fy)) - T.at(TN_(Fy0))) * fyb);
    vsxinb = fma(T.at(TN_(dw)) * (T.at(TN_(vsxin)) >= 0 ? 1.0 : -1.0), wb, vsxinb);
    // Fx = f sx isc, Fy = f sy isc
    const double sx = T.at(TN_(sx)), sy = T.at(TN_(sy));
    double fb = 0, sxb = 0, syb = 0, iscb = 0;
    if (T.at(TN_(sc)) > 0.0) {
        const double f = T.at(TN_(f)), isc = T.at(TN_(isc));
        const double pr = fma(sx, Fxb, sy * Fyb);
        fb = isc * pr;
        sxb = f * isc * Fxb;
        syb = f * isc * Fyb;
        iscb = f * pr;
    }
    // f = fos s on every regime of tmxy_combined
    double scb = T.at(TN_(fos)) * fb, df0b = 0, smb = 0, fmb = 0, ssb = 0, fsb = 0;
    tmxy_rev(T.at(TN_(sc)), T.at(TN_(df0)), T.at(TN_(sm)), T.at(TN_(fm)), T.at(TN_(ss)), T.at(TN_(fs)),
             T.at(TN_(sc)) * fb, scb, df0b, smb, fmb, ssb, fsb);
    // curve magnitudes: df0 = |(dfx0 ca, dfy0 sa)|, fm = mu |(fxm ca, fym sa)|, ...
    const double ca = T.at(TN_(calpha)), sa = T.at(TN_(salpha));
    double cab = 0, sab = 0;
    double dfx0b = 0, dfy0b = 0, fxmb = 0, fymb = 0, fxsb = 0, fysb = 0, sxmb = 0, symb = 0, sxsb = 0, sysb = 0;
    auto hyp_rev = [&](double p, double q, double h, double hb, double& pb_, double& qb_, double& cab_,
                       double& sab_) {
        if (h > 0 && hb != 0.0) {  // h = |(p ca, q sa)|
            const double t = hb / h;
            pb_ = fma(ca * (p * ca), t, pb_);
            qb_ = fma(sa * (q * sa), t, qb_);
            cab_ = fma(p * (p * ca), t, cab_);
            sab_ = fma(q * (q * sa), t, sab_);
        }
    };
    hyp_rev(T.at(TN_(dfx0)), T.at(TN_(dfy0)), T.at(TN_(df0)), df0b, dfx0b, dfy0b, cab, sab);
    hyp_rev(T.at(TN_(fxm)), T.at(TN_(fym)), T.at(TN_(hfm)), mu * fmb, fxmb, fymb, cab, sab);
    hyp_rev(T.at(TN_(sxm)), T.at(TN_(sym)), T.at(TN_(hsm)), mu * smb, sxmb, symb, cab, sab);
    hyp_rev(T.at(TN_(fxs)), T.at(TN_(fys)), T.at(TN_(hfs)), mu * fsb, fxsb, fysb, cab, sab);
    hyp_rev(T.at(TN_(sxs)), T.at(TN_(sys)), T.at(TN_(hss)), mu * ssb, sxsb, sysb, cab, sab);
    // ca = sx isc, sa = sy isc, sc = q isc, isc = q^-1/2, q = sx^2 + sy^2
    if (T.at(TN_(qpos)) != 0.0) {
        const double isc = T.at(TN_(isc)), q = T.at(TN_(q));
        sxb = fma(isc, cab, sxb);
        syb = fma(isc, sab, syb);
        iscb = fma(sx, cab, fma(sy, sab, iscb));
        iscb = fma(q, scb, iscb);
        const double qb = fma(isc, scb, -0.5 * isc * isc * isc * iscb);
        sxb = fma(2.0 * sx, qb, sxb);
        syb = fma(2.0 * sy, qb, syb);
    }
    // curve parameters from the normalised load
    const double fzn = T.at(TN_(fzn));
    double fznb = 0;
    fznb = fma(fma(-2.0 * K(K_Q2DFX0), fzn, K(K_Q1DFX0)), dfx0b, fznb);
    fznb = fma(fma(-2.0 * K(K_Q2DFY0), fzn, K(K_Q1DFY0)), dfy0b, fznb);
    fznb = fma(fma(-2.0 * K(K_Q2FXM), fzn, K(K_Q1FXM)), fxmb, fznb);
    fznb = fma(fma(-2.0 * K(K_Q2FYM), fzn, K(K_Q1FYM)), fymb, fznb);
    fznb = fma(fma(-2.0 * K(K_Q2FXS), fzn, K(K_Q1FXS)), fxsb, fznb);
    fznb = fma(fma(-2.0 * K(K_Q2FYS), fzn, K(K_Q1FYS)), fysb, fznb);
    kb.at(KB_Q1FXM) = fma(fzn, fxmb, kb.at(KB_Q1FXM));
    kb.at(KB_Q2FXM) = fma(-fzn * fzn, fxmb, kb.at(KB_Q2FXM));
    kb.at(KB_Q1FYM) = fma(fzn, fymb, kb.at(KB_Q1FYM));
    kb.at(KB_Q2FYM) = fma(-fzn * fzn, fymb, kb.at(KB_Q2FYM));
    kb.at(KB_Q1FXS) = fma(fzn, fxsb, kb.at(KB_Q1FXS));
    kb.at(KB_Q2FXS) = fma(-fzn * fzn, fxsb, kb.at(KB_Q2FXS));
    kb.at(KB_Q1FYS) = fma(fzn, fysb, kb.at(KB_Q1FYS));
    kb.at(KB_Q2FYS) = fma(-fzn * fzn, fysb, kb.at(KB_Q2FYS));
    fznb = fma(K(K_DSXM), sxmb, fma(K(K_DSYM), symb, fma(K(K_DSXS), sxsb, fma(K(K_DSYS), sysb, fznb))));
    fzcb = fma(K(K_INVPN), fznb, fzcb);
    if (T.at(TN_(fzcl)) == 0.0) fzb += fzcb;
    // slips
    const double vta = T.at(TN_(vta)), ivta = 1.0 / vta;
    double vsxb = -ivta * sxb;
    double vtab = T.at(TN_(vsx)) * ivta * ivta * sxb;
    if (kSteered) {
        const double iD = 1.0 / T.at(TN_(D));
        const double Nb = -syb * iD, Db = T.at(TN_(N)) * (iD * iD) * syb;
        vsyb = fma(c, Nb, fma(s, Db, vsyb));
        vtab = fma(-s, Nb, fma(c, Db, vtab));
        cb = fma(T.at(TN_(vsy)), Nb, fma(vta, Db, cb));
        sb_ = fma(-vta, Nb, fma(T.at(TN_(vsy)), Db, sb_));
    } else {
        vsyb = fma(-ivta, syb, vsyb);
        vtab = fma(T.at(TN_(vsy)) * ivta * ivta, syb, vtab);
    }
    // Coulomb force: (a, b) = (tx, ty) fz mu, clamped to the circle of radius fz mu
    {
        const double fz = T.at(TN_(fz));
        double ab = Fx0b, bb = Fy0b;
        if (T.at(TN_(clamp)) != 0.0) {
            const double a0 = T.at(TN_(a0)), b0 = T.at(TN_(b0)), h0 = T.at(TN_(h0));
            const double ih = 1.0 / h0, g = fz * mu * ih;
            const double dot = fma(a0, Fx0b, b0 * Fy0b);
            ab = g * fma(-a0 * ih * ih, dot, Fx0b);
            bb = g * fma(-b0 * ih * ih, dot, Fy0b);
            fzb = fma(mu * ih, dot, fzb);
        }
        const double tx = T.at(TN_(tx)), ty = T.at(TN_(ty));
        fzb = fma(mu, fma(tx, ab, ty * bb), fzb);
        const double k2 = -2.0 / K(K_VCOUL);
        vsxb = fma(fma(-tx, tx, 1.0) * k2, fz * mu * ab, vsxb);
        vsyb = fma(fma(-ty, ty, 1.0) * k2, fz * mu * bb, vsyb);
    }
    // vsx = vsxin - omega r_eff, vta = r_eff |omega| + 0.01
    const double om = T.at(TN_(om)), r_eff = T.at(TN_(r_eff));
    double reffb = fabs(om) * vtab;
    omb = fma(r_eff * (om > 0 ? 1.0 : (om < 0 ? -1.0 : 0.0)), vtab, omb);
    vsxinb += vsxb;
    omb = fma(-r_eff, vsxb, omb);
    reffb = fma(-om, vsxb, reffb);
    // r_eff = rdynco xt + rStat, rStat = r0 - xt, xt = fz / kt
    double xtb = T.at(TN_(rdynco)) * reffb;
    rStatb += reffb;
    if (T.at(TN_(fzrd)) != 0.0) fzb += K(K_DRD) * K(K_INVPN) * (T.at(TN_(xt)) * reffb);
    xtb += -rStatb;
    fzb = fma(K(K_INVKT), xtb, fzb);
    kb.at(KB_INVKT) = fma(T.at(TN_(fz)), xtb, kb.at(KB_INVKT));
}

// Reverse of one right-hand-side evaluation (rhsFun): from the adjoints of its outputs (udotb,
// vdotb, wxdotb, wzdotb: chassis accelerations; dOcb: crank acceleration with a torque converter;
// crank_outb: the crank speed the powertrain computes from the wheel speeds without one; dOmb,
// xedotnb, yedotnb: wheel accelerations and deflection rates) to those of the state it reads, which
// are added to ub, vb, wxb, wzb, phib, crankb and om_midb; L.xe/L.ye hold on entry what the caller
// carries for the deflections and receive (with L.om, L.xedot, L.yedot, L.udot, L.vdot) the
// totals. The adjoints of the controls are added to steerb/thrb/brkb, those of the parameter
// constants to kb.
template <bool kNr = false>
__device__ __forceinline__ void rev18_rhs(const TapeRef& T, const KView& K, const ClassDev18& C, const KBar& kb,
                                          const double udotb, const double vdotb, const double wxdotb,
                                          const double wzdotb, const double dOcb, double crank_outb,
                                          const double* dOmb, const double* xedotnb, const double* yedotnb,
                                          double& ub, double& vb, double& wxb, double& wzb, double& phib,
                                          double& crankb, double* om_midb, Adj18& L, double& steerb, double& thrb,
                                          double& brkb) {
    const int g = (int)T.at(TS_(gear));
    // vehicle RHS
    double fxrb[4], fyrb[4];
    {
        const double innerb = K(K_INVMT) * udotb;
        kb.at(KB_INVMT) = fma(T.at(TS_(inner)), udotb, kb.at(KB_INVMT));
        wzb = fma(T.at(TS_(v)), udotb, wzb);
        vb = fma(T.at(TS_(wz)), udotb, vb);
        wzb = fma((fma(2.0 * K(K_UWZ2), T.at(TS_(wz)), -K(K_UWZWX) * T.at(TS_(wx)))), innerb, wzb);
        wxb = fma(-K(K_UWZWX) * T.at(TS_(wz)), innerb, wxb);
        kb.at(KB_UWZ2) = fma(T.at(TS_(wz)) * T.at(TS_(wz)), innerb, kb.at(KB_UWZ2));
        kb.at(KB_UWZWX) = fma(-T.at(TS_(wz)) * T.at(TS_(wx)), innerb, kb.at(KB_UWZWX));
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            fxrb[k] = innerb;
            fyrb[k] = 0;
        }
        const double E1b = fma(K(K_CV1), vdotb, fma(K(K_CV3), wxdotb, K(K_CV2) * wzdotb));
        const double E2b = fma(K(K_CV2), vdotb, fma(K(K_CX2), wxdotb, K(K_CZ2) * wzdotb));
        const double E3b = fma(K(K_CV3), vdotb, fma(K(K_CX3), wxdotb, K(K_CX2) * wzdotb));
        kb.at(KB_CV1) = fma(T.at(TS_(E1)), vdotb, kb.at(KB_CV1));
        kb.at(KB_CV2) = fma(T.at(TS_(E2)), vdotb, fma(T.at(TS_(E1)), wzdotb, kb.at(KB_CV2)));
        kb.at(KB_CV3) = fma(T.at(TS_(E3)), vdotb, fma(T.at(TS_(E1)), wxdotb, kb.at(KB_CV3)));
        kb.at(KB_CX2) = fma(T.at(TS_(E2)), wxdotb, fma(T.at(TS_(E3)), wzdotb, kb.at(KB_CX2)));
        kb.at(KB_CX3) = fma(T.at(TS_(E3)), wxdotb, kb.at(KB_CX3));
        kb.at(KB_CZ2) = fma(T.at(TS_(E2)), wzdotb, kb.at(KB_CZ2));
        double wub = K(K_E3WU) * E3b;
        phib = fma(K(K_E3PHI), E3b, phib);
        wxb = fma(K(K_E3WX), E3b, wxb);
        kb.at(KB_E3WU) = fma(T.at(TS_(wu)), E3b, kb.at(KB_E3WU));
        kb.at(KB_E3PHI) = fma(T.at(TS_(phi)), E3b, kb.at(KB_E3PHI));
        const double fyf = T.at(TS_(fyr) + 0) + T.at(TS_(fyr) + 1), fyr = T.at(TS_(fyr) + 2) + T.at(TS_(fyr) + 3);
        wub = fma(K(K_E2WU), E2b, wub);
        fxrb[3] = fma(K(K_CR2), E2b, fxrb[3]);
        fxrb[2] -= K(K_CR2) * E2b;
        fxrb[1] = fma(K(K_CF2), E2b, fxrb[1]);
        fxrb[0] -= K(K_CF2) * E2b;
        double fyfb = K(K_A) * E2b, fyrb_ = -K(K_B) * E2b;
        kb.at(KB_E2WU) = fma(T.at(TS_(wu)), E2b, kb.at(KB_E2WU));
        kb.at(KB_A) = fma(fyf, E2b, kb.at(KB_A));
        wub = fma(-K(K_MT), E1b, wub);
        fyfb += E1b;
        fyrb_ += E1b;
        kb.at(KB_MT) = fma(-T.at(TS_(wu)), E1b, kb.at(KB_MT));
        (void)fyr;
        fyrb[0] += fyfb;
        fyrb[1] += fyfb;
        fyrb[2] += fyrb_;
        fyrb[3] += fyrb_;
        wzb = fma(T.at(TS_(u)), wub, wzb);
        ub = fma(T.at(TS_(wz)), wub, ub);
    }
    // front forces rotated into the vehicle frame
    double fxb[4], fyb[4], cdb = 0, sdb = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (k < 2) {
            const double fx = tire_ref(T, k).at(TT_(fx)), fy = tire_ref(T, k).at(TT_(fy));
            fxb[k] = fma(T.at(TS_(cd)), fxrb[k], T.at(TS_(sd)) * fyrb[k]);
            fyb[k] = fma(-T.at(TS_(sd)), fxrb[k], T.at(TS_(cd)) * fyrb[k]);
            cdb += fma(fx, fxrb[k], fy * fyrb[k]);
            sdb += fma(-fy, fxrb[k], fx * fyrb[k]);
        } else {
            fxb[k] = fxrb[k];
            fyb[k] = fyrb[k];
        }
    }
    // powertrain
    double Myb[4], rStatb[4], engb[4], brakeb = 0;
    double om_mid[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        om_mid[k] = tire_ref(T, k).at(TT_(on)) != 0.0 ? tire_ref(T, k).at(TT_(om)) : 0.0;
        const double gk = K(K_INVJW) * dOmb[k];
        engb[k] = gk;
        Myb[k] = gk;
        brakeb = fma(-sgnd(om_mid[k]), gk, brakeb);
        fxb[k] = fma(-tire_ref(T, k).at(TT_(rStat)), gk, fxb[k]);
        rStatb[k] = -tire_ref(T, k).at(TT_(fx)) * gk;
    }
    brkb = fma(K(K_MAXBRAKE), brakeb, brkb);
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
    const double tfb = split_rev(T.at(TS_(tf)), T.at(TS_(alf)), T.at(TS_(dalf)), T.at(TS_(slowf)), engb[0], engb[1], om_mid[0], om_mid[1], om_midb[0],
                                 om_midb[1]);
    const double trrb = split_rev(T.at(TS_(trr)), T.at(TS_(alr)), T.at(TS_(dalr)), T.at(TS_(slowr)), engb[2], engb[3], om_mid[2], om_mid[3], om_midb[2],
                                  om_midb[3]);
    double torque_tb = C.driveType ? 0.5 * (tfb + trrb) : (C.whichWheels ? trrb : tfb);
    if (T.at(TS_(tclip)) != 0.0) torque_tb = 0;
    if (C.tcbool) {
        const double torque_outb = C.invgear[g] * torque_tb;
        double torque_inb = 0, trb = 0;
        if (T.at(TS_(rev)) != 0.0) {
            torque_inb += -torque_outb;
        } else {
            trb = -T.at(TS_(torque_in)) * torque_outb;
            torque_inb = fma(-T.at(TS_(tr)), torque_outb, torque_inb);
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
            omega_outb = fma(sr0b, iin, omega_outb);
            omega_inb = fma(-T.at(TS_(omega_out)) * iin * iin, sr0b, omega_inb);
        }
        const double omega_tb = omega_outb * C.invgear[g];
#pragma unroll
        for (int k = 0; k < 4; ++k) om_midb[k] += 0.25 * omega_tb;
        crankb += omega_inb;
    } else {
        const double dtqb = C.invgear[g] * torque_tb;
        thrb = fma(T.at(TS_(dt_map)), dtqb, thrb);
        crank_outb = fma(T.at(TS_(dt_slope)), dtqb, crank_outb);
#pragma unroll
        for (int k = 0; k < 4; ++k) om_midb[k] += 0.25 * crank_outb * C.invgear[g];
    }
    // tires
    double vsxinb[4], vsyb[4], fzb[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        vsxinb[k] = vsyb[k] = fzb[k] = 0;
        if (tire_ref(T, k).at(TT_(on)) != 0.0) {
            double xeb = L.xe[k], yeb = L.ye[k], omb = om_midb[k];
            if (kNr) {
                xeb = yeb = 0;
                if (k < 2)
                    tire_rev_nr<true>(tire_ref(T, k), K, kb, fxb[k], fyb[k], Myb[k], rStatb[k], omb, vsxinb[k], vsyb[k],
                                      fzb[k], cdb, sdb, T.at(TS_(cd)), T.at(TS_(sd)));
                else {
                    double cdum = 0, sdum = 0;
                    tire_rev_nr<false>(tire_ref(T, k), K, kb, fxb[k], fyb[k], Myb[k], rStatb[k], omb, vsxinb[k],
                                       vsyb[k], fzb[k], cdum, sdum, 1.0, 0.0);
                }
            } else if (k < 2)
                tire_rev<true>(tire_ref(T, k), K, kb, xedotnb[k], yedotnb[k], fxb[k], fyb[k], Myb[k], rStatb[k], xeb, yeb,
                               omb, vsxinb[k], vsyb[k], fzb[k], cdb, sdb, T.at(TS_(cd)), T.at(TS_(sd)));
            else {
                double cdum = 0, sdum = 0;
                tire_rev<false>(tire_ref(T, k), K, kb, xedotnb[k], yedotnb[k], fxb[k], fyb[k], Myb[k], rStatb[k], xeb, yeb,
                                omb, vsxinb[k], vsyb[k], fzb[k], cdum, sdum, 1.0, 0.0);
            }
            L.xe[k] = xeb;
            L.ye[k] = yeb;
            L.om[k] = omb;
            L.xedot[k] = 0;
            L.yedot[k] = 0;
        } else {  // lifted wheel: xe, ye, omega were zeroed; the stale rates carry
            L.xe[k] = 0;
            L.ye[k] = 0;
            L.om[k] = 0;
            L.xedot[k] = xedotnb[k];
            L.yedot[k] = yedotnb[k];
        }
    }
    // vehicle-to-tire transform
    {
        const double vsyfb = fma(T.at(TS_(sd)), (vsxinb[0] + vsxinb[1]), vsyb[0] + vsyb[1]);
        sdb = fma(T.at(TS_(vsyf)), (vsxinb[0] + vsxinb[1]), sdb);
        cdb = fma((T.at(TS_(u)) - T.at(TS_(wcf))), vsxinb[0], fma((T.at(TS_(u)) + T.at(TS_(wcf))), vsxinb[1], cdb));
        ub = fma(T.at(TS_(cd)), (vsxinb[0] + vsxinb[1]), ub + vsxinb[2] + vsxinb[3]);
        const double wcfb = T.at(TS_(cd)) * (vsxinb[1] - vsxinb[0]);
        const double wcrb = vsxinb[3] - vsxinb[2];
        const double vsyrb = vsyb[2] + vsyb[3];
        wzb = fma(K(K_A), vsyfb, fma(-K(K_B), vsyrb, fma(K(K_CF2), wcfb, fma(K(K_CR2), wcrb, wzb))));
        vb += vsyfb + vsyrb;
        kb.at(KB_A) = fma(T.at(TS_(wz)), vsyfb, kb.at(KB_A));
    }
    // wheel angle
    steerb = fma(T.at(TS_(dslope)), (fma(T.at(TS_(cd)), sdb, -(T.at(TS_(sd))) * cdb)), steerb);
    // tire loads (with the previous step's accelerations)
    double udot_oldb, vdot_oldb;
    {
        const double g0 = T.at(TS_(fzarg) + 0) > 0 ? 1.0 : 0.0, g1 = T.at(TS_(fzarg) + 1) > 0 ? 1.0 : 0.0;
        const double g2 = T.at(TS_(fzarg) + 2) > 0 ? 1.0 : 0.0, g3 = T.at(TS_(fzarg) + 3) > 0 ? 1.0 : 0.0;
        const double Afb = fma(fzb[0], g0, fzb[1] * g1), Bfb = fma(-fzb[0], g0, fzb[1] * g1);
        const double Arb = fma(fzb[2], g2, fzb[3] * g3), Brb = fma(-fzb[2], g2, fzb[3] * g3);
        const double Z4b = -Afb + Arb;
        kb.add(KB_Z1F, Afb);
        kb.add(KB_Z1R, Arb);
        const double latb = fma(K(K_Z2F), Bfb, K(K_Z2R) * Brb);
        kb.at(KB_Z2F) = fma(T.at(TS_(lat)), Bfb, kb.at(KB_Z2F));
        kb.at(KB_Z2R) = fma(T.at(TS_(lat)), Brb, kb.at(KB_Z2R));
        phib = fma(K(K_Z3FK), Bfb, fma(K(K_Z3RK), Brb, phib));
        wxb = fma(K(K_Z3FB), Bfb, fma(K(K_Z3RB), Brb, wxb));
        const double lonb = K(K_Z4) * Z4b;
        kb.at(KB_Z4) = fma(T.at(TS_(lon)), Z4b, kb.at(KB_Z4));
        wzb = fma(T.at(TS_(u)), latb, fma(-(T.at(TS_(v))), lonb, wzb));
        ub = fma(T.at(TS_(wz)), latb, ub);
        vb = fma(-T.at(TS_(wz)), lonb, vb);
        vdot_oldb = latb;
        udot_oldb = lonb;
    }
    L.udot = udot_oldb;
    L.vdot = vdot_oldb;
}

// One step's reverse sweep. L: on entry the adjoint of the state after the step, on return that of
// the state before it; the adjoints of the step's controls are added to steerb/thrb/brkb and those
// of the differentiable constants to kb.
__device__ __forceinline__ void rev18(const TapeRef& T, const KView& K, const ClassDev18& C, const KBar& kb,
                                      double dt, Adj18& L, double& steerb, double& thrb, double& brkb) {
    // half-implicit update: x, y with the updated speeds and the old yaw; yaw and roll with the
    // updated rates
    double u1b = dt * fma(T.at(TS_(cp)), L.x, T.at(TS_(sp)) * L.y);
    double v1b = dt * fma(-T.at(TS_(sp)), L.x, T.at(TS_(cp)) * L.y);
    double psib = fma(dt, (fma((fma(-T.at(TS_(u1)), T.at(TS_(sp)), -(T.at(TS_(v1))) * T.at(TS_(cp)))), L.x, (fma(T.at(TS_(u1)), T.at(TS_(cp)), -(T.at(TS_(v1))) * T.at(TS_(sp)))) * L.y)), L.psi);
    double wz1b = fma(dt, L.psi, L.wz);
    double wx1b = fma(dt, L.phi, L.wx);
    const double phib0 = L.phi;
    u1b += L.u;
    v1b += L.v;
    double ub = u1b, vb = v1b, wxb = wx1b, wzb = wz1b, phib = phib0;
    const double udotb = fma(dt, u1b, L.udot);  // the new accelerations are also carried to the next step
    const double vdotb = fma(dt, v1b, L.vdot);
    const double wxdotb = dt * wx1b, wzdotb = dt * wz1b;
    double crankb = 0, dOcb = 0, crank_outb = 0;
    if (C.tcbool) {
        crankb = L.crank;
        dOcb = dt * L.crank;
    } else {
        crank_outb = L.crank;
    }
    double om_midb[4], dOmb[4], xedotnb[4], yedotnb[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        om_midb[k] = L.om[k];
        dOmb[k] = dt * L.om[k];
        xedotnb[k] = fma(dt, L.xe[k], L.xedot[k]);
        yedotnb[k] = fma(dt, L.ye[k], L.yedot[k]);
    }
    rev18_rhs(T, K, C, kb, udotb, vdotb, wxdotb, wzdotb, dOcb, crank_outb, dOmb, xedotnb, yedotnb, ub, vb, wxb, wzb,
              phib, crankb, om_midb, L, steerb, thrb, brkb);
    // L.x, L.y are unchanged (x and y enter the next state with unit weight)
    L.u = ub;
    L.v = vb;
    L.psi = psib;
    L.wz = wzb;
    L.phi = phib;
    L.wx = wxb;
    L.crank = C.tcbool ? crankb : 0.0;
}

}  // namespace lfdm
