/*
 * ORACLE — test infrastructure only (see lfdm_oracle.h). Never linked into the product.
 *
 * Plain-C FP64 restatement of the reference's 18-DOF half-implicit stepper. Each function keeps
 * the reference's expression order and parenthesisation so that, compiled without FMA
 * contraction, it reproduces the reference CPU solver bit for bit (checked against
 * tests/golden/). Reference files cited by path inside wheeled_vehicle_models/.
 */
#define _GNU_SOURCE
#include "lfdm_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

static const double C_PI = 3.141592653589793238462643383279;
static const double C_2PI = 6.283185307179586476925286766559;
static const double G = 9.81;

/* ---------------------------------------------------------------------------------------------- */
/* utils (utils/utils_gpu.cuh, utils/utils_gpu.cu)                                                */

/* InterpL, InterpQ: utils_gpu.cuh:86-93 */
static double InterpL(double fz, double w1, double w2, double pn) { return w1 + (w2 - w1) * (fz / pn - 1.); }
static double InterpQ(double fz, double w1, double w2, double pn) {
    return (fz / pn) * (2. * w1 - 0.5 * w2 - (w1 - 0.5 * w2) * (fz / pn));
}
/* sgn: utils_gpu.cuh:96-99 */
static int sgn(double v) { return (0. < v) - (v < 0.); }
/* clamp: utils_gpu.cuh:104-111 */
static double clampd(double v, double lo, double hi) {
    if (v < lo) return lo;
    if (v > hi) return hi;
    return v;
}
/* sineStep: utils_gpu.cu:78-88 */
static double sineStep(double x, double x1, double y1, double x2, double y2) {
    if (x <= x1) return y1;
    if (x >= x2) return y2;
    double dx = x2 - x1;
    double dy = y2 - y1;
    double y = y1 + dy * (x - x1) / dx - (dy / C_2PI) * sin(C_2PI * (x - x1) / dx);
    return y;
}
/* lower_bound over {x, y} pairs keyed on x: utils_gpu.cu:109-121 (std::lower_bound on CPU) */
static int lower_bound_key(const double* a, int n, int stride, double x) {
    int l = 0, h = n;
    while (l < h) {
        int mid = l + (h - l) / 2;
        if (x <= a[(size_t)mid * stride]) h = mid;
        else l = mid + 1;
    }
    return l;
}
/* getMapY: utils_gpu.cu:60-75 */
double oracle_map_y(const double* map, int n, double x) {
    if (x <= map[0]) return map[1];
    else if (x >= map[2 * (n - 1)]) return map[2 * (n - 1) + 1];
    int right = lower_bound_key(map, n, 2, x);
    int left = right - 1;
    double mbar = (x - map[2 * left]) / (map[2 * right] - map[2 * left]);
    return (map[2 * left + 1] + mbar * (map[2 * right + 1] - map[2 * left + 1]));
}
/* GetDriverInput: utils_gpu.cu:34-56; out = {time, steering, throttle, braking} */
void oracle_driver_input(double t, const double* d, int len, double* out) {
    if (t <= d[0]) {
        memcpy(out, d, 4 * sizeof(double));
    } else if (t >= d[4 * (len - 1)]) {
        memcpy(out, d + 4 * (len - 1), 4 * sizeof(double));
    } else {
        int right = lower_bound_key(d, len, 4, t);
        int left = right - 1;
        const double* L = d + 4 * left;
        const double* R = d + 4 * right;
        double tbar = (t - L[0]) / (R[0] - L[0]);
        out[0] = t;
        out[1] = L[1] + tbar * (R[1] - L[1]);
        out[2] = L[2] + tbar * (R[2] - L[2]);
        out[3] = L[3] + tbar * (R[3] - L[3]);
    }
}

/* ---------------------------------------------------------------------------------------------- */
/* state views                                                                                     */
typedef struct {
    double xe, ye, xedot, yedot, omega, dOmega, xt, rStat, fx, fy, fz, vsx, vsy, My, engTor;
} Tire;
typedef struct {
    double x, y, u, v, psi, wz, phi, wx, udot, vdot, wxdot, wzdot, crankOmega, dOmega_crank;
    int current_gr;
} Veh;
typedef struct {
    const double* p;        /* flat params */
    const lfdm_class18* c;  /* class */
} Par;

#define P(i) (pp->p[(i)])

static void tire_init(double* p) {
    /* tireInit: 18dof-gpu/dof18_gpu.cu:227-233 */
    p[LFDM_P_FZRDYNCO] = (p[LFDM_P_PN] * (p[LFDM_P_RDYNCOP2N] - 2.0 * p[LFDM_P_RDYNCOPN] + 1.)) /
                         (2. * (p[LFDM_P_RDYNCOP2N] - p[LFDM_P_RDYNCOPN]));
    p[LFDM_P_RDYNCOCRIT] = InterpL(p[LFDM_P_FZRDYNCO], p[LFDM_P_RDYNCOPN], p[LFDM_P_RDYNCOP2N], p[LFDM_P_PN]);
}
void oracle_tire_init(double* params) { tire_init(params); }

/* steering input -> wheel angle: the head of vehToTireTransform etc. (dof18_gpu.cu:79-87) */
static double wheel_angle(const Par* pp, double steering) {
    if (pp->c->nonLinearSteer) return oracle_map_y(&pp->c->steerMap[0][0], pp->c->steerMapSize, steering);
    return steering * P(LFDM_P_MAXSTEER);
}

/* driveTorque: dof18_gpu.cu:15-38. throttleMod scales a private copy of the map, as the CPU     */
/* solver does (18dof/dof18.cpp:23-29); the GPU solver scales the shared map in place.           */
static double driveTorque(const Par* pp, double throttle, double motor_speed) {
    double motor_torque = 0.;
    const lfdm_class18* c = pp->c;
    if (c->throttleMod) {
        double m[LFDM_MAX_MAP][2];
        int len = c->powertrainMapSize;
        for (int i = 0; i < len; i++) {
            m[i][0] = c->powertrainMap[i][0] * throttle;
            m[i][1] = c->powertrainMap[i][1] * throttle;
        }
        motor_torque = oracle_map_y(&m[0][0], len, motor_speed);
        double motor_losses = oracle_map_y(&c->lossesMap[0][0], c->lossesMapSize, motor_speed);
        motor_torque = motor_torque + motor_losses;
    } else {
        motor_torque = oracle_map_y(&c->powertrainMap[0][0], c->powertrainMapSize, motor_speed);
        double motor_losses = oracle_map_y(&c->lossesMap[0][0], c->lossesMapSize, motor_speed);
        motor_torque = motor_torque * throttle + motor_losses;
    }
    return motor_torque;
}

/* differentialSplit: dof18_gpu.cu:42-69 */
static void differentialSplit(double torque, double max_bias, double speed_left, double speed_right,
                              double* torque_left, double* torque_right) {
    double diff = fabs(speed_left - speed_right);
    double bias = 1;
    if (diff > 0.5) bias = max_bias;
    else if (diff > 0.25) bias = 4 * (max_bias - 1) * diff + (2 - max_bias);
    double alpha = bias / (1 + bias);
    double slow = alpha * torque;
    double fast = torque - slow;
    if (fabs(speed_left) < fabs(speed_right)) {
        *torque_left = slow;
        *torque_right = fast;
    } else {
        *torque_left = fast;
        *torque_right = slow;
    }
}

/* vehToTireTransform: dof18_gpu.cu:71-109 */
static void vehToTireTransform(Tire* t, const Veh* v, const double* loads, const Par* pp, double steering) {
    double delta = wheel_angle(pp, steering);
    t[0].fz = loads[0];
    t[0].vsy = v->v + v->wz * P(LFDM_P_A);
    t[0].vsx = (v->u - (v->wz * P(LFDM_P_CF)) / 2.) * cos(delta) + t[0].vsy * sin(delta);
    t[1].fz = loads[1];
    t[1].vsy = v->v + v->wz * P(LFDM_P_A);
    t[1].vsx = (v->u + (v->wz * P(LFDM_P_CF)) / 2.) * cos(delta) + t[1].vsy * sin(delta);
    t[2].fz = loads[2];
    t[2].vsy = v->v - v->wz * P(LFDM_P_B);
    t[2].vsx = v->u - (v->wz * P(LFDM_P_CR)) / 2.;
    t[3].fz = loads[3];
    t[3].vsy = v->v - v->wz * P(LFDM_P_B);
    t[3].vsx = v->u + (v->wz * P(LFDM_P_CR)) / 2.;
}

/* tireToVehTransform: dof18_gpu.cu:152-185 (front tires rotated by the wheel angle) */
static void tireToVehTransform(Tire* t, const Par* pp, double steering) {
    double delta = wheel_angle(pp, steering);
    for (int k = 0; k < 2; ++k) {
        double fx = t[k].fx * cos(delta) - t[k].fy * sin(delta);
        double fy = t[k].fx * sin(delta) + t[k].fy * cos(delta);
        t[k].fx = fx;
        t[k].fy = fy;
    }
}

/* tmxy_combined: dof18_gpu.cu:243-285 */
static void tmxy_combined(double* f, double* fos, double s, double df0, double sm, double fm, double ss, double fs) {
    double df0loc = 0.0;
    if (sm > 0.0) df0loc = fmax(2.0 * fm / sm, df0);
    if (s > 0.0 && df0loc > 0.0) {
        if (s > ss) {
            *f = fs;
            *fos = *f / s;
        } else {
            if (s < sm) {
                double p = df0loc * sm / fm - 2.0;
                double sn = s / sm;
                double dn = 1.0 + (sn + p) * sn;
                *f = df0loc * sm * sn / dn;
                *fos = df0loc / dn;
            } else {
                double a = pow(fm / sm, 2.0) / (df0loc * sm);
                double sstar = sm + (fm - fs) / (a * (ss - sm));
                if (sstar <= ss) {
                    if (s <= sstar) {
                        *f = fm - a * (s - sm) * (s - sm);
                    } else {
                        double b = a * (sstar - sm) / (ss - sstar);
                        *f = fs + b * (ss - s) * (ss - s);
                    }
                } else {
                    double sn = (s - sm) / (ss - sm);
                    *f = fm - (fm - fs) * sn * sn * (3.0 - 2.0 * sn);
                }
                *fos = *f / s;
            }
        }
    } else {
        *f = 0.0;
        *fos = 0.0;
    }
}

/* computeCombinedCoulombForce: dof18_gpu.cu:287-303 */
static void coulomb(double* fx, double* fy, double mu, double vsx, double vsy, double fz, double vcoulomb) {
    *fx = tanh(-2.0 * vsx / vcoulomb) * fz * mu;
    *fy = tanh(-2.0 * vsy / vcoulomb) * fz * mu;
    if (hypot(*fx, *fy) > fz * mu) {
        double f = fz * mu / hypot(*fx, *fy);
        *fx *= f;
        *fy *= f;
    }
}

/* computeTireLoads: dof18_gpu.cu:305-340 (identical for both tire types) */
static void computeTireLoads(double* loads, const Veh* v, const Par* pp) {
    double huf = P(LFDM_P_R0);
    double hur = P(LFDM_P_R0);
    const double a = P(LFDM_P_A), b = P(LFDM_P_B), m = P(LFDM_P_M), h = P(LFDM_P_H);
    const double muf = P(LFDM_P_MUF), mur = P(LFDM_P_MUR), cf = P(LFDM_P_CF), cr = P(LFDM_P_CR);
    double Z1 = (m * G * b) / (2. * (a + b)) + (muf * G) / 2.;
    double Z2 = ((muf * huf) / cf + m * b * (h - P(LFDM_P_HRCF)) / (cf * (a + b))) * (v->vdot + v->wz * v->u);
    double Z3 = (P(LFDM_P_KROF) * v->phi + P(LFDM_P_BROF) * v->wx) / cf;
    double Z4 = ((m * h + muf * huf + mur * hur) * (v->udot - v->wz * v->v)) / (2. * (a + b));
    loads[0] = (Z1 - Z2 - Z3 - Z4) > 0. ? (Z1 - Z2 - Z3 - Z4) : 0.;
    loads[1] = (Z1 + Z2 + Z3 - Z4) > 0. ? (Z1 + Z2 + Z3 - Z4) : 0.;
    Z1 = (m * G * a) / (2. * (a + b)) + (mur * G) / 2.;
    Z2 = ((mur * hur) / cr + m * a * (h - P(LFDM_P_HRCR)) / (cr * (a + b))) * (v->vdot + v->wz * v->u);
    Z3 = (P(LFDM_P_KROR) * v->phi + P(LFDM_P_BROR) * v->wx) / cr;
    loads[2] = (Z1 - Z2 - Z3 + Z4) > 0. ? (Z1 - Z2 - Z3 + Z4) : 0.;
    loads[3] = (Z1 + Z2 + Z3 + Z4) > 0. ? (Z1 + Z2 + Z3 + Z4) : 0.;
}

/* computeTireRHS, TMeasy: dof18_gpu.cu:379-530 */
static void tireRHS_TM(Tire* ts, const Par* pp, double steering) {
    double delta = wheel_angle(pp, steering);
    double fz = ts->fz;
    double vsy = ts->vsy;
    double vsx = ts->vsx;
    if (fz <= 0) {
        ts->xe = 0;
        ts->ye = 0;
        ts->omega = 0;
        ts->xt = 0;
        ts->rStat = P(LFDM_P_R0);
        ts->fx = 0;
        ts->fy = 0;
        ts->My = 0;
        return;
    }
    const double pn = P(LFDM_P_PN), r0 = P(LFDM_P_R0);
    ts->xt = fz / P(LFDM_P_KT);
    ts->rStat = r0 - ts->xt;
    double r_eff, rdynco;
    if (fz <= P(LFDM_P_FZRDYNCO)) {
        rdynco = InterpL(fz, P(LFDM_P_RDYNCOPN), P(LFDM_P_RDYNCOP2N), pn);
        r_eff = rdynco * r0 + (1. - rdynco) * ts->rStat;
    } else {
        rdynco = P(LFDM_P_RDYNCOCRIT);
        r_eff = rdynco * r0 + (1. - rdynco) * ts->rStat;
    }
    vsx = vsx - (ts->omega * r_eff);
    double vta = r_eff * fabs(ts->omega) + 0.01;
    double sx = -vsx / vta;
    double alpha = atan2(vsy, vta) - delta;
    double sy = -tan(alpha);
    if (fz > P(LFDM_P_PNMAX)) fz = P(LFDM_P_PNMAX);
    double dfx0 = InterpQ(fz, P(LFDM_P_DFX0PN), P(LFDM_P_DFX0P2N), pn);
    double dfy0 = InterpQ(fz, P(LFDM_P_DFY0PN), P(LFDM_P_DFY0P2N), pn);
    double fxm = InterpQ(fz, P(LFDM_P_FXMPN), P(LFDM_P_FXMP2N), pn);
    double fym = InterpQ(fz, P(LFDM_P_FYMPN), P(LFDM_P_FYMP2N), pn);
    double fxs = InterpQ(fz, P(LFDM_P_FXSPN), P(LFDM_P_FXSP2N), pn);
    double fys = InterpQ(fz, P(LFDM_P_FYSPN), P(LFDM_P_FYSP2N), pn);
    double sxm = InterpL(fz, P(LFDM_P_SXMPN), P(LFDM_P_SXMP2N), pn);
    double sym = InterpL(fz, P(LFDM_P_SYMPN), P(LFDM_P_SYMP2N), pn);
    double sxs = InterpL(fz, P(LFDM_P_SXSPN), P(LFDM_P_SXSP2N), pn);
    double sys = InterpL(fz, P(LFDM_P_SYSPN), P(LFDM_P_SYSP2N), pn);
    double hsxn = sxm / (sxm + sym) + (fxm / dfx0) / (fxm / dfx0 + fym / dfy0);
    double hsyn = sym / (sxm + sym) + (fym / dfy0) / (fxm / dfx0 + fym / dfy0);
    double sxn = sx / hsxn;
    double syn = sy / hsyn;
    double sc = hypot(sxn, syn);
    double calpha, salpha;
    if (sc > 0) {
        calpha = sxn / sc;
        salpha = syn / sc;
    } else {
        calpha = sqrt(2.) / 2.;
        salpha = sqrt(2.) / 2.;
    }
    double df0 = hypot(dfx0 * calpha * hsxn, dfy0 * salpha * hsyn);
    double fm = hypot(fxm * calpha, fym * salpha);
    double sm = hypot(sxm * calpha / hsxn, sym * salpha / hsyn);
    double fs = hypot(fxs * calpha, fys * salpha);
    double ss = hypot(sxs * calpha / hsxn, sys * salpha / hsyn);
    double f, fos;
    tmxy_combined(&f, &fos, sc, df0, sm, fm, ss, fs);
    /* rolling resistance; sineStep(vta, 0, 0, 0, 1) with vx_min = vx_max = 0 */
    double vx_min = 0., vx_max = 0.;
    ts->My = -sineStep(vta, vx_min, 0., vx_max, 1.) * P(LFDM_P_RR) * fz * ts->rStat * sgn(ts->omega);
    double vtxs = r_eff * fabs(ts->omega) * hsxn + 0.01;
    double vtys = r_eff * fabs(ts->omega) * hsyn + 0.01;
    const double cx = P(LFDM_P_CX), cy = P(LFDM_P_CY), dx = P(LFDM_P_DX), dy = P(LFDM_P_DY);
    ts->xedot = (-vtxs * cx * ts->xe - fos * vsx) / (vtxs * dx + fos);
    ts->yedot = (-vtys * cy * ts->ye - fos * (-sy * vta)) / (vtys * dy + fos);
    double fxdyn = dx * (-vtxs * cx * ts->xe - fos * vsx) / (vtxs * dx + fos) + cx * ts->xe;
    double fydyn = dy * ((-vtys * cy * ts->ye - fos * (-sy * vta)) / (vtys * dy + fos)) + (cy * ts->ye);
    double fxstr = clampd(ts->xe * cx + ts->xedot * dx, -P(LFDM_P_FXMP2N), P(LFDM_P_FXMP2N));
    double fystr = clampd(ts->ye * cy + ts->yedot * dy, -P(LFDM_P_FYMP2N), P(LFDM_P_FYMP2N));
    double weightx = sineStep(fabs(vsx), 1., 1., 1.5, 0.);
    double weighty = sineStep(fabs(-sy * vta), 1., 1., 1.5, 0.);
    ts->fx = weightx * fxstr + (1. - weightx) * fxdyn;
    ts->fy = weighty * fystr + (1. - weighty) * fydyn;
}

/* computeTireRHS, TMeasyNr: dof18_gpu.cu:532-662 */
/* The TMeasyNr tire from the effective radius on (dof18_gpu.cu:532-662; 24dof/dof24.cpp:988-1108):
   fz > 0 is the unclamped load, r_eff the effective radius, rStat the loaded radius. */
static void tireNr_core(double* fx_out, double* fy_out, double* My_out, double fz, double r_eff, double rStat,
                        double omega, double vsx_in, double vsy, double vsx_raw, double delta, const Par* pp) {
    const double pn = P(LFDM_P_PN), mu = P(LFDM_P_MU);
    double vsx = vsx_in - (omega * r_eff);
    double vta = r_eff * fabs(omega) + 0.01;
    double Fx0 = 0, Fy0 = 0;
    coulomb(&Fx0, &Fy0, mu, vsx, vsy, fz, P(LFDM_P_VCOULOMB));
    double sx = -vsx / vta;
    double alpha = atan2(vsy, vta) - delta;
    double sy = -tan(alpha);
    if (fz > P(LFDM_P_PNMAX)) fz = P(LFDM_P_PNMAX);
    double dfx0 = InterpQ(fz, P(LFDM_P_DFX0PN), P(LFDM_P_DFX0P2N), pn);
    double dfy0 = InterpQ(fz, P(LFDM_P_DFY0PN), P(LFDM_P_DFY0P2N), pn);
    double fxm = InterpQ(fz, P(LFDM_P_FXMPN), P(LFDM_P_FXMP2N), pn);
    double fym = InterpQ(fz, P(LFDM_P_FYMPN), P(LFDM_P_FYMP2N), pn);
    double fxs = InterpQ(fz, P(LFDM_P_FXSPN), P(LFDM_P_FXSP2N), pn);
    double fys = InterpQ(fz, P(LFDM_P_FYSPN), P(LFDM_P_FYSP2N), pn);
    double sxm = InterpL(fz, P(LFDM_P_SXMPN), P(LFDM_P_SXMP2N), pn);
    double sym = InterpL(fz, P(LFDM_P_SYMPN), P(LFDM_P_SYMP2N), pn);
    double sxs = InterpL(fz, P(LFDM_P_SXSPN), P(LFDM_P_SXSP2N), pn);
    double sys = InterpL(fz, P(LFDM_P_SYSPN), P(LFDM_P_SYSP2N), pn);
    double frblend = sineStep(fabs(vsx_raw), P(LFDM_P_FRBLEND_BEGIN), 0., P(LFDM_P_FRBLEND_END), 1.);
    double sc = hypot(sx, sy);
    double salpha = 0, calpha = 0;
    if (sc > 0) {
        calpha = sx / sc;
        salpha = sy / sc;
    } else {
        calpha = sqrt(2.) / 2.;
        salpha = sqrt(2.) / 2.;
    }
    double df0 = hypot(dfx0 * calpha, dfy0 * salpha);
    double fm = mu * hypot(fxm * calpha, fym * salpha);
    double sm = mu * hypot(sxm * calpha, sym * salpha);
    double fs = mu * hypot(fxs * calpha, fys * salpha);
    double ss = mu * hypot(sxs * calpha, sys * salpha);
    double f, fos;
    tmxy_combined(&f, &fos, sc, df0, sm, fm, ss, fs);
    double Fx, Fy;
    if (sc > 0.) {
        Fx = f * sx / sc;
        Fy = f * sy / sc;
    } else {
        Fx = 0.;
        Fy = 0.;
    }
    Fx = (1.0 - frblend) * Fx0 + frblend * Fx;
    Fy = (1.0 - frblend) * Fy0 + frblend * Fy;
    *My_out = -P(LFDM_P_RR) * fz * rStat * tanh(omega);
    *fx_out = Fx;
    *fy_out = Fy;
}


static void tireRHS_Nr(Tire* ts, const Par* pp, double steering) {
    double delta = wheel_angle(pp, steering);
    double fz = ts->fz;
    if (fz <= 0) {
        ts->omega = 0;
        ts->xt = 0;
        ts->rStat = P(LFDM_P_R0);
        ts->fx = 0;
        ts->fy = 0;
        ts->My = 0;
        return;
    }
    const double pn = P(LFDM_P_PN), r0 = P(LFDM_P_R0);
    ts->xt = fz / P(LFDM_P_KT);
    ts->rStat = r0 - ts->xt;
    double r_eff, rdynco;
    if (fz <= P(LFDM_P_FZRDYNCO)) {
        rdynco = InterpL(fz, P(LFDM_P_RDYNCOPN), P(LFDM_P_RDYNCOP2N), pn);
        r_eff = rdynco * r0 + (1. - rdynco) * ts->rStat;
    } else {
        rdynco = P(LFDM_P_RDYNCOCRIT);
        r_eff = rdynco * r0 + (1. - rdynco) * ts->rStat;
    }
    tireNr_core(&ts->fx, &ts->fy, &ts->My, fz, r_eff, ts->rStat, ts->omega, ts->vsx, ts->vsy, ts->vsx, delta, pp);
}

/* computePowertrainRHS: dof18_gpu.cu:664-839 (same body for both tire types) */
static void powertrainRHS(Veh* v, Tire* t, const Par* pp, const double* controls) {
    const lfdm_class18* c = pp->c;
    double torque_t = 0;
    double max_bias = 2;
    const double throttle = controls[2], braking = controls[3];
    if (c->tcbool) {
        int tc_reverse_flow = 0;
        double omega_t = 0.25 * (t[0].omega + t[1].omega + t[2].omega + t[3].omega);
        double omega_out = omega_t / (c->gearRatios[v->current_gr]);
        double omega_in = v->crankOmega;
        double sr, cf, tr;
        if ((omega_out < 1e-9) || (omega_in < 1e-9)) {
            sr = 0;
            cf = oracle_map_y(&c->CFmap[0][0], c->CFmapSize, sr);
            tr = oracle_map_y(&c->TRmap[0][0], c->TRmapSize, sr);
        } else {
            sr = omega_out / omega_in;
            if (sr > 1.) {
                sr = 1. - (sr - 1.);
                tc_reverse_flow = 1;
            }
            if (sr < 0) sr = 0;
            cf = oracle_map_y(&c->CFmap[0][0], c->CFmapSize, sr);
            tr = oracle_map_y(&c->TRmap[0][0], c->TRmapSize, sr);
        }
        double torque_in = -pow((omega_in / cf), 2);
        if (tc_reverse_flow) torque_in = -torque_in;
        double torque_out;
        if (tc_reverse_flow) torque_out = -torque_in;
        else torque_out = -tr * torque_in;
        torque_t = torque_out / c->gearRatios[v->current_gr];
        /* reference: abs((u - 0) < 1e-9) && (torque_t < 0) — abs() of the comparison's result */
        if ((v->u - 0) < 1e-9 && (torque_t < 0)) torque_t = 0;
        v->dOmega_crank = (1. / P(LFDM_P_CRANKINERTIA)) * (driveTorque(pp, throttle, v->crankOmega) + torque_in);
        if (omega_out > c->shiftMap[v->current_gr][1]) {
            if (v->current_gr < c->noGears - 1) v->current_gr++;
        } else if (omega_out < c->shiftMap[v->current_gr][0]) {
            if (v->current_gr > 0) v->current_gr--;
        }
    } else {
        v->crankOmega =
            0.25 * (t[0].omega + t[1].omega + t[2].omega + t[3].omega) / c->gearRatios[v->current_gr];
        torque_t = driveTorque(pp, throttle, v->crankOmega) / c->gearRatios[v->current_gr];
        if ((v->u - 0) < 1e-9 && (torque_t < 0)) torque_t = 0;
        if (v->crankOmega > c->shiftMap[v->current_gr][1]) {
            if (v->current_gr < c->noGears - 1) v->current_gr++;
        } else if (v->crankOmega < c->shiftMap[v->current_gr][0]) {
            if (v->current_gr > 0) v->current_gr--;
        }
    }
    double torque_front = 0, torque_rear = 0;
    if (c->driveType) {
        torque_front = torque_t * 0.5;
        torque_rear = torque_t * 0.5;
    } else {
        if (c->whichWheels) {
            torque_front = 0;
            torque_rear = torque_t;
        } else {
            torque_front = torque_t;
            torque_rear = 0;
        }
    }
    differentialSplit(torque_front, max_bias, t[0].omega, t[1].omega, &t[0].engTor, &t[1].engTor);
    differentialSplit(torque_rear, max_bias, t[2].omega, t[3].omega, &t[2].engTor, &t[3].engTor);
    const double jw = P(LFDM_P_JW);
    const double brake = P(LFDM_P_MAXBRAKETORQUE) * braking; /* brakeTorque: dof18_gpu.cuh:1069-1071 */
    for (int k = 0; k < 4; ++k)
        t[k].dOmega = (1 / jw) * (t[k].engTor + t[k].My - sgn(t[k].omega) * brake - t[k].fx * t[k].rStat);
}

/* computeVehRHS: dof18_gpu.cu:1017-1068 */
static void vehRHS(Veh* v, const Par* pp, const double* fx, const double* fy) {
    const double a = P(LFDM_P_A), b = P(LFDM_P_B), m = P(LFDM_P_M), muf = P(LFDM_P_MUF), mur = P(LFDM_P_MUR);
    const double jx = P(LFDM_P_JX), jz = P(LFDM_P_JZ), jxz = P(LFDM_P_JXZ);
    double mt = m + 2 * (muf + mur);
    double hrc = (P(LFDM_P_HRCF) * b + P(LFDM_P_HRCR) * a) / (a + b);
    double E1 = -mt * v->wz * v->u + (fy[0] + fy[1] + fy[2] + fy[3]);
    double E2 = (fy[0] + fy[1]) * a - (fy[2] + fy[3]) * b + (fx[1] - fx[0]) * P(LFDM_P_CF) / 2 +
                (fx[3] - fx[2]) * P(LFDM_P_CR) / 2 + (-muf * a + mur * b) * v->wz * v->u;
    double E3 = m * G * hrc * v->phi - (P(LFDM_P_KROF) + P(LFDM_P_KROR)) * v->phi -
                (P(LFDM_P_BROF) + P(LFDM_P_BROR)) * v->wx + hrc * m * v->wz * v->u;
    double A1 = mur * b - muf * a;
    double A2 = jx + m * pow(hrc, 2);
    double A3 = hrc * m;
    v->udot = v->wz * v->v +
              (1 / mt) * ((fx[0] + fx[1] + fx[2] + fx[3]) + (-mur * b + muf * a) * pow(v->wz, 2) -
                          2. * hrc * m * v->wz * v->wx);
    double denom = (A2 * pow(A1, 2) - 2. * A1 * A3 * jxz + jz * pow(A3, 2) + mt * pow(jxz, 2) - A2 * jz * mt);
    v->vdot = (E1 * pow(jxz, 2) - A1 * A2 * E2 + A1 * E3 * jxz + A3 * E2 * jxz - A2 * E1 * jz - A3 * E3 * jz) / denom;
    v->wxdot = (pow(A1, 2) * E3 - A1 * A3 * E2 + A1 * E1 * jxz - A3 * E1 * jz + E2 * jxz * mt - E3 * jz * mt) / denom;
    v->wzdot = (pow(A3, 2) * E2 - A1 * A2 * E1 - A1 * A3 * E3 + A3 * E1 * jxz - A2 * E2 * mt + E3 * jxz * mt) / denom;
}

/* ---------------------------------------------------------------------------------------------- */
/* one vehicle                                                                                     */

static void load_state(const double* s, Veh* v, Tire* t) {
    v->x = s[LFDM_S_X];
    v->y = s[LFDM_S_Y];
    v->u = s[LFDM_S_U];
    v->v = s[LFDM_S_V];
    v->psi = s[LFDM_S_PSI];
    v->wz = s[LFDM_S_WZ];
    v->phi = s[LFDM_S_PHI];
    v->wx = s[LFDM_S_WX];
    v->udot = s[LFDM_S_UDOT];
    v->vdot = s[LFDM_S_VDOT];
    v->wxdot = s[LFDM_S_WXDOT];
    v->wzdot = s[LFDM_S_WZDOT];
    v->crankOmega = s[LFDM_S_CRANKOMEGA];
    v->dOmega_crank = s[LFDM_S_DOMEGA_CRANK];
    v->current_gr = (int)s[LFDM_S_CURRENT_GR];
    for (int k = 0; k < 4; ++k) memcpy(&t[k], s + LFDM_S_TIRE0 + k * LFDM_S_TIRE_STRIDE, sizeof(Tire));
}
static void store_state(double* s, const Veh* v, const Tire* t) {
    s[LFDM_S_X] = v->x;
    s[LFDM_S_Y] = v->y;
    s[LFDM_S_U] = v->u;
    s[LFDM_S_V] = v->v;
    s[LFDM_S_PSI] = v->psi;
    s[LFDM_S_WZ] = v->wz;
    s[LFDM_S_PHI] = v->phi;
    s[LFDM_S_WX] = v->wx;
    s[LFDM_S_UDOT] = v->udot;
    s[LFDM_S_VDOT] = v->vdot;
    s[LFDM_S_WXDOT] = v->wxdot;
    s[LFDM_S_WZDOT] = v->wzdot;
    s[LFDM_S_CRANKOMEGA] = v->crankOmega;
    s[LFDM_S_DOMEGA_CRANK] = v->dOmega_crank;
    s[LFDM_S_CURRENT_GR] = (double)v->current_gr;
    for (int k = 0; k < 4; ++k) memcpy(s + LFDM_S_TIRE0 + k * LFDM_S_TIRE_STRIDE, &t[k], sizeof(Tire));
}

/* rhsFun: 18dof-gpu/dof18_halfImplicit_gpu.cu:685-729 */
static void rhs(Veh* v, Tire* t, const Par* pp, const double* controls, int nr) {
    double loads[4] = {0., 0., 0., 0.};
    computeTireLoads(loads, v, pp);
    vehToTireTransform(t, v, loads, pp, controls[1]);
    if (nr) {
        tireRHS_Nr(&t[0], pp, controls[1]);
        tireRHS_Nr(&t[1], pp, controls[1]);
        tireRHS_Nr(&t[2], pp, 0);
        tireRHS_Nr(&t[3], pp, 0);
    } else {
        tireRHS_TM(&t[0], pp, controls[1]);
        tireRHS_TM(&t[1], pp, controls[1]);
        tireRHS_TM(&t[2], pp, 0);
        tireRHS_TM(&t[3], pp, 0);
    }
    powertrainRHS(v, t, pp, controls);
    tireToVehTransform(t, pp, controls[1]);
    double fx[4] = {t[0].fx, t[1].fx, t[2].fx, t[3].fx};
    double fy[4] = {t[0].fy, t[1].fy, t[2].fy, t[3].fy};
    vehRHS(v, pp, fx, fy);
}

/* PerturbRhsFun (18dof/dof18_halfImplicit.cpp:679-745) with unpackY / packYDOT (:879-1101): the
   right-hand side at the packed states y, unpacked into a fresh state (all fields 0, first gear) or
   into full_state. TMeasyNr tires carry no deflection states. */
static int perturb18(const Par* pp, const double* full_state, const double* y, const double* ctl, double* ydot,
                     int nr) {
    Veh v;
    Tire t[4];
    memset(&v, 0, sizeof v);
    memset(t, 0, sizeof t);
    if (full_state) load_state(full_state, &v, t);
    const int tc = pp->c->tcbool != 0;
    int i = 0;
    if (!nr)
        for (int k = 0; k < 4; ++k) {
            t[k].xe = y[i++];
            t[k].ye = y[i++];
        }
    for (int k = 0; k < 4; ++k) t[k].omega = y[i++];
    if (tc) v.crankOmega = y[i++];
    v.x = y[i++];
    v.y = y[i++];
    v.u = y[i++];
    v.v = y[i++];
    v.psi = y[i++];
    v.wz = y[i++];
    v.phi = y[i++];
    v.wx = y[i++];
    const double controls[4] = {0.0, ctl[0], ctl[1], ctl[2]};
    rhs(&v, t, pp, controls, nr);
    i = 0;
    if (!nr)
        for (int k = 0; k < 4; ++k) {
            ydot[i++] = t[k].xedot;
            ydot[i++] = t[k].yedot;
        }
    for (int k = 0; k < 4; ++k) ydot[i++] = t[k].dOmega;
    if (tc) ydot[i++] = v.dOmega_crank;
    ydot[i++] = (v.u * cos(v.psi) - v.v * sin(v.psi)); /* computeVehRHS, 18dof/dof18.cpp:1075-1077 */
    ydot[i++] = (v.u * sin(v.psi) + v.v * cos(v.psi));
    ydot[i++] = v.udot;
    ydot[i++] = v.vdot;
    ydot[i++] = v.wz;
    ydot[i++] = v.wzdot;
    ydot[i++] = v.wx;
    ydot[i++] = v.wxdot;
    return i;
}

int oracle18_rhs(const lfdm_class18* cls, const double* params, const double* full_state, const double* y,
                 const double* ctl, double* ydot) {
    Par pp = {params, cls};
    return perturb18(&pp, full_state, y, ctl, ydot, 0);
}

/* half-implicit update: dof18_halfImplicit_gpu.cu:913-946 */
static void update(Veh* v, Tire* t, const Par* pp, double step, int nr) {
    for (int k = 0; k < 4; ++k) {
        if (!nr) {
            t[k].xe += t[k].xedot * step;
            t[k].ye += t[k].yedot * step;
        }
        t[k].omega += t[k].dOmega * step;
    }
    if (pp->c->tcbool) v->crankOmega += v->dOmega_crank * step;
    v->u += v->udot * step;
    v->v += v->vdot * step;
    v->wx += v->wxdot * step;
    v->wz += v->wzdot * step;
    v->x += (v->u * cos(v->psi) - v->v * sin(v->psi)) * step;
    v->y += (v->u * sin(v->psi) + v->v * cos(v->psi)) * step;
    v->psi += v->wz * step;
    v->phi += v->wx * step;
}

static void controls_at(const oracle18_args* a, int i, double t, double* c) {
    if (a->drv_rows) {
        oracle_driver_input(t, a->drv_rows + 4 * a->drv_off[i], a->drv_len[i], c);
    } else {
        c[0] = t;
        c[1] = a->ctl[3 * i + 0];
        c[2] = a->ctl[3 * i + 1];
        c[3] = a->ctl[3 * i + 2];
    }
}

/* one GPU launch window for vehicle i: Integrate, dof18_halfImplicit_gpu.cu:882-977 */
static void window(const oracle18_args* a, int i, Veh* v, Tire* t, const Par* pp, double current_time,
                   int64_t sample_base) {
    const int nr = a->tire_type == LFDM_TIRE_TMEASY_NR;
    const double step = a->dt;
    double tt = current_time;
    double kernel_time = 0;
    int64_t stored = 0;
    const double end_time = (tt + a->ksim) - step / 10.;
    while (tt < end_time) {
        double c[4];
        controls_at(a, i, tt, c);
        rhs(v, t, pp, c, nr);
        update(v, t, pp, step, nr);
        tt += step;
        kernel_time += step;
        if (a->resp && a->dtout > 0) {
            if (fabs(kernel_time - (stored + 1) * a->dtout) < 1e-7) {
                int64_t smp = sample_base + stored;
                if (stored < a->samples_per_window && smp < a->resp_samples) {
                    double* r = a->resp + (size_t)smp * LFDM18_RESP_CHANNELS * a->n;
                    const double ch[LFDM18_RESP_CHANNELS] = {tt,     v->x,  v->y,  v->u,       v->v,
                                                             v->phi, v->psi, v->wx, v->wz,      t[0].omega,
                                                             t[1].omega, t[2].omega, t[3].omega};
                    for (int k = 0; k < LFDM18_RESP_CHANNELS; ++k) r[(size_t)k * a->n + i] = ch[k];
                }
                stored++;
            }
        }
    }
}

static void run_vehicle(const oracle18_args* a, int i) {
    Veh v;
    Tire t[4];
    Par pp = {a->params + (size_t)i * LFDM_P_COUNT, &a->classes[a->class_of[i]]};
    const int nr = a->tire_type == LFDM_TIRE_TMEASY_NR;
    load_state(a->states + (size_t)i * LFDM_S_COUNT, &v, t);
    if (a->schedule == 0) {
        /* d18SolverHalfImplicit::Integrate, 18dof/dof18_halfImplicit.cpp:163-242 */
        double tt = a->t0;
        while (tt < (a->tend - a->dt / 10.)) {
            double c[4];
            controls_at(a, i, tt, c);
            rhs(&v, t, &pp, c, nr);
            update(&v, t, &pp, a->dt, nr);
            tt += a->dt;
        }
    } else if (a->schedule == 1) {
        /* d18SolverHalfImplicitGPU::Solve, dof18_halfImplicit_gpu.cu:438-463 */
        double current_time = a->t0;
        int64_t w = 0;
        while (current_time < a->tend) {
            window(a, i, &v, t, &pp, current_time, w * a->samples_per_window);
            current_time = current_time + a->ksim;
            ++w;
        }
    } else {
        window(a, i, &v, t, &pp, a->t0, 0);
    }
    store_state(a->states + (size_t)i * LFDM_S_COUNT, &v, t);
}

/* ---------------------------------------------------------------------------------------------- */
/* 11-DOF model (11dof-gpu/dof11_gpu.cu, 11dof-gpu/dof11_halfImplicit_gpu.cu). The tire RHS,       */
/* tmxy_combined, driveTorque and the lookups are the same functions as in the 18-DOF model.        */

typedef struct {
    double x, y, u, v, psi, wz, udot, vdot, wzdot, crankOmega, dOmega_crank;
    int current_gr;
} Veh11;

/* computeTireLoads: dof11_gpu.cu:234-252 */
static void computeTireLoads11(double* loads, const Veh11* v, const Par* pp) {
    double huf = P(LFDM_P_R0);
    double hur = P(LFDM_P_R0);
    const double a = P(LFDM_P_A), b = P(LFDM_P_B), m = P(LFDM_P_M), h = P(LFDM_P_H);
    const double muf = P(LFDM_P_MUF), mur = P(LFDM_P_MUR);
    double Z1 = (m * G * b) / (2. * (a + b)) + (muf * G) / 2.;
    double Z2 = ((m * h + muf * huf + mur * hur) * (v->udot - v->wz * v->v)) / (2. * (a + b));
    loads[0] = (Z1 - Z2) > 0. ? (Z1 - Z2) : 0.;
    double Z3 = (m * G * a) / (2. * (a + b)) + (mur * G) / 2.;
    loads[1] = (Z3 + Z2) > 0. ? (Z3 + Z2) : 0.;
}

/* vehToTireTransform: dof11_gpu.cu:41-68 */
static void vehToTireTransform11(Tire* t, const Veh11* v, const double* loads, const Par* pp, double steering) {
    double delta = wheel_angle(pp, steering);
    t[0].fz = loads[0];
    t[0].vsy = v->v + v->wz * P(LFDM_P_A);
    t[0].vsx = v->u * cos(delta) + t[0].vsy * sin(delta);
    t[1].fz = loads[1];
    t[1].vsy = v->v - v->wz * P(LFDM_P_B);
    t[1].vsx = v->u;
}

/* tireToVehTransform: 11dof/dof11.cpp:100-124 — both front forces rotated by the wheel angle and  */
/* stored back, as the GPU twin does too (11dof-gpu/dof11_gpu.cu:98-123, stores at :117-121).       */
static void tireToVehTransform11(Tire* t, const Par* pp, double steering) {
    double delta = wheel_angle(pp, steering);
    double fx = t[0].fx * cos(delta) - t[0].fy * sin(delta);
    double fy = t[0].fx * sin(delta) + t[0].fy * cos(delta);
    t[0].fx = fx;
    t[0].fy = fy;
}

/* differentialSplit: dof11_gpu.cu:276-315 */
static void differentialSplit11(double torque, double max_bias, double speed_rear, double speed_front,
                                double* torque_rear, double* torque_front, int split, int whichWheels) {
    double diff = fabs(speed_rear - speed_front);
    if (split) {
        double bias = 1;
        if (diff > 0.5) bias = max_bias;
        else if (diff > 0.25) bias = 4 * (max_bias - 1) * diff + (2 - max_bias);
        double alpha = bias / (1 + bias);
        double slow = alpha * torque;
        double fast = torque - slow;
        if (fabs(speed_rear) < fabs(speed_front)) {
            *torque_rear = slow;
            *torque_front = fast;
        } else {
            *torque_rear = fast;
            *torque_front = slow;
        }
    } else {
        if (whichWheels) {
            *torque_rear = torque;
            *torque_front = 0;
        } else {
            *torque_rear = 0;
            *torque_front = torque;
        }
    }
}

/* computePowertrainRHS: dof11_gpu.cu:601-745 */
static void powertrainRHS11(Veh11* v, Tire* t, const Par* pp, const double* controls) {
    const lfdm_class18* c = pp->c;
    double torque_t = 0;
    double max_bias = 2;
    const double throttle = controls[2], braking = controls[3];
    if (c->tcbool) {
        int tc_reverse_flow = 0;
        double omega_t = 0.5 * (t[0].omega + t[1].omega);
        double omega_out = omega_t / (c->gearRatios[v->current_gr]);
        double omega_in = v->crankOmega;
        double sr, cf, tr;
        if ((omega_out < 1e-9) || (omega_in < 1e-9)) {
            sr = 0;
            cf = oracle_map_y(&c->CFmap[0][0], c->CFmapSize, sr);
            tr = oracle_map_y(&c->TRmap[0][0], c->TRmapSize, sr);
        } else {
            sr = omega_out / omega_in;
            if (sr > 1.) {
                sr = 1. - (sr - 1.);
                tc_reverse_flow = 1;
            }
            if (sr < 0) sr = 0;
            cf = oracle_map_y(&c->CFmap[0][0], c->CFmapSize, sr);
            tr = oracle_map_y(&c->TRmap[0][0], c->TRmapSize, sr);
        }
        double torque_in = -pow((omega_in / cf), 2);
        if (tc_reverse_flow) torque_in = -torque_in;
        double torque_out;
        if (tc_reverse_flow) torque_out = -torque_in;
        else torque_out = -tr * torque_in;
        torque_t = torque_out / c->gearRatios[v->current_gr];
        if ((v->u - 0) < 1e-9 && (torque_t < 0)) torque_t = 0;
        v->dOmega_crank = (1. / P(LFDM_P_CRANKINERTIA)) * (driveTorque(pp, throttle, v->crankOmega) + torque_in);
        if (omega_out > c->shiftMap[v->current_gr][1]) {
            if (v->current_gr < c->noGears - 1) v->current_gr++;
        } else if (omega_out < c->shiftMap[v->current_gr][0]) {
            if (v->current_gr > 0) v->current_gr--;
        }
    } else {
        v->crankOmega = 0.5 * (t[0].omega + t[1].omega) / c->gearRatios[v->current_gr];
        torque_t = driveTorque(pp, throttle, v->crankOmega) / c->gearRatios[v->current_gr];
        if ((v->u - 0) < 1e-9 && (torque_t < 0)) torque_t = 0;
        if (v->crankOmega > c->shiftMap[v->current_gr][1]) {
            if (v->current_gr < c->noGears - 1) v->current_gr++;
        } else if (v->crankOmega < c->shiftMap[v->current_gr][0]) {
            if (v->current_gr > 0) v->current_gr--;
        }
    }
    differentialSplit11(torque_t, max_bias, t[1].omega, t[0].omega, &t[1].engTor, &t[0].engTor, c->driveType,
                        c->whichWheels);
    const double jw = P(LFDM_P_JW);
    const double brake = P(LFDM_P_MAXBRAKETORQUE) * braking;
    for (int k = 0; k < 2; ++k)
        t[k].dOmega = (1 / jw) * (t[k].engTor + t[k].My - sgn(t[k].omega) * brake - t[k].fx * t[k].rStat);
}

/* computeVehRHS: dof11_gpu.cu:893-909 */
static void vehRHS11(Veh11* v, const Par* pp, const double* fx, const double* fy) {
    double mt = P(LFDM_P_M) + 2 * (P(LFDM_P_MUF) + P(LFDM_P_MUR));
    v->vdot = -v->u * v->wz + (fy[0] + fy[1]) / mt;
    v->udot = v->v * v->wz + (fx[0] + fx[1]) / mt;
    v->wzdot = (P(LFDM_P_A) * fy[0] - P(LFDM_P_B) * fy[1]) / P(LFDM_P_JZ);
}

static void load_state11(const double* s, Veh11* v, Tire* t) {
    v->x = s[LFDM11_S_X];
    v->y = s[LFDM11_S_Y];
    v->u = s[LFDM11_S_U];
    v->v = s[LFDM11_S_V];
    v->psi = s[LFDM11_S_PSI];
    v->wz = s[LFDM11_S_WZ];
    v->udot = s[LFDM11_S_UDOT];
    v->vdot = s[LFDM11_S_VDOT];
    v->wzdot = s[LFDM11_S_WZDOT];
    v->crankOmega = s[LFDM11_S_CRANKOMEGA];
    v->dOmega_crank = s[LFDM11_S_DOMEGA_CRANK];
    v->current_gr = (int)s[LFDM11_S_CURRENT_GR];
    for (int k = 0; k < 2; ++k) memcpy(&t[k], s + LFDM11_S_TIRE0 + k * LFDM_S_TIRE_STRIDE, sizeof(Tire));
}
static void store_state11(double* s, const Veh11* v, const Tire* t) {
    s[LFDM11_S_X] = v->x;
    s[LFDM11_S_Y] = v->y;
    s[LFDM11_S_U] = v->u;
    s[LFDM11_S_V] = v->v;
    s[LFDM11_S_PSI] = v->psi;
    s[LFDM11_S_WZ] = v->wz;
    s[LFDM11_S_UDOT] = v->udot;
    s[LFDM11_S_VDOT] = v->vdot;
    s[LFDM11_S_WZDOT] = v->wzdot;
    s[LFDM11_S_CRANKOMEGA] = v->crankOmega;
    s[LFDM11_S_DOMEGA_CRANK] = v->dOmega_crank;
    s[LFDM11_S_CURRENT_GR] = (double)v->current_gr;
    for (int k = 0; k < 2; ++k) memcpy(s + LFDM11_S_TIRE0 + k * LFDM_S_TIRE_STRIDE, &t[k], sizeof(Tire));
}

/* rhsFun: 11dof-gpu/dof11_halfImplicit_gpu.cu:663-700 */
static void rhs11(Veh11* v, Tire* t, const Par* pp, const double* controls, int nr) {
    double loads[2] = {0., 0.};
    computeTireLoads11(loads, v, pp);
    vehToTireTransform11(t, v, loads, pp, controls[1]);
    if (nr) {
        tireRHS_Nr(&t[0], pp, controls[1]);
        tireRHS_Nr(&t[1], pp, 0);
    } else {
        tireRHS_TM(&t[0], pp, controls[1]);
        tireRHS_TM(&t[1], pp, 0);
    }
    powertrainRHS11(v, t, pp, controls);
    tireToVehTransform11(t, pp, controls[1]);
    double fx[2] = {t[0].fx, t[1].fx};
    double fy[2] = {t[0].fy, t[1].fy};
    vehRHS11(v, pp, fx, fy);
}

/* half-implicit update: 11dof-gpu/dof11_halfImplicit_gpu.cu:863-880 */
static void update11(Veh11* v, Tire* t, const Par* pp, double step, int nr) {
    for (int k = 0; k < 2; ++k) {
        if (!nr) {
            t[k].xe += t[k].xedot * step;
            t[k].ye += t[k].yedot * step;
        }
        t[k].omega += t[k].dOmega * step;
    }
    if (pp->c->tcbool) v->crankOmega += v->dOmega_crank * step;
    v->u += v->udot * step;
    v->v += v->vdot * step;
    v->wz += v->wzdot * step;
    v->x += (v->u * cos(v->psi) - v->v * sin(v->psi)) * step;
    v->y += (v->u * sin(v->psi) + v->v * cos(v->psi)) * step;
    v->psi += v->wz * step;
}

static void window11(const oracle18_args* a, int i, Veh11* v, Tire* t, const Par* pp, double current_time,
                     int64_t sample_base) {
    const int nr = a->tire_type == LFDM_TIRE_TMEASY_NR;
    const double step = a->dt;
    double tt = current_time;
    double kernel_time = 0;
    int64_t stored = 0;
    const double end_time = (tt + a->ksim) - step / 10.;
    while (tt < end_time) {
        double c[4];
        controls_at(a, i, tt, c);
        rhs11(v, t, pp, c, nr);
        update11(v, t, pp, step, nr);
        tt += step;
        kernel_time += step;
        if (a->resp && a->dtout > 0) {
            if (fabs(kernel_time - (stored + 1) * a->dtout) < 1e-7) {
                int64_t smp = sample_base + stored;
                if (stored < a->samples_per_window && smp < a->resp_samples) {
                    double* r = a->resp + (size_t)smp * LFDM11_RESP_CHANNELS * a->n;
                    const double ch[LFDM11_RESP_CHANNELS] = {tt, v->x, v->y, v->u, v->v, v->psi, v->wz,
                                                             t[0].omega, t[1].omega};
                    for (int k = 0; k < LFDM11_RESP_CHANNELS; ++k) r[(size_t)k * a->n + i] = ch[k];
                }
                stored++;
            }
        }
    }
}

static void run_vehicle11(const oracle18_args* a, int i) {
    Veh11 v;
    Tire t[2];
    Par pp = {a->params + (size_t)i * LFDM_P_COUNT, &a->classes[a->class_of[i]]};
    const int nr = a->tire_type == LFDM_TIRE_TMEASY_NR;
    load_state11(a->states + (size_t)i * LFDM11_S_COUNT, &v, t);
    if (a->schedule == 0) {
        /* d11SolverHalfImplicit::Integrate (11dof/dof11_halfImplicit.cpp) */
        double tt = a->t0;
        while (tt < (a->tend - a->dt / 10.)) {
            double c[4];
            controls_at(a, i, tt, c);
            rhs11(&v, t, &pp, c, nr);
            update11(&v, t, &pp, a->dt, nr);
            tt += a->dt;
        }
    } else if (a->schedule == 1) {
        double current_time = a->t0;
        int64_t w = 0;
        while (current_time < a->tend) {
            window11(a, i, &v, t, &pp, current_time, w * a->samples_per_window);
            current_time = current_time + a->ksim;
            ++w;
        }
    } else {
        window11(a, i, &v, t, &pp, a->t0, 0);
    }
    store_state11(a->states + (size_t)i * LFDM11_S_COUNT, &v, t);
}

/* ---------------------------------------------------------------------------------------------- */
/* 24-DOF model (24dof/dof24.cpp, 24dof/dof24_halfImplicit.cpp; GPU twins 24dof-gpu/dof24_gpu.cu    */
/* and 24dof-gpu/dof24_halfImplicit_gpu.cu, identical arithmetic except that the GPU driveTorque   */
/* scales the shared engine map in place under throttleMod). TMeasy tires. Field order of the      */
/* structs below is the reference structs' (24dof-gpu/dof24_gpu.cuh).                              */
typedef struct {
    double x, y, z, u, v, w, psi, wz, phi, wx, theta, wy, udot, vdot, wdot, wxdot, wydot, wzdot, dtheta, dphi,
        dpsi, crankOmega, dOmega_crank;
    int current_gr;
} Veh24;
typedef struct {
    double xe, ye, xedot, yedot, omega, dOmega, xt, dxt, rStat, fx, fy, fz, fxg, fyg, fzg, vgx, vgy, vgz, vsx, vsy,
        vsz, My, engTor;
} Tire24;
typedef struct {
    double xs, xsi, dxs, ls, lsi, us, vs, ws, dus, dvs, dws, uu, vu, wu, duu, dvu, dwu, fxs, fys, fzs, fzd, mx, my,
        mz;
} Sus24;

_Static_assert(sizeof(Tire24) == LFDM24_T_COUNT * sizeof(double), "Tire24 is the flat tire block");
_Static_assert(sizeof(Sus24) == LFDM24_SUS_COUNT * sizeof(double), "Sus24 is the flat suspension block");

static void load_state24(const double* s, Veh24* v, Tire24* t, Sus24* su) {
    memcpy(v, s, LFDM24_S_CURRENT_GR * sizeof(double)); /* the doubles before current_gr */
    v->current_gr = (int)s[LFDM24_S_CURRENT_GR];
    for (int c = 0; c < 4; ++c) {
        memcpy(&t[c], s + LFDM24_S_TIRE0 + c * LFDM24_T_COUNT, sizeof(Tire24));
        memcpy(&su[c], s + LFDM24_S_SUS0 + c * LFDM24_SUS_COUNT, sizeof(Sus24));
    }
}
static void store_state24(double* s, const Veh24* v, const Tire24* t, const Sus24* su) {
    memcpy(s, v, LFDM24_S_CURRENT_GR * sizeof(double));
    s[LFDM24_S_CURRENT_GR] = (double)v->current_gr;
    for (int c = 0; c < 4; ++c) {
        memcpy(s + LFDM24_S_TIRE0 + c * LFDM24_T_COUNT, &t[c], sizeof(Tire24));
        memcpy(s + LFDM24_S_SUS0 + c * LFDM24_SUS_COUNT, &su[c], sizeof(Sus24));
    }
}

/* initializeTireSus: dof24.cpp:34-88 (GPU: dof24_gpu.cu:34-90, called by Initialize) */
static void init_tire_sus24(Veh24* v, Tire24* t, Sus24* su, const double* p) {
    const double a = p[LFDM_P_A], b = p[LFDM_P_B], m = p[LFDM_P_M], ks = p[LFDM_P_KS];
    double weight_split = ((m * G * b) / (2 * (a + b)) + p[LFDM_P_MUF] * G);
    t[0].fz = t[1].fz = weight_split;
    weight_split = ((m * G * a) / (2 * (a + b)) + p[LFDM_P_MUR] * G);
    t[2].fz = t[3].fz = weight_split;
    for (int c = 0; c < 4; ++c) t[c].xt = t[c].fz / p[LFDM_P_KT];
    su[0].xsi = (m * G * b) / (2 * (a + b) * ks);
    su[2].xsi = (m * G * a) / (2 * (a + b) * ks);
    su[1].xsi = su[0].xsi;
    su[3].xsi = su[2].xsi;
    for (int c = 0; c < 4; ++c) su[c].xs = su[c].xsi;
    for (int c = 0; c < 4; ++c) su[c].lsi = p[LFDM_P_H] - (p[LFDM_P_R0] - t[c].xt);
    for (int c = 0; c < 4; ++c) su[c].ls = su[c].lsi;
    for (int c = 0; c < 4; ++c) su[c].wu = v->w;
}

/* vehToSusTransform: dof24.cpp:148-229. Corner signs: LF (-cf/2, +a), RF (+cf/2, +a),           */
/* LR (-cr/2, -b), RR (+cr/2, -b); uses the previous step's accelerations and dxs.                  */
static void vehToSus24(const Veh24* v, Sus24* su, const Par* pp) {
    const double cf = P(LFDM_P_CF), cr = P(LFDM_P_CR), a = P(LFDM_P_A), b = P(LFDM_P_B);
    su[0].us = (-cf * v->wz / 2.) + v->u;
    su[0].vs = a * v->wz + v->v;
    su[0].ws = (cf * v->wx / 2.) - (a * v->wy) + v->w;
    su[1].us = (cf * v->wz / 2.) + v->u;
    su[1].vs = a * v->wz + v->v;
    su[1].ws = (-cf * v->wx / 2.) - (a * v->wy) + v->w;
    su[2].us = (-cr * v->wz / 2.) + v->u;
    su[2].vs = -b * v->wz + v->v;
    su[2].ws = (cr * v->wx / 2.) + b * v->wy + v->w;
    su[3].us = (cr * v->wz / 2.) + v->u;
    su[3].vs = -b * v->wz + v->v;
    su[3].ws = (-cr * v->wx / 2.) + b * v->wy + v->w;
    for (int c = 0; c < 4; ++c) su[c].ls = su[c].lsi - (su[c].xs - su[c].xsi);
    for (int c = 0; c < 4; ++c) su[c].uu = su[c].us - su[c].ls * v->wy;
    for (int c = 0; c < 4; ++c) su[c].vu = su[c].vs + su[c].ls * v->wx;
    su[0].dus = (-cf * v->wzdot) / 2 + v->udot;
    su[0].dvs = a * v->wzdot + v->vdot;
    su[1].dus = (cf * v->wzdot) / 2 + v->udot;
    su[1].dvs = a * v->wzdot + v->vdot;
    su[2].dus = (-cr * v->wzdot) / 2 + v->udot;
    su[2].dvs = -b * v->wzdot + v->vdot;
    su[3].dus = (cr * v->wzdot) / 2 + v->udot;
    su[3].dvs = (-b * v->wzdot) + v->vdot;
    for (int c = 0; c < 4; ++c) {
        su[c].duu = su[c].dus - (-su[c].dxs * v->wy + su[c].ls * v->wydot);
        su[c].dvu = su[c].dvs + (-su[c].dxs * v->wx + su[c].ls * v->wxdot);
    }
}

/* vehToTireTransform: dof24.cpp:313-384. The contact-patch lateral velocity is vgy unrotated. */
static void vehToTire24(const Veh24* v, Tire24* t, const Sus24* su, const Par* pp, double steering) {
    double delta = wheel_angle(pp, steering);
    for (int c = 0; c < 4; ++c) {
        t[c].vgx = cos(v->theta) * (su[c].uu - v->wy * t[c].rStat) +
                   sin(v->theta) * (su[c].wu * cos(v->phi) + sin(v->phi) * (v->wx * t[c].rStat + su[c].vu));
        t[c].vgy = cos(v->phi) * (su[c].vu + v->wx * t[c].rStat) - su[c].wu * sin(v->phi);
    }
    for (int c = 0; c < 2; ++c) {
        t[c].vsy = t[c].vgy;
        t[c].vsx = t[c].vgx * cos(delta) + t[c].vgy * sin(delta);
    }
    for (int c = 2; c < 4; ++c) {
        t[c].vsy = t[c].vgy;
        t[c].vsx = t[c].vgx;
    }
}

/* computeTireRHS (TMeasy): dof24.cpp:827-986. Differs from the 18-DOF tire in the load (fz from */
/* the integrated compression xt) and the loaded radius (divided by cos(theta) cos(phi)).         */
static void tireRHS24(const Veh24* v, Tire24* ts, const Par* pp, double steering) {
    double delta = wheel_angle(pp, steering);
    ts->fz = ts->xt * P(LFDM_P_KT);
    double fz = ts->fz;
    double vsy = ts->vsy;
    double vsx = ts->vsx;
    const double pn = P(LFDM_P_PN), r0 = P(LFDM_P_R0);
    ts->rStat = (r0 - ts->xt) / (cos(v->theta) * cos(v->phi));
    if (fz <= 0) {
        ts->xe = 0;
        ts->ye = 0;
        ts->omega = 0;
        ts->xt = 0;
        ts->rStat = r0;
        ts->fz = 0;
        ts->fx = 0;
        ts->fy = 0;
        ts->My = 0;
        return;
    }
    double r_eff, rdynco;
    if (fz <= P(LFDM_P_FZRDYNCO)) {
        rdynco = InterpL(fz, P(LFDM_P_RDYNCOPN), P(LFDM_P_RDYNCOP2N), pn);
        r_eff = rdynco * r0 + (1. - rdynco) * ts->rStat;
    } else {
        rdynco = P(LFDM_P_RDYNCOCRIT);
        r_eff = rdynco * r0 + (1. - rdynco) * ts->rStat;
    }
    vsx = vsx - (ts->omega * r_eff);
    double vta = r_eff * fabs(ts->omega) + 0.01;
    double sx = -vsx / vta;
    double alpha = atan2(vsy, vta) - delta;
    double sy = -tan(alpha);
    if (fz > P(LFDM_P_PNMAX)) fz = P(LFDM_P_PNMAX);
    double dfx0 = InterpQ(fz, P(LFDM_P_DFX0PN), P(LFDM_P_DFX0P2N), pn);
    double dfy0 = InterpQ(fz, P(LFDM_P_DFY0PN), P(LFDM_P_DFY0P2N), pn);
    double fxm = InterpQ(fz, P(LFDM_P_FXMPN), P(LFDM_P_FXMP2N), pn);
    double fym = InterpQ(fz, P(LFDM_P_FYMPN), P(LFDM_P_FYMP2N), pn);
    double fxs = InterpQ(fz, P(LFDM_P_FXSPN), P(LFDM_P_FXSP2N), pn);
    double fys = InterpQ(fz, P(LFDM_P_FYSPN), P(LFDM_P_FYSP2N), pn);
    double sxm = InterpL(fz, P(LFDM_P_SXMPN), P(LFDM_P_SXMP2N), pn);
    double sym = InterpL(fz, P(LFDM_P_SYMPN), P(LFDM_P_SYMP2N), pn);
    double sxs = InterpL(fz, P(LFDM_P_SXSPN), P(LFDM_P_SXSP2N), pn);
    double sys = InterpL(fz, P(LFDM_P_SYSPN), P(LFDM_P_SYSP2N), pn);
    double hsxn = sxm / (sxm + sym) + (fxm / dfx0) / (fxm / dfx0 + fym / dfy0);
    double hsyn = sym / (sxm + sym) + (fym / dfy0) / (fxm / dfx0 + fym / dfy0);
    double sxn = sx / hsxn;
    double syn = sy / hsyn;
    double sc = hypot(sxn, syn);
    double calpha, salpha;
    if (sc > 0) {
        calpha = sxn / sc;
        salpha = syn / sc;
    } else {
        calpha = sqrt(2.) / 2.;
        salpha = sqrt(2.) / 2.;
    }
    double df0 = hypot(dfx0 * calpha * hsxn, dfy0 * salpha * hsyn);
    double fm = hypot(fxm * calpha, fym * salpha);
    double sm = hypot(sxm * calpha / hsxn, sym * salpha / hsyn);
    double fs = hypot(fxs * calpha, fys * salpha);
    double ss = hypot(sxs * calpha / hsxn, sys * salpha / hsyn);
    double f, fos;
    tmxy_combined(&f, &fos, sc, df0, sm, fm, ss, fs);
    double vx_min = 0., vx_max = 0.;
    ts->My = -sineStep(vta, vx_min, 0., vx_max, 1.) * P(LFDM_P_RR) * fz * ts->rStat * sgn(ts->omega);
    double vtxs = r_eff * fabs(ts->omega) * hsxn + 0.01;
    double vtys = r_eff * fabs(ts->omega) * hsyn + 0.01;
    const double cx = P(LFDM_P_CX), cy = P(LFDM_P_CY), dx = P(LFDM_P_DX), dy = P(LFDM_P_DY);
    ts->xedot = (-vtxs * cx * ts->xe - fos * vsx) / (vtxs * dx + fos);
    ts->yedot = (-vtys * cy * ts->ye - fos * (-sy * vta)) / (vtys * dy + fos);
    double fxdyn = dx * (-vtxs * cx * ts->xe - fos * vsx) / (vtxs * dx + fos) + cx * ts->xe;
    double fydyn = dy * ((-vtys * cy * ts->ye - fos * (-sy * vta)) / (vtys * dy + fos)) + (cy * ts->ye);
    double fxstr = clampd(ts->xe * cx + ts->xedot * dx, -P(LFDM_P_FXMP2N), P(LFDM_P_FXMP2N));
    double fystr = clampd(ts->ye * cy + ts->yedot * dy, -P(LFDM_P_FYMP2N), P(LFDM_P_FYMP2N));
    double weightx = sineStep(fabs(vsx), 1., 1., 1.5, 0.);
    double weighty = sineStep(fabs(-sy * vta), 1., 1., 1.5, 0.);
    ts->fx = weightx * fxstr + (1. - weightx) * fxdyn;
    ts->fy = weighty * fystr + (1. - weighty) * fydyn;
}

/* computeTireRHS, TMeasyNr: 24dof/dof24.cpp:988-1108 (GPU 24dof-gpu/dof24_gpu.cu:990-1119) */
static void tireRHS24_Nr(const Veh24* v, Tire24* ts, const Par* pp, double steering) {
    double delta = wheel_angle(pp, steering);
    ts->fz = ts->xt * P(LFDM_P_KT);
    double fz = ts->fz;
    const double pn = P(LFDM_P_PN), r0 = P(LFDM_P_R0);
    ts->rStat = (r0 - ts->xt) / (cos(v->theta) * cos(v->phi));
    if (fz <= 0) {
        ts->omega = 0;
        ts->xt = 0;
        ts->rStat = r0;
        ts->fx = 0;
        ts->fy = 0;
        ts->fz = 0;
        ts->My = 0;
        return;
    }
    double r_eff, rdynco;
    if (fz <= P(LFDM_P_FZRDYNCO)) {
        rdynco = InterpL(fz, P(LFDM_P_RDYNCOPN), P(LFDM_P_RDYNCOP2N), pn);
        r_eff = rdynco * r0 + (1. - rdynco) * ts->rStat;
    } else {
        rdynco = P(LFDM_P_RDYNCOCRIT);
        r_eff = rdynco * r0 + (1. - rdynco) * ts->rStat;
    }
    tireNr_core(&ts->fx, &ts->fy, &ts->My, fz, r_eff, ts->rStat, ts->omega, ts->vsx, ts->vsy, ts->vsx, delta, pp);
}

/* computeTireCompressionVelocity: dof24.cpp:1122-1150 */
static void tireCompression24(const Veh24* v, Tire24* t, const Sus24* su) {
    for (int c = 0; c < 4; ++c)
        t[c].dxt = t[c].vsz - (cos(v->theta) * (su[c].wu * cos(v->phi) + su[c].vu * sin(v->phi)) -
                               su[c].uu * sin(v->theta));
}

/* computePowertrainRHS: dof24.cpp:1338-1508 (the 18-DOF powertrain on the 24-DOF structs) */
static void powertrain24(Veh24* v, Tire24* t, const Par* pp, const double* controls) {
    const lfdm_class18* c = pp->c;
    double torque_t = 0;
    double max_bias = 2;
    const double throttle = controls[2], braking = controls[3];
    if (c->tcbool) {
        int tc_reverse_flow = 0;
        double omega_t = 0.25 * (t[0].omega + t[1].omega + t[2].omega + t[3].omega);
        double omega_out = omega_t / (c->gearRatios[v->current_gr]);
        double omega_in = v->crankOmega;
        double sr, cf, tr;
        if ((omega_out < 1e-9) || (omega_in < 1e-9)) {
            sr = 0;
            cf = oracle_map_y(&c->CFmap[0][0], c->CFmapSize, sr);
            tr = oracle_map_y(&c->TRmap[0][0], c->TRmapSize, sr);
        } else {
            sr = omega_out / omega_in;
            if (sr > 1.) {
                sr = 1. - (sr - 1.);
                tc_reverse_flow = 1;
            }
            if (sr < 0) sr = 0;
            cf = oracle_map_y(&c->CFmap[0][0], c->CFmapSize, sr);
            tr = oracle_map_y(&c->TRmap[0][0], c->TRmapSize, sr);
        }
        double torque_in = -pow((omega_in / cf), 2);
        if (tc_reverse_flow) torque_in = -torque_in;
        double torque_out;
        if (tc_reverse_flow) torque_out = -torque_in;
        else torque_out = -tr * torque_in;
        torque_t = torque_out / c->gearRatios[v->current_gr];
        /* reference: abs((u - 0) < 1e-9) && (torque_t < 0) — abs() of the comparison's result */
        if ((v->u - 0) < 1e-9 && (torque_t < 0)) torque_t = 0;
        v->dOmega_crank = (1. / P(LFDM_P_CRANKINERTIA)) * (driveTorque(pp, throttle, v->crankOmega) + torque_in);
        if (omega_out > c->shiftMap[v->current_gr][1]) {
            if (v->current_gr < c->noGears - 1) v->current_gr++;
        } else if (omega_out < c->shiftMap[v->current_gr][0]) {
            if (v->current_gr > 0) v->current_gr--;
        }
    } else {
        v->crankOmega =
            0.25 * (t[0].omega + t[1].omega + t[2].omega + t[3].omega) / c->gearRatios[v->current_gr];
        torque_t = driveTorque(pp, throttle, v->crankOmega) / c->gearRatios[v->current_gr];
        if ((v->u - 0) < 1e-9 && (torque_t < 0)) torque_t = 0;
        if (v->crankOmega > c->shiftMap[v->current_gr][1]) {
            if (v->current_gr < c->noGears - 1) v->current_gr++;
        } else if (v->crankOmega < c->shiftMap[v->current_gr][0]) {
            if (v->current_gr > 0) v->current_gr--;
        }
    }
    double torque_front = 0, torque_rear = 0;
    if (c->driveType) {
        torque_front = torque_t * 0.5;
        torque_rear = torque_t * 0.5;
    } else {
        if (c->whichWheels) {
            torque_front = 0;
            torque_rear = torque_t;
        } else {
            torque_front = torque_t;
            torque_rear = 0;
        }
    }
    differentialSplit(torque_front, max_bias, t[0].omega, t[1].omega, &t[0].engTor, &t[1].engTor);
    differentialSplit(torque_rear, max_bias, t[2].omega, t[3].omega, &t[2].engTor, &t[3].engTor);
    const double jw = P(LFDM_P_JW);
    const double brake = P(LFDM_P_MAXBRAKETORQUE) * braking; /* brakeTorque: dof24.h:1484-1486 */
    for (int k = 0; k < 4; ++k)
        t[k].dOmega = (1 / jw) * (t[k].engTor + t[k].My - sgn(t[k].omega) * brake - t[k].fx * t[k].rStat);
}

/* tireToVehTransform: dof24.cpp:459-527 (front forces rotated by the wheel angle and stored back, */
/* then all four expressed in the chassis frame through pitch and roll)                          */
static void tireToVeh24(const Veh24* v, Tire24* t, const Par* pp, double steering) {
    double delta = wheel_angle(pp, steering);
    for (int k = 0; k < 2; ++k) {
        double fx = t[k].fx * cos(delta) - t[k].fy * sin(delta);
        double fy = t[k].fx * sin(delta) + t[k].fy * cos(delta);
        t[k].fx = fx;
        t[k].fy = fy;
    }
    for (int k = 0; k < 4; ++k) {
        t[k].fxg = t[k].fx * cos(v->theta) - t[k].fz * sin(v->theta);
        t[k].fyg = t[k].fx * sin(v->phi) * sin(v->theta) + t[k].fy * cos(v->phi) +
                   t[k].fz * sin(v->phi) * cos(v->theta);
        t[k].fzg = t[k].fx * sin(v->theta) * cos(v->phi) - t[k].fy * sin(v->phi) +
                   t[k].fz * cos(v->phi) * cos(v->theta);
    }
}

/* computeSusRHS: dof24.cpp:1182-1228 (uses the previous step's jacking force fzd and dxs, then   */
/* sets the new dxs)                                                                              */
static void susRHS24(const Veh24* v, const Tire24* t, Sus24* su, const Par* pp) {
    const double theta = v->theta, phi = v->phi;
    const double ks = P(LFDM_P_KS), bs = P(LFDM_P_BS);
    for (int c = 0; c < 4; ++c) {
        const double mu = c < 2 ? P(LFDM_P_MUF) : P(LFDM_P_MUR);
        su[c].dwu = (1 / mu) * (cos(phi) * (cos(theta) * (t[c].fz - mu * G) + sin(theta) * t[c].fx) -
                                sin(phi) * t[c].fy - su[c].fzd - su[c].xs * ks - su[c].dxs * bs -
                                mu * (su[c].vu * v->wx - su[c].uu * v->wy));
    }
    for (int c = 0; c < 4; ++c) su[c].dxs = -su[c].ws + su[c].wu;
}

/* computeForcesThroughSus: dof24.cpp:599-679. The rear-right lateral force omits the cos(theta) */
/* factor of the other three corners (:639 as in the reference; GPU twin dof24_gpu.cu:649).       */
static void forcesThroughSus24(const Veh24* v, const Tire24* t, Sus24* su, const Par* pp) {
    const double ks = P(LFDM_P_KS), bs = P(LFDM_P_BS);
    for (int c = 0; c < 4; ++c) {
        const double mu = c < 2 ? P(LFDM_P_MUF) : P(LFDM_P_MUR);
        su[c].fxs = t[c].fxg + mu * G * sin(v->theta) - mu * su[c].duu + mu * v->wz * su[c].vu -
                    mu * v->wy * su[c].wu;
        if (c < 3)
            su[c].fys = t[c].fyg - mu * G * sin(v->phi) * cos(v->theta) - mu * su[c].dvu + mu * v->wx * su[c].wu -
                        mu * v->wz * su[c].uu;
        else
            su[c].fys = t[c].fyg - mu * G * sin(v->phi) - mu * su[c].dvu + mu * v->wx * su[c].wu -
                        mu * v->wz * su[c].uu;
        su[c].fzs = su[c].xs * ks + su[c].dxs * bs;
    }
    su[1].fzd = (t[1].fyg * t[1].rStat + su[1].fys * su[1].ls + t[0].fyg * t[0].rStat + su[0].fys * su[0].ls -
                 (su[1].fys + su[0].fys) * P(LFDM_P_HRCF)) /
                P(LFDM_P_CF);
    su[0].fzd = -su[1].fzd;
    su[3].fzd = (t[3].fyg * t[3].rStat + su[3].fys * su[3].ls + t[2].fyg * t[2].rStat + su[2].fys * su[2].ls -
                 (su[3].fys + su[2].fys) * P(LFDM_P_HRCR)) /
                P(LFDM_P_CR);
    su[2].fzd = -su[3].fzd;
    for (int c = 0; c < 4; ++c) su[c].mx = su[c].fys * (c < 2 ? P(LFDM_P_HRCF) : P(LFDM_P_HRCR));
    for (int c = 0; c < 4; ++c) su[c].my = -(t[c].fxg * t[c].rStat + su[c].fxs * su[c].ls);
    for (int c = 0; c < 4; ++c) su[c].mz = 0;
}

/* computeVehicleRHS: dof24.cpp:1682-1732 (the global dx, dy that only the Sundials solver reads are */
/* not part of the GPU state and are left out)                                                      */
static void vehRHS24(Veh24* v, const Sus24* su, const Par* pp) {
    const double m = P(LFDM_P_M), a = P(LFDM_P_A), b = P(LFDM_P_B), cf = P(LFDM_P_CF), cr = P(LFDM_P_CR);
    v->udot = v->wz * v->v - v->wy * v->w + (1 / m) * (su[0].fxs + su[1].fxs + su[2].fxs + su[3].fxs) +
              G * sin(v->theta);
    v->vdot = v->wx * v->w - v->wz * v->u + (1 / m) * (su[0].fys + su[1].fys + su[2].fys + su[3].fys) -
              G * sin(v->phi) * cos(v->theta);
    v->wdot = v->wy * v->u - v->wx * v->v +
              (1 / m) * (su[0].fzs + su[1].fzs + su[2].fzs + su[3].fzs + su[0].fzd + su[1].fzd + su[2].fzd +
                         su[3].fzd) -
              G * cos(v->phi) * cos(v->theta);
    v->wxdot = (1 / P(LFDM_P_JX)) * ((su[0].mx + su[1].mx + su[2].mx + su[3].mx) + (su[0].fzs - su[1].fzs) * (cf / 2.) +
                                     (su[2].fzs - su[3].fzs) * (cr / 2.));
    v->wydot = (1 / P(LFDM_P_JY)) *
               ((su[0].my + su[1].my + su[2].my + su[3].my) + (su[2].fzs + su[3].fzs) * b - (su[0].fzs + su[1].fzs) * a);
    v->wzdot = (1 / P(LFDM_P_JZ)) * ((su[0].mz + su[1].mz + su[2].mz + su[3].mz) + (su[0].fys + su[1].fys) * a -
                                     (su[2].fys + su[3].fys) * b + (-su[0].fxs + su[1].fxs) * (cf / 2.) +
                                     (-su[2].fxs + su[3].fxs) * (cr / 2.));
    v->dtheta = v->wy * cos(v->phi) - v->wz * sin(v->phi);
    v->dpsi = (v->wy * sin(v->phi) / cos(v->theta)) + (v->wz * cos(v->phi) / cos(v->theta));
    v->dphi = v->wx + v->wy * sin(v->phi) * tan(v->theta) + v->wz * cos(v->phi) * tan(v->theta);
}

/* rhsFun: 24dof-gpu/dof24_halfImplicit_gpu.cu:728-775 (CPU 24dof/dof24_halfImplicit.cpp:594-650) */
static void rhs24(Veh24* v, Tire24* t, Sus24* su, const Par* pp, const double* controls, int nr) {
    const double steering = controls[1];
    vehToSus24(v, su, pp);
    vehToTire24(v, t, su, pp, steering);
    if (nr) {
        tireRHS24_Nr(v, &t[0], pp, steering);
        tireRHS24_Nr(v, &t[1], pp, steering);
        tireRHS24_Nr(v, &t[2], pp, 0);
        tireRHS24_Nr(v, &t[3], pp, 0);
    } else {
        tireRHS24(v, &t[0], pp, steering);
        tireRHS24(v, &t[1], pp, steering);
        tireRHS24(v, &t[2], pp, 0);
        tireRHS24(v, &t[3], pp, 0);
    }
    tireCompression24(v, t, su);
    powertrain24(v, t, pp, controls);
    tireToVeh24(v, t, pp, steering);
    susRHS24(v, t, su, pp);
    forcesThroughSus24(v, t, su, pp);
    vehRHS24(v, su, pp);
}

/* half-implicit update: 24dof-gpu/dof24_halfImplicit_gpu.cu:1016-1081 (CPU :199-283). Angles use  */
/* the updated body rates, and x, y the updated yaw.                                              */
static void update24(Veh24* v, Tire24* t, Sus24* su, const Par* pp, double step, int nr) {
    for (int k = 0; k < 4; ++k) {
        if (!nr) {
            t[k].xe += t[k].xedot * step;
            t[k].ye += t[k].yedot * step;
        }
        t[k].xt += t[k].dxt * step;
        t[k].omega += t[k].dOmega * step;
    }
    for (int k = 0; k < 4; ++k) {
        su[k].wu += su[k].dwu * step;
        su[k].xs += su[k].dxs * step;
    }
    if (pp->c->tcbool) v->crankOmega += v->dOmega_crank * step;
    v->u += v->udot * step;
    v->v += v->vdot * step;
    v->w += v->wdot * step;
    v->wx += v->wxdot * step;
    v->wy += v->wydot * step;
    v->wz += v->wzdot * step;
    v->dtheta = v->wy * cos(v->phi) - v->wz * sin(v->phi);
    v->dpsi = (v->wy * sin(v->phi) / cos(v->theta)) + (v->wz * cos(v->phi) / cos(v->theta));
    v->dphi = v->wx + v->wy * sin(v->phi) * tan(v->theta) + v->wz * cos(v->phi) * tan(v->theta);
    v->theta += v->dtheta * step;
    v->psi += v->dpsi * step;
    v->phi += v->dphi * step;
    v->x += (v->u * cos(v->psi) - v->v * sin(v->psi)) * step;
    v->y += (v->u * sin(v->psi) + v->v * cos(v->psi)) * step;
}

/* one GPU launch window (Integrate, 24dof-gpu/dof24_halfImplicit_gpu.cu:955-1113) */
static void window24(const oracle18_args* a, int i, Veh24* v, Tire24* t, Sus24* su, const Par* pp,
                     double current_time, int64_t sample_base) {
    const double step = a->dt;
    double tt = current_time;
    double kernel_time = 0;
    int64_t stored = 0;
    const double end_time = (tt + a->ksim) - step / 10.;
    const int nr = a->tire_type == LFDM_TIRE_TMEASY_NR;
    while (tt < end_time) {
        double c[4];
        controls_at(a, i, tt, c);
        rhs24(v, t, su, pp, c, nr);
        update24(v, t, su, pp, step, nr);
        tt += step;
        kernel_time += step;
        if (a->resp && a->dtout > 0) {
            if (fabs(kernel_time - (stored + 1) * a->dtout) < 1e-7) {
                int64_t smp = sample_base + stored;
                if (stored < a->samples_per_window && smp < a->resp_samples) {
                    double* r = a->resp + (size_t)smp * LFDM24_RESP_CHANNELS * a->n;
                    const double ch[LFDM24_RESP_CHANNELS] = {tt,         v->x,       v->y,       v->u,      v->v,
                                                             v->phi,     v->psi,     v->theta,   v->wx,     v->wz,
                                                             v->wy,      t[0].omega, t[1].omega, t[2].omega, t[3].omega};
                    for (int k = 0; k < LFDM24_RESP_CHANNELS; ++k) r[(size_t)k * a->n + i] = ch[k];
                }
                stored++;
            }
        }
    }
}

static void run_vehicle24(const oracle18_args* a, int i) {
    Veh24 v;
    Tire24 t[4];
    Sus24 su[4];
    Par pp = {a->params + (size_t)i * LFDM_P_COUNT, &a->classes[a->class_of[i]]};
    load_state24(a->states + (size_t)i * LFDM24_S_COUNT, &v, t, su);
    if (a->schedule == 0) {
        /* d24SolverHalfImplicit::Integrate, 24dof/dof24_halfImplicit.cpp:188-297 */
        double tt = a->t0;
        const int nr = a->tire_type == LFDM_TIRE_TMEASY_NR;
        while (tt < (a->tend - a->dt / 10.)) {
            double c[4];
            controls_at(a, i, tt, c);
            rhs24(&v, t, su, &pp, c, nr);
            update24(&v, t, su, &pp, a->dt, nr);
            tt += a->dt;
        }
    } else if (a->schedule == 1) {
        double current_time = a->t0;
        int64_t w = 0;
        while (current_time < a->tend) {
            window24(a, i, &v, t, su, &pp, current_time, w * a->samples_per_window);
            current_time = current_time + a->ksim;
            ++w;
        }
    } else {
        window24(a, i, &v, t, su, &pp, a->t0, 0);
    }
    store_state24(a->states + (size_t)i * LFDM24_S_COUNT, &v, t, su);
}

void oracle24_init_state(const double* params, double* state) {
    Veh24 v;
    Tire24 t[4];
    Sus24 su[4];
    load_state24(state, &v, t, su);
    init_tire_sus24(&v, t, su, params);
    store_state24(state, &v, t, su);
}

typedef void (*vehicle_fn)(const oracle18_args*, int);

typedef struct {
    const oracle18_args* a;
    vehicle_fn fn;
    int lo, hi;
} Chunk;

static void* worker(void* p) {
    Chunk* c = (Chunk*)p;
    for (int i = c->lo; i < c->hi; ++i) c->fn(c->a, i);
    return NULL;
}

static int run_all(const oracle18_args* a, vehicle_fn fn) {
    if (!a || a->n < 0 || !a->classes || !a->class_of || !a->params || !a->states) return 1;
    if (!a->drv_rows && !a->ctl) return 1;
    if (a->drv_rows && (!a->drv_off || !a->drv_len)) return 1;
    if (a->schedule != 0 && !(a->ksim > 0)) return 1;
    int nt = a->nthreads < 1 ? 1 : a->nthreads;
    if (nt > a->n) nt = a->n > 0 ? a->n : 1;
    if (nt == 1) {
        for (int i = 0; i < a->n; ++i) fn(a, i);
        return 0;
    }
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * nt);
    Chunk* ch = (Chunk*)malloc(sizeof(Chunk) * nt);
    for (int k = 0; k < nt; ++k) {
        ch[k].a = a;
        ch[k].fn = fn;
        ch[k].lo = (int)((long)a->n * k / nt);
        ch[k].hi = (int)((long)a->n * (k + 1) / nt);
        pthread_create(&th[k], NULL, worker, &ch[k]);
    }
    for (int k = 0; k < nt; ++k) pthread_join(th[k], NULL);
    free(th);
    free(ch);
    return 0;
}

int oracle18_run(const oracle18_args* a) { return run_all(a, run_vehicle); }
int oracle11_run(const oracle18_args* a) { return run_all(a, run_vehicle11); }
int oracle24_run(const oracle18_args* a) { return run_all(a, run_vehicle24); }

/* ---------------------------------------------------------------------------------------------- */
/* PerturbRhsFun of the 11- and 24-DOF solvers and IntegrateStepWithJacobian's central differences  */

/* 11dof/dof11_halfImplicit.cpp:606-667 with packY / packYDOT / unpackY (:769-929) */
static int perturb11(const Par* pp, const double* full_state, const double* y, const double* ctl, double* ydot,
                     int nr) {
    Veh11 v;
    Tire t[2];
    memset(&v, 0, sizeof v);
    memset(t, 0, sizeof t);
    if (full_state) load_state11(full_state, &v, t);
    const int tc = pp->c->tcbool != 0;
    int i = 0;
    if (!nr)
        for (int k = 0; k < 2; ++k) {
            t[k].xe = y[i++];
            t[k].ye = y[i++];
        }
    for (int k = 0; k < 2; ++k) t[k].omega = y[i++];
    if (tc) v.crankOmega = y[i++];
    v.x = y[i++];
    v.y = y[i++];
    v.u = y[i++];
    v.v = y[i++];
    v.psi = y[i++];
    v.wz = y[i++];
    const double controls[4] = {0.0, ctl[0], ctl[1], ctl[2]};
    rhs11(&v, t, pp, controls, nr);
    i = 0;
    if (!nr)
        for (int k = 0; k < 2; ++k) {
            ydot[i++] = t[k].xedot;
            ydot[i++] = t[k].yedot;
        }
    for (int k = 0; k < 2; ++k) ydot[i++] = t[k].dOmega;
    if (tc) ydot[i++] = v.dOmega_crank;
    ydot[i++] = v.u * cos(v.psi) - v.v * sin(v.psi); /* computeVehRHS, 11dof/dof11.cpp:904-905 */
    ydot[i++] = v.u * sin(v.psi) + v.v * cos(v.psi);
    ydot[i++] = v.udot;
    ydot[i++] = v.vdot;
    ydot[i++] = v.wz;
    ydot[i++] = v.wzdot;
    return i;
}

/* 24dof/dof24_halfImplicit.cpp:787-880 with packY / packYDOT / unpackY (:1015-1386). The reference's
   TMeasyNr branch of PerturbRhsFun evaluates default-constructed states without unpacking y (its
   state Jacobian is identically zero); here both branches unpack y. */
static int perturb24(const Par* pp, const double* full_state, const double* y, const double* ctl, double* ydot,
                     int nr) {
    Veh24 v;
    Tire24 t[4];
    Sus24 su[4];
    memset(&v, 0, sizeof v);
    memset(t, 0, sizeof t);
    memset(su, 0, sizeof su);
    if (full_state) load_state24(full_state, &v, t, su);
    const int tc = pp->c->tcbool != 0;
    int i = 0;
    for (int c = 0; c < 4; ++c) {
        if (!nr) {
            t[c].xe = y[i++];
            t[c].ye = y[i++];
        }
        t[c].xt = y[i++];
    }
    for (int c = 0; c < 4; ++c) t[c].omega = y[i++];
    for (int c = 0; c < 4; ++c) {
        su[c].wu = y[i++];
        su[c].xs = y[i++];
    }
    if (tc) v.crankOmega = y[i++];
    v.x = y[i++];
    v.y = y[i++];
    v.u = y[i++];
    v.v = y[i++];
    v.w = y[i++];
    v.wz = y[i++];
    v.wx = y[i++];
    v.wy = y[i++];
    v.psi = y[i++];
    v.phi = y[i++];
    v.theta = y[i++];
    const double controls[4] = {0.0, ctl[0], ctl[1], ctl[2]};
    rhs24(&v, t, su, pp, controls, nr);
    i = 0;
    for (int c = 0; c < 4; ++c) {
        if (!nr) {
            ydot[i++] = t[c].xedot;
            ydot[i++] = t[c].yedot;
        }
        ydot[i++] = t[c].dxt;
    }
    for (int c = 0; c < 4; ++c) ydot[i++] = t[c].dOmega;
    for (int c = 0; c < 4; ++c) {
        ydot[i++] = su[c].dwu;
        ydot[i++] = su[c].dxs;
    }
    if (tc) ydot[i++] = v.dOmega_crank;
    ydot[i++] = (v.u * cos(v.psi) - v.v * sin(v.psi)); /* computeVehicleRHS, 24dof/dof24.cpp:1729-1731 */
    ydot[i++] = (v.u * sin(v.psi) + v.v * cos(v.psi));
    ydot[i++] = v.udot;
    ydot[i++] = v.vdot;
    ydot[i++] = v.wdot;
    ydot[i++] = v.wzdot;
    ydot[i++] = v.wxdot;
    ydot[i++] = v.wydot;
    ydot[i++] = v.dpsi;
    ydot[i++] = v.dphi;
    ydot[i++] = v.dtheta;
    return i;
}

/* packY of a flat state (the same field order as the unpacking above) */
static int pack_state(int model, int nr, int tc, const double* s, double* y) {
    int i = 0;
    if (model == LFDM_MODEL_18) {
        Veh v;
        Tire t[4];
        load_state(s, &v, t);
        if (!nr)
            for (int k = 0; k < 4; ++k) {
                y[i++] = t[k].xe;
                y[i++] = t[k].ye;
            }
        for (int k = 0; k < 4; ++k) y[i++] = t[k].omega;
        if (tc) y[i++] = v.crankOmega;
        const double r[8] = {v.x, v.y, v.u, v.v, v.psi, v.wz, v.phi, v.wx};
        for (int k = 0; k < 8; ++k) y[i++] = r[k];
    } else if (model == LFDM_MODEL_11) {
        Veh11 v;
        Tire t[2];
        load_state11(s, &v, t);
        if (!nr)
            for (int k = 0; k < 2; ++k) {
                y[i++] = t[k].xe;
                y[i++] = t[k].ye;
            }
        for (int k = 0; k < 2; ++k) y[i++] = t[k].omega;
        if (tc) y[i++] = v.crankOmega;
        const double r[6] = {v.x, v.y, v.u, v.v, v.psi, v.wz};
        for (int k = 0; k < 6; ++k) y[i++] = r[k];
    } else {
        Veh24 v;
        Tire24 t[4];
        Sus24 su[4];
        load_state24(s, &v, t, su);
        for (int c = 0; c < 4; ++c) {
            if (!nr) {
                y[i++] = t[c].xe;
                y[i++] = t[c].ye;
            }
            y[i++] = t[c].xt;
        }
        for (int c = 0; c < 4; ++c) y[i++] = t[c].omega;
        for (int c = 0; c < 4; ++c) {
            y[i++] = su[c].wu;
            y[i++] = su[c].xs;
        }
        if (tc) y[i++] = v.crankOmega;
        const double r[11] = {v.x, v.y, v.u, v.v, v.w, v.wz, v.wx, v.wy, v.psi, v.phi, v.theta};
        for (int k = 0; k < 11; ++k) y[i++] = r[k];
    }
    return i;
}

int oracle_rhs(int model, int tire_type, const lfdm_class18* cls, const double* params, const double* full_state,
               const double* y, const double* ctl, double* ydot) {
    Par pp = {params, cls};
    const int nr = tire_type == LFDM_TIRE_TMEASY_NR;
    if (model == LFDM_MODEL_18) return perturb18(&pp, full_state, y, ctl, ydot, nr);
    if (model == LFDM_MODEL_11) return perturb11(&pp, full_state, y, ctl, ydot, nr);
    if (model == LFDM_MODEL_24) return perturb24(&pp, full_state, y, ctl, ydot, nr);
    return -1;
}

/* IntegrateStepWithJacobian's Jacobian block (18dof/dof18_halfImplicit.cpp:356-449; the 11- and
   24-DOF solvers repeat it, 11dof/dof11_halfImplicit.cpp:335-429, 24dof/dof24_halfImplicit.cpp:402-494):
   each packed state perturbed by +-|1e-3 y_i| (1e-3 where that is below 1e-8), steering and throttle
   by +-1e-3 with braking 0. */
int oracle_jacobian_fd(int model, int tire_type, const lfdm_class18* cls, const double* params, const double* state,
                       const double* ctl, int full_point, double* jac_state, double* jac_ctl) {
    enum { MAXY = 40 };
    const int nr = tire_type == LFDM_TIRE_TMEASY_NR;
    double y[MAXY], yp[MAXY], ym[MAXY], dp[MAXY], dm[MAXY];
    const int ny = pack_state(model, nr, cls->tcbool != 0, state, y);
    const double* full = full_point ? state : NULL;
    for (int i = 0; i < ny; ++i) {
        double del = fabs(y[i] * 1e-3);
        if (del < 1e-8) del = 1e-3;
        memcpy(yp, y, sizeof(double) * ny);
        memcpy(ym, y, sizeof(double) * ny);
        yp[i] = yp[i] + del;
        ym[i] = ym[i] - del;
        if (oracle_rhs(model, tire_type, cls, params, full, yp, ctl, dp) != ny) return -1;
        if (oracle_rhs(model, tire_type, cls, params, full, ym, ctl, dm) != ny) return -1;
        for (int j = 0; j < ny; ++j) jac_state[j * ny + i] = (dp[j] - dm[j]) / (2 * del);
    }
    for (int i = 0; i < 2; ++i) {
        double cp[3] = {ctl[0], ctl[1], 0.0}, cm[3] = {ctl[0], ctl[1], 0.0};
        cp[i] = cp[i] + 1e-3;
        cm[i] = cm[i] - 1e-3;
        if (oracle_rhs(model, tire_type, cls, params, full, y, cp, dp) != ny) return -1;
        if (oracle_rhs(model, tire_type, cls, params, full, y, cm, dm) != ny) return -1;
        for (int j = 0; j < ny; ++j) jac_ctl[j * 2 + i] = (dp[j] - dm[j]) / (2 * 1e-3);
    }
    return ny;
}

typedef struct {
    int model, tire_type, full_point, lo, hi, rc;
    const lfdm_class18* cls;
    const double *params, *states, *ctl;
    double *jac_state, *jac_ctl;
} JacChunk;

static void* jac_worker(void* p) {
    JacChunk* c = (JacChunk*)p;
    const int sc = c->model == LFDM_MODEL_18 ? LFDM_S_COUNT : c->model == LFDM_MODEL_11 ? LFDM11_S_COUNT : LFDM24_S_COUNT;
    for (int i = c->lo; i < c->hi; ++i) {
        const double ctl[3] = {c->ctl[3 * i], c->ctl[3 * i + 1], c->ctl[3 * i + 2]};
        if (oracle_jacobian_fd(c->model, c->tire_type, c->cls, c->params + (size_t)i * LFDM_P_COUNT,
                               c->states + (size_t)i * sc, ctl, c->full_point, c->jac_state + (size_t)i * 36 * 36,
                               c->jac_ctl + (size_t)i * 36 * 2) < 0)
            c->rc = 1;
    }
    return NULL;
}

int oracle_jacobian_fd_batch(int model, int tire_type, const lfdm_class18* cls, const double* params,
                             const double* states, const double* ctl, int n, int full_point, int nthreads,
                             double* jac_state, double* jac_ctl) {
    if (n < 0 || !cls || !params || !states || !ctl || !jac_state || !jac_ctl) return 1;
    if (model != LFDM_MODEL_11 && model != LFDM_MODEL_18 && model != LFDM_MODEL_24) return 1;
    int nt = nthreads < 1 ? 1 : nthreads;
    if (nt > n) nt = n > 0 ? n : 1;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * nt);
    JacChunk* ch = (JacChunk*)malloc(sizeof(JacChunk) * nt);
    for (int k = 0; k < nt; ++k) {
        JacChunk c = {model, tire_type, full_point, (int)((long)n * k / nt), (int)((long)n * (k + 1) / nt), 0,
                      cls, params, states, ctl, jac_state, jac_ctl};
        ch[k] = c;
        pthread_create(&th[k], NULL, jac_worker, &ch[k]);
    }
    int rc = 0;
    for (int k = 0; k < nt; ++k) {
        pthread_join(th[k], NULL);
        rc |= ch[k].rc;
    }
    free(th);
    free(ch);
    return rc;
}

