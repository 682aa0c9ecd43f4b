/*
 * ORACLE — test infrastructure only. Nothing in the product links, loads or calls this.
 *
 * CPU restatement (plain C, FP64, no FMA contraction) of the reference's batched half-implicit
 * stepper for the 18-, 11- and 24-DOF models with TMeasy and TMeasyNr tires. The CUDA path is
 * compared against it in tests/ and smoke(); bench.py's CPU-baseline leg times it. It is pinned against the reference's own CPU solvers (oracle/refrun{11,18,24}.cpp,
 * built by `make ref`) through the golden fixtures in tests/golden/.
 */
#ifndef LFDM_ORACLE_H
#define LFDM_ORACLE_H

#include <stdint.h>
#include "../include/lfdm.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int n;                        /* vehicles */
    int tire_type;                /* LFDM_TIRE_TMEASY / LFDM_TIRE_TMEASY_NR */
    const lfdm_class18* classes;  /* class table */
    const int32_t* class_of;      /* [n] class index of each vehicle */
    const double* params;         /* [n][LFDM_P_COUNT] */
    double* states;               /* [n][LFDM_S_COUNT], advanced in place */
    /* controls: driver tables (rows of {t, steering, throttle, braking}) ... */
    const double* drv_rows;       /* concatenated rows, or NULL */
    const int64_t* drv_off;       /* [n] first row of each vehicle's table */
    const int32_t* drv_len;       /* [n] rows of each vehicle's table */
    /* ... or constant per-vehicle controls for the whole window (SolveStep) */
    const double* ctl;            /* [n][3] {steering, throttle, braking}, used when drv_rows == NULL */
    double dt;                    /* integration step */
    double t0;                    /* start time */
    double tend;                  /* end time (schedule 0 and 1) */
    double ksim;                  /* window length (schedule 1 and 2) */
    int schedule;                 /* 0: CPU solver (t from t0 while t < tend - dt/10)
                                     1: GPU Solve (windows from t0 while window start < tend)
                                     2: GPU SolveStep (exactly one window from t0) */
    double dtout;                 /* output interval, <= 0 for none (schedules 1 and 2) */
    double* resp;                 /* [samples][13][n], window w writes samples w*spw ... */
    int64_t resp_samples;         /* capacity in samples */
    int64_t samples_per_window;   /* spw = ceil(ksim / dtout) */
    int nthreads;                 /* host threads (>= 1) */
} oracle18_args;

/* Returns 0 on success, nonzero on bad arguments. */
int oracle18_run(const oracle18_args* a);
/* The 11-DOF model with the same arguments: states [n][LFDM11_S_COUNT], resp [samples][9][n]. */
int oracle11_run(const oracle18_args* a);
/* The 24-DOF model: states [n][LFDM24_S_COUNT], resp [samples][15][n]. */
int oracle24_run(const oracle18_args* a);
/* initializeTireSus (24dof/dof24.cpp:34-88) applied to one flat 24-DOF state, as Initialize does. */
void oracle24_init_state(const double* params, double* state);

/* PerturbRhsFun (18dof/dof18_halfImplicit.cpp:679-745): the 18-DOF right-hand side at the packed
   states y (packY order: {xe, ye} x 4 tires, omega x 4, crank speed with a torque converter, x, y, u,
   v, psi, wz, phi, wx) with ctl {steering, throttle, braking}, into ydot (packYDOT order). The other
   state fields come from full_state [LFDM_S_COUNT] when given, else are those of a freshly
   constructed state (0, first gear), as in the reference. TMeasy tires. Returns the count. */
int oracle18_rhs(const lfdm_class18* cls, const double* params, const double* full_state, const double* y,
                 const double* ctl, double* ydot);

/* PerturbRhsFun of the model (LFDM_MODEL_11/18/24) and tire type: the right-hand side at packed
   states y (the reference's packY order; TMeasyNr tires have no deflection states) into ydot
   (packYDOT order), with the other fields from full_state or a fresh state. Returns the count. */
int oracle_rhs(int model, int tire_type, const lfdm_class18* cls, const double* params, const double* full_state,
               const double* y, const double* ctl, double* ydot);

/* IntegrateStepWithJacobian's central-difference Jacobians at the flat state `state`:
   jac_state [ny][ny] (d ydot_j / d y_i at [j][i]) and jac_ctl [ny][2] (steering, throttle), each
   right-hand side evaluated at a fresh state (full_point 0, as the reference) or on top of `state`
   (full_point 1). Returns ny, or -1. */
int oracle_jacobian_fd(int model, int tire_type, const lfdm_class18* cls, const double* params, const double* state,
                       const double* ctl, int full_point, double* jac_state, double* jac_ctl);

/* oracle_jacobian_fd for n vehicles of one class on nthreads host threads: params [n][LFDM_P_COUNT],
   states [n][state count of the model], ctl [n][3]; jac_state [n][36 * 36] and jac_ctl [n][36 * 2]
   (the first ny * ny and ny * 2 values of each block used). Returns 0, or 1 on bad arguments. */
int oracle_jacobian_fd_batch(int model, int tire_type, const lfdm_class18* cls, const double* params,
                             const double* states, const double* ctl, int n, int full_point, int nthreads,
                             double* jac_state, double* jac_ctl);

/* tireInit (18dof-gpu/dof18_gpu.cu:227-241) on one flat parameter vector. */
void oracle_tire_init(double* params);

/* Driver-table interpolation of one vehicle at time t (utils/utils_gpu.cu:34-56); out[4]. */
void oracle_driver_input(double t, const double* rows, int len, double* out);

/* Map lookup (utils/utils_gpu.cu:60-75) on [n][2] points. */
double oracle_map_y(const double* map, int n, double x);

#ifdef __cplusplus
}
#endif
#endif
