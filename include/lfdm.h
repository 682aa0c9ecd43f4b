/*
 * lfdm.h — C ABI of the GB300-native batched half-implicit vehicle stepper.
 *
 * This is the drop-in boundary for the reference's GPU solver classes
 *   d18SolverHalfImplicitGPU  (18dof-gpu/dof18_halfImplicit_gpu.cuh:15-343)
 *   d11SolverHalfImplicitGPU  (11dof-gpu/dof11_halfImplicit_gpu.cuh:16)
 *   d24SolverHalfImplicitGPU  (24dof-gpu/dof24_halfImplicit_gpu.cuh:15)
 * The reference has no C ABI: its callers compile against those C++ classes. The header-only
 * C++ classes in include/lfdm/ keep the reference's class names, overloads and struct field
 * names and forward every method to the functions below, so an FFI binding (ctypes, cgo, JNI)
 * binds exactly this file.
 *
 * Conventions: every function returns an lfdm_status; on failure lfdm_last_error() returns a
 * message. All pointers are host pointers unless a name ends in _dev. Sizes are in elements.
 * One solver handle per host thread; calls on a handle are serialised by the caller. Every
 * solve call returns after its work (including requested device-to-host copies) has completed.
 */
#ifndef LFDM_H
#define LFDM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------------------------ */
/* Status codes. The reference prints and continues (utils/utils_gpu.cuh:18-25) or exits       */
/* (18dof-gpu/dof18_halfImplicit_gpu.cu:502-507); here every failure is a returned code.        */
typedef enum {
    LFDM_OK = 0,
    LFDM_ERR_ARG = 1,      /* bad argument (null pointer, out-of-range index, size mismatch) */
    LFDM_ERR_IO = 2,       /* file cannot be opened */
    LFDM_ERR_PARSE = 3,    /* malformed JSON or driver table, missing required key */
    LFDM_ERR_CUDA = 4,     /* CUDA runtime error (message carries cudaGetErrorString) */
    LFDM_ERR_STATE = 5,    /* call order violated (e.g. Solve before Construct/Initialize) */
    LFDM_ERR_CAPACITY = 6, /* more vehicles/classes/map points than the solver was sized for */
    LFDM_ERR_NUMERIC = 7,  /* a vehicle produced a non-finite state (see lfdm_get_status_words) */
    LFDM_ERR_NODEVICE = 8  /* no CUDA device / extension not usable */
} lfdm_status;

typedef enum { LFDM_MODEL_11 = 11, LFDM_MODEL_18 = 18, LFDM_MODEL_24 = 24 } lfdm_model;

/* TireType (18dof-gpu/dof18_gpu.cuh:12) */
typedef enum { LFDM_TIRE_TMEASY = 0, LFDM_TIRE_TMEASY_NR = 1 } lfdm_tire_type;

/* Arithmetic of the stepper. FP64 reproduces the reference; MIXED (18-DOF, TMeasy) runs the RHS  */
/* and tire math in FP32 and keeps FP64 in the X/Y/yaw accumulation and the tire slip and         */
/* transport velocities; MIXED_TIRE (11/18/24-DOF, TMeasy and TMeasyNr) runs only the tire core   */
/* (load interpolation, combined slip, force curve, relaxation or Coulomb blend) in FP32 and       */
/* everything else in FP64.                                                                        */
typedef enum { LFDM_PREC_FP64 = 0, LFDM_PREC_MIXED = 1, LFDM_PREC_MIXED_TIRE = 2 } lfdm_precision;

/* ------------------------------------------------------------------------------------------ */
/* Flat per-vehicle parameter vector (doubles). Vehicle part follows VehicleParam               */
/* (18dof-gpu/dof18_gpu.cuh:502-709); tire part is a superset of TMeasyParam (:25-153) and        */
/* TMeasyNrParam (:263-400). Index names drop the leading underscore of the reference fields.    */
enum {
    LFDM_P_A = 0, LFDM_P_B, LFDM_P_H, LFDM_P_M, LFDM_P_JZ, LFDM_P_JX, LFDM_P_JXZ, LFDM_P_CF, LFDM_P_CR,
    LFDM_P_MUF, LFDM_P_MUR, LFDM_P_HRCF, LFDM_P_HRCR, LFDM_P_KROF, LFDM_P_KROR, LFDM_P_BROF, LFDM_P_BROR,
    LFDM_P_MAXSTEER, LFDM_P_CRANKINERTIA, LFDM_P_MAXBRAKETORQUE,
    /* tire block */
    LFDM_P_JW = 20, LFDM_P_RR, LFDM_P_MU, LFDM_P_R0, LFDM_P_PN, LFDM_P_PNMAX, LFDM_P_CX, LFDM_P_CY, LFDM_P_KT,
    LFDM_P_DX, LFDM_P_DY, LFDM_P_RDYNCOPN, LFDM_P_RDYNCOP2N, LFDM_P_FZRDYNCO, LFDM_P_RDYNCOCRIT,
    LFDM_P_DFX0PN, LFDM_P_DFX0P2N, LFDM_P_FXMPN, LFDM_P_FXMP2N, LFDM_P_FXSPN, LFDM_P_FXSP2N, LFDM_P_SXMPN,
    LFDM_P_SXMP2N, LFDM_P_SXSPN, LFDM_P_SXSP2N, LFDM_P_DFY0PN, LFDM_P_DFY0P2N, LFDM_P_FYMPN, LFDM_P_FYMP2N,
    LFDM_P_FYSPN, LFDM_P_FYSP2N, LFDM_P_SYMPN, LFDM_P_SYMP2N, LFDM_P_SYSPN, LFDM_P_SYSP2N,
    /* TMeasyNr-only fields */
    LFDM_P_WIDTH, LFDM_P_RIM_RADIUS, LFDM_P_VCOULOMB, LFDM_P_FRBLEND_BEGIN, LFDM_P_FRBLEND_END,
    LFDM_P_BEARINGCAPACITY, LFDM_P_LI, LFDM_P_P_LI, LFDM_P_P_USE,
    /* 24-DOF only: pitch inertia (24dof-gpu/dof24_gpu.cuh VehicleParam::_jy) and the suspension  */
    /* spring stiffness and damping (SuspensionParam::_ks, _bs)                                   */
    LFDM_P_JY, LFDM_P_KS, LFDM_P_BS,
    LFDM_P_COUNT /* = 67 */
};

/* Per-class data shared by all vehicles built from one vehicle JSON: flags, gears and maps.     */
/* Map x units are those the reference stores after loading (rad/s for engine/shift maps,        */
/* dof18_gpu.cu:1132-1174). Maps hold at most LFDM_MAX_MAP points, gears LFDM_MAX_GEARS.          */
#define LFDM_MAX_MAP 32
#define LFDM_MAX_GEARS 16
typedef struct {
    int32_t nonLinearSteer, tcbool, throttleMod, driveType, whichWheels;
    int32_t noGears, steerMapSize, powertrainMapSize, lossesMapSize, CFmapSize, TRmapSize, pad_;
    double gearRatios[LFDM_MAX_GEARS];
    double shiftMap[LFDM_MAX_GEARS][2];       /* [gear] = {downshift, upshift} rad/s */
    double steerMap[LFDM_MAX_MAP][2];         /* {normalised input, wheel angle} */
    double powertrainMap[LFDM_MAX_MAP][2];    /* {crank rad/s, torque N m} */
    double lossesMap[LFDM_MAX_MAP][2];        /* {crank rad/s, loss torque N m} */
    double CFmap[LFDM_MAX_MAP][2];            /* {speed ratio, capacity factor} */
    double TRmap[LFDM_MAX_MAP][2];            /* {speed ratio, torque ratio} */
} lfdm_class18;

/* Flat per-vehicle state vector (doubles), 18-DOF. Field order follows VehicleState            */
/* (dof18_gpu.cuh:719-810) then 4 x TMeasyState (:164-253) in LF, RF, LR, RR order. current_gr is */
/* stored as a double holding an integer. TMeasyNr vehicles leave xe, ye, xedot, yedot at 0.      */
enum {
    LFDM_S_X = 0, LFDM_S_Y, LFDM_S_U, LFDM_S_V, LFDM_S_PSI, LFDM_S_WZ, LFDM_S_PHI, LFDM_S_WX,
    LFDM_S_UDOT, LFDM_S_VDOT, LFDM_S_WXDOT, LFDM_S_WZDOT, LFDM_S_CRANKOMEGA, LFDM_S_DOMEGA_CRANK,
    LFDM_S_CURRENT_GR,
    LFDM_S_TIRE0 = 15, /* tire k starts at LFDM_S_TIRE0 + k*LFDM_S_TIRE_STRIDE */
    LFDM_S_TIRE_STRIDE = 15,
    LFDM_S_COUNT = 75
};
enum { /* offsets inside one tire block */
    LFDM_T_XE = 0, LFDM_T_YE, LFDM_T_XEDOT, LFDM_T_YEDOT, LFDM_T_OMEGA, LFDM_T_DOMEGA, LFDM_T_XT, LFDM_T_RSTAT,
    LFDM_T_FX, LFDM_T_FY, LFDM_T_FZ, LFDM_T_VSX, LFDM_T_VSY, LFDM_T_MY, LFDM_T_ENGTOR
};

/* Flat per-vehicle state vector, 11-DOF: VehicleState (11dof-gpu/dof11_gpu.cuh:704-765) then      */
/* TMeasyState of the front and the rear tire (same 15-field block as the 18-DOF model).            */
enum {
    LFDM11_S_X = 0, LFDM11_S_Y, LFDM11_S_U, LFDM11_S_V, LFDM11_S_PSI, LFDM11_S_WZ, LFDM11_S_UDOT, LFDM11_S_VDOT,
    LFDM11_S_WZDOT, LFDM11_S_CRANKOMEGA, LFDM11_S_DOMEGA_CRANK, LFDM11_S_CURRENT_GR,
    LFDM11_S_TIRE0 = 12, /* front tire block; rear tire at LFDM11_S_TIRE0 + LFDM_S_TIRE_STRIDE */
    LFDM11_S_COUNT = 42
};
/* Flat per-vehicle state vector, 24-DOF: VehicleState (24dof-gpu/dof24_gpu.cuh), then 4 x        */
/* TMeasyState (23 fields) and 4 x SuspensionState (24 fields), LF, RF, LR, RR, in the field order */
/* of the reference structs. current_gr is stored as a double holding an integer.                  */
enum {
    LFDM24_S_X = 0, LFDM24_S_Y, LFDM24_S_Z, LFDM24_S_U, LFDM24_S_V, LFDM24_S_W, LFDM24_S_PSI, LFDM24_S_WZ,
    LFDM24_S_PHI, LFDM24_S_WX, LFDM24_S_THETA, LFDM24_S_WY, LFDM24_S_UDOT, LFDM24_S_VDOT, LFDM24_S_WDOT,
    LFDM24_S_WXDOT, LFDM24_S_WYDOT, LFDM24_S_WZDOT, LFDM24_S_DTHETA, LFDM24_S_DPHI, LFDM24_S_DPSI,
    LFDM24_S_CRANKOMEGA, LFDM24_S_DOMEGA_CRANK, LFDM24_S_CURRENT_GR,
    LFDM24_S_TIRE0 = 24, /* tire k at LFDM24_S_TIRE0 + k * LFDM24_T_COUNT */
    LFDM24_S_SUS0 = 116, /* suspension k at LFDM24_S_SUS0 + k * LFDM24_SUS_COUNT */
    LFDM24_S_COUNT = 212
};
enum { /* TMeasyState of the 24-DOF model (24dof-gpu/dof24_gpu.cuh) */
    LFDM24_T_XE = 0, LFDM24_T_YE, LFDM24_T_XEDOT, LFDM24_T_YEDOT, LFDM24_T_OMEGA, LFDM24_T_DOMEGA, LFDM24_T_XT,
    LFDM24_T_DXT, LFDM24_T_RSTAT, LFDM24_T_FX, LFDM24_T_FY, LFDM24_T_FZ, LFDM24_T_FXG, LFDM24_T_FYG,
    LFDM24_T_FZG, LFDM24_T_VGX, LFDM24_T_VGY, LFDM24_T_VGZ, LFDM24_T_VSX, LFDM24_T_VSY, LFDM24_T_VSZ,
    LFDM24_T_MY, LFDM24_T_ENGTOR,
    LFDM24_T_COUNT = 23
};
enum { /* SuspensionState (24dof-gpu/dof24_gpu.cuh) */
    LFDM24_SUS_XS = 0, LFDM24_SUS_XSI, LFDM24_SUS_DXS, LFDM24_SUS_LS, LFDM24_SUS_LSI, LFDM24_SUS_US,
    LFDM24_SUS_VS, LFDM24_SUS_WS, LFDM24_SUS_DUS, LFDM24_SUS_DVS, LFDM24_SUS_DWS, LFDM24_SUS_UU, LFDM24_SUS_VU,
    LFDM24_SUS_WU, LFDM24_SUS_DUU, LFDM24_SUS_DVU, LFDM24_SUS_DWU, LFDM24_SUS_FXS, LFDM24_SUS_FYS,
    LFDM24_SUS_FZS, LFDM24_SUS_FZD, LFDM24_SUS_MX, LFDM24_SUS_MY, LFDM24_SUS_MZ,
    LFDM24_SUS_COUNT = 24
};
/* 24-DOF response channels (24dof-gpu/dof24_halfImplicit_gpu.cu:1086-1106): time, x, y, u, v,      */
/* phi (roll), psi (yaw), theta (pitch), wx, wz, wy, wheel speeds LF, RF, LR, RR.                    */
#define LFDM24_RESP_CHANNELS 15

/* 11-DOF response channels (11dof-gpu/dof11_halfImplicit_gpu.cu:893-904): time, x, y, u, v, psi, wz, */
/* front wheel speed, rear wheel speed.                                                              */
#define LFDM11_RESP_CHANNELS 9

/* Response channels written every output sample, in this order (dof18_halfImplicit_gpu.cu:954-974): */
/* time, x, y, u(vx), v(vy), phi(roll), psi(yaw), wx(roll rate), wz(yaw rate), wlf, wrf, wlr, wrr.  */
#define LFDM18_RESP_CHANNELS 13

/* Driver table row = DriverInput (utils/utils_gpu.cuh:28-41): {time, steering, throttle, braking}. */
#define LFDM_DRIVER_COLS 4

/* ------------------------------------------------------------------------------------------ */
typedef struct lfdm_solver lfdm_solver;

/* ctor d18SolverHalfImplicitGPU(unsigned total_num_vehicles) (dof18_halfImplicit_gpu.cu:14-37). */
/* Device 0 is used, as in the reference (:35-36); lfdm_create_on_device picks another.         */
int lfdm_create(int model, unsigned total_num_vehicles, lfdm_solver** out);
int lfdm_create_on_device(int model, unsigned total_num_vehicles, int device, lfdm_solver** out);
/* ~d18SolverHalfImplicitGPU (:38-50) */
int lfdm_destroy(lfdm_solver* h);
/* Message of the last failing call on h (or of the last failing lfdm_create when h is NULL). */
const char* lfdm_last_error(const lfdm_solver* h);

/* Construct(veh, tire, n, driver[, TireType]) and Construct(veh, tire, n[, TireType])          */
/* (dof18_halfImplicit_gpu.cu:53-285). sus_json is the 24-DOF suspension file                  */
/* (24dof-gpu/dof24_halfImplicit_gpu.cu:53-57), NULL otherwise. driver_file may be NULL (vehicles */
/* then need SolveStep controls). Each call appends n vehicles of one new parameter class.        */
int lfdm_construct(lfdm_solver* h, const char* veh_json, const char* tire_json, const char* sus_json,
                   unsigned num_vehicles, const char* driver_file, int tire_type);

/* Extension (replaces writing the reference's public m_sim_data[i] members directly):          */
/* append n vehicles of a class given as data. params is [n][LFDM_P_COUNT]; the tire block must   */
/* already hold fzRdynco/rdyncoCrit (tireInit, dof18_gpu.cu:227-241) or lfdm_tire_init fills it.  */
int lfdm_construct_class(lfdm_solver* h, const lfdm_class18* cls, unsigned num_vehicles, const double* params,
                         int tire_type);
/* Overwrite parameters of vehicles [first, first+count), [count][LFDM_P_COUNT]. */
int lfdm_set_params(lfdm_solver* h, unsigned first, unsigned count, const double* params);
int lfdm_get_params(lfdm_solver* h, unsigned first, unsigned count, double* params);
/* tireInit (dof18_gpu.cu:227-241) applied to one flat parameter vector in place. */
int lfdm_tire_init(double* params);

/* Driver tables. One table shared by vehicles [first, first+count) (rows: [nrows][4]), or one    */
/* table per vehicle with equal row counts (rows: [count][nrows][4]). Times must be              */
/* non-decreasing. Replaces the per-vehicle managed copies of dof18_halfImplicit_gpu.cu:84-94.    */
int lfdm_set_driver_table(lfdm_solver* h, unsigned first, unsigned count, const double* rows, unsigned nrows);
int lfdm_set_driver_tables(lfdm_solver* h, unsigned first, unsigned count, const double* rows, unsigned nrows);

/* Initialize(VehicleState&, TMeasyState& x4, n) (dof18_halfImplicit_gpu.cu:290-313): copy one    */
/* flat state [LFDM_S_COUNT] to the next n vehicles.                                              */
int lfdm_initialize(lfdm_solver* h, const double* state, unsigned num_vehicles);
/* Per-vehicle states [count][LFDM_S_COUNT] (extension; GetSimState reads one, :667-682). */
int lfdm_set_states(lfdm_solver* h, unsigned first, unsigned count, const double* states);
int lfdm_get_states(lfdm_solver* h, unsigned first, unsigned count, double* states);

/* Setters of dof18_halfImplicit_gpu.cuh:93-110. */
int lfdm_set_time_step(lfdm_solver* h, double step);
int lfdm_set_end_time(lfdm_solver* h, double tend);
int lfdm_set_kernel_sim_time(lfdm_solver* h, double time);
int lfdm_set_host_dump_time(lfdm_solver* h, double time);
int lfdm_set_threads_per_block(lfdm_solver* h, unsigned threads);
int lfdm_get_step(lfdm_solver* h, double* step);
int lfdm_get_end_time(lfdm_solver* h, double* tend);
int lfdm_get_tire_type(lfdm_solver* h, int* tire_type);
int lfdm_get_num_vehicles(lfdm_solver* h, unsigned* total, unsigned* constructed, unsigned* initialized);
/* Extension: arithmetic of the stepper (default LFDM_PREC_FP64). */
int lfdm_set_precision(lfdm_solver* h, int precision);

/* SetOutput(file, freq, store_all=false, no_outs=50) (dof18_halfImplicit_gpu.cu:342-399):       */
/* per-vehicle CSV files <file>_<idx>.csv written by Solve, byte-compatible with the reference.   */
int lfdm_set_output(lfdm_solver* h, const char* output_file, double output_freq, int store_all,
                    unsigned no_outs);
/* Extension: stream the SoA response [sample][channels][N] of Solve into caller memory instead  */
/* of (or as well as) CSV files. dst holds capacity doubles; Solve fails with LFDM_ERR_CAPACITY   */
/* when the run needs more. Page-locked dst (cudaHostRegister'ed by lfdm_register_host) lets the  */
/* copies overlap the next window's compute. Sample k (k >= 1) is the state at t = k/output_freq.  */
int lfdm_set_response_buffer(lfdm_solver* h, double* dst, size_t capacity, double output_freq);
int lfdm_response_samples(lfdm_solver* h, size_t* samples_written);
int lfdm_register_host(void* ptr, size_t bytes);
int lfdm_unregister_host(void* ptr);

/* Extension: like lfdm_set_response_buffer, but dst is device memory of the solver's GPU and the   */
/* stepping kernel writes samples straight into it (no copy). capacity (doubles) must hold a whole */
/* number of windows (samples per window = ceil(kernel_sim_time * output_freq)); samples wrap.      */
int lfdm_set_response_device(lfdm_solver* h, double* dst_dev, size_t capacity, double output_freq);

/* Solve() (dof18_halfImplicit_gpu.cu:404-494): integrate all vehicles from t = 0 to end time in */
/* windows of kernel_sim_time.                                                                     */
int lfdm_solve(lfdm_solver* h);
/* Extension: the part of Solve() whose windows start in [t_begin, t_end): window starts are      */
/* 0, k, 2k, ... (k = kernel_sim_time) exactly as in Solve, so consecutive ranges reproduce one     */
/* Solve() call; lfdm_solve(h) == lfdm_solve_range(h, 0, end time) plus CSV output.                */
int lfdm_solve_range(lfdm_solver* h, double t_begin, double t_end);
/* SolveStep(t, steering, throttle, braking) (:497-550): one window with constant controls;       */
/* *t_out receives t + kernel_sim_time.                                                            */
int lfdm_solve_step(lfdm_solver* h, double t, double steering, double throttle, double braking, double* t_out);
/* Extension: one window with per-vehicle constant controls, arrays of total_num_vehicles.        */
int lfdm_solve_step_controls(lfdm_solver* h, double t, const double* steering, const double* throttle,
                             const double* braking, double* t_out);

/* GetSimState(i) (dof18_halfImplicit_gpu.cu:667-682) as a flat state vector. */
int lfdm_get_sim_state(lfdm_solver* h, unsigned vehicle_index, double* state);

/* Per-vehicle status words after the last solve: bit 0 = non-finite state seen. */
int lfdm_get_status_words(lfdm_solver* h, unsigned first, unsigned count, uint32_t* words);

/* Device time in milliseconds of the last lfdm_solve / lfdm_solve_step* call's stepping kernels  */
/* (CUDA events on the solver's stream), and how many stepping kernels it launched.               */
int lfdm_last_kernel_ms(lfdm_solver* h, double* ms, unsigned* launches);

/* Library build information (arch, version). */
const char* lfdm_version(void);

/* Measurement helper (no counterpart in the reference): FP64 fused-multiply-add instruction rate of */
/* a device, measured with a throughput kernel (the FP64 issue roofline of the stepping kernel).     */
int lfdm_measure_fp64_peak(int device, double* dfma_per_s);
/* The same probe with the SM clock it ran at (GHz, from the SM clock counter over the global       */
/* nanosecond timer), which normalises the rate to DFMA per clock per SM.                          */
int lfdm_measure_fp64_peak_clock(int device, double* dfma_per_s, double* sm_ghz);
/* The same probe on FP32 FMA chains: lane FFMA per second and the SM clock it ran at (the FP32     */
/* issue roofline of the mixed-precision steppers).                                                */
int lfdm_measure_fp32_peak_clock(int device, double* ffma_per_s, double* sm_ghz);

/* Host-only utilities (no device needed). setVehParamsJSON + setTireParamsJSON + tireInit        */
/* (dof18_gpu.cu:1075-1330, :227-241) into a class record and a flat parameter vector, and        */
/* LoadDriverData (utils/utils_gpu.cu:7-31) into rows [capacity_rows][4].                          */
int lfdm_parse_vehicle18(const char* veh_json, const char* tire_json, int tire_type, lfdm_class18* cls,
                         double* params, char* err, size_t err_len);
int lfdm_load_driver_file(const char* path, double* rows, unsigned capacity_rows, unsigned* nrows, char* err,
                          size_t err_len);
/* The loaders of any model: 11 (11dof-gpu/dof11_gpu.cu:910-1099), 18, or 24 with its suspension   */
/* file (24dof-gpu/dof24_gpu.cu setVehParamsJSON/setTireParamsJSON/setSuspensionParamsJSON).       */
int lfdm_parse_vehicle(int model, const char* veh_json, const char* tire_json, const char* sus_json, int tire_type,
                       lfdm_class18* cls, double* params, char* err, size_t err_len);

/* Extension: one window whose controls follow a per-step schedule shared by all vehicles          */
/* (ctl: [nsteps][3] {steering, throttle, braking}), the C-ABI form of the reference's functor      */
/* SolveStep (dof18_halfImplicit_gpu.cuh:234-287): the C++ header evaluates the functor at the      */
/* window's step times and passes the schedule. ctl_on_device says whether ctl is a device pointer. */
/* Fails with LFDM_ERR_ARG when nsteps differs from the window's step count (lfdm_window_steps).    */
int lfdm_solve_step_schedule(lfdm_solver* h, double t, const double* ctl, unsigned nsteps, int ctl_on_device,
                             double* t_out);
/* Step count and step start times of the window starting at t (times: [capacity] or NULL). */
int lfdm_window_steps(lfdm_solver* h, double t, unsigned* nsteps, double* times, unsigned capacity);

/* ------------------------------------------------------------------------------------------ */
/* Differentiable 18-DOF rollout (no counterpart in the reference; its Sundials solver offers     */
/* forward sensitivities for map parameters only, 18dof/dof18_sundials.h:42-49). nsteps FP64       */
/* steps of dt from the solver's current states (unchanged) with per-step controls ctl            */
/* [nsteps][3][N] = {steering, throttle, braking} (DEVICE pointers, row stride N); per vehicle      */
/* loss[N] = sum over steps of e_lat^2 + e_head^2 + weight_u*|u_k|^2 on the state after each step, */
/* e_lat = -(x - xr) sin(psir) + (y - yr) cos(psir), e_head = psi - psir, ref [nsteps][3][N] =    */
/* {xr, yr, psir}. The forward stores a checkpoint every ckpt_every steps and the last segment's   */
/* step tape; the backward (same arguments) recomputes each earlier segment and runs the           */
/* hand-written adjoint of the step: grad_ctl                                                      */
/* [nsteps][3][N], grad_params [5][N] (mass, Jz, CG-to-front distance a with b held, tire friction */
/* scale on fxmPn..fysP2n at scale 1, tire vertical stiffness kt), grad_state0 [31][N] or NULL     */
/* (adjoint of x, y, u, v, psi, wz, phi, wx, udot, vdot, crank, then xe, ye, xedot, yedot, omega   */
/* of the 4 tires, each block of 4). 18-DOF TMeasy, throttleMod off.                               */
int lfdm_traj18_forward(lfdm_solver* h, const double* ctl, const double* ref, unsigned nsteps, double weight_u,
                        unsigned ckpt_every, double* loss);
int lfdm_traj18_backward(lfdm_solver* h, const double* ctl, const double* ref, unsigned nsteps, double weight_u,
                         unsigned ckpt_every, double* grad_ctl, double* grad_params, double* grad_state0);
/* CUDA-event times of the last forward and backward kernels. */
int lfdm_traj18_last_ms(lfdm_solver* h, double* forward_ms, double* backward_ms);
/* Branch signature of the rollout lfdm_traj18_forward runs with the same controls: per vehicle a   */
/* 64-bit hash of every discrete decision of every step (tire lift-off, tmxy_combined regime, clamps, */
/* sineStep bands, wheel-speed sign, map segments, converter mode and flow direction, gear,          */
/* differential bias bands). Two rollouts whose signatures are equal took the same branches, so a    */
/* central difference between them does not straddle a kink of the loss. ctl [nsteps][3][N] and     */
/* sig [N] are DEVICE arrays. (Extension: test instrumentation for the adjoint's derivative checks.) */
int lfdm_traj18_branch_signature(lfdm_solver* h, const double* ctl, unsigned nsteps, uint64_t* sig);

/* Exact Jacobians of the 18-DOF right-hand side for every vehicle (extension; the reference's GPU  */
/* solver has none, its CPU solver takes central differences: IntegrateStepWithJacobian,           */
/* GetJacobianState, GetJacobianControls, 18dof/dof18_halfImplicit.cpp:356-520). At each vehicle's  */
/* current state and the controls ctl [3][N] (DEVICE, steering/throttle/braking; braking enters no  */
/* derivative): jac_state [ny][ny][N] = d rhs_r / d y_c and jac_ctl [ny][2][N] = d rhs_r /          */
/* d (steering, throttle), DEVICE arrays, in the reference's packed order (packY/packYDOT, :879-1018): */
/* y = {xe, ye} of LF, RF, LR, RR, omega x 4, crank speed (torque converter only), x, y, u, v, psi,  */
/* wz, phi, wx; ny = 21 with a torque converter, 20 without (*ny); with TMeasyNr tires (no          */
/* deflection states) y = omega x 4, crank speed, x, y, u, v, psi, wz, phi, wx and ny = 13 or 12.     */
/* reference_point = 1 differentiates where PerturbRhsFun does (a fresh vehicle state: previous      */
/* accelerations 0, first gear); 0 at the full current state. All vehicles with or all without a    */
/* torque converter.                                                                                */
int lfdm_rhs_jacobian18(lfdm_solver* h, const double* ctl, int reference_point, double* jac_state, double* jac_ctl,
                        int* ny);

/* Exact Jacobians of every model (replaces the Jacobian blocks of 11dof/dof11_halfImplicit.cpp:     */
/* 335-429 and 24dof/dof24_halfImplicit.cpp:402-494 as well): the same call for an 11-, 18- or      */
/* 24-DOF solver, each in its model's packed order (the difference scheme's, below); 11-DOF ny = 13 */
/* / 12 (TMeasy), 9 / 8 (TMeasyNr); 24-DOF TMeasy tires only, ny = 36 / 35.                         */
int lfdm_rhs_jacobian_exact(lfdm_solver* h, const double* ctl, int reference_point, double* jac_state,
                            double* jac_ctl, int* ny);

/* The reference's own Jacobian scheme for every model and tire type, batched over vehicles        */
/* (replaces IntegrateStepWithJacobian's Jacobian block: 11dof/dof11_halfImplicit.cpp:335-429,     */
/* 18dof/dof18_halfImplicit.cpp:356-449, 24dof/dof24_halfImplicit.cpp:402-494): every packed state   */
/* perturbed by +-|1e-3 y_i| (1e-3 where that is below 1e-8), steering and throttle by +-1e-3 with   */
/* braking 0, central differences of PerturbRhsFun. Same arguments and layout as                    */
/* lfdm_rhs_jacobian18, in each model's packed order (packY/packYDOT): 11-DOF {xe, ye} x 2, omega  */
/* x 2, crank, x, y, u, v, psi, wz (ny 13/12 TMeasy, 9/8 TMeasyNr); 18-DOF as above (ny 21/20,     */
/* 13/12); 24-DOF {xe, ye, xt} x 4, omega x 4, {wu, xs} x 4, crank, x, y, u, v, w, wz, wx, wy, psi, */
/* phi, theta (ny 36/35 TMeasy, 28/27 TMeasyNr with xt only). The crank speed is a state only with */
/* a torque converter. The reference's 24-DOF TMeasyNr PerturbRhsFun does not unpack the perturbed  */
/* states (its state Jacobian is zero); this one does.                                              */
int lfdm_rhs_jacobian_fd(lfdm_solver* h, const double* ctl, int reference_point, double* jac_state, double* jac_ctl,
                         int* ny);

/* Either Jacobian with HOST buffers, laid out per vehicle as the reference's CPU solvers return     */
/* them (GetJacobianState / GetJacobianControls): ctl [3][N] = {steering, throttle, braking},       */
/* jac_state [N][ny][ny], jac_ctl [N][ny][2]. exact = 1 selects lfdm_rhs_jacobian_exact (11- and  */
/* 18-DOF), 0 the reference's difference scheme (lfdm_rhs_jacobian_fd). With jac_state and jac_ctl  */
/* both NULL only *ny is set (ny <= 36 for every model). The solver's configuration is checked      */
/* first, so the size query fails (LFDM_ERR_ARG) for a configuration the chosen Jacobian does not  */
/* support, before any buffer is allocated.                                                         */
int lfdm_rhs_jacobian_host(lfdm_solver* h, int exact, const double* ctl, int reference_point, double* jac_state,
                           double* jac_ctl, int* ny);

/* ------------------------------------------------------------------------------------------ */
/* Mixed-DOF fleets (no counterpart class in the reference, whose solvers hold one model and one */
/* end time each: d18SolverHalfImplicitGPU, d24SolverHalfImplicitGPU). A fleet holds 18-DOF and   */
/* 24-DOF TMeasy vehicles of any number of parameter classes, each with its own end time, and      */
/* steps them in one persistent launch (a CUDA graph of one or a few launches). Every vehicle gets */
/* what the reference's Solve() computes for it with m_tend = its end time and the fleet's         */
/* kernel_sim_time (dof18_halfImplicit_gpu.cu:404-494): same step times, steps and output samples. */
typedef struct lfdm_fleet lfdm_fleet;
int lfdm_fleet_create(int device, lfdm_fleet** out);
int lfdm_fleet_destroy(lfdm_fleet* f);
const char* lfdm_fleet_last_error(const lfdm_fleet* f);
/* Appends n vehicles of one model (LFDM_MODEL_18 or LFDM_MODEL_24) and one class: params          */
/* [n][LFDM_P_COUNT], states [n][model's state count], end times [n] (s), driver rows [nrows][4]   */
/* with each vehicle's first row and row count (vehicles may share a table). With rows == NULL the */
/* row offsets index the rows already added by lfdm_fleet_add_rows (tables shared across calls).   */
int lfdm_fleet_add(lfdm_fleet* f, int model, const lfdm_class18* cls, unsigned n, const double* params,
                   const double* states, const double* horizons, const double* rows, size_t nrows,
                   const int64_t* row_off, const int32_t* row_len);
/* Appends driver rows [nrows][4] shared by later lfdm_fleet_add calls; *first_row = their index. */
int lfdm_fleet_add_rows(lfdm_fleet* f, const double* rows, size_t nrows, int64_t* first_row);
int lfdm_fleet_set_time_step(lfdm_fleet* f, double dt);
int lfdm_fleet_set_kernel_sim_time(lfdm_fleet* f, double ksim);
/* Output interval of the device response buffers (0: none); samples as SetOutput's (:342-399). */
int lfdm_fleet_set_output(lfdm_fleet* f, double dtout);
/* Launch configuration: threads per block (32..128), resident blocks per SM (0: as many as fit)  */
/* and steps per launch (0: the whole horizon in one launch).                                      */
int lfdm_fleet_set_launch(lfdm_fleet* f, unsigned threads, unsigned blocks_per_sm, unsigned steps_per_launch);
int lfdm_fleet_get_launch(lfdm_fleet* f, unsigned* threads, unsigned* blocks_per_sm, unsigned* steps_per_launch);
/* Model affinity (default off; lfdm_fleet_tune tries both): the SMs are split between the 18-DOF */
/* and 24-DOF tiles in proportion to their estimated work (steps x per-step cost) and each warp    */
/* drains its SM's home list before it helps with the other. Off: one list of both models' tiles  */
/* by estimated cost. *frac18 receives the 18-DOF share of the work of the prepared fleet (1 before */
/* the first solve or tune).                                                                        */
int lfdm_fleet_set_affinity(lfdm_fleet* f, int on);
/* Arithmetic of the fleet kernel: LFDM_PREC_FP64 (default) or LFDM_PREC_MIXED_TIRE.               */
int lfdm_fleet_set_precision(lfdm_fleet* f, int precision);
int lfdm_fleet_get_affinity(lfdm_fleet* f, int* on, double* frac18);
/* Autotuner: times the candidate configurations on the first pilot_steps steps (states restored) */
/* and keeps the fastest; *best_ms receives its pilot time.                                        */
int lfdm_fleet_tune(lfdm_fleet* f, unsigned pilot_steps, double* best_ms);
/* Steps every vehicle from its current state over its horizon. */
int lfdm_fleet_solve(lfdm_fleet* f);
int lfdm_fleet_last_ms(lfdm_fleet* f, double* ms, unsigned* launches);
int lfdm_fleet_info(lfdm_fleet* f, unsigned* n18, unsigned* n24, long long* total_steps, double* vehicle_steps,
                    unsigned* nsamples);
/* States of one model's vehicles in the order they were added. */
int lfdm_fleet_get_states(lfdm_fleet* f, int model, unsigned first, unsigned count, double* out);
int lfdm_fleet_set_states(lfdm_fleet* f, int model, unsigned first, unsigned count, const double* states);
/* Response of one model, [nsamples][channels][n] in add order (out NULL: only *nsamples). */
int lfdm_fleet_get_response(lfdm_fleet* f, int model, double* out, size_t capacity, unsigned* nsamples);
int lfdm_fleet_get_status_words(lfdm_fleet* f, int model, uint32_t* out);

/* Extension: the 11-DOF model's split-warp window kernel, which runs each vehicle's two tires on two */
/* warps (for fleets too small to fill the GPU, whose time is set by one vehicle's FP64 instruction  */
/* chain; results are bit for bit those of the one-warp kernel). mode -1 (default): used when the    */
/* fleet needs at most 2 blocks of 64 threads per SM; 0: never; 1: always. Other models ignore it.  */
int lfdm_set_split_warps(lfdm_solver* h, int mode);

/* One stepping window run by a kernel the CALLER compiles: the C++ drop-in's SolveStep(t, func)     */
/* with a __device__ functor (18dof-gpu/dof18_halfImplicit_gpu.cuh:234-287, the functor kernels at  */
/* :455-640 and rhsFun at :646-694; include/lfdm/device/functor_window.cuh). begin uploads what has  */
/* changed, clears the status words and describes the device data of the window that starts at t;   */
/* the caller enqueues its kernel on view->stream, then end waits for that stream, marks the device  */
/* states as the current ones and checks the status words (LFDM_ERR_NUMERIC on a non-finite state).  */
/* FP64 only; refused with CSV output set, as SolveStep is. No responses are written.               */
typedef struct {
    int32_t model, tire_type, n, npad, nclasses, nsteps, kcount, pad_;
    double t0, dt;              /* window start and step                                          */
    const double* K;            /* [kcount][npad] derived per-vehicle constants                   */
    const void* classes;        /* [nclasses] device class records (lfdm::ClassDev18)              */
    const int32_t* class_of;    /* [n] class of each vehicle                                       */
    double* S;                  /* [state count][npad] states (SoA), stepped in place              */
    uint32_t* status;           /* [n] status words; bit 0 = the state became non-finite           */
    void* stream;               /* cudaStream_t to enqueue the window on                           */
} lfdm_device_window;
int lfdm_device_window_begin(lfdm_solver* h, double t, lfdm_device_window* view);
int lfdm_device_window_end(lfdm_solver* h, double t, double* t_out);

/* No counterpart in the reference (its solver owns and allocates all of its memory). For callers   */
/* that cannot allocate device memory on their call path (a real-time control loop, a host that    */
/* hands the GPU over with a fixed memory budget): one 18-DOF FP64 window of nsteps steps of dt     */
/* from t0 over n <= LFDM_NOALLOC_MAX_VEHICLES device-resident vehicles of one class, with           */
/* per-vehicle constant controls, that allocates nothing. Its scratch (derived constants, SoA state */
/* and controls, class index and status words, class table) is one static device array of exactly   */
/* LFDM_NOALLOC_SCRATCH_BYTES bytes (18.8 MiB), reserved on every device where the library is        */
/* loaded. params [n][LFDM_P_COUNT], states [n][LFDM_S_COUNT] (in/out) and steering/throttle/braking */
/* [n] are DEVICE pointers; the work is enqueued on `stream` (a cudaStream_t, NULL = legacy default */
/* stream), and the call waits for that stream at the end to read one status word: it returns       */
/* LFDM_ERR_NUMERIC when a vehicle's state became non-finite (the states are still written back).   */
/* Larger n fails with LFDM_ERR_CAPACITY. Every call on a device shares that scratch, so calls that  */
/* overlap on the GPU race: serialise them. err (err_len bytes, may be NULL) receives a message on   */
/* failure.                                                                                          */
#define LFDM_NOALLOC_MAX_VEHICLES 16384
#define LFDM_NOALLOC_SCRATCH_BYTES 19669504
int lfdm_step18_noalloc(const lfdm_class18* cls, int tire_type, const double* params, double* states,
                        const double* steering, const double* throttle, const double* braking, unsigned n, double t0,
                        double dt, unsigned nsteps, void* stream, char* err, size_t err_len);

#ifdef __cplusplus
}
#endif
#endif /* LFDM_H */
