// C++ drop-in layer over liblfdm's C ABI (../lfdm.h). The three model headers beside this one,
// dof11_halfImplicit_gpu.cuh, dof18_halfImplicit_gpu.cuh and dof24_halfImplicit_gpu.cuh, carry the
// names the reference's GPU solver headers export (11dof-gpu/dof11_halfImplicit_gpu.cuh:16,
// 18dof-gpu/dof18_halfImplicit_gpu.cuh:15-343, 24dof-gpu/dof24_halfImplicit_gpu.cuh:15): the
// classes d11/d18/d24SolverHalfImplicitGPU with the same constructor, Construct/Initialize
// overloads, setters, Solve, SolveStep, GetSimState and GetTireType, and the state structs of the
// namespaces d11GPU/d18GPU/d24GPU with the same field names. Code written against the reference
// compiles against these headers (add include/lfdm to the include path) and links with
// -llfdm; every method forwards to one or two lfdm_* calls.
//
// Header-only, plain C++17: a caller compiles with a host compiler, or with nvcc for the device
// functor SolveStep below.
//
// Errors. The reference prints CUDA errors and carries on (utils/utils_gpu.cuh CHECK_CUDA_ERROR),
// asserts (compiled out in Release) or calls exit() (SolveStep with CSV output set). Here every
// failing lfdm_* call prints "lfdm: <method>: <message>" to stderr and the method returns, so a
// program behaves as it did against the reference; define LFDM_CPP_THROW before including to get a
// std::runtime_error instead.
//
// SolveStep(t, func) with a functor (18dof-gpu/dof18_halfImplicit_gpu.cuh:234-287):
//  - compiled with nvcc, the reference's way: a kernel instantiated for the functor's type (in
//    device/functor_window.cuh, over the library's device headers in device/) calls the __device__
//    functor at every step of the window and runs the library's step with those controls, on the
//    solver's stream, over its device states (lfdm_device_window_begin/_end of lfdm.h). Compile
//    with --fmad=false to get the states of the library's own kernels bit for bit.
//  - compiled with a host compiler (or with LFDM_HOST_FUNCTOR defined), the functor is called on
//    the host once per step of the window at the step's start time, and the window runs with that
//    control schedule; its operator() must then be callable on the host.
//
// Differences a caller can see:
//  - The public m_sim_data / m_sim_states arrays are not exposed; parameters and states of
//    individual vehicles are read and written through handle() and the lfdm_get/set_params and
//    lfdm_get/set_states extensions of lfdm.h.
#pragma once

#include <cstddef>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "../lfdm.h"

#if defined(__CUDACC__) && !defined(LFDM_HOST_FUNCTOR)
#define LFDM_DEVICE_FUNCTOR 1
#endif
#if defined(__CUDACC__)
#define LFDM_HD __host__ __device__
#else
#define LFDM_HD
#endif

#ifndef LFDM_TIRE_TYPE_DEFINED
#define LFDM_TIRE_TYPE_DEFINED
// 18dof-gpu/dof18_gpu.cuh:12 (the 11- and 24-DOF headers declare the same enum; here it is
// declared once, so several model headers can be included together).
enum class TireType { TMeasy, TMeasyNr };
#endif

#ifndef LFDM_DRIVER_INPUT_DEFINED
#define LFDM_DRIVER_INPUT_DEFINED
// utils/utils_gpu.cuh:29-40: one row of a driver table, and what a SolveStep functor fills in.
struct DriverInput {
    LFDM_HD DriverInput() : m_time(0), m_steering(0), m_throttle(0), m_braking(0) {}
    LFDM_HD DriverInput(double time, double steering, double throttle, double braking)
        : m_time(time), m_steering(steering), m_throttle(throttle), m_braking(braking) {}
    double m_time;
    double m_steering;
    double m_throttle;
    double m_braking;
};
#endif

#ifdef LFDM_DEVICE_FUNCTOR
#include "device/functor_window.cuh"
#endif

namespace lfdm_cpp {

inline void check(int rc, const lfdm_solver* h, const char* what) {
    if (rc == LFDM_OK) return;
    const char* m = lfdm_last_error(h);
    const std::string msg = std::string(what) + ": " + (m ? m : "error");
#ifdef LFDM_CPP_THROW
    throw std::runtime_error(msg);
#else
    std::fprintf(stderr, "lfdm: %s\n", msg.c_str());
#endif
}

// An argument error found by the wrapper itself, reported like the library's.
inline void check_message(const char* what, const char* msg) {
#ifdef LFDM_CPP_THROW
    throw std::runtime_error(std::string(what) + ": " + msg);
#else
    std::fprintf(stderr, "lfdm: %s: %s\n", what, msg);
#endif
}

inline int tire_code(TireType t) { return t == TireType::TMeasyNr ? LFDM_TIRE_TMEASY_NR : LFDM_TIRE_TMEASY; }

// Copy between a struct's double fields (listed as member pointers, in the struct's field order)
// and a slice of the flat per-vehicle state vector of lfdm.h.
template <typename S, std::size_t N>
inline void put(const S& s, double S::*const (&fields)[N], double* dst) {
    for (std::size_t i = 0; i < N; ++i) dst[i] = s.*fields[i];
}
template <typename S, std::size_t N>
inline void get(S& s, double S::*const (&fields)[N], const double* src) {
    for (std::size_t i = 0; i < N; ++i) s.*fields[i] = src[i];
}

// What the three solver classes share: lifetime, setters, Solve and SolveStep.
template <int Model>
class SolverBase {
  public:
    explicit SolverBase(unsigned int total_num_vehicles) {
        check(lfdm_create(Model, total_num_vehicles, &h_), nullptr, "constructor");
    }
    ~SolverBase() {
        if (h_) lfdm_destroy(h_);
    }
    SolverBase(const SolverBase&) = delete;
    SolverBase& operator=(const SolverBase&) = delete;

    void SetEndTime(double tend) { check(lfdm_set_end_time(h_, tend), h_, "SetEndTime"); }
    void SetTimeStep(double step) { check(lfdm_set_time_step(h_, step), h_, "SetTimeStep"); }
    void SetKernelSimTime(double time) { check(lfdm_set_kernel_sim_time(h_, time), h_, "SetKernelSimTime"); }
    void SetHostDumpTime(double time) { check(lfdm_set_host_dump_time(h_, time), h_, "SetHostDumpTime"); }
    void SetThreadsPerBlock(unsigned int threads) {
        check(lfdm_set_threads_per_block(h_, threads), h_, "SetThreadsPerBlock");
    }
    double GetStep() {
        double v = 0;
        check(lfdm_get_step(h_, &v), h_, "GetStep");
        return v;
    }
    double GetEndTime() {
        double v = 0;
        check(lfdm_get_end_time(h_, &v), h_, "GetEndTime");
        return v;
    }
    void SetOutput(const std::string& output_file, double output_freq, bool store_all = false,
                   unsigned int no_outs = 50) {
        check(lfdm_set_output(h_, output_file.c_str(), output_freq, store_all ? 1 : 0, no_outs), h_, "SetOutput");
    }
    void Solve() { check(lfdm_solve(h_), h_, "Solve"); }
    double SolveStep(double t, double steering, double throttle, double braking) {
        double t_out = t;
        check(lfdm_solve_step(h_, t, steering, throttle, braking, &t_out), h_, "SolveStep");
        return t_out;
    }
    // Functor form (18dof-gpu/dof18_halfImplicit_gpu.cuh:234-287): func(t, DriverInput*) gives the
    // controls at each step start time of the window [t, t + kernel_sim_time); on the device when
    // compiled with nvcc, else on the host (see the top of this file).
    template <typename Func>
    double SolveStep(double t, Func func) {
#ifdef LFDM_DEVICE_FUNCTOR
        lfdm_device_window view;
        int rc = lfdm_device_window_begin(h_, t, &view);
        check(rc, h_, "SolveStep");
        if (rc != LFDM_OK) return t;
        const cudaError_t e = lfdm::launch_functor_window<Model>(view, func);
        if (e != cudaSuccess) check_message("SolveStep", cudaGetErrorString(e));
        double t_out = t;
        check(lfdm_device_window_end(h_, t, &t_out), h_, "SolveStep");
        return t_out;
#else
        unsigned int n = 0;
        check(lfdm_window_steps(h_, t, &n, nullptr, 0), h_, "SolveStep");
        std::vector<double> times(n), ctl(3 * static_cast<std::size_t>(n));
        if (n) check(lfdm_window_steps(h_, t, &n, times.data(), n), h_, "SolveStep");
        for (unsigned int k = 0; k < n; ++k) {
            DriverInput d(times[k], 0.0, 0.0, 0.0);
            func(times[k], &d);
            ctl[3 * k] = d.m_steering;
            ctl[3 * k + 1] = d.m_throttle;
            ctl[3 * k + 2] = d.m_braking;
        }
        double t_out = t;
        check(lfdm_solve_step_schedule(h_, t, ctl.data(), n, 0, &t_out), h_, "SolveStep");
        return t_out;
#endif
    }
    TireType GetTireType() const {
        int t = LFDM_TIRE_TMEASY;
        check(lfdm_get_tire_type(h_, &t), h_, "GetTireType");
        return t == LFDM_TIRE_TMEASY_NR ? TireType::TMeasyNr : TireType::TMeasy;
    }
    // Extension: right-hand-side Jacobians of every vehicle at its current state, each as the
    // reference's CPU solver returns one (GetJacobianState / GetJacobianControls after
    // IntegrateStepWithJacobian): jac_state[i] is vehicle i's ny x ny matrix, jac_controls[i] its ny x 2
    // one, in the packed order. exact: the exact Jacobian (24-DOF: TMeasy tires) instead of the reference's
    // central differences; reference_point: the packed states in a fresh state, as PerturbRhsFun.
    // Controls hold one value per vehicle. Returns ny (0 on error).
    int GetRhsJacobians(const std::vector<double>& steering, const std::vector<double>& throttle,
                        const std::vector<double>& braking,
                        std::vector<std::vector<std::vector<double>>>& jac_state,
                        std::vector<std::vector<std::vector<double>>>& jac_controls, bool exact = false,
                        bool reference_point = true) {
        unsigned int total = 0, constructed = 0, initialized = 0;
        int rc = lfdm_get_num_vehicles(h_, &total, &constructed, &initialized);
        check(rc, h_, "GetRhsJacobians");
        const std::size_t n = total;
        if (rc != LFDM_OK || steering.size() != n || throttle.size() != n || braking.size() != n) {
            if (rc == LFDM_OK) check_message("GetRhsJacobians", "one control value per vehicle is needed");
            return 0;
        }
        int ny = 0;
        rc = lfdm_rhs_jacobian_host(h_, exact ? 1 : 0, nullptr, 0, nullptr, nullptr, &ny);
        check(rc, h_, "GetRhsJacobians");
        if (rc != LFDM_OK) return 0;
        std::vector<double> ctl;
        ctl.reserve(3 * n);
        ctl.insert(ctl.end(), steering.begin(), steering.end());
        ctl.insert(ctl.end(), throttle.begin(), throttle.end());
        ctl.insert(ctl.end(), braking.begin(), braking.end());
        const std::size_t m = static_cast<std::size_t>(ny);
        std::vector<double> js(n * m * m), ju(n * m * 2);
        rc = lfdm_rhs_jacobian_host(h_, exact ? 1 : 0, ctl.data(), reference_point ? 1 : 0, js.data(), ju.data(), &ny);
        check(rc, h_, "GetRhsJacobians");
        if (rc != LFDM_OK) return 0;
        jac_state.assign(n, std::vector<std::vector<double>>(m, std::vector<double>(m)));
        jac_controls.assign(n, std::vector<std::vector<double>>(m, std::vector<double>(2)));
        for (std::size_t i = 0; i < n; ++i)
            for (std::size_t r = 0; r < m; ++r) {
                for (std::size_t c = 0; c < m; ++c) jac_state[i][r][c] = js[(i * m + r) * m + c];
                jac_controls[i][r][0] = ju[(i * m + r) * 2];
                jac_controls[i][r][1] = ju[(i * m + r) * 2 + 1];
            }
        return ny;
    }
    // Extension: the C-ABI handle, for the lfdm_* calls that have no method here (per-vehicle
    // parameters, states and controls, response buffers, precision, timing).
    lfdm_solver* handle() const { return h_; }

  protected:
    void construct(const std::string& veh, const std::string& tire, const std::string* sus, unsigned int n,
                   const std::string* driver, TireType type) {
        check(lfdm_construct(h_, veh.c_str(), tire.c_str(), sus ? sus->c_str() : nullptr, n,
                             driver ? driver->c_str() : nullptr, tire_code(type)),
              h_, "Construct");
    }
    void initialize(const std::vector<double>& flat, unsigned int n) {
        check(lfdm_initialize(h_, flat.data(), n), h_, "Initialize");
    }
    std::vector<double> flat_state(unsigned int i, std::size_t count) {
        std::vector<double> s(count, 0.0);
        check(lfdm_get_sim_state(h_, i, s.data()), h_, "GetSimState");
        return s;
    }

    lfdm_solver* h_ = nullptr;
};

}  // namespace lfdm_cpp
