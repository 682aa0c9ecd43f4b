// Stepping windows driven by a caller's __device__ functor: the kernels behind the C++ drop-in's
// SolveStep(t, func) when the caller is compiled with nvcc (the reference's functor Integrate
// kernels, 18dof-gpu/dof18_halfImplicit_gpu.cuh:455-640, with rhsFun calling func(t, &controls) at
// every step, :646-694; the 11- and 24-DOF solvers have the same pair).
//
// One thread per vehicle, over the device data of lfdm_device_window (lfdm.h): the vehicle's state
// is loaded from the SoA state columns into registers, then for every step of the window
// func(t, &controls) is called with the step's start time and the step of the model runs with those
// controls (the same device functions as the library's own window kernels), and the state is
// stored back. The step times are t0, t0 + dt, ... accumulated in FP64 as the reference's kernel
// and the library's schedule replay do.
//
// Rounding: the library's kernels are compiled with --fmad=false (only the fma() calls written in
// the model code fuse). A caller that compiles with --fmad=false too gets the states of the
// library's own SolveStep paths bit for bit; with contraction on, they agree to rounding level.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

#include "dof11_device.cuh"
#include "dof18_device.cuh"
#include "dof24_device.cuh"

#ifndef LFDM_DRIVER_INPUT_DEFINED
#define LFDM_DRIVER_INPUT_DEFINED
// utils/utils_gpu.cuh:29-40: one row of a driver table, and what a SolveStep functor fills in (the
// same struct as in ../lfdm_solver.hpp, which includes this header under nvcc).
struct DriverInput {
    __host__ __device__ DriverInput() : m_time(0), m_steering(0), m_throttle(0), m_braking(0) {}
    __host__ __device__ DriverInput(double time, double steering, double throttle, double braking)
        : m_time(time), m_steering(steering), m_throttle(throttle), m_braking(braking) {}
    double m_time;
    double m_steering;
    double m_throttle;
    double m_braking;
};
#endif

namespace lfdm {

constexpr int kFunctorThreads = 128;

template <bool kNr, typename Func>
__global__ void __launch_bounds__(kFunctorThreads) functor_window18(const lfdm_device_window w, Func func) {
    const int vid = blockIdx.x * blockDim.x + threadIdx.x;
    if (vid >= w.n) return;
    const KView K{w.K + vid, w.npad};
    const ClassDev18& C = static_cast<const ClassDev18*>(w.classes)[__ldg(w.class_of + vid)];
    const size_t np = (size_t)w.npad;
    double* S = w.S + vid;
    VehC v;
    VehAux va;
    TireC ts[4];
    TireAux ta[4];
    load_state18(S, np, v, va, ts, ta);
    double t = w.t0;
    for (int s = 0; s < w.nsteps; ++s) {
        DriverInput c;
        func(t, &c);
        step18<kNr>(v, va, ts, ta, K, C, c.m_steering, c.m_throttle, c.m_braking, w.dt);
        t += w.dt;
    }
    store_state18(S, np, v, va, ts, ta);
    if (!state18_finite(v, ts)) w.status[vid] |= 1u;
}

template <bool kNr, typename Func>
__global__ void __launch_bounds__(kFunctorThreads) functor_window11(const lfdm_device_window w, Func func) {
    const int vid = blockIdx.x * blockDim.x + threadIdx.x;
    if (vid >= w.n) return;
    const KView K{w.K + vid, w.npad};
    const ClassDev18& C = static_cast<const ClassDev18*>(w.classes)[__ldg(w.class_of + vid)];
    const size_t np = (size_t)w.npad;
    double* S = w.S + vid;
    Veh11 v;
    Veh11Aux va;
    TireC ts[2];
    TireAux ta[2];
    load_state11(S, np, v, va, ts, ta);
    double t = w.t0;
    for (int s = 0; s < w.nsteps; ++s) {
        DriverInput c;
        func(t, &c);
        step11<kNr>(v, va, ts, ta, K, C, c.m_steering, c.m_throttle, c.m_braking, w.dt);
        t += w.dt;
    }
    store_state11(S, np, v, va, ts, ta);
    if (!state11_finite(v, ts)) w.status[vid] |= 1u;
}

template <bool kNr, typename Func>
__global__ void __launch_bounds__(kFunctorThreads) functor_window24(const lfdm_device_window w, Func func) {
    const int vid = blockIdx.x * blockDim.x + threadIdx.x;
    if (vid >= w.n) return;
    const KView K{w.K + vid, w.npad};
    const ClassDev18& C = static_cast<const ClassDev18*>(w.classes)[__ldg(w.class_of + vid)];
    const size_t np = (size_t)w.npad;
    double* S = w.S + vid;
    VehC v;
    Veh24X vx;
    VehAux va;
    TireC ts[4];
    TireAux ta[4];
    Sus24C su[4];
    Corner24K ck[4];
    load_state24(S, np, v, vx, va, ts, ta, su, ck);
    double t = w.t0;
    const int last = w.nsteps - 1;
    for (int s = 0; s <= last; ++s) {
        DriverInput c;
        func(t, &c);
        // the last step also writes the values the reference leaves in its state structs
        step24<kNr>(v, vx, va, ts, ta, su, ck, K, C, c.m_steering, c.m_throttle, c.m_braking, w.dt, S, np, s == last);
        t += w.dt;
    }
    store_state24(S, np, v, vx, va, ts, ta, su, C.tcbool);
    if (!state24_finite(v, vx, ts)) w.status[vid] |= 1u;
}

// Enqueues the window of `view` on view.stream: the kernel of model Model (LFDM_MODEL_11/18/24) for
// the tire type the view describes.
template <int Model, typename Func>
inline cudaError_t launch_functor_window(const lfdm_device_window& view, Func func) {
    if (view.n <= 0 || view.nsteps <= 0) return cudaSuccess;
    if (view.model != Model) return cudaErrorInvalidValue;
    const unsigned blocks = (unsigned)((view.n + kFunctorThreads - 1) / kFunctorThreads);
    cudaStream_t st = static_cast<cudaStream_t>(view.stream);
    const bool nr = view.tire_type == LFDM_TIRE_TMEASY_NR;
    if constexpr (Model == LFDM_MODEL_11) {
        if (nr) functor_window11<true><<<blocks, kFunctorThreads, 0, st>>>(view, func);
        else functor_window11<false><<<blocks, kFunctorThreads, 0, st>>>(view, func);
    } else if constexpr (Model == LFDM_MODEL_24) {
        if (nr) functor_window24<true><<<blocks, kFunctorThreads, 0, st>>>(view, func);
        else functor_window24<false><<<blocks, kFunctorThreads, 0, st>>>(view, func);
    } else {
        if (nr) functor_window18<true><<<blocks, kFunctorThreads, 0, st>>>(view, func);
        else functor_window18<false><<<blocks, kFunctorThreads, 0, st>>>(view, func);
    }
    return cudaGetLastError();
}

}  // namespace lfdm
