// Mixed-DOF fleet kernel: one persistent launch steps a fleet of 18-DOF and 24-DOF vehicles with
// different parameter classes and horizons.
//
// The reference solves one model, one end time and (per Construct) one parameter set per solver
// (d18SolverHalfImplicitGPU / d24SolverHalfImplicitGPU, m_tend global), so an uneven fleet needs one
// solver run per model and horizon group. Here the vehicles of each model are sorted by their step
// count (longest first) and cut into tiles of 32 (one warp). The tiles of both models form one work
// list ordered by estimated cost (steps x vehicles x per-step cost of the model), largest first. A
// persistent grid (SMs x resident blocks) pulls tiles with one atomic per tile and runs each tile's
// vehicles over the steps of this launch, keeping their state in registers, so long-horizon
// vehicles start first and short ones fill the tail (longest-processing-time-first scheduling).
// Model affinity (an autotuner choice): each model's tiles in a list of its own, and the SMs split in
// proportion to the two models' estimated work; a warp first drains its SM's home list and then
// helps with the other one, so that an SM runs one model's code for most of the launch instead of
// interleaving the two step functions (together larger than the instruction cache).
//
// Each vehicle follows exactly the reference's per-vehicle schedule: the step start times are the
// ones the reference's Solve loop produces (windows of kernel_sim_time from t = 0, t restarting at
// each window start; computed on the host in the same FP64 arithmetic), the vehicle runs the steps
// of the windows that start before its own end time, and response samples are taken at the steps
// the reference samples. A launch covers a contiguous range of global steps; the host may split a
// horizon over several launches (steps per launch is a tuning knob). Per-warp shared memory holds
// the tile's derived constants; class tables are read through L1.
#include <cuda_runtime.h>

#include "../../include/lfdm/device/dof24_device.cuh"
#include "fleet.h"
#include "window_common.cuh"

namespace lfdm {

constexpr int kFleetKMax = (int)K18_COUNT > (int)K24_COUNT ? (int)K18_COUNT : (int)K24_COUNT;

// per warp: the tile's derived constants in FP64, and their FP32 copies for the FP32 tire core
size_t fleet_smem_per_warp(bool f32) {
    return (size_t)kFleetKMax * 32 * (sizeof(double) + (f32 ? sizeof(float) : 0));
}

template <bool kF32>
__device__ __forceinline__ void run_tile18(const FleetLaunch& L, const FleetTile& T, double* ks, float* fks, int lane) {
    const FleetModelDev& M = L.m18;
    if (lane >= T.count) return;
    const int i = T.first + lane;
    const int nst = min(__ldg(M.nsteps + i), L.s_end);
    if (nst <= L.s_begin) return;
    const size_t np = (size_t)M.npad;
#pragma unroll 4
    for (int k = 0; k < K18_COUNT; ++k) {
        const double x = __ldg(M.K + (size_t)k * np + i);
        ks[k * 32 + lane] = x;
        if (kF32) fks[k * 32 + lane] = (float)x;
    }
    const KView K{ks + lane, 32, kF32 ? fks + lane : nullptr};
    const ClassDev18& C = M.classes[__ldg(M.class_of + i)];
    double* S = M.S + i;
    VehC v;
    VehAux va;
    TireC ts[4];
    TireAux ta[4];
    load_state18(S, np, v, va, ts, ta);
    DriverCursor cur;
    driver_begin(cur, L.rows + 4 * __ldg(M.row_off + i), __ldg(M.row_len + i), __ldg(L.step_t + L.s_begin));
    double steer, thr, brk;
    for (int s = L.s_begin; s < nst; ++s) {
        const double t = __ldg(L.step_t + s);
        driver_at(cur, t, steer, thr, brk);
        step18<false, kF32>(v, va, ts, ta, K, C, steer, thr, brk, L.dt);
        const int k = __ldg(L.step_sample + s);
        if (M.resp && k >= 0 && k < L.nsamples) {
            double* r = M.resp + (size_t)k * LFDM18_RESP_CHANNELS * M.n + i;
            const size_t n = (size_t)M.n;
            r[0 * n] = t + L.dt;
            r[1 * n] = v.x;
            r[2 * n] = v.y;
            r[3 * n] = v.u;
            r[4 * n] = v.v;
            r[5 * n] = v.phi;
            r[6 * n] = v.psi;
            r[7 * n] = v.wx;
            r[8 * n] = v.wz;
            r[9 * n] = ts[0].omega;
            r[10 * n] = ts[1].omega;
            r[11 * n] = ts[2].omega;
            r[12 * n] = ts[3].omega;
        }
    }
    store_state18(S, np, v, va, ts, ta);
    if (!state18_finite(v, ts)) M.status[i] |= 1u;
}

template <bool kF32>
__device__ __forceinline__ void run_tile24(const FleetLaunch& L, const FleetTile& T, double* ks, float* fks, int lane) {
    const FleetModelDev& M = L.m24;
    if (lane >= T.count) return;
    const int i = T.first + lane;
    const int nst = min(__ldg(M.nsteps + i), L.s_end);
    if (nst <= L.s_begin) return;
    const size_t np = (size_t)M.npad;
#pragma unroll 4
    for (int k = 0; k < K24_COUNT; ++k) {
        const double x = __ldg(M.K + (size_t)k * np + i);
        ks[k * 32 + lane] = x;
        if (kF32) fks[k * 32 + lane] = (float)x;
    }
    const KView K{ks + lane, 32, kF32 ? fks + lane : nullptr};
    const ClassDev18& C = M.classes[__ldg(M.class_of + i)];
    double* S = M.S + i;
    VehC v;
    Veh24X vx;
    VehAux va;
    TireC ts[4];
    TireAux ta[4];
    Sus24C su[4];
    Corner24K ck[4];
    load_state24(S, np, v, vx, va, ts, ta, su, ck);
    DriverCursor cur;
    driver_begin(cur, L.rows + 4 * __ldg(M.row_off + i), __ldg(M.row_len + i), __ldg(L.step_t + L.s_begin));
    double steer, thr, brk;
    auto sample = [&](int s, double t) {
        const int k = __ldg(L.step_sample + s);
        if (M.resp && k >= 0 && k < L.nsamples) {
            double* r = M.resp + (size_t)k * LFDM24_RESP_CHANNELS * M.n + i;
            const size_t n = (size_t)M.n;
            r[0 * n] = t + L.dt;
            r[1 * n] = v.x;
            r[2 * n] = v.y;
            r[3 * n] = v.u;
            r[4 * n] = v.v;
            r[5 * n] = v.phi;
            r[6 * n] = v.psi;
            r[7 * n] = vx.theta;
            r[8 * n] = v.wx;
            r[9 * n] = v.wz;
            r[10 * n] = vx.wy;
            r[11 * n] = ts[0].omega;
            r[12 * n] = ts[1].omega;
            r[13 * n] = ts[2].omega;
            r[14 * n] = ts[3].omega;
        }
    };
    const int last = nst - 1;
    for (int s = L.s_begin; s <= last; ++s) {
        const double t = __ldg(L.step_t + s);
        driver_at(cur, t, steer, thr, brk);
        // the step that ends this launch's range for the vehicle also writes the values the
        // reference leaves in its state structs (as the window kernel does for a window's last step)
        step24<false, kF32>(v, vx, va, ts, ta, su, ck, K, C, steer, thr, brk, L.dt, S, np, s == last);
        sample(s, t);
    }
    store_state24(S, np, v, vx, va, ts, ta, su, C.tcbool);
    if (!state24_finite(v, vx, ts)) M.status[i] |= 1u;
}

// kF32: the TMeasy tire core in FP32 (precision LFDM_PREC_MIXED_TIRE)
template <bool kF32>
__global__ void __launch_bounds__(128) fleet_kernel(const FleetLaunch L) {
    extern __shared__ __align__(16) double fleet_smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double* ks = fleet_smem + (size_t)warp * kFleetKMax * 32;
    float* fks = reinterpret_cast<float*>(fleet_smem + (size_t)(blockDim.x >> 5) * kFleetKMax * 32) +
                 (size_t)warp * kFleetKMax * 32;
    if (!L.affinity) {
        for (;;) {
            int tile = 0;
            if (lane == 0) tile = atomicAdd(L.queue, 1);
            tile = __shfl_sync(0xffffffffu, tile, 0);
            if (tile >= L.ntiles) break;
            const FleetTile T = L.merged[tile];
            if (T.nsteps_max > L.s_begin) {
                if (T.model == LFDM_MODEL_24) run_tile24<kF32>(L, T, ks, fks, lane);
                else run_tile18<kF32>(L, T, ks, fks, lane);
            }
            __syncwarp();
        }
        return;
    }
    unsigned smid, nsmid;
    asm("mov.u32 %0, %%smid;" : "=r"(smid));
    asm("mov.u32 %0, %%nsmid;" : "=r"(nsmid));
    const int home = (float)smid < L.home18 * (float)nsmid ? 0 : 1;  // 0: 18-DOF list, 1: 24-DOF list
    const int base[2] = {0, L.ntiles18};
    const int count[2] = {L.ntiles18, L.ntiles - L.ntiles18};
    // each list is taken until its counter passes its length (a counter already past it is seen
    // with a plain read, saving the atomic); then the other list; then the warp is done
    for (int pass = 0; pass < 2; ++pass) {
        const int q = pass == 0 ? home : 1 - home;
        if (count[q] == 0) continue;
        for (;;) {
            int tile = count[q];
            if (lane == 0 && *(volatile int*)(L.queue + q) < count[q]) tile = atomicAdd(L.queue + q, 1);
            tile = __shfl_sync(0xffffffffu, tile, 0);
            if (tile >= count[q]) break;
            const FleetTile T = L.tiles[base[q] + tile];
            if (T.nsteps_max > L.s_begin) {
                if (T.model == LFDM_MODEL_24) run_tile24<kF32>(L, T, ks, fks, lane);
                else run_tile18<kF32>(L, T, ks, fks, lane);
            }
            __syncwarp();
        }
    }
}

// Raises the kernels' dynamic shared-memory limits to what 4 warps per block need (every
// configuration uses at most that); called before any launch or occupancy query, outside capture.
cudaError_t fleet_kernel_setup() {
    cudaError_t e = cudaFuncSetAttribute(fleet_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(fleet_smem_per_warp(false) * 4));
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(fleet_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(fleet_smem_per_warp(true) * 4));
}

cudaError_t fleet_occupancy(int threads, bool f32, int* blocks_per_sm) {
    const size_t smem = fleet_smem_per_warp(f32) * (threads / 32);
    return f32 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, fleet_kernel<true>, threads, smem)
               : cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, fleet_kernel<false>, threads, smem);
}

cudaError_t launch_fleet(const FleetLaunch& L, int blocks, int threads, bool f32, cudaStream_t stream) {
    if (threads <= 0 || threads > 128 || (threads & 31) || blocks <= 0) return cudaErrorInvalidValue;
    const size_t smem = fleet_smem_per_warp(f32) * (threads / 32);
    if (f32) fleet_kernel<true><<<blocks, threads, smem, stream>>>(L);
    else fleet_kernel<false><<<blocks, threads, smem, stream>>>(L);
    return cudaGetLastError();
}

}  // namespace lfdm
