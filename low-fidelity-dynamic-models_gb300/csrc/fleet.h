// Device-side description of a mixed-DOF fleet launch (fleet.cu) and its host launchers.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

#include "../../include/lfdm.h"

namespace lfdm {

struct ClassDev18;

// 32 consecutive vehicles (in the model's step-count order) of one model: one warp's work item.
struct FleetTile {
    int model;       // LFDM_MODEL_18 or LFDM_MODEL_24
    int first;       // first vehicle (index into the model's arrays)
    int count;       // vehicles in the tile (<= 32)
    int nsteps_max;  // steps of the tile's longest horizon
};

// One model's share of the fleet; vehicles are stored in the model's step-count order.
struct FleetModelDev {
    int n = 0, npad = 0;
    const double* K = nullptr;             // [K count][npad] derived constants
    double* S = nullptr;                   // [states][npad] SoA state, in/out
    const int32_t* class_of = nullptr;     // [n]
    const ClassDev18* classes = nullptr;   // class tables of this model
    const int64_t* row_off = nullptr;      // [n] first driver row of each vehicle
    const int32_t* row_len = nullptr;      // [n]
    const int32_t* nsteps = nullptr;       // [n] steps of each vehicle's horizon
    double* resp = nullptr;                // [nsamples][channels][n] or nullptr
    uint32_t* status = nullptr;            // [n] OR-ed status bits (1: non-finite state)
};

struct FleetLaunch {
    FleetModelDev m18, m24;
    const double* rows = nullptr;          // driver rows {t, steering, throttle, braking}
    const FleetTile* tiles = nullptr;      // the 18-DOF tiles [0, ntiles18), then the 24-DOF ones
    const FleetTile* merged = nullptr;     // the same tiles in one list by estimated cost (both models)
    int ntiles = 0;
    int ntiles18 = 0;
    int* queue = nullptr;                  // this launch's two tile counters, zero at its start
    int affinity = 0;                      // 0: one list by cost (merged, counter 0); 1: model affinity
    float home18 = 0.0f;                   // with affinity: SMs with smid < home18 * nsmid start on the
                                           // 18-DOF tiles, the others on the 24-DOF tiles
    const double* step_t = nullptr;        // [total steps] start time of each global step
    const int32_t* step_sample = nullptr;  // [total steps] sample index taken after the step, or -1
    int s_begin = 0, s_end = 0;            // global steps [s_begin, s_end) of this launch
    double dt = 1e-3;
    int nsamples = 0;                      // samples the response buffers hold
};

// f32: the kernel with the FP32 TMeasy tire core (precision LFDM_PREC_MIXED_TIRE)
size_t fleet_smem_per_warp(bool f32);
cudaError_t fleet_kernel_setup();
cudaError_t fleet_occupancy(int threads, bool f32, int* blocks_per_sm);
cudaError_t launch_fleet(const FleetLaunch& L, int blocks, int threads, bool f32, cudaStream_t stream);

}  // namespace lfdm
