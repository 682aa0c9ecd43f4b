// Host-side declarations of the CUDA kernels' launchers (implemented in kernels18.cu).
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

#include "../../include/lfdm.h"

namespace lfdm {

struct ClassDev18;
struct ClassDev18F;

// Control source of a window.
enum CtlMode : int { CTL_TABLE = 0, CTL_SCALAR = 1, CTL_ARRAY = 2, CTL_SCHEDULE = 3 };

struct Window18 {
    int n = 0;           // vehicles
    int npad = 0;        // SoA row stride (multiple of 32, >= grid coverage)
    int tire_nr = 0;     // TMeasyNr tires
    int precision = LFDM_PREC_FP64;
    double t0 = 0, dt = 1e-3;
    int nsteps = 0;      // steps in this window (host-simulated loop of the reference)
    const double* K = nullptr;           // [K18_COUNT][npad] derived constants
    const ClassDev18* classes = nullptr; // [nclasses]
    const ClassDev18F* classes_f = nullptr;  // FP32 copies for the mixed kernel
    int nclasses = 0;
    const int32_t* class_of = nullptr;   // [n]
    double* S = nullptr;                 // [LFDM_S_COUNT][npad] state, in/out
    int ctl_mode = CTL_TABLE;
    const double* rows = nullptr;        // driver rows {t, steer, thr, brk}
    const int64_t* row_off = nullptr;    // [n]
    const int32_t* row_len = nullptr;    // [n]
    double steer = 0, thr = 0, brk = 0;  // CTL_SCALAR
    const double* ctl = nullptr;         // CTL_ARRAY: [3][npad]
    const double* sched = nullptr;       // CTL_SCHEDULE: [nsteps][3] shared by all vehicles
    double* resp = nullptr;              // [spw][13][n] or nullptr
    int nsamples = 0;                    // samples this window writes
    const int32_t* sample_steps = nullptr;  // [nsamples] 1-based step index after which sample k is taken
    uint32_t* status = nullptr;          // [n] OR-ed status bits
    int threads = 128;
    int split = -1;                      // 11-DOF split-warp kernel: -1 small fleets, 0 never, 1 always
};

// Launch one stepping window on `stream`. Returns cudaSuccess or the launch error.
cudaError_t launch_window18(const Window18& w, cudaStream_t stream);

// Dynamic shared memory one block of `threads` needs for `nclasses` classes; 0 if it cannot fit.
size_t window18_smem(int threads, int nclasses, bool f32 = false);

// Derived per-vehicle constants: params AoS [n][LFDM_P_COUNT] (device) -> K SoA [K18_COUNT][npad].
cudaError_t launch_prepare18(const double* params_dev, int n, int npad, double* K_dev, cudaStream_t stream);

// AoS [n][ns] <-> SoA [ns][npad] (device buffers); ns = doubles per state vector of the model.
cudaError_t launch_states_to_soa(const double* aos, int n, int ns, int npad, double* soa, cudaStream_t stream);
cudaError_t launch_states_to_aos(const double* soa, int n, int ns, int npad, double* aos, cudaStream_t stream);

// 11-DOF window (same Window18 fields; states in the LFDM11_S_* layout, 9 response channels).
cudaError_t launch_window11(const Window18& w, cudaStream_t stream);

// 24-DOF window (states in the LFDM24_S_* layout, 15 response channels, K from launch_prepare24).
cudaError_t launch_window24(const Window18& w, cudaStream_t stream);
cudaError_t launch_prepare24(const double* params_dev, int n, int npad, double* K_dev, cudaStream_t stream);
int k24_count();

// Counts table rows whose time is smaller than the previous row's (per vehicle, equal-length tables
// of nrows rows each; shared != 0: one table). *bad_dev must be zeroed by the caller.
cudaError_t launch_check_tables(const double* rows, long long ntables, int nrows, unsigned* bad_dev,
                                cudaStream_t stream);

// Measured FP64 fused-multiply-add throughput of the current device, in DFMA lane operations per
// second (a kernel of independent chains timed with CUDA events), and the SM clock it ran at in GHz
// (clock counter over the global timer; sm_ghz may be null).
cudaError_t measure_dfma_rate(double* dfma_per_s, double* sm_ghz);
cudaError_t measure_ffma_rate(double* ffma_per_s, double* sm_ghz);

// Host-side conversion of a class record into the device table (computes segment reciprocals).
void build_class_dev18(const lfdm_class18& c, ClassDev18* out);
size_t class_dev18_size();
void build_class_dev18f(const lfdm_class18& c, ClassDev18F* out);
size_t class_dev18f_size();

int k18_count();

}  // namespace lfdm
