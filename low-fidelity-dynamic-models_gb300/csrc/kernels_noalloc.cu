// lfdm_step18_noalloc: one 18-DOF FP64 stepping window over device-resident vehicles that
// allocates nothing. It has no counterpart in the reference (whose solver owns and allocates all
// of its memory); it serves callers that keep their own device buffers and cannot allow an
// allocation on the call path.
//
// The window kernel needs memory beyond its inputs and outputs: the derived per-vehicle constants
// K [K18_COUNT][npad], the SoA state [LFDM_S_COUNT][npad] it steps in place, the SoA controls
// [3][npad], the class index per vehicle and the class table. All of that lives in ONE file-scope
// `static __device__` array, `g_noalloc_scratch`, of a fixed size that holds kNoAllocMaxVehicles
// vehicles; larger calls are rejected. Every call on a device shares that device's array, so
// calls that overlap on the GPU (different streams, or host threads racing) race on it: the
// caller serialises them. Nothing in it has to start at zero: each call writes every element it
// later reads (the class-index words are cleared by a memset on the call's stream).
//
// Per device, at the first call with that device current, cudaGetSymbolAddress gives the array's
// address, which is then passed to the kernels. No cudaMalloc, cudaFree, cudaMallocAsync or
// allocating library routine is called; copies and memsets are enqueued on the caller's stream.

#include <cstdio>
#include <cstring>
#include <mutex>

#include "dof18_device.cuh"
#include "kernels.h"

namespace lfdm {
namespace {

constexpr int kNoAllocMaxVehicles = LFDM_NOALLOC_MAX_VEHICLES;
static_assert(kNoAllocMaxVehicles % 128 == 0, "the vehicle capacity is a whole number of 128-thread blocks");

// Layout of the scratch array, in bytes from its start (each part 256-byte aligned).
constexpr size_t kAlign = 256;
constexpr size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }
constexpr size_t kOffK = 0;
constexpr size_t kOffS = align_up(kOffK + sizeof(double) * (size_t)K18_COUNT * kNoAllocMaxVehicles);
constexpr size_t kOffCtl = align_up(kOffS + sizeof(double) * (size_t)LFDM_S_COUNT * kNoAllocMaxVehicles);
constexpr size_t kOffClassOf = align_up(kOffCtl + sizeof(double) * 3 * (size_t)kNoAllocMaxVehicles);
constexpr size_t kOffClass = align_up(kOffClassOf + sizeof(int32_t) * (size_t)kNoAllocMaxVehicles);
constexpr size_t kScratchBytes = align_up(kOffClass + sizeof(ClassDev18));

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char* g_scratch_ptr[kMaxDevices] = {};

void set_err(char* err, size_t err_len, const char* msg) {
    if (err && err_len) {
        std::snprintf(err, err_len, "%s", msg);
    }
}

}  // namespace
}  // namespace lfdm

using namespace lfdm;

#define NA_CK(call)                                                                          \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) {                                                             \
            char m_[256];                                                                    \
            std::snprintf(m_, sizeof(m_), "%s: %s", #call, cudaGetErrorString(e_));          \
            set_err(err, err_len, m_);                                                       \
            return LFDM_ERR_CUDA;                                                            \
        }                                                                                    \
    } while (0)

extern "C" int lfdm_step18_noalloc(const lfdm_class18* cls, int tire_type, const double* params, double* states,
                                   const double* steering, const double* throttle, const double* braking,
                                   unsigned n, double t0, double dt, unsigned nsteps, void* stream, char* err,
                                   size_t err_len) {
    set_err(err, err_len, "");
    if (n == 0) return LFDM_OK;
    if (n > (unsigned)kNoAllocMaxVehicles) {
        char m[160];
        std::snprintf(m, sizeof(m), "lfdm_step18_noalloc: %u vehicles exceed the fixed scratch capacity of %d vehicles",
                      n, kNoAllocMaxVehicles);
        set_err(err, err_len, m);
        return LFDM_ERR_CAPACITY;
    }
    if (!cls || !params || !states || !steering || !throttle || !braking) {
        set_err(err, err_len, "lfdm_step18_noalloc: null class, parameter, state or control pointer");
        return LFDM_ERR_ARG;
    }
    if (tire_type != LFDM_TIRE_TMEASY && tire_type != LFDM_TIRE_TMEASY_NR) {
        set_err(err, err_len, "lfdm_step18_noalloc: unknown tire type");
        return LFDM_ERR_ARG;
    }
    if (!(dt > 0) || !(dt < 1e300) || !(t0 > -1e300 && t0 < 1e300) || nsteps == 0 || nsteps > (1u << 30)) {
        set_err(err, err_len, "lfdm_step18_noalloc: dt must be positive and finite, t0 finite, nsteps in [1, 2^30]");
        return LFDM_ERR_ARG;
    }
    const lfdm_class18& c = *cls;
    bool maps_ok = c.noGears >= 1 && c.noGears <= LFDM_MAX_GEARS && c.powertrainMapSize >= 1 &&
                   c.powertrainMapSize <= LFDM_MAX_MAP && c.lossesMapSize >= 1 && c.lossesMapSize <= LFDM_MAX_MAP;
    if (c.tcbool)
        maps_ok = maps_ok && c.CFmapSize >= 1 && c.CFmapSize <= LFDM_MAX_MAP && c.TRmapSize >= 1 &&
                  c.TRmapSize <= LFDM_MAX_MAP;
    if (c.nonLinearSteer) maps_ok = maps_ok && c.steerMapSize >= 1 && c.steerMapSize <= LFDM_MAX_MAP;
    if (!maps_ok) {
        set_err(err, err_len, "lfdm_step18_noalloc: gear count or map sizes out of range");
        return LFDM_ERR_ARG;
    }

    int dev = 0;
    NA_CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        set_err(err, err_len, "lfdm_step18_noalloc: device ordinal out of range");
        return LFDM_ERR_ARG;
    }
    unsigned char* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        if (!g_scratch_ptr[dev]) {
            void* p = nullptr;
            NA_CK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
            g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
        }
        base = g_scratch_ptr[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int ni = (int)n;
    const int npad = (ni + 127) / 128 * 128;  // <= kNoAllocMaxVehicles
    double* K = reinterpret_cast<double*>(base + kOffK);
    double* S = reinterpret_cast<double*>(base + kOffS);
    double* ctl = reinterpret_cast<double*>(base + kOffCtl);
    int32_t* class_of = reinterpret_cast<int32_t*>(base + kOffClassOf);
    ClassDev18* cdev = reinterpret_cast<ClassDev18*>(base + kOffClass);

    ClassDev18 host_cls;
    build_class_dev18(c, &host_cls);
    // Pageable source: the copy has taken the bytes when cudaMemcpyAsync returns.
    NA_CK(cudaMemcpyAsync(cdev, &host_cls, sizeof(ClassDev18), cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemsetAsync(class_of, 0, sizeof(int32_t) * n, st));
    NA_CK(launch_prepare18(params, ni, npad, K, st));
    NA_CK(launch_states_to_soa(states, ni, LFDM_S_COUNT, npad, S, st));
    NA_CK(cudaMemcpyAsync(ctl, steering, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    NA_CK(cudaMemcpyAsync(ctl + npad, throttle, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    NA_CK(cudaMemcpyAsync(ctl + 2 * (size_t)npad, braking, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));

    Window18 w;
    w.n = ni;
    w.npad = npad;
    w.tire_nr = tire_type == LFDM_TIRE_TMEASY_NR;
    w.precision = LFDM_PREC_FP64;
    w.t0 = t0;
    w.dt = dt;
    w.nsteps = (int)nsteps;
    w.K = K;
    w.classes = cdev;
    w.nclasses = 1;
    w.class_of = class_of;
    w.S = S;
    w.ctl_mode = CTL_ARRAY;
    w.ctl = ctl;
    w.threads = 128;
    NA_CK(launch_window18(w, st));
    NA_CK(launch_states_to_aos(S, ni, LFDM_S_COUNT, npad, states, st));
    return LFDM_OK;
}
