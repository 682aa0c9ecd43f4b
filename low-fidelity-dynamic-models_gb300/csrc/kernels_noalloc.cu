// lfdm_step18_noalloc: one 18-DOF FP64 stepping window over device-resident vehicles that
// allocates nothing. It has no counterpart in the reference (whose solver owns and allocates all
// of its memory); it serves callers that keep their own device buffers and cannot allow an
// allocation on the call path.
//
// The window kernel needs memory beyond its inputs and outputs: the derived per-vehicle constants
// K [K18_COUNT][npad], the SoA state [LFDM_S_COUNT][npad] it steps in place, the SoA controls
// [3][npad], the class index and status word per vehicle, one summary status word and the class
// table. All of that lives in ONE file-scope `static __device__` array, `g_noalloc_scratch`, of
// exactly LFDM_NOALLOC_SCRATCH_BYTES bytes, which holds LFDM_NOALLOC_MAX_VEHICLES vehicles; larger
// calls are rejected. The array is reserved on every device where the library's module is loaded,
// whether or not this entry point is called. Every call on a device shares that device's array,
// so calls that overlap on the GPU (different streams, or host threads racing) race on it: the
// caller serialises them. The class-index, status and summary words are cleared by memsets on the
// call's stream; every other element is written before it is read.
//
// At every call, with the call's device current, cudaGetSymbolAddress gives the array's device
// address (cheap, allocates nothing, and stays right if the device's context was torn down and
// recreated in between), which is then passed to the kernels. No cudaMalloc, cudaFree,
// cudaMallocAsync or allocating library routine is called; copies, memsets and kernels are
// enqueued on the caller's stream, and the call waits for that stream at the end to read the
// summary status word (LFDM_ERR_NUMERIC if any vehicle's state became non-finite, as in the
// solver).

#include <cstdio>
#include <cstring>

#include "../../include/lfdm/device/dof18_device.cuh"
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
constexpr size_t kOffStatus = align_up(kOffClassOf + sizeof(int32_t) * (size_t)kNoAllocMaxVehicles);
constexpr size_t kOffAny = align_up(kOffStatus + sizeof(uint32_t) * (size_t)kNoAllocMaxVehicles);
constexpr size_t kOffClass = align_up(kOffAny + sizeof(uint32_t));
constexpr size_t kScratchBytes = align_up(kOffClass + sizeof(ClassDev18));
static_assert(kScratchBytes == LFDM_NOALLOC_SCRATCH_BYTES,
              "LFDM_NOALLOC_SCRATCH_BYTES in include/lfdm.h states the scratch array's exact size");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kAnyThreads = 256;

// OR of the n per-vehicle status words into one summary word (one block).
__global__ void __launch_bounds__(kAnyThreads) status_any_kernel(const uint32_t* status, int n, uint32_t* any) {
    uint32_t bits = 0;
    for (int i = threadIdx.x; i < n; i += kAnyThreads) bits |= status[i];
    bits = __reduce_or_sync(0xffffffffu, bits);
    if ((threadIdx.x & 31) == 0 && bits) atomicOr(any, bits);
}

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

    unsigned char* base = nullptr;
    {
        void* p = nullptr;
        NA_CK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        base = static_cast<unsigned char*>(p);
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int ni = (int)n;
    const int npad = (ni + 127) / 128 * 128;  // <= kNoAllocMaxVehicles
    double* K = reinterpret_cast<double*>(base + kOffK);
    double* S = reinterpret_cast<double*>(base + kOffS);
    double* ctl = reinterpret_cast<double*>(base + kOffCtl);
    int32_t* class_of = reinterpret_cast<int32_t*>(base + kOffClassOf);
    uint32_t* status = reinterpret_cast<uint32_t*>(base + kOffStatus);
    uint32_t* any = reinterpret_cast<uint32_t*>(base + kOffAny);
    ClassDev18* cdev = reinterpret_cast<ClassDev18*>(base + kOffClass);

    ClassDev18 host_cls;
    build_class_dev18(c, &host_cls);
    // Pageable source: the copy has taken the bytes when cudaMemcpyAsync returns.
    NA_CK(cudaMemcpyAsync(cdev, &host_cls, sizeof(ClassDev18), cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemsetAsync(class_of, 0, sizeof(int32_t) * n, st));
    NA_CK(cudaMemsetAsync(status, 0, sizeof(uint32_t) * n, st));
    NA_CK(cudaMemsetAsync(any, 0, sizeof(uint32_t), st));
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
    w.status = status;
    w.threads = 128;
    NA_CK(launch_window18(w, st));
    NA_CK(launch_states_to_aos(S, ni, LFDM_S_COUNT, npad, states, st));
    status_any_kernel<<<1, kAnyThreads, 0, st>>>(status, ni, any);
    NA_CK(cudaGetLastError());
    uint32_t any_host = 0;
    NA_CK(cudaMemcpyAsync(&any_host, any, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    NA_CK(cudaStreamSynchronize(st));
    if (any_host & 1u) {
        set_err(err, err_len, "lfdm_step18_noalloc: a vehicle's state became non-finite");
        return LFDM_ERR_NUMERIC;
    }
    return LFDM_OK;
}
