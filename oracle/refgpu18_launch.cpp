// Test infrastructure only: runs the REFERENCE's own GPU kernel for the 18-DOF model.
//
// The reference's device code (18dof-gpu/dof18_halfImplicit_gpu.cu, dof18_gpu.cu,
// utils/utils_gpu.cu) is compiled from its sources and device-linked into oracle/_ref/ref18.cubin
// by `make refgpu` where the reference checkout exists. This launcher (no reference code in it)
// builds the reference's managed per-vehicle records (layout in refgpu18_layout.h), loads the cubin
// with the CUDA driver API and launches the table-driven Integrate kernel window by window the way
// d18SolverHalfImplicitGPU::Solve does (dof18_halfImplicit_gpu.cu:404-494): windows of ksim from
// t = 0 while the window start is below tend, threads_per_block threads per block.
//
// usage: refgpu18_launch <cubin> <input.bin> <output.bin>
// input.bin : int32 n, nrows, tpb, pad; double dt, ksim, tend, dtout; lfdm_class18;
//             params [n][LFDM_P_COUNT]; tables [n][nrows][4]; states [n][LFDM_S_COUNT]
// output.bin: states [n][LFDM_S_COUNT] after the run
// stdout    : one JSON line with per-window kernel times (CUDA events).
#include <cuda.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../include/lfdm.h"
#include "refgpu18_layout.h"

using namespace refgpu18;

#define DRV(x)                                                                  \
    do {                                                                        \
        CUresult r_ = (x);                                                      \
        if (r_ != CUDA_SUCCESS) {                                               \
            const char* s_ = nullptr;                                           \
            cuGetErrorString(r_, &s_);                                          \
            std::fprintf(stderr, "%s failed: %s\n", #x, s_ ? s_ : "?");         \
            return 1;                                                           \
        }                                                                       \
    } while (0)

template <typename T>
static bool rd(FILE* f, T* p, size_t n) {
    return std::fread(p, sizeof(T), n, f) == n;
}

template <typename T>
static T* managed(size_t n) {
    CUdeviceptr p = 0;
    if (cuMemAllocManaged(&p, sizeof(T) * (n ? n : 1), CU_MEM_ATTACH_GLOBAL) != CUDA_SUCCESS) return nullptr;
    return reinterpret_cast<T*>(p);
}

static MapEntry* map_copy(const double (*pts)[2], int n, double xs = 1.0) {
    MapEntry* m = managed<MapEntry>(n);
    for (int i = 0; i < n; ++i) m[i] = MapEntry{pts[i][0] * xs, pts[i][1]};
    return m;
}

int main(int argc, char** argv) {
    if (argc != 4) {
        std::fprintf(stderr, "usage: %s <cubin> <input.bin> <output.bin>\n", argv[0]);
        return 2;
    }
    FILE* f = std::fopen(argv[2], "rb");
    if (!f) return 2;
    int32_t hdr[4];
    double dh[4];
    lfdm_class18 cls;
    if (!rd(f, hdr, 4) || !rd(f, dh, 4) || !rd(f, &cls, 1)) return 2;
    const int n = hdr[0], nrows = hdr[1], tpb = hdr[2];
    const double dt = dh[0], ksim = dh[1], tend = dh[2], dtout = dh[3];
    std::vector<double> P((size_t)n * LFDM_P_COUNT), T((size_t)n * nrows * 4), S((size_t)n * LFDM_S_COUNT);
    if (!rd(f, P.data(), P.size()) || !rd(f, T.data(), T.size()) || !rd(f, S.data(), S.size())) return 2;
    std::fclose(f);

    DRV(cuInit(0));
    CUdevice dev;
    DRV(cuDeviceGet(&dev, 0));
    CUcontext ctx;
    DRV(cuDevicePrimaryCtxRetain(&ctx, dev));
    DRV(cuCtxSetCurrent(ctx));
    CUmodule mod;
    DRV(cuModuleLoad(&mod, argv[1]));
    CUfunction fn;
    DRV(cuModuleGetFunction(&fn, mod, kIntegrateName));

    // one set of maps for the class (the reference allocates them per Construct call)
    MapEntry* steer = cls.nonLinearSteer ? map_copy(cls.steerMap, cls.steerMapSize) : nullptr;
    double* gears = managed<double>(cls.noGears);
    for (int g = 0; g < cls.noGears; ++g) gears[g] = cls.gearRatios[g];
    MapEntry* shift = map_copy(cls.shiftMap, cls.noGears);
    MapEntry* pt = map_copy(cls.powertrainMap, cls.powertrainMapSize);
    MapEntry* loss = map_copy(cls.lossesMap, cls.lossesMapSize);
    MapEntry* cf = cls.tcbool ? map_copy(cls.CFmap, cls.CFmapSize) : nullptr;
    MapEntry* tr = cls.tcbool ? map_copy(cls.TRmap, cls.TRmapSize) : nullptr;
    DriverInput* rows = managed<DriverInput>((size_t)n * nrows);
    std::memcpy(rows, T.data(), T.size() * sizeof(double));
    SimData* data = managed<SimData>(n);
    SimState* st = managed<SimState>(n);
    if (!gears || !shift || !pt || !loss || !rows || !data || !st) return 3;
    for (int i = 0; i < n; ++i) {
        const double* p = &P[(size_t)i * LFDM_P_COUNT];
        VehicleParam& v = data[i].veh;
        std::memset(&data[i], 0, sizeof(SimData));
        v.a = p[LFDM_P_A]; v.b = p[LFDM_P_B]; v.h = p[LFDM_P_H]; v.m = p[LFDM_P_M]; v.jz = p[LFDM_P_JZ];
        v.jx = p[LFDM_P_JX]; v.jxz = p[LFDM_P_JXZ]; v.cf = p[LFDM_P_CF]; v.cr = p[LFDM_P_CR];
        v.muf = p[LFDM_P_MUF]; v.mur = p[LFDM_P_MUR]; v.hrcf = p[LFDM_P_HRCF]; v.hrcr = p[LFDM_P_HRCR];
        v.krof = p[LFDM_P_KROF]; v.kror = p[LFDM_P_KROR]; v.brof = p[LFDM_P_BROF]; v.bror = p[LFDM_P_BROR];
        v.nonLinearSteer = cls.nonLinearSteer != 0;
        v.steerMap = steer;
        v.steerMapSize = cls.steerMapSize;
        v.maxSteer = p[LFDM_P_MAXSTEER];
        v.crankInertia = p[LFDM_P_CRANKINERTIA];
        v.gearRatios = gears;
        v.noGears = cls.noGears;
        v.shiftMap = shift;
        v.tcbool = cls.tcbool != 0;
        v.maxBrakeTorque = p[LFDM_P_MAXBRAKETORQUE];
        v.throttleMod = cls.throttleMod != 0;
        v.powertrainMap = pt;
        v.powertrainMapSize = cls.powertrainMapSize;
        v.lossesMap = loss;
        v.lossesMapSize = cls.lossesMapSize;
        v.CFmap = cf;
        v.CFmapSize = cls.CFmapSize;
        v.TRmap = tr;
        v.TRmapSize = cls.TRmapSize;
        v.driveType = cls.driveType != 0;
        v.whichWheels = cls.whichWheels != 0;
        std::memcpy(data[i].tire.v, p + LFDM_P_JW, 35 * sizeof(double));
        data[i].driver_data = rows + (size_t)i * nrows;
        data[i].driver_data_len = (unsigned)nrows;
        const double* s = &S[(size_t)i * LFDM_S_COUNT];
        std::memcpy(st[i].veh.v, s, 14 * sizeof(double));
        st[i].veh.current_gr = (int)s[LFDM_S_CURRENT_GR];
        for (int k = 0; k < 4; ++k)
            std::memcpy(st[i].tire[k].v, s + LFDM_S_TIRE0 + k * LFDM_S_TIRE_STRIDE, 15 * sizeof(double));
    }
    CUmemLocation loc;
    loc.type = CU_MEM_LOCATION_TYPE_DEVICE;
    loc.id = (int)dev;
    DRV(cuMemPrefetchAsync((CUdeviceptr)data, sizeof(SimData) * n, loc, 0, 0));
    DRV(cuMemPrefetchAsync((CUdeviceptr)st, sizeof(SimState) * n, loc, 0, 0));
    DRV(cuMemPrefetchAsync((CUdeviceptr)rows, sizeof(DriverInput) * (size_t)n * nrows, loc, 0, 0));
    DRV(cuCtxSynchronize());

    const bool output = dtout > 0;
    const unsigned collection_states = 13;
    const size_t spw = output ? (size_t)(ksim / dtout + 0.999999) : 1;
    CUdeviceptr resp = 0;
    DRV(cuMemAlloc(&resp, sizeof(double) * (size_t)n * collection_states * spw));
    CUevent e0, e1;
    DRV(cuEventCreate(&e0, CU_EVENT_DEFAULT));
    DRV(cuEventCreate(&e1, CU_EVENT_DEFAULT));
    std::vector<float> ms;
    double current = 0.0;
    unsigned total = (unsigned)n;
    const unsigned blocks = (total + tpb - 1) / tpb;
    while (current < tend) {
        double t0 = current, ks = ksim, step = dt, dto = output ? dtout : 1.0;
        bool out = output;
        double* rp = reinterpret_cast<double*>(resp);
        SimData* dp = data;
        SimState* sp = st;
        unsigned cs = collection_states;
        void* args[] = {&t0, &ks, &step, &out, &total, &cs, &dto, &rp, &dp, &sp};
        DRV(cuEventRecord(e0, 0));
        DRV(cuLaunchKernel(fn, blocks, 1, 1, tpb, 1, 1, 0, 0, args, nullptr));
        DRV(cuEventRecord(e1, 0));
        DRV(cuEventSynchronize(e1));
        float t = 0;
        DRV(cuEventElapsedTime(&t, e0, e1));
        ms.push_back(t);
        current = current + ksim;
    }
    DRV(cuCtxSynchronize());
    FILE* o = std::fopen(argv[3], "wb");
    if (!o) return 2;
    for (int i = 0; i < n; ++i) {
        double s[LFDM_S_COUNT] = {0};
        std::memcpy(s, st[i].veh.v, 14 * sizeof(double));
        s[LFDM_S_CURRENT_GR] = st[i].veh.current_gr;
        for (int k = 0; k < 4; ++k)
            std::memcpy(s + LFDM_S_TIRE0 + k * LFDM_S_TIRE_STRIDE, st[i].tire[k].v, 15 * sizeof(double));
        std::fwrite(s, sizeof(double), LFDM_S_COUNT, o);
    }
    std::fclose(o);
    std::printf("{\"n\": %d, \"tpb\": %d, \"windows\": %zu, \"window_ms\": [", n, tpb, ms.size());
    for (size_t k = 0; k < ms.size(); ++k) std::printf("%s%.4f", k ? ", " : "", ms[k]);
    std::printf("]}\n");
    return 0;
}
