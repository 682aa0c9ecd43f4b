// Test infrastructure only: runs the REFERENCE's own GPU kernels of the 11-, 18- and 24-DOF models.
//
// The reference's device code (<m>dof-gpu/dof<m>_halfImplicit_gpu.cu, dof<m>_gpu.cu,
// utils/utils_gpu.cu) is compiled from its sources and device-linked into oracle/_ref/ref<m>.cubin
// by `make refgpu` where the reference checkout exists. This launcher (no reference code in it)
// builds the reference's managed per-vehicle records (layouts in refgpu<m>_layout.h), loads the
// cubin with the CUDA driver API and launches the table-driven Integrate kernel window by window the
// way d<m>SolverHalfImplicitGPU::Solve does (e.g. 18dof-gpu/dof18_halfImplicit_gpu.cu:404-494):
// windows of ksim from t = 0 while the window start is below tend, threads_per_block threads per
// block, the response buffer sized for one window.
//
// usage: refgpu_launch <cubin> <input.bin> <output.bin>
// input.bin : int32 model (11, 18, 24), n, nrows, tpb; double dt, ksim, tend, dtout; lfdm_class18;
//             params [n][LFDM_P_COUNT]; tables [n][nrows][4]; states [n][state count of the model]
// output.bin: states [n][state count of the model] after the run
// stdout    : one JSON line with per-window kernel times (CUDA events).
#include <cuda.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../include/lfdm.h"
#include "refgpu11_layout.h"
#include "refgpu18_layout.h"
#include "refgpu24_layout.h"

#define DRV(x)                                                                  \
    do {                                                                        \
        CUresult r_ = (x);                                                      \
        if (r_ != CUDA_SUCCESS) {                                               \
            const char* s_ = nullptr;                                           \
            cuGetErrorString(r_, &s_);                                          \
            std::fprintf(stderr, "%s failed: %s\n", #x, s_ ? s_ : "?");         \
            std::exit(1);                                                       \
        }                                                                       \
    } while (0)

using refgpu18::DriverInput;
using refgpu18::MapEntry;

template <typename T>
static bool rd(FILE* f, T* p, size_t n) {
    return std::fread(p, sizeof(T), n, f) == n;
}

template <typename T>
static T* managed(size_t n) {
    CUdeviceptr p = 0;
    DRV(cuMemAllocManaged(&p, sizeof(T) * (n ? n : 1), CU_MEM_ATTACH_GLOBAL));
    return reinterpret_cast<T*>(p);
}

static MapEntry* map_copy(const double (*pts)[2], int n) {
    MapEntry* m = managed<MapEntry>(n);
    for (int i = 0; i < n; ++i) m[i] = MapEntry{pts[i][0], pts[i][1]};
    return m;
}

// The class's maps, allocated once (the reference allocates them per Construct call).
struct Maps {
    MapEntry *steer = nullptr, *shift = nullptr, *pt = nullptr, *loss = nullptr, *cf = nullptr, *tr = nullptr;
    double* gears = nullptr;
    explicit Maps(const lfdm_class18& c) {
        if (c.nonLinearSteer) steer = map_copy(c.steerMap, c.steerMapSize);
        gears = managed<double>(c.noGears);
        for (int g = 0; g < c.noGears; ++g) gears[g] = c.gearRatios[g];
        shift = map_copy(c.shiftMap, c.noGears);
        pt = map_copy(c.powertrainMap, c.powertrainMapSize);
        loss = map_copy(c.lossesMap, c.lossesMapSize);
        if (c.tcbool) {
            cf = map_copy(c.CFmap, c.CFmapSize);
            tr = map_copy(c.TRmap, c.TRmapSize);
        }
    }
};

// The flags, maps and scalar fields every model's VehicleParam has after its model-specific head.
template <typename VP>
static void fill_tail(VP& v, const lfdm_class18& c, const Maps& m, const double* p) {
    v.nonLinearSteer = c.nonLinearSteer != 0;
    v.steerMap = m.steer;
    v.steerMapSize = c.steerMapSize;
    v.maxSteer = p[LFDM_P_MAXSTEER];
    v.crankInertia = p[LFDM_P_CRANKINERTIA];
    v.gearRatios = m.gears;
    v.noGears = c.noGears;
    v.shiftMap = m.shift;
    v.tcbool = c.tcbool != 0;
    v.maxBrakeTorque = p[LFDM_P_MAXBRAKETORQUE];
    v.throttleMod = c.throttleMod != 0;
    v.powertrainMap = m.pt;
    v.powertrainMapSize = c.powertrainMapSize;
    v.lossesMap = m.loss;
    v.lossesMapSize = c.lossesMapSize;
    v.CFmap = m.cf;
    v.CFmapSize = c.CFmapSize;
    v.TRmap = m.tr;
    v.TRmapSize = c.TRmapSize;
    v.driveType = c.driveType != 0;
    v.whichWheels = c.whichWheels != 0;
}

static void fill_data(refgpu18::SimData& d, const lfdm_class18& c, const Maps& m, const double* p) {
    refgpu18::VehicleParam& v = d.veh;
    v.a = p[LFDM_P_A]; v.b = p[LFDM_P_B]; v.h = p[LFDM_P_H]; v.m = p[LFDM_P_M]; v.jz = p[LFDM_P_JZ];
    v.jx = p[LFDM_P_JX]; v.jxz = p[LFDM_P_JXZ]; v.cf = p[LFDM_P_CF]; v.cr = p[LFDM_P_CR];
    v.muf = p[LFDM_P_MUF]; v.mur = p[LFDM_P_MUR]; v.hrcf = p[LFDM_P_HRCF]; v.hrcr = p[LFDM_P_HRCR];
    v.krof = p[LFDM_P_KROF]; v.kror = p[LFDM_P_KROR]; v.brof = p[LFDM_P_BROF]; v.bror = p[LFDM_P_BROR];
    fill_tail(v, c, m, p);
    std::memcpy(d.tire.v, p + LFDM_P_JW, 35 * sizeof(double));
}

static void fill_data(refgpu11::SimData& d, const lfdm_class18& c, const Maps& m, const double* p) {
    refgpu11::VehicleParam& v = d.veh;
    v.a = p[LFDM_P_A]; v.b = p[LFDM_P_B]; v.h = p[LFDM_P_H]; v.m = p[LFDM_P_M]; v.jz = p[LFDM_P_JZ];
    v.muf = p[LFDM_P_MUF]; v.mur = p[LFDM_P_MUR];
    fill_tail(v, c, m, p);
    std::memcpy(d.tire.v, p + LFDM_P_JW, 35 * sizeof(double));
}

static void fill_data(refgpu24::SimData& d, const lfdm_class18& c, const Maps& m, const double* p) {
    refgpu24::VehicleParam& v = d.veh;
    v.a = p[LFDM_P_A]; v.b = p[LFDM_P_B]; v.h = p[LFDM_P_H]; v.m = p[LFDM_P_M]; v.jz = p[LFDM_P_JZ];
    v.jx = p[LFDM_P_JX]; v.jy = p[LFDM_P_JY]; v.cf = p[LFDM_P_CF]; v.cr = p[LFDM_P_CR];
    v.muf = p[LFDM_P_MUF]; v.mur = p[LFDM_P_MUR]; v.hrcf = p[LFDM_P_HRCF]; v.hrcr = p[LFDM_P_HRCR];
    fill_tail(v, c, m, p);
    std::memcpy(d.tire.v, p + LFDM_P_JW, 35 * sizeof(double));
    d.sus.ks = p[LFDM_P_KS];
    d.sus.bs = p[LFDM_P_BS];
}

// Flat state vector <-> the model's SimState: every model's flat vector is its SimState's fields in
// order, one double slot each, with current_gr held as a double in the int's slot.
template <typename SS>
static void state_in(SS& s, const double* flat, int gear_slot) {
    std::memcpy(&s, flat, sizeof(SS));
    int g = (int)flat[gear_slot];
    std::memcpy(reinterpret_cast<char*>(&s) + gear_slot * sizeof(double), &g, sizeof(int));
}
template <typename SS>
static void state_out(const SS& s, double* flat, int gear_slot) {
    std::memcpy(flat, &s, sizeof(SS));
    int g = 0;
    std::memcpy(&g, reinterpret_cast<const char*>(&s) + gear_slot * sizeof(double), sizeof(int));
    flat[gear_slot] = g;
}

struct Run {
    int n, nrows, tpb;
    double dt, ksim, tend, dtout;
    lfdm_class18 cls;
    std::vector<double> P, T, S;
};

template <typename SD, typename SS>
static int launch(const Run& r, int ns, int gear_slot, unsigned channels, const char* cubin, const char* kernel,
                  std::vector<double>& out, std::vector<float>& ms) {
    DRV(cuInit(0));
    CUdevice dev;
    DRV(cuDeviceGet(&dev, 0));
    CUcontext ctx;
    DRV(cuDevicePrimaryCtxRetain(&ctx, dev));
    DRV(cuCtxSetCurrent(ctx));
    CUmodule mod;
    DRV(cuModuleLoad(&mod, cubin));
    CUfunction fn;
    DRV(cuModuleGetFunction(&fn, mod, kernel));
    const int n = r.n;
    Maps maps(r.cls);
    DriverInput* rows = managed<DriverInput>((size_t)n * r.nrows);
    std::memcpy(rows, r.T.data(), r.T.size() * sizeof(double));
    SD* data = managed<SD>(n);
    SS* st = managed<SS>(n);
    for (int i = 0; i < n; ++i) {
        std::memset(&data[i], 0, sizeof(SD));
        fill_data(data[i], r.cls, maps, &r.P[(size_t)i * LFDM_P_COUNT]);
        data[i].driver_data = rows + (size_t)i * r.nrows;
        data[i].driver_data_len = (unsigned)r.nrows;
        state_in(st[i], &r.S[(size_t)i * ns], gear_slot);
    }
    CUmemLocation loc;
    loc.type = CU_MEM_LOCATION_TYPE_DEVICE;
    loc.id = (int)dev;
    DRV(cuMemPrefetchAsync((CUdeviceptr)data, sizeof(SD) * n, loc, 0, 0));
    DRV(cuMemPrefetchAsync((CUdeviceptr)st, sizeof(SS) * n, loc, 0, 0));
    DRV(cuMemPrefetchAsync((CUdeviceptr)rows, sizeof(DriverInput) * (size_t)n * r.nrows, loc, 0, 0));
    DRV(cuCtxSynchronize());

    const bool output = r.dtout > 0;
    const size_t spw = output ? (size_t)(r.ksim / r.dtout + 0.999999) : 1;
    CUdeviceptr resp = 0;
    DRV(cuMemAlloc(&resp, sizeof(double) * (size_t)n * channels * spw));
    CUevent e0, e1;
    DRV(cuEventCreate(&e0, CU_EVENT_DEFAULT));
    DRV(cuEventCreate(&e1, CU_EVENT_DEFAULT));
    double current = 0.0;
    unsigned total = (unsigned)n;
    const unsigned blocks = (total + r.tpb - 1) / r.tpb;
    while (current < r.tend) {
        double t0 = current, ks = r.ksim, step = r.dt, dto = output ? r.dtout : 1.0;
        bool o = output;
        double* rp = reinterpret_cast<double*>(resp);
        SD* dp = data;
        SS* sp = st;
        unsigned cs = channels;
        void* args[] = {&t0, &ks, &step, &o, &total, &cs, &dto, &rp, &dp, &sp};
        DRV(cuEventRecord(e0, 0));
        DRV(cuLaunchKernel(fn, blocks, 1, 1, r.tpb, 1, 1, 0, 0, args, nullptr));
        DRV(cuEventRecord(e1, 0));
        DRV(cuEventSynchronize(e1));
        float t = 0;
        DRV(cuEventElapsedTime(&t, e0, e1));
        ms.push_back(t);
        current = current + r.ksim;
    }
    DRV(cuCtxSynchronize());
    out.assign((size_t)n * ns, 0.0);
    for (int i = 0; i < n; ++i) state_out(st[i], &out[(size_t)i * ns], gear_slot);
    return 0;
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
    Run r;
    if (!rd(f, hdr, 4) || !rd(f, dh, 4) || !rd(f, &r.cls, 1)) return 2;
    const int model = hdr[0];
    r.n = hdr[1];
    r.nrows = hdr[2];
    r.tpb = hdr[3];
    r.dt = dh[0];
    r.ksim = dh[1];
    r.tend = dh[2];
    r.dtout = dh[3];
    const int ns = model == 11 ? (int)LFDM11_S_COUNT : model == 24 ? (int)LFDM24_S_COUNT : (int)LFDM_S_COUNT;
    if ((model != 11 && model != 18 && model != 24) || r.n <= 0 || r.nrows <= 0 || r.tpb <= 0) return 2;
    r.P.resize((size_t)r.n * LFDM_P_COUNT);
    r.T.resize((size_t)r.n * r.nrows * 4);
    r.S.resize((size_t)r.n * ns);
    if (!rd(f, r.P.data(), r.P.size()) || !rd(f, r.T.data(), r.T.size()) || !rd(f, r.S.data(), r.S.size())) return 2;
    std::fclose(f);
    std::vector<double> out;
    std::vector<float> ms;
    int rc;
    if (model == 11)
        rc = launch<refgpu11::SimData, refgpu11::SimState>(r, ns, LFDM11_S_CURRENT_GR, 9, argv[1],
                                                           refgpu11::kIntegrateName, out, ms);
    else if (model == 24)
        rc = launch<refgpu24::SimData, refgpu24::SimState>(r, ns, LFDM24_S_CURRENT_GR, 15, argv[1],
                                                           refgpu24::kIntegrateName, out, ms);
    else
        rc = launch<refgpu18::SimData, refgpu18::SimState>(r, ns, LFDM_S_CURRENT_GR, 13, argv[1],
                                                           refgpu18::kIntegrateName, out, ms);
    if (rc) return rc;
    FILE* o = std::fopen(argv[3], "wb");
    if (!o) return 2;
    std::fwrite(out.data(), sizeof(double), out.size(), o);
    std::fclose(o);
    std::printf("{\"model\": %d, \"n\": %d, \"tpb\": %d, \"windows\": %zu, \"window_ms\": [", model, r.n, r.tpb,
                ms.size());
    for (size_t k = 0; k < ms.size(); ++k) std::printf("%s%.4f", k ? ", " : "", ms[k]);
    std::printf("]}\n");
    return 0;
}
