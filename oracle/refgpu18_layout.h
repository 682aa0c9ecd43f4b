// Test infrastructure only. Memory layout of the reference GPU solver's per-vehicle records
// (d18GPU::SimData / SimState, 18dof-gpu/dof18_gpu.cuh:25-905), written out so that a launcher
// without the reference headers can build the records its Integrate kernel reads.
// refgpu18_check.cu compares every offset with the reference headers where they exist.
#pragma once
#include <cstddef>

namespace refgpu18 {

struct MapEntry {
    double x, y;
};
struct DriverInput {
    double t, steering, throttle, braking;
};
struct TMeasyParam {  // 35 doubles in the field order of d18GPU::TMeasyParam (== LFDM_P_JW..LFDM_P_SYSP2N)
    double v[35];
};
struct VehicleParam {
    double a, b, h, m, jz, jx, jxz, cf, cr, muf, mur, hrcf, hrcr, krof, kror, brof, bror;
    bool nonLinearSteer;
    MapEntry* steerMap;
    int steerMapSize;
    double maxSteer;
    double crankInertia;
    double* gearRatios;
    int noGears;
    MapEntry* shiftMap;
    bool tcbool;
    double maxBrakeTorque;
    bool throttleMod;
    MapEntry* powertrainMap;
    int powertrainMapSize;
    MapEntry* lossesMap;
    int lossesMapSize;
    MapEntry* CFmap;
    int CFmapSize;
    MapEntry* TRmap;
    int TRmapSize;
    bool driveType;
    bool whichWheels;
};
struct SimData {
    VehicleParam veh;
    TMeasyParam tire;
    DriverInput* driver_data;
    unsigned driver_data_len;
};
struct VehicleState {  // 14 doubles + int, field order of d18GPU::VehicleState (== LFDM_S_X..CURRENT_GR)
    double v[14];
    int current_gr;
};
struct TMeasyState {  // 15 doubles (== LFDM_T_XE..LFDM_T_ENGTOR)
    double v[15];
};
struct SimState {
    VehicleState veh;
    TMeasyState tire[4];
};

static_assert(sizeof(VehicleParam) == 288, "VehicleParam layout");
static_assert(sizeof(TMeasyParam) == 280, "TMeasyParam layout");
static_assert(sizeof(SimData) == 584, "SimData layout");
static_assert(sizeof(SimState) == 600, "SimState layout");

// Mangled name of the table-driven kernel
// Integrate(double, double, double, bool, unsigned, unsigned, double, double*, SimData*, SimState*)
// (18dof-gpu/dof18_halfImplicit_gpu.cu:882-977).
constexpr const char* kIntegrateName = "_Z9IntegratedddbjjdPdPN6d18GPU7SimDataEPNS0_8SimStateE";

}  // namespace refgpu18
