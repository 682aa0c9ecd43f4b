// Test infrastructure only. Memory layout of the reference 24-DOF GPU solver's per-vehicle records
// (d24GPU::SimData / SimState, 24dof-gpu/dof24_gpu.cuh:25-1230), written out so that a launcher
// without the reference headers can build the records its Integrate kernel reads.
// refgpu24_check.cu compares every offset with the reference headers where they exist.
#pragma once
#include <cstddef>

#include "refgpu18_layout.h"  // MapEntry, DriverInput, TMeasyParam are the same records

namespace refgpu24 {

using refgpu18::DriverInput;
using refgpu18::MapEntry;
using refgpu18::TMeasyParam;

struct VehicleParam {
    double a, b, h, m, jz, jx, jy, cf, cr, muf, mur, hrcf, hrcr;
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
struct SuspensionParam {
    double ks, bs;
};
struct SimData {
    VehicleParam veh;
    TMeasyParam tire;
    SuspensionParam sus;
    DriverInput* driver_data;
    unsigned driver_data_len;
};
struct VehicleState {  // 23 doubles + int (== LFDM24_S_X..CURRENT_GR)
    double v[23];
    int current_gr;
};
struct TMeasyState {  // 23 doubles (== LFDM24_T_*)
    double v[23];
};
struct SuspensionState {  // 24 doubles (== LFDM24_SUS_*)
    double v[24];
};
struct SimState {  // == the flat LFDM24_S_* vector (212 slots)
    VehicleState veh;
    TMeasyState tire[4];          // LF, RF, LR, RR
    SuspensionState sus[4];       // LF, RF, LR, RR
};

static_assert(sizeof(SimState) == 212 * sizeof(double), "SimState layout");

// Integrate(double, double, double, bool, unsigned, unsigned, double, double*, SimData*, SimState*)
// (24dof-gpu/dof24_halfImplicit_gpu.cu:982-1113).
constexpr const char* kIntegrateName = "_Z9IntegratedddbjjdPdPN6d24GPU7SimDataEPNS0_8SimStateE";

}  // namespace refgpu24
