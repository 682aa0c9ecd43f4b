// Test infrastructure only. Memory layout of the reference 11-DOF GPU solver's per-vehicle records
// (d11GPU::SimData / SimState, 11dof-gpu/dof11_gpu.cuh:24-840), written out so that a launcher
// without the reference headers can build the records its Integrate kernel reads.
// refgpu11_check.cu compares every offset with the reference headers where they exist.
#pragma once
#include <cstddef>

#include "refgpu18_layout.h"  // MapEntry, DriverInput, TMeasyParam, TMeasyState are the same records

namespace refgpu11 {

using refgpu18::DriverInput;
using refgpu18::MapEntry;
using refgpu18::TMeasyParam;
using refgpu18::TMeasyState;

struct VehicleParam {
    double a, b, h, m, jz, muf, mur;
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
struct VehicleState {  // 11 doubles + int, field order of d11GPU::VehicleState (== LFDM11_S_X..CURRENT_GR)
    double v[11];
    int current_gr;
};
struct SimState {  // == the flat LFDM11_S_* vector (42 slots)
    VehicleState veh;
    TMeasyState tire[2];  // front, rear
};

static_assert(sizeof(SimState) == 42 * sizeof(double), "SimState layout");

// Integrate(double, double, double, bool, unsigned, unsigned, double, double*, SimData*, SimState*)
// (11dof-gpu/dof11_halfImplicit_gpu.cu:837-916).
constexpr const char* kIntegrateName = "_Z9IntegratedddbjjdPdPN6d11GPU7SimDataEPNS0_8SimStateE";

}  // namespace refgpu11
