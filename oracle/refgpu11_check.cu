// Test infrastructure only: compile-time check (where the reference checkout exists) that
// refgpu11_layout.h matches the reference's d11GPU structs field by field. Built by `make refgpu`.
#include <cstdio>

#include "dof11_gpu.cuh"
#include "refgpu11_layout.h"

#define SAME(R, M, F) static_assert(offsetof(d11GPU::R, _##F) == offsetof(refgpu11::M, F), #R "::" #F)
SAME(VehicleParam, VehicleParam, a);
SAME(VehicleParam, VehicleParam, mur);
SAME(VehicleParam, VehicleParam, nonLinearSteer);
SAME(VehicleParam, VehicleParam, steerMap);
SAME(VehicleParam, VehicleParam, steerMapSize);
SAME(VehicleParam, VehicleParam, maxSteer);
SAME(VehicleParam, VehicleParam, crankInertia);
SAME(VehicleParam, VehicleParam, gearRatios);
SAME(VehicleParam, VehicleParam, noGears);
SAME(VehicleParam, VehicleParam, shiftMap);
SAME(VehicleParam, VehicleParam, tcbool);
SAME(VehicleParam, VehicleParam, maxBrakeTorque);
SAME(VehicleParam, VehicleParam, throttleMod);
SAME(VehicleParam, VehicleParam, powertrainMap);
SAME(VehicleParam, VehicleParam, powertrainMapSize);
SAME(VehicleParam, VehicleParam, lossesMap);
SAME(VehicleParam, VehicleParam, lossesMapSize);
SAME(VehicleParam, VehicleParam, CFmap);
SAME(VehicleParam, VehicleParam, CFmapSize);
SAME(VehicleParam, VehicleParam, TRmap);
SAME(VehicleParam, VehicleParam, TRmapSize);
SAME(VehicleParam, VehicleParam, driveType);
SAME(VehicleParam, VehicleParam, whichWheels);
static_assert(sizeof(d11GPU::VehicleParam) == sizeof(refgpu11::VehicleParam), "VehicleParam size");
static_assert(sizeof(d11GPU::TMeasyParam) == sizeof(refgpu11::TMeasyParam), "TMeasyParam size");
static_assert(offsetof(d11GPU::TMeasyParam, _kt) == 8 * sizeof(double), "TMeasyParam order");
static_assert(offsetof(d11GPU::TMeasyParam, _sysP2n) == 34 * sizeof(double), "TMeasyParam order");
static_assert(offsetof(d11GPU::SimData, _tireTM_param) == offsetof(refgpu11::SimData, tire), "SimData");
static_assert(offsetof(d11GPU::SimData, _driver_data) == offsetof(refgpu11::SimData, driver_data), "SimData");
static_assert(offsetof(d11GPU::SimData, _driver_data_len) == offsetof(refgpu11::SimData, driver_data_len), "SimData");
static_assert(sizeof(d11GPU::SimData) == sizeof(refgpu11::SimData), "SimData size");
static_assert(offsetof(d11GPU::VehicleState, _dOmega_crank) == 10 * sizeof(double), "VS order");
static_assert(offsetof(d11GPU::VehicleState, _current_gr) == offsetof(refgpu11::VehicleState, current_gr), "VS");
static_assert(sizeof(d11GPU::TMeasyState) == sizeof(refgpu11::TMeasyState), "TS size");
static_assert(offsetof(d11GPU::TMeasyState, _engTor) == 14 * sizeof(double), "TS order");
static_assert(offsetof(d11GPU::SimState, _tirer_state) == offsetof(refgpu11::SimState, tire[1]), "SimState");
static_assert(sizeof(d11GPU::SimState) == sizeof(refgpu11::SimState), "SimState size");

int main() {
    std::printf("refgpu11 layout matches the reference headers\n");
    return 0;
}
