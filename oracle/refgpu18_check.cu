// Test infrastructure only: compile-time check (where the reference checkout exists) that
// refgpu18_layout.h matches the reference's d18GPU structs field by field. Built by `make refgpu`.
#include <cstdio>

#include "dof18_gpu.cuh"
#include "refgpu18_layout.h"

#define SAME(R, M, F) static_assert(offsetof(d18GPU::R, _##F) == offsetof(refgpu18::M, F), #R "::" #F)
SAME(VehicleParam, VehicleParam, a);
SAME(VehicleParam, VehicleParam, bror);
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
static_assert(sizeof(d18GPU::VehicleParam) == sizeof(refgpu18::VehicleParam), "VehicleParam size");
static_assert(sizeof(d18GPU::TMeasyParam) == sizeof(refgpu18::TMeasyParam), "TMeasyParam size");
static_assert(offsetof(d18GPU::TMeasyParam, _sysP2n) == 34 * sizeof(double), "TMeasyParam order");
static_assert(offsetof(d18GPU::TMeasyParam, _kt) == 8 * sizeof(double), "TMeasyParam order");
static_assert(offsetof(d18GPU::SimData, _tireTM_param) == offsetof(refgpu18::SimData, tire), "SimData");
static_assert(offsetof(d18GPU::SimData, _driver_data) == offsetof(refgpu18::SimData, driver_data), "SimData");
static_assert(offsetof(d18GPU::SimData, _driver_data_len) == offsetof(refgpu18::SimData, driver_data_len), "SimData");
static_assert(sizeof(d18GPU::SimData) == sizeof(refgpu18::SimData), "SimData size");
static_assert(offsetof(d18GPU::VehicleState, _current_gr) == offsetof(refgpu18::VehicleState, current_gr), "VS");
static_assert(offsetof(d18GPU::VehicleState, _dOmega_crank) == 13 * sizeof(double), "VS order");
static_assert(offsetof(d18GPU::TMeasyState, _engTor) == 14 * sizeof(double), "TS order");
static_assert(offsetof(d18GPU::SimState, _tirerr_state) == offsetof(refgpu18::SimState, tire[3]), "SimState");
static_assert(sizeof(d18GPU::SimState) == sizeof(refgpu18::SimState), "SimState size");

int main() {
    std::printf("refgpu18 layout matches the reference headers\n");
    return 0;
}
