// Test infrastructure only: compile-time check (where the reference checkout exists) that
// refgpu24_layout.h matches the reference's d24GPU structs field by field. Built by `make refgpu`.
#include <cstdio>

#include "dof24_gpu.cuh"
#include "refgpu24_layout.h"

#define SAME(R, M, F) static_assert(offsetof(d24GPU::R, _##F) == offsetof(refgpu24::M, F), #R "::" #F)
SAME(VehicleParam, VehicleParam, a);
SAME(VehicleParam, VehicleParam, jy);
SAME(VehicleParam, VehicleParam, hrcr);
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
static_assert(sizeof(d24GPU::VehicleParam) == sizeof(refgpu24::VehicleParam), "VehicleParam size");
static_assert(sizeof(d24GPU::TMeasyParam) == sizeof(refgpu24::TMeasyParam), "TMeasyParam size");
static_assert(offsetof(d24GPU::TMeasyParam, _kt) == 8 * sizeof(double), "TMeasyParam order");
static_assert(offsetof(d24GPU::TMeasyParam, _sysP2n) == 34 * sizeof(double), "TMeasyParam order");
static_assert(offsetof(d24GPU::SuspensionParam, _bs) == offsetof(refgpu24::SuspensionParam, bs), "Sus");
static_assert(offsetof(d24GPU::SimData, _tireTM_params) == offsetof(refgpu24::SimData, tire), "SimData");
static_assert(offsetof(d24GPU::SimData, _sus_params) == offsetof(refgpu24::SimData, sus), "SimData");
static_assert(offsetof(d24GPU::SimData, _driver_data) == offsetof(refgpu24::SimData, driver_data), "SimData");
static_assert(offsetof(d24GPU::SimData, _driver_data_len) == offsetof(refgpu24::SimData, driver_data_len), "SimData");
static_assert(sizeof(d24GPU::SimData) == sizeof(refgpu24::SimData), "SimData size");
static_assert(offsetof(d24GPU::VehicleState, _dOmega_crank) == 22 * sizeof(double), "VS order");
static_assert(offsetof(d24GPU::VehicleState, _current_gr) == offsetof(refgpu24::VehicleState, current_gr), "VS");
static_assert(sizeof(d24GPU::TMeasyState) == sizeof(refgpu24::TMeasyState), "TS size");
static_assert(offsetof(d24GPU::TMeasyState, _engTor) == 22 * sizeof(double), "TS order");
static_assert(sizeof(d24GPU::SuspensionState) == sizeof(refgpu24::SuspensionState), "SusState size");
static_assert(offsetof(d24GPU::SuspensionState, _mz) == 23 * sizeof(double), "SusState order");
static_assert(offsetof(d24GPU::SimState, _tirelf_st) == offsetof(refgpu24::SimState, tire[0]), "SimState");
static_assert(offsetof(d24GPU::SimState, _tirerr_st) == offsetof(refgpu24::SimState, tire[3]), "SimState");
static_assert(offsetof(d24GPU::SimState, _suslf_st) == offsetof(refgpu24::SimState, sus[0]), "SimState");
static_assert(offsetof(d24GPU::SimState, _susrr_st) == offsetof(refgpu24::SimState, sus[3]), "SimState");
static_assert(sizeof(d24GPU::SimState) == sizeof(refgpu24::SimState), "SimState size");

int main() {
    std::printf("refgpu24 layout matches the reference headers\n");
    return 0;
}
