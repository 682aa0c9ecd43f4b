// d11SolverHalfImplicitGPU over liblfdm (11dof-gpu/dof11_halfImplicit_gpu.cuh:16 of the reference)
// and the 11-DOF state structs of namespace d11GPU (11dof-gpu/dof11_gpu.cuh:704-765 and the tire
// state structs before it). See lfdm_solver.hpp for the error behaviour and the functor SolveStep.
// The library steps the 11-DOF model with TMeasy tires; Construct with TireType::TMeasyNr reports
// an error.
#pragma once

#include "lfdm_solver.hpp"

namespace d11GPU {

struct TMeasyState {
    double _xe = 0, _ye = 0, _xedot = 0, _yedot = 0, _omega = 0, _dOmega = 0, _xt = 0, _rStat = 0, _fx = 0,
           _fy = 0, _fz = 0, _vsx = 0, _vsy = 0, _My = 0, _engTor = 0;
};
struct TMeasyNrState {
    double _omega = 0, _dOmega = 0, _xt = 0, _rStat = 0, _fx = 0, _fy = 0, _fz = 0, _vsx = 0, _vsy = 0, _My = 0,
           _engTor = 0;
};
struct VehicleState {
    double _x = 0, _y = 0, _u = 0, _v = 0, _psi = 0, _wz = 0, _udot = 0, _vdot = 0, _wzdot = 0, _crankOmega = 0,
           _dOmega_crank = 0;
    int _current_gr = 0;
};
struct SimState {
    VehicleState _veh_state;
    TMeasyState _tiref_state, _tirer_state;
};
struct SimStateNr {
    VehicleState _veh_state;
    TMeasyNrState _tiref_state, _tirer_state;
};

namespace detail {
constexpr double VehicleState::*const kVeh[] = {
    &VehicleState::_x,    &VehicleState::_y,     &VehicleState::_u,          &VehicleState::_v,
    &VehicleState::_psi,  &VehicleState::_wz,    &VehicleState::_udot,       &VehicleState::_vdot,
    &VehicleState::_wzdot, &VehicleState::_crankOmega, &VehicleState::_dOmega_crank};
constexpr double TMeasyState::*const kTire[] = {
    &TMeasyState::_xe,  &TMeasyState::_ye,  &TMeasyState::_xedot, &TMeasyState::_yedot, &TMeasyState::_omega,
    &TMeasyState::_dOmega, &TMeasyState::_xt, &TMeasyState::_rStat, &TMeasyState::_fx,  &TMeasyState::_fy,
    &TMeasyState::_fz,  &TMeasyState::_vsx, &TMeasyState::_vsy,   &TMeasyState::_My,    &TMeasyState::_engTor};
constexpr double TMeasyNrState::*const kTireNr[] = {
    &TMeasyNrState::_omega, &TMeasyNrState::_dOmega, &TMeasyNrState::_xt,  &TMeasyNrState::_rStat,
    &TMeasyNrState::_fx,    &TMeasyNrState::_fy,     &TMeasyNrState::_fz,  &TMeasyNrState::_vsx,
    &TMeasyNrState::_vsy,   &TMeasyNrState::_My,     &TMeasyNrState::_engTor};
static_assert(sizeof(kVeh) / sizeof(kVeh[0]) == LFDM11_S_CURRENT_GR, "vehicle block of the flat state");

inline void put_vehicle(const VehicleState& v, double* s) {
    lfdm_cpp::put(v, kVeh, s);
    s[LFDM11_S_CURRENT_GR] = static_cast<double>(v._current_gr);
}
inline void get_vehicle(VehicleState& v, const double* s) {
    lfdm_cpp::get(v, kVeh, s);
    v._current_gr = static_cast<int>(s[LFDM11_S_CURRENT_GR]);
}
inline double* tire(double* s, int k) { return s + LFDM11_S_TIRE0 + k * LFDM_S_TIRE_STRIDE; }
}  // namespace detail

}  // namespace d11GPU

class d11SolverHalfImplicitGPU : public lfdm_cpp::SolverBase<LFDM_MODEL_11> {
  public:
    explicit d11SolverHalfImplicitGPU(unsigned int total_num_vehicles) : SolverBase(total_num_vehicles) {}

    void Construct(const std::string& veh_params_file, const std::string& tire_params_file,
                   unsigned int num_vehicles, const std::string& driver_file) {
        construct(veh_params_file, tire_params_file, nullptr, num_vehicles, &driver_file, TireType::TMeasy);
    }
    void Construct(const std::string& vehicle_params_file, const std::string& tire_params_file,
                   unsigned int num_vehicles, const std::string& driver_inputs_file, TireType type) {
        construct(vehicle_params_file, tire_params_file, nullptr, num_vehicles, &driver_inputs_file, type);
    }
    void Construct(const std::string& vehicle_params_file, const std::string& tire_params_file,
                   unsigned int num_vehicles) {
        construct(vehicle_params_file, tire_params_file, nullptr, num_vehicles, nullptr, TireType::TMeasy);
    }
    void Construct(const std::string& vehicle_params_file, const std::string& tire_params_file,
                   unsigned int num_vehicles, TireType type) {
        construct(vehicle_params_file, tire_params_file, nullptr, num_vehicles, nullptr, type);
    }

    void Initialize(d11GPU::VehicleState& vehicle_states, d11GPU::TMeasyState& tire_states_F,
                    d11GPU::TMeasyState& tire_states_R, unsigned int num_vehicles) {
        std::vector<double> s(LFDM11_S_COUNT, 0.0);
        d11GPU::detail::put_vehicle(vehicle_states, s.data());
        lfdm_cpp::put(tire_states_F, d11GPU::detail::kTire, d11GPU::detail::tire(s.data(), 0));
        lfdm_cpp::put(tire_states_R, d11GPU::detail::kTire, d11GPU::detail::tire(s.data(), 1));
        initialize(s, num_vehicles);
    }
    void Initialize(d11GPU::VehicleState& vehicle_states, d11GPU::TMeasyNrState& tire_states_F,
                    d11GPU::TMeasyNrState& tire_states_R, unsigned int num_vehicles) {
        std::vector<double> s(LFDM11_S_COUNT, 0.0);
        d11GPU::detail::put_vehicle(vehicle_states, s.data());
        lfdm_cpp::put(tire_states_F, d11GPU::detail::kTireNr, d11GPU::detail::tire(s.data(), 0) + LFDM_T_OMEGA);
        lfdm_cpp::put(tire_states_R, d11GPU::detail::kTireNr, d11GPU::detail::tire(s.data(), 1) + LFDM_T_OMEGA);
        initialize(s, num_vehicles);
    }

    d11GPU::SimState GetSimState(unsigned int vehicle_index) {
        std::vector<double> s = flat_state(vehicle_index, LFDM11_S_COUNT);
        d11GPU::SimState out;
        d11GPU::detail::get_vehicle(out._veh_state, s.data());
        lfdm_cpp::get(out._tiref_state, d11GPU::detail::kTire, d11GPU::detail::tire(s.data(), 0));
        lfdm_cpp::get(out._tirer_state, d11GPU::detail::kTire, d11GPU::detail::tire(s.data(), 1));
        return out;
    }
};
