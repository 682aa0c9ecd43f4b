// d18SolverHalfImplicitGPU over liblfdm (18dof-gpu/dof18_halfImplicit_gpu.cuh:15-343 of the
// reference) and the 18-DOF state structs of namespace d18GPU (18dof-gpu/dof18_gpu.cuh:164-253,
// :719-810, :861-905). See lfdm_solver.hpp for the error behaviour and the functor SolveStep.
#pragma once

#include "lfdm_solver.hpp"

namespace d18GPU {

// TMeasyState (dof18_gpu.cuh:164-253); the flat tire block of lfdm.h (LFDM_T_*) in this order.
struct TMeasyState {
    double _xe = 0, _ye = 0, _xedot = 0, _yedot = 0, _omega = 0, _dOmega = 0, _xt = 0, _rStat = 0, _fx = 0,
           _fy = 0, _fz = 0, _vsx = 0, _vsy = 0, _My = 0, _engTor = 0;
};
// TMeasyNrState: the TMeasy fields from _omega on (the TMeasyNr tire has no deflection states).
struct TMeasyNrState {
    double _omega = 0, _dOmega = 0, _xt = 0, _rStat = 0, _fx = 0, _fy = 0, _fz = 0, _vsx = 0, _vsy = 0, _My = 0,
           _engTor = 0;
};
// VehicleState (dof18_gpu.cuh:719-810).
struct VehicleState {
    double _x = 0, _y = 0, _u = 0, _v = 0, _psi = 0, _wz = 0, _phi = 0, _wx = 0, _udot = 0, _vdot = 0, _wxdot = 0,
           _wzdot = 0, _crankOmega = 0, _dOmega_crank = 0;
    int _current_gr = 0;
};
struct SimState {
    VehicleState _veh_state;
    TMeasyState _tirelf_state, _tirerf_state, _tirelr_state, _tirerr_state;
};
struct SimStateNr {
    VehicleState _veh_state;
    TMeasyNrState _tirelf_state, _tirerf_state, _tirelr_state, _tirerr_state;
};

namespace detail {
constexpr double VehicleState::*const kVeh[] = {
    &VehicleState::_x,    &VehicleState::_y,     &VehicleState::_u,     &VehicleState::_v,
    &VehicleState::_psi,  &VehicleState::_wz,    &VehicleState::_phi,   &VehicleState::_wx,
    &VehicleState::_udot, &VehicleState::_vdot,  &VehicleState::_wxdot, &VehicleState::_wzdot,
    &VehicleState::_crankOmega, &VehicleState::_dOmega_crank};
constexpr double TMeasyState::*const kTire[] = {
    &TMeasyState::_xe,  &TMeasyState::_ye,  &TMeasyState::_xedot, &TMeasyState::_yedot, &TMeasyState::_omega,
    &TMeasyState::_dOmega, &TMeasyState::_xt, &TMeasyState::_rStat, &TMeasyState::_fx,  &TMeasyState::_fy,
    &TMeasyState::_fz,  &TMeasyState::_vsx, &TMeasyState::_vsy,   &TMeasyState::_My,    &TMeasyState::_engTor};
constexpr double TMeasyNrState::*const kTireNr[] = {
    &TMeasyNrState::_omega, &TMeasyNrState::_dOmega, &TMeasyNrState::_xt,  &TMeasyNrState::_rStat,
    &TMeasyNrState::_fx,    &TMeasyNrState::_fy,     &TMeasyNrState::_fz,  &TMeasyNrState::_vsx,
    &TMeasyNrState::_vsy,   &TMeasyNrState::_My,     &TMeasyNrState::_engTor};
static_assert(sizeof(kVeh) / sizeof(kVeh[0]) == LFDM_S_CURRENT_GR, "vehicle block of the flat state");
static_assert(sizeof(kTire) / sizeof(kTire[0]) == LFDM_S_TIRE_STRIDE, "tire block of the flat state");

inline void put_vehicle(const VehicleState& v, double* s) {
    lfdm_cpp::put(v, kVeh, s);
    s[LFDM_S_CURRENT_GR] = static_cast<double>(v._current_gr);
}
inline void get_vehicle(VehicleState& v, const double* s) {
    lfdm_cpp::get(v, kVeh, s);
    v._current_gr = static_cast<int>(s[LFDM_S_CURRENT_GR]);
}
inline double* tire(double* s, int k) { return s + LFDM_S_TIRE0 + k * LFDM_S_TIRE_STRIDE; }
}  // namespace detail

}  // namespace d18GPU

class d18SolverHalfImplicitGPU : public lfdm_cpp::SolverBase<LFDM_MODEL_18> {
  public:
    explicit d18SolverHalfImplicitGPU(unsigned int total_num_vehicles) : SolverBase(total_num_vehicles) {}

    // Construct overloads (dof18_halfImplicit_gpu.cuh:34-87): each call appends num_vehicles
    // vehicles of the parameter files, driven by the driver file when one is given.
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

    // Initialize (dof18_halfImplicit_gpu.cuh:172-195): the next num_vehicles vehicles start from
    // these states.
    void Initialize(d18GPU::VehicleState& vehicle_states, d18GPU::TMeasyState& tire_states_LF,
                    d18GPU::TMeasyState& tire_states_RF, d18GPU::TMeasyState& tire_states_LR,
                    d18GPU::TMeasyState& tire_states_RR, unsigned int num_vehicles) {
        std::vector<double> s(LFDM_S_COUNT, 0.0);
        d18GPU::detail::put_vehicle(vehicle_states, s.data());
        const d18GPU::TMeasyState* t[4] = {&tire_states_LF, &tire_states_RF, &tire_states_LR, &tire_states_RR};
        for (int k = 0; k < 4; ++k) lfdm_cpp::put(*t[k], d18GPU::detail::kTire, d18GPU::detail::tire(s.data(), k));
        initialize(s, num_vehicles);
    }
    void Initialize(d18GPU::VehicleState& vehicle_states, d18GPU::TMeasyNrState& tire_states_LF,
                    d18GPU::TMeasyNrState& tire_states_RF, d18GPU::TMeasyNrState& tire_states_LR,
                    d18GPU::TMeasyNrState& tire_states_RR, unsigned int num_vehicles) {
        std::vector<double> s(LFDM_S_COUNT, 0.0);
        d18GPU::detail::put_vehicle(vehicle_states, s.data());
        const d18GPU::TMeasyNrState* t[4] = {&tire_states_LF, &tire_states_RF, &tire_states_LR, &tire_states_RR};
        for (int k = 0; k < 4; ++k)
            lfdm_cpp::put(*t[k], d18GPU::detail::kTireNr, d18GPU::detail::tire(s.data(), k) + LFDM_T_OMEGA);
        initialize(s, num_vehicles);
    }

    // GetSimState (dof18_halfImplicit_gpu.cu:667-682). TMeasyNr vehicles report zero deflections.
    d18GPU::SimState GetSimState(unsigned int vehicle_index) {
        std::vector<double> s = flat_state(vehicle_index, LFDM_S_COUNT);
        d18GPU::SimState out;
        d18GPU::detail::get_vehicle(out._veh_state, s.data());
        d18GPU::TMeasyState* t[4] = {&out._tirelf_state, &out._tirerf_state, &out._tirelr_state, &out._tirerr_state};
        for (int k = 0; k < 4; ++k) lfdm_cpp::get(*t[k], d18GPU::detail::kTire, d18GPU::detail::tire(s.data(), k));
        return out;
    }
};
