// d24SolverHalfImplicitGPU over liblfdm (24dof-gpu/dof24_halfImplicit_gpu.cuh:15 of the reference)
// and the 24-DOF state structs of namespace d24GPU (24dof-gpu/dof24_gpu.cuh: TMeasyState,
// TMeasyNrState, VehicleState, SuspensionState, SimState). See lfdm_solver.hpp for the error
// behaviour and the functor SolveStep. Initialize fills the tire and suspension states from the
// vehicle's parameters as the reference's initializeTireSus does (24dof-gpu/dof24_gpu.cu:34-90),
// so the vehicles must be constructed first. The library steps the 24-DOF model with TMeasy tires;
// Construct with TireType::TMeasyNr reports an error.
#pragma once

#include "lfdm_solver.hpp"

namespace d24GPU {

struct TMeasyState {
    double _xe = 0, _ye = 0, _xedot = 0, _yedot = 0, _omega = 0, _dOmega = 0, _xt = 0, _dxt = 0, _rStat = 0,
           _fx = 0, _fy = 0, _fz = 0, _fxg = 0, _fyg = 0, _fzg = 0, _vgx = 0, _vgy = 0, _vgz = 0, _vsx = 0,
           _vsy = 0, _vsz = 0, _My = 0, _engTor = 0;
};
struct TMeasyNrState {
    double _omega = 0, _dOmega = 0, _xt = 0, _dxt = 0, _rStat = 0, _fx = 0, _fy = 0, _fz = 0, _fxg = 0, _fyg = 0,
           _fzg = 0, _vgx = 0, _vgy = 0, _vgz = 0, _vsx = 0, _vsy = 0, _vsz = 0, _My = 0, _engTor = 0;
};
struct VehicleState {
    double _x = 0, _y = 0, _z = 0, _u = 0, _v = 0, _w = 0, _psi = 0, _wz = 0, _phi = 0, _wx = 0, _theta = 0,
           _wy = 0, _udot = 0, _vdot = 0, _wdot = 0, _wxdot = 0, _wydot = 0, _wzdot = 0, _dtheta = 0, _dphi = 0,
           _dpsi = 0, _crankOmega = 0, _dOmega_crank = 0;
    int _current_gr = 0;
};
struct SuspensionState {
    double _xs = 0, _xsi = 0, _dxs = 0, _ls = 0, _lsi = 0, _us = 0, _vs = 0, _ws = 0, _dus = 0, _dvs = 0,
           _dws = 0, _uu = 0, _vu = 0, _wu = 0, _duu = 0, _dvu = 0, _dwu = 0, _fxs = 0, _fys = 0, _fzs = 0,
           _fzd = 0, _mx = 0, _my = 0, _mz = 0;
};
struct SimState {
    SimState() {}
    SimState(VehicleState v_states, TMeasyState tirelf_st, TMeasyState tirerf_st, TMeasyState tirelr_st,
             TMeasyState tirerr_st, SuspensionState suslf_st, SuspensionState susrf_st, SuspensionState suslr_st,
             SuspensionState susrr_st)
        : _v_states(v_states), _tirelf_st(tirelf_st), _tirerf_st(tirerf_st), _tirelr_st(tirelr_st),
          _tirerr_st(tirerr_st), _suslf_st(suslf_st), _susrf_st(susrf_st), _suslr_st(suslr_st),
          _susrr_st(susrr_st) {}
    VehicleState _v_states;
    TMeasyState _tirelf_st, _tirerf_st, _tirelr_st, _tirerr_st;
    SuspensionState _suslf_st, _susrf_st, _suslr_st, _susrr_st;
};
struct SimStateNr {
    SimStateNr() {}
    SimStateNr(VehicleState v_states, TMeasyNrState tirelf_st, TMeasyNrState tirerf_st, TMeasyNrState tirelr_st,
               TMeasyNrState tirerr_st, SuspensionState suslf_st, SuspensionState susrf_st,
               SuspensionState suslr_st, SuspensionState susrr_st)
        : _v_states(v_states), _tirelf_st(tirelf_st), _tirerf_st(tirerf_st), _tirelr_st(tirelr_st),
          _tirerr_st(tirerr_st), _suslf_st(suslf_st), _susrf_st(susrf_st), _suslr_st(suslr_st),
          _susrr_st(susrr_st) {}
    VehicleState _v_states;
    TMeasyNrState _tirelf_st, _tirerf_st, _tirelr_st, _tirerr_st;
    SuspensionState _suslf_st, _susrf_st, _suslr_st, _susrr_st;
};

namespace detail {
using V = VehicleState;
constexpr double V::*const kVeh[] = {&V::_x,      &V::_y,      &V::_z,     &V::_u,      &V::_v,       &V::_w,
                                     &V::_psi,    &V::_wz,     &V::_phi,   &V::_wx,     &V::_theta,   &V::_wy,
                                     &V::_udot,   &V::_vdot,   &V::_wdot,  &V::_wxdot,  &V::_wydot,   &V::_wzdot,
                                     &V::_dtheta, &V::_dphi,   &V::_dpsi,  &V::_crankOmega, &V::_dOmega_crank};
using T = TMeasyState;
constexpr double T::*const kTire[] = {&T::_xe,  &T::_ye,  &T::_xedot, &T::_yedot, &T::_omega, &T::_dOmega,
                                      &T::_xt,  &T::_dxt, &T::_rStat, &T::_fx,    &T::_fy,    &T::_fz,
                                      &T::_fxg, &T::_fyg, &T::_fzg,   &T::_vgx,   &T::_vgy,   &T::_vgz,
                                      &T::_vsx, &T::_vsy, &T::_vsz,   &T::_My,    &T::_engTor};
using TN = TMeasyNrState;
constexpr double TN::*const kTireNr[] = {&TN::_omega, &TN::_dOmega, &TN::_xt,  &TN::_dxt, &TN::_rStat,
                                         &TN::_fx,    &TN::_fy,     &TN::_fz,  &TN::_fxg, &TN::_fyg,
                                         &TN::_fzg,   &TN::_vgx,    &TN::_vgy, &TN::_vgz, &TN::_vsx,
                                         &TN::_vsy,   &TN::_vsz,    &TN::_My,  &TN::_engTor};
using S = SuspensionState;
constexpr double S::*const kSus[] = {&S::_xs,  &S::_xsi, &S::_dxs, &S::_ls,  &S::_lsi, &S::_us,  &S::_vs,  &S::_ws,
                                     &S::_dus, &S::_dvs, &S::_dws, &S::_uu,  &S::_vu,  &S::_wu,  &S::_duu, &S::_dvu,
                                     &S::_dwu, &S::_fxs, &S::_fys, &S::_fzs, &S::_fzd, &S::_mx,  &S::_my,  &S::_mz};
static_assert(sizeof(kVeh) / sizeof(kVeh[0]) == LFDM24_S_CURRENT_GR, "vehicle block of the flat state");
static_assert(sizeof(kTire) / sizeof(kTire[0]) == LFDM24_T_COUNT, "tire block of the flat state");
static_assert(sizeof(kSus) / sizeof(kSus[0]) == LFDM24_SUS_COUNT, "suspension block of the flat state");

inline void put_vehicle(const VehicleState& v, double* s) {
    lfdm_cpp::put(v, kVeh, s);
    s[LFDM24_S_CURRENT_GR] = static_cast<double>(v._current_gr);
}
inline void get_vehicle(VehicleState& v, const double* s) {
    lfdm_cpp::get(v, kVeh, s);
    v._current_gr = static_cast<int>(s[LFDM24_S_CURRENT_GR]);
}
inline double* tire(double* s, int k) { return s + LFDM24_S_TIRE0 + k * LFDM24_T_COUNT; }
inline double* sus(double* s, int k) { return s + LFDM24_S_SUS0 + k * LFDM24_SUS_COUNT; }
}  // namespace detail

}  // namespace d24GPU

class d24SolverHalfImplicitGPU : public lfdm_cpp::SolverBase<LFDM_MODEL_24> {
  public:
    explicit d24SolverHalfImplicitGPU(unsigned int num_vehicles) : SolverBase(num_vehicles) {}

    // Construct overloads (24dof-gpu/dof24_halfImplicit_gpu.cuh): the suspension file follows the
    // tire file.
    void Construct(const std::string& veh_params_file, const std::string& tire_params_file,
                   const std::string& sus_params_file, unsigned int num_vehicles, const std::string& driver_file) {
        construct(veh_params_file, tire_params_file, &sus_params_file, num_vehicles, &driver_file, TireType::TMeasy);
    }
    void Construct(const std::string& vehicle_params_file, const std::string& tire_params_file,
                   const std::string& sus_params_file, unsigned int num_vehicles,
                   const std::string& driver_inputs_file, TireType type) {
        construct(vehicle_params_file, tire_params_file, &sus_params_file, num_vehicles, &driver_inputs_file, type);
    }
    void Construct(const std::string& vehicle_params_file, const std::string& tire_params_file,
                   const std::string& sus_params_file, unsigned int num_vehicles) {
        construct(vehicle_params_file, tire_params_file, &sus_params_file, num_vehicles, nullptr, TireType::TMeasy);
    }
    void Construct(const std::string& vehicle_params_file, const std::string& tire_params_file,
                   const std::string& sus_params_file, unsigned int num_vehicles, TireType type) {
        construct(vehicle_params_file, tire_params_file, &sus_params_file, num_vehicles, nullptr, type);
    }

    void Initialize(d24GPU::VehicleState& vehicle_states, d24GPU::TMeasyState& tire_states_LF,
                    d24GPU::TMeasyState& tire_states_RF, d24GPU::TMeasyState& tire_states_LR,
                    d24GPU::TMeasyState& tire_states_RR, d24GPU::SuspensionState& sus_states_LF,
                    d24GPU::SuspensionState& sus_states_RF, d24GPU::SuspensionState& sus_states_LR,
                    d24GPU::SuspensionState& sus_states_RR, unsigned int num_vehicles) {
        std::vector<double> s(LFDM24_S_COUNT, 0.0);
        d24GPU::detail::put_vehicle(vehicle_states, s.data());
        const d24GPU::TMeasyState* t[4] = {&tire_states_LF, &tire_states_RF, &tire_states_LR, &tire_states_RR};
        for (int k = 0; k < 4; ++k) lfdm_cpp::put(*t[k], d24GPU::detail::kTire, d24GPU::detail::tire(s.data(), k));
        put_sus(s.data(), sus_states_LF, sus_states_RF, sus_states_LR, sus_states_RR);
        initialize(s, num_vehicles);
    }
    void Initialize(d24GPU::VehicleState& vehicle_states, d24GPU::TMeasyNrState& tire_states_LF,
                    d24GPU::TMeasyNrState& tire_states_RF, d24GPU::TMeasyNrState& tire_states_LR,
                    d24GPU::TMeasyNrState& tire_states_RR, d24GPU::SuspensionState& sus_states_LF,
                    d24GPU::SuspensionState& sus_states_RF, d24GPU::SuspensionState& sus_states_LR,
                    d24GPU::SuspensionState& sus_states_RR, unsigned int num_vehicles) {
        std::vector<double> s(LFDM24_S_COUNT, 0.0);
        d24GPU::detail::put_vehicle(vehicle_states, s.data());
        const d24GPU::TMeasyNrState* t[4] = {&tire_states_LF, &tire_states_RF, &tire_states_LR, &tire_states_RR};
        for (int k = 0; k < 4; ++k)
            lfdm_cpp::put(*t[k], d24GPU::detail::kTireNr, d24GPU::detail::tire(s.data(), k) + LFDM24_T_OMEGA);
        put_sus(s.data(), sus_states_LF, sus_states_RF, sus_states_LR, sus_states_RR);
        initialize(s, num_vehicles);
    }

    d24GPU::SimState GetSimState(unsigned int vehicle_index) {
        std::vector<double> s = flat_state(vehicle_index, LFDM24_S_COUNT);
        d24GPU::SimState out;
        d24GPU::detail::get_vehicle(out._v_states, s.data());
        d24GPU::TMeasyState* t[4] = {&out._tirelf_st, &out._tirerf_st, &out._tirelr_st, &out._tirerr_st};
        d24GPU::SuspensionState* u[4] = {&out._suslf_st, &out._susrf_st, &out._suslr_st, &out._susrr_st};
        for (int k = 0; k < 4; ++k) {
            lfdm_cpp::get(*t[k], d24GPU::detail::kTire, d24GPU::detail::tire(s.data(), k));
            lfdm_cpp::get(*u[k], d24GPU::detail::kSus, d24GPU::detail::sus(s.data(), k));
        }
        return out;
    }

  private:
    static void put_sus(double* s, const d24GPU::SuspensionState& lf, const d24GPU::SuspensionState& rf,
                        const d24GPU::SuspensionState& lr, const d24GPU::SuspensionState& rr) {
        const d24GPU::SuspensionState* u[4] = {&lf, &rf, &lr, &rr};
        for (int k = 0; k < 4; ++k) lfdm_cpp::put(*u[k], d24GPU::detail::kSus, d24GPU::detail::sus(s, k));
    }
};
