// Test infrastructure only (golden-vector generator). Not part of the product.
//
// Drives the reference's own CPU 24-DOF half-implicit solver (class d24SolverHalfImplicit,
// 24dof/dof24_halfImplicit.h) compiled from the reference sources by oracle/Makefile, and prints
// full-precision trajectories for golden fixtures (TMeasy tires).
//
// Integrate() (24dof/dof24_halfImplicit.cpp:188-297) is replayed step by step through
// IntegrateStep() (:299-400) with controls from the reference's GetDriverInput
// (utils/utils.cpp:34-56); IntegrateStep runs the same rhsFun and update as Integrate, so the
// trajectory is the reference's own. Two time schedules:
//   ksim == 0 : the CPU solver's (t accumulates from 0 while t < tend - dt/10),
//   ksim  > 0 : the GPU solver's (24dof-gpu/dof24_halfImplicit_gpu.cu): windows of length ksim,
//               t restarts at k*ksim, each window runs while t < k*ksim + ksim - dt/10.
//
// Job format (stdin, whitespace separated, several jobs per stream):
//   veh <json> | tire <json> | sus <json> | tiretype 0|1 | driver <txt> | dt <v> | tend <v> | ksim <v>
//   vp <field> <v> | tp <field> <v> | sp <field> <v> | vs <field> <v> | ts <tire 0..3> <field> <v>
//   gear <initial gear> | sample <every n steps> | jac 0|1 | run
// Parameters are set before Initialize, which applies initializeTireSus (dof24.cpp:34-88).
// Output per job: "S step t x y u v phi psi theta wx wz wy wlf wrf wlr wrr" rows, one "F ..." row
// with the state in the GPU struct layout (212 doubles: VehicleState without the CPU-only dx, dy,
// tor; 4 x TMeasyState; 4 x SuspensionState) and "E" on its own line; with jac 1, the
// reference's Jacobians at that final state (print_jacobian) come before "E".
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <map>
#include <string>
#include <vector>

#include "dof24.h"
#include "dof24_halfImplicit.h"

using namespace d24;

namespace {

struct Job {
    std::string veh, tire, sus, driver;
    int tiretype = 0;  // 0 TMeasy, 1 TMeasyNr
    double dt = 1e-3, tend = -1, ksim = 0;
    int sample = 0;
    std::vector<std::pair<std::string, double>> vp, tp, sp, vs;
    std::vector<std::pair<std::pair<int, std::string>, double>> ts;
    int gear = -1;
    int jac = 0;
};

template <typename T>
double* field(T& obj, const std::map<std::string, size_t>& off, const std::string& k, const char* what) {
    auto it = off.find(k);
    if (it == off.end()) {
        std::fprintf(stderr, "unknown %s %s\n", what, k.c_str());
        std::exit(2);
    }
    return reinterpret_cast<double*>(reinterpret_cast<char*>(&obj) + it->second);
}

#define F(T, n) {#n, offsetof(T, _##n)}
const std::map<std::string, size_t> kVehParam = {
    F(VehicleParam, a),  F(VehicleParam, b),   F(VehicleParam, h),   F(VehicleParam, m),
    F(VehicleParam, jz), F(VehicleParam, jx),  F(VehicleParam, jy),  F(VehicleParam, muf),
    F(VehicleParam, mur), F(VehicleParam, maxSteer), F(VehicleParam, crankInertia),
    F(VehicleParam, maxBrakeTorque),
};
const std::map<std::string, size_t> kTireParam = {
    F(TMeasyParam, jw),      F(TMeasyParam, rr),      F(TMeasyParam, r0),       F(TMeasyParam, pn),
    F(TMeasyParam, pnmax),   F(TMeasyParam, cx),      F(TMeasyParam, cy),       F(TMeasyParam, kt),
    F(TMeasyParam, dx),      F(TMeasyParam, dy),      F(TMeasyParam, rdyncoPn), F(TMeasyParam, rdyncoP2n),
    F(TMeasyParam, dfx0Pn),  F(TMeasyParam, dfx0P2n), F(TMeasyParam, fxmPn),    F(TMeasyParam, fxmP2n),
    F(TMeasyParam, fxsPn),   F(TMeasyParam, fxsP2n),  F(TMeasyParam, sxmPn),    F(TMeasyParam, sxmP2n),
    F(TMeasyParam, sxsPn),   F(TMeasyParam, sxsP2n),  F(TMeasyParam, dfy0Pn),   F(TMeasyParam, dfy0P2n),
    F(TMeasyParam, fymPn),   F(TMeasyParam, fymP2n),  F(TMeasyParam, fysPn),    F(TMeasyParam, fysP2n),
    F(TMeasyParam, symPn),   F(TMeasyParam, symP2n),  F(TMeasyParam, sysPn),    F(TMeasyParam, sysP2n),
};
const std::map<std::string, size_t> kSusParam = {F(SuspensionParam, ks), F(SuspensionParam, bs)};
const std::map<std::string, size_t> kVehState = {
    F(VehicleState, x), F(VehicleState, y), F(VehicleState, u), F(VehicleState, v), F(VehicleState, w),
    F(VehicleState, psi), F(VehicleState, wz), F(VehicleState, crankOmega),
};
const std::map<std::string, size_t> kTireState = {F(TMeasyState, omega), F(TMeasyState, xe), F(TMeasyState, ye)};
#undef F

void print_veh(const VehicleState& s) {
    const double d[] = {s._x,     s._y,     s._z,     s._u,      s._v,      s._w,      s._psi,    s._wz,
                        s._phi,   s._wx,    s._theta, s._wy,     s._udot,   s._vdot,   s._wdot,   s._wxdot,
                        s._wydot, s._wzdot, s._dtheta, s._dphi,  s._dpsi,   s._crankOmega, s._dOmega_crank};
    for (double x : d) std::printf(" %.17g", x);
    std::printf(" %d", s._current_gr);
}
void print_tire(const TMeasyState& s) {
    const double d[] = {s._xe,  s._ye,  s._xedot, s._yedot, s._omega, s._dOmega, s._xt,  s._dxt,
                        s._rStat, s._fx, s._fy,   s._fz,    s._fxg,   s._fyg,    s._fzg,  s._vgx,
                        s._vgy, s._vgz, s._vsx,   s._vsy,   s._vsz,   s._My,     s._engTor};
    for (double x : d) std::printf(" %.17g", x);
}
// TMeasyNr: the same 23-field block with the deflections and their rates at 0
void print_tire(const TMeasyNrState& s) {
    const double d[] = {0.0,    0.0,     0.0,     0.0,    s._omega, s._dOmega, s._xt,  s._dxt,
                        s._rStat, s._fx, s._fy,   s._fz,  s._fxg,   s._fyg,    s._fzg, s._vgx,
                        s._vgy, s._vgz,  s._vsx,  s._vsy, s._vsz,   s._My,     s._engTor};
    for (double x : d) std::printf(" %.17g", x);
}
void print_sus(const SuspensionState& s) {
    const double d[] = {s._xs,  s._xsi, s._dxs, s._ls,  s._lsi, s._us,  s._vs,  s._ws,  s._dus, s._dvs, s._dws, s._uu,
                        s._vu,  s._wu,  s._duu, s._dvu, s._dwu, s._fxs, s._fys, s._fzs, s._fzd, s._mx,  s._my,  s._mz};
    for (double x : d) std::printf(" %.17g", x);
}

template <typename TS>
void run_job(const Job& job, d24SolverHalfImplicit& solver, TS* const tires[4]);

void run(const Job& job) {
    d24SolverHalfImplicit solver;
    solver.SetTimeStep(job.dt);
    const bool nr = job.tiretype != 0;
    solver.Construct(job.veh, job.tire, job.sus, job.driver, nr ? d24::TireType::TMeasyNr : d24::TireType::TMeasy);
    for (auto& kv : job.vp) *field(solver.m_veh_param, kVehParam, kv.first, "vehicle param") = kv.second;
    if (!job.tp.empty()) {
        if (nr) {
            std::fprintf(stderr, "tire parameter overrides are for TMeasy jobs\n");
            std::exit(2);
        }
        for (auto& kv : job.tp) *field(solver.m_tireTM_param, kTireParam, kv.first, "tire param") = kv.second;
        tireInit(solver.m_tireTM_param);
    }
    for (auto& kv : job.sp) *field(solver.m_sus_param, kSusParam, kv.first, "suspension param") = kv.second;
    VehicleState vs;
    for (auto& kv : job.vs) *field(vs, kVehState, kv.first, "vehicle state") = kv.second;
    if (job.gear >= 0) vs._current_gr = job.gear;
    SuspensionState ss[4];
    if (!nr) {
        TMeasyState ts[4];
        for (auto& kv : job.ts) *field(ts[kv.first.first], kTireState, kv.first.second, "tire state") = kv.second;
        solver.Initialize(vs, ts[0], ts[1], ts[2], ts[3], ss[0], ss[1], ss[2], ss[3]);
        TMeasyState* const tires[4] = {&solver.m_tireTMlf_state, &solver.m_tireTMrf_state, &solver.m_tireTMlr_state,
                                       &solver.m_tireTMrr_state};
        run_job(job, solver, tires);
    } else {
        TMeasyNrState ts[4];
        for (auto& kv : job.ts) {
            if (kv.first.second != "omega") {
                std::fprintf(stderr, "TMeasyNr tire state %s\n", kv.first.second.c_str());
                std::exit(2);
            }
            ts[kv.first.first]._omega = kv.second;
        }
        solver.Initialize(vs, ts[0], ts[1], ts[2], ts[3], ss[0], ss[1], ss[2], ss[3]);
        TMeasyNrState* const tires[4] = {&solver.m_tireTMNrlf_state, &solver.m_tireTMNrrf_state,
                                         &solver.m_tireTMNrlr_state, &solver.m_tireTMNrrr_state};
        run_job(job, solver, tires);
    }
}

// The reference's own finite-difference Jacobians (IntegrateStepWithJacobian) at the current state
// with the driver's controls at time t: "C steering throttle braking", then "JS" with the state
// Jacobian row-major (GetJacobianState) and "JC" with the control Jacobian (GetJacobianControls).
template <typename Solver>
void print_jacobian(Solver& solver, const DriverData& drv, double t) {
    DriverInput c = GetDriverInput(t, drv);
    solver.IntegrateStepWithJacobian(t, c.m_throttle, c.m_steering, c.m_braking, true);
    std::printf("\nC %.17g %.17g %.17g\nJS", c.m_steering, c.m_throttle, c.m_braking);
    for (const auto& row : solver.GetJacobianState())
        for (double x : row) std::printf(" %.17g", x);
    std::printf("\nJC");
    for (const auto& row : solver.GetJacobianControls())
        for (double x : row) std::printf(" %.17g", x);
}

template <typename TS>
void run_job(const Job& job, d24SolverHalfImplicit& solver, TS* const tires[4]) {
    VehicleState& v = solver.m_veh_state;
    SuspensionState* const sus[4] = {&solver.m_suslf_state, &solver.m_susrf_state, &solver.m_suslr_state,
                                      &solver.m_susrr_state};
    DriverData drv;
    LoadDriverData(drv, job.driver);
    const double dt = job.dt;
    const double tend = job.tend > 0 ? job.tend : drv.back().m_time;
    long step = 0;
    double t_last = 0;
    auto one = [&](double t) {
        DriverInput c = GetDriverInput(t, drv);
        double tn = solver.IntegrateStep(t, c.m_throttle, c.m_steering, c.m_braking);
        t_last = tn;
        ++step;
        if (job.sample > 0 && step % job.sample == 0)
            std::printf("S %ld %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g\n",
                        step, tn, v._x, v._y, v._u, v._v, v._phi, v._psi, v._theta, v._wx, v._wz, v._wy,
                        tires[0]->_omega, tires[1]->_omega, tires[2]->_omega, tires[3]->_omega);
        return tn;
    };
    if (job.ksim <= 0) {
        double t = 0;
        while (t < (tend - dt / 10.)) t = one(t);
    } else {
        double t0 = 0;
        while (t0 < tend) {
            double t = t0;
            const double end_time = (t0 + job.ksim) - dt / 10.;
            while (t < end_time) t = one(t);
            t0 = t0 + job.ksim;
        }
    }
    std::printf("F");
    print_veh(v);
    for (int i = 0; i < 4; ++i) print_tire(*tires[i]);
    for (int i = 0; i < 4; ++i) print_sus(*sus[i]);
    if (job.jac) print_jacobian(solver, drv, t_last);
    std::printf("\nE\n");
    std::fflush(stdout);
}

}  // namespace

int main() {
    Job job;
    std::string key;
    while (std::cin >> key) {
        if (key == "veh") std::cin >> job.veh;
        else if (key == "tire") std::cin >> job.tire;
        else if (key == "sus") std::cin >> job.sus;
        else if (key == "driver") std::cin >> job.driver;
        else if (key == "tiretype") std::cin >> job.tiretype;
        else if (key == "dt") std::cin >> job.dt;
        else if (key == "tend") std::cin >> job.tend;
        else if (key == "ksim") std::cin >> job.ksim;
        else if (key == "sample") std::cin >> job.sample;
        else if (key == "gear") std::cin >> job.gear;
        else if (key == "jac") std::cin >> job.jac;
        else if (key == "vp" || key == "tp" || key == "sp" || key == "vs") {
            std::string f;
            double v;
            std::cin >> f >> v;
            (key == "vp" ? job.vp : key == "tp" ? job.tp : key == "sp" ? job.sp : job.vs).push_back({f, v});
        } else if (key == "ts") {
            int i;
            std::string f;
            double v;
            std::cin >> i >> f >> v;
            job.ts.push_back({{i, f}, v});
        } else if (key == "run") {
            run(job);
            job = Job();
        } else {
            std::fprintf(stderr, "bad key %s\n", key.c_str());
            return 2;
        }
    }
    return 0;
}
