// Test infrastructure only (golden-vector generator). Not part of the product.
//
// Drives the reference's own CPU 11-DOF half-implicit solver (class d11SolverHalfImplicit,
// 11dof/dof11_halfImplicit.h) compiled from the reference sources by oracle/Makefile,
// and prints full-precision trajectories for golden fixtures.
//
// The reference's Integrate() (11dof/dof11_halfImplicit.cpp) is replayed step by step
// through IntegrateStep() with controls taken from the reference's GetDriverInput
// (utils/utils.cpp:34-56); rhsFun(t, controls) is the same computation as rhsFun(t) once the controls are equal, so the trajectory is the reference's own. Two time
// schedules are offered:
//   ksim == 0 : the CPU solver's schedule (t accumulates from 0 while t < tend - dt/10),
//   ksim  > 0 : the GPU solver's schedule (11dof-gpu/dof11_halfImplicit_gpu.cu): windows of length ksim, t restarts at k*ksim, each window runs
//               while t < k*ksim + ksim - dt/10.
//
// Job format (stdin, whitespace separated, several jobs per stream):
//   veh <json> | tire <json> | tiretype 0|1 | driver <txt> | dt <v> | tend <v> | ksim <v>
//   vp <field> <v> | tp <field> <v> | vs <field> <v> | ts <tire 0..1> <field> <v>
//   gear <initial gear> | sample <every n steps> | jac 0|1 | run
// Output per job: "S step t x y u v phi psi wx wz wlf wrf wlr wrr" rows, then one "F ..." row
// with the full packed state (42 doubles, TMeasy) and "E" on its own line; with jac 1, the
// reference's Jacobians at that final state (print_jacobian) come before "E".
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <map>
#include <string>
#include <vector>

#include "dof11.h"
#include "dof11_halfImplicit.h"

using namespace d11;

namespace {

struct Job {
    std::string veh, tire, driver;
    int tiretype = 0;
    double dt = 1e-3, tend = -1, ksim = 0;
    int sample = 0;
    std::vector<std::pair<std::string, double>> vp, tp, vs;
    std::vector<std::pair<std::pair<int, std::string>, double>> ts;
    int gear = -1;
    int jac = 0;
};

double* vparam_field(VehicleParam& p, const std::string& k) {
    if (k == "a") return &p._a;
    if (k == "b") return &p._b;
    if (k == "h") return &p._h;
    if (k == "m") return &p._m;
    if (k == "jz") return &p._jz;
    if (k == "muf") return &p._muf;
    if (k == "mur") return &p._mur;
    if (k == "maxSteer") return &p._maxSteer;
    if (k == "crankInertia") return &p._crankInertia;
    if (k == "maxBrakeTorque") return &p._maxBrakeTorque;
    std::fprintf(stderr, "unknown vehicle param %s\n", k.c_str());
    std::exit(2);
}

template <typename TP>
double* tparam_field(TP& p, const std::string& k) {
#define F(n) {#n, offsetof(TP, _##n)}
    static const std::map<std::string, size_t> off = {
        F(jw),     F(rr),      F(mu),       F(r0),       F(pn),         F(pnmax),  F(kt),
        F(rdyncoPn), F(rdyncoP2n), F(fzRdynco), F(rdyncoCrit), F(dfx0Pn), F(dfx0P2n), F(fxmPn),
        F(fxmP2n), F(fxsPn),   F(fxsP2n),   F(sxmPn),    F(sxmP2n),     F(sxsPn),  F(sxsP2n),
        F(dfy0Pn), F(dfy0P2n), F(fymPn),    F(fymP2n),   F(fysPn),      F(fysP2n), F(symPn),
        F(symP2n), F(sysPn),   F(sysP2n),
    };
#undef F
    auto it = off.find(k);
    if (it != off.end())
        return reinterpret_cast<double*>(reinterpret_cast<char*>(&p) + it->second);
    std::fprintf(stderr, "unknown tire param %s\n", k.c_str());
    std::exit(2);
}

double* tm_extra_field(TMeasyParam& p, const std::string& k) {
    if (k == "cx") return &p._cx;
    if (k == "cy") return &p._cy;
    if (k == "dx") return &p._dx;
    if (k == "dy") return &p._dy;
    return tparam_field(p, k);
}

double* vstate_field(VehicleState& s, const std::string& k) {
    if (k == "x") return &s._x;
    if (k == "y") return &s._y;
    if (k == "u") return &s._u;
    if (k == "v") return &s._v;
    if (k == "psi") return &s._psi;
    if (k == "wz") return &s._wz;
    if (k == "udot") return &s._udot;
    if (k == "vdot") return &s._vdot;
    if (k == "crankOmega") return &s._crankOmega;
    std::fprintf(stderr, "unknown vehicle state %s\n", k.c_str());
    std::exit(2);
}

template <typename TS>
double* tstate_field(TS& s, const std::string& k) {
    if (k == "omega") return &s._omega;
    std::fprintf(stderr, "unknown tire state %s\n", k.c_str());
    std::exit(2);
}
double* tstate_field(TMeasyState& s, const std::string& k) {
    if (k == "xe") return &s._xe;
    if (k == "ye") return &s._ye;
    if (k == "omega") return &s._omega;
    std::fprintf(stderr, "unknown tire state %s\n", k.c_str());
    std::exit(2);
}

void print_tm(const TMeasyState& s) {
    std::printf(" %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g",
                s._xe, s._ye, s._xedot, s._yedot, s._omega, s._dOmega, s._xt, s._rStat, s._fx, s._fy, s._fz,
                s._vsx, s._vsy, s._My, s._engTor);
}
void print_tm(const TMeasyNrState& s) {
    std::printf(" %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g", 0.0,
                0.0, 0.0, 0.0, s._omega, s._dOmega, s._xt, s._rStat, s._fx, s._fy, s._fz, s._vsx, s._vsy, s._My,
                s._engTor);
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
void run_job(const Job& job, d11SolverHalfImplicit& solver, TS* const tires[2]) {
    VehicleState& v = solver.m_veh_state;
    DriverData drv;
    LoadDriverData(drv, job.driver);
    const double dt = job.dt;
    const double tend = job.tend > 0 ? job.tend : drv.back().m_time;
    long step = 0;
    auto sample = [&](double t) {
        std::printf("S %ld %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g\n", step, t, v._x, v._y, v._u, v._v,
                    v._psi, v._wz, tires[0]->_omega, tires[1]->_omega);
    };
    double t_last = 0;
    auto one = [&](double t) {
        DriverInput c = GetDriverInput(t, drv);
        double tn = solver.IntegrateStep(t, c.m_throttle, c.m_steering, c.m_braking);
        t_last = tn;
        ++step;
        if (job.sample > 0 && step % job.sample == 0)
            sample(tn);
        return tn;
    };
    if (job.ksim <= 0) {
        double t = 0;
        while (t < (tend - dt / 10.))
            t = one(t);
    } else {
        double t0 = 0;
        while (t0 < tend) {
            double t = t0;
            const double end_time = (t0 + job.ksim) - dt / 10.;
            while (t < end_time)
                t = one(t);
            t0 = t0 + job.ksim;
        }
    }
    std::printf("F %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %d", v._x, v._y, v._u, v._v,
                v._psi, v._wz, v._udot, v._vdot, v._wzdot, v._crankOmega, v._dOmega_crank, v._current_gr);
    for (int i = 0; i < 2; ++i)
        print_tm(*tires[i]);
    if (job.jac) print_jacobian(solver, drv, t_last);
    std::printf("\nE\n");
    std::fflush(stdout);
}

void run(const Job& job) {
    d11SolverHalfImplicit solver;
    solver.SetTimeStep(job.dt);
    const TireType tt = job.tiretype == 0 ? TireType::TMeasy : TireType::TMeasyNr;
    solver.Construct(job.veh, job.tire, job.driver, tt);
    for (auto& kv : job.vp)
        *vparam_field(solver.m_veh_param, kv.first) = kv.second;
    VehicleState vs;
    for (auto& kv : job.vs)
        *vstate_field(vs, kv.first) = kv.second;
    if (job.gear >= 0)
        vs._current_gr = job.gear;
    if (tt == TireType::TMeasy) {
        for (auto& kv : job.tp)
            *tm_extra_field(solver.m_tireTM_param, kv.first) = kv.second;
        if (!job.tp.empty())
            tireInit(solver.m_tireTM_param);
        TMeasyState ts[2];
        for (auto& kv : job.ts)
            *tstate_field(ts[kv.first.first], kv.first.second) = kv.second;
        solver.Initialize(vs, ts[0], ts[1]);
        TMeasyState* const tires[2] = {&solver.m_tireTMf_state, &solver.m_tireTMr_state};
        run_job(job, solver, tires);
    } else {
        for (auto& kv : job.tp)
            *tparam_field(solver.m_tireTMNr_param, kv.first) = kv.second;
        if (!job.tp.empty())
            tireInit(solver.m_tireTMNr_param);
        TMeasyNrState ts[2];
        for (auto& kv : job.ts)
            *tstate_field(ts[kv.first.first], kv.first.second) = kv.second;
        solver.Initialize(vs, ts[0], ts[1]);
        TMeasyNrState* const tires[2] = {&solver.m_tireTMNrf_state, &solver.m_tireTMNrr_state};
        run_job(job, solver, tires);
    }
}

}  // namespace

int main() {
    Job job;
    std::string key;
    while (std::cin >> key) {
        if (key == "veh") std::cin >> job.veh;
        else if (key == "tire") std::cin >> job.tire;
        else if (key == "driver") std::cin >> job.driver;
        else if (key == "tiretype") std::cin >> job.tiretype;
        else if (key == "dt") std::cin >> job.dt;
        else if (key == "tend") std::cin >> job.tend;
        else if (key == "ksim") std::cin >> job.ksim;
        else if (key == "sample") std::cin >> job.sample;
        else if (key == "gear") std::cin >> job.gear;
        else if (key == "jac") std::cin >> job.jac;
        else if (key == "vp" || key == "tp" || key == "vs") {
            std::string f;
            double v;
            std::cin >> f >> v;
            (key == "vp" ? job.vp : key == "tp" ? job.tp : job.vs).push_back({f, v});
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
