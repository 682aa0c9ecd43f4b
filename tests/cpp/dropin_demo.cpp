// A program written the way the reference's GPU tests and demos use the solver classes
// (tests/18dof_gpu.cu, tests/24dof_gpu.cu, 18dof-gpu/demos/HMMWV/demo_hmmwv_step_18gpu.cu,
// demo_hmmwv_controlsFunctor_18gpu.cu), compiled against the C++ drop-in headers of include/lfdm.
// It prints named state fields as "<name> <value>" lines for tests/test_cpp_dropin.py to compare
// with the Python binding of the same library.
//
//   dropin_demo solve 18 <veh> <tire> - <driver> <n> <tend>
//   dropin_demo solve 11 <veh> <tire> - <driver> <n> <tend>
//   dropin_demo solve 24 <veh> <tire> <sus> <driver> <n> <tend>
//   dropin_demo step <veh> <tire> <n>
//   dropin_demo jac <veh> <tire> <n>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "dof11_halfImplicit_gpu.cuh"
#include "dof18_halfImplicit_gpu.cuh"
#include "dof24_halfImplicit_gpu.cuh"

static void out(const char* name, double v) { std::printf("%s %.17g\n", name, v); }

static void print18(const char* tag, const d18GPU::SimState& s) {
    std::string p(tag);
    out((p + ".x").c_str(), s._veh_state._x);
    out((p + ".y").c_str(), s._veh_state._y);
    out((p + ".u").c_str(), s._veh_state._u);
    out((p + ".v").c_str(), s._veh_state._v);
    out((p + ".psi").c_str(), s._veh_state._psi);
    out((p + ".wz").c_str(), s._veh_state._wz);
    out((p + ".phi").c_str(), s._veh_state._phi);
    out((p + ".wx").c_str(), s._veh_state._wx);
    out((p + ".crankOmega").c_str(), s._veh_state._crankOmega);
    out((p + ".current_gr").c_str(), s._veh_state._current_gr);
    out((p + ".lf.omega").c_str(), s._tirelf_state._omega);
    out((p + ".rr.omega").c_str(), s._tirerr_state._omega);
    out((p + ".lf.xe").c_str(), s._tirelf_state._xe);
    out((p + ".rr.ye").c_str(), s._tirerr_state._ye);
    out((p + ".lr.fz").c_str(), s._tirelr_state._fz);
}

static int solve18(const char* veh, const char* tire, const char* drv, unsigned n, double tend) {
    d18SolverHalfImplicitGPU solver(n);
    solver.Construct(veh, tire, n, drv);
    solver.SetThreadsPerBlock(32);
    solver.SetTimeStep(1e-3);
    d18GPU::VehicleState veh_st;
    d18GPU::TMeasyState tirelf_st, tirerf_st, tirelr_st, tirerr_st;
    solver.Initialize(veh_st, tirelf_st, tirerf_st, tirelr_st, tirerr_st, n);
    solver.SetEndTime(tend);
    solver.Solve();
    out("step", solver.GetStep());
    out("end_time", solver.GetEndTime());
    out("tire_nr", solver.GetTireType() == TireType::TMeasyNr ? 1.0 : 0.0);
    print18("first", solver.GetSimState(0));
    print18("last", solver.GetSimState(n - 1));
    return 0;
}

static int solve11(const char* veh, const char* tire, const char* drv, unsigned n, double tend) {
    d11SolverHalfImplicitGPU solver(n);
    solver.Construct(veh, tire, n, drv);
    solver.SetThreadsPerBlock(32);
    solver.SetTimeStep(1e-3);
    d11GPU::VehicleState veh_st;
    d11GPU::TMeasyState tiref_st, tirer_st;
    solver.Initialize(veh_st, tiref_st, tirer_st, n);
    solver.SetEndTime(tend);
    solver.Solve();
    const d11GPU::SimState s = solver.GetSimState(n - 1);
    out("last.x", s._veh_state._x);
    out("last.y", s._veh_state._y);
    out("last.u", s._veh_state._u);
    out("last.psi", s._veh_state._psi);
    out("last.wz", s._veh_state._wz);
    out("last.current_gr", s._veh_state._current_gr);
    out("last.f.omega", s._tiref_state._omega);
    out("last.r.omega", s._tirer_state._omega);
    out("last.f.xe", s._tiref_state._xe);
    return 0;
}

static int solve24(const char* veh, const char* tire, const char* sus, const char* drv, unsigned n, double tend) {
    d24SolverHalfImplicitGPU solver(n);
    solver.Construct(veh, tire, sus, n, drv);
    solver.SetThreadsPerBlock(32);
    solver.SetTimeStep(1e-3);
    d24GPU::VehicleState veh_st;
    d24GPU::TMeasyState tirelf_st, tirerf_st, tirelr_st, tirerr_st;
    d24GPU::SuspensionState suslf_st, susrf_st, suslr_st, susrr_st;
    solver.Initialize(veh_st, tirelf_st, tirerf_st, tirelr_st, tirerr_st, suslf_st, susrf_st, suslr_st, susrr_st,
                      n);
    const d24GPU::SimState s0 = solver.GetSimState(0);  // after initializeTireSus
    out("init.z", s0._v_states._z);
    out("init.lf.xt", s0._tirelf_st._xt);
    out("init.rr.xs", s0._susrr_st._xs);
    out("init.lf.ls", s0._suslf_st._ls);
    solver.SetEndTime(tend);
    solver.Solve();
    const d24GPU::SimState s = solver.GetSimState(n - 1);
    out("last.x", s._v_states._x);
    out("last.y", s._v_states._y);
    out("last.z", s._v_states._z);
    out("last.theta", s._v_states._theta);
    out("last.psi", s._v_states._psi);
    out("last.current_gr", s._v_states._current_gr);
    out("last.lf.omega", s._tirelf_st._omega);
    out("last.rr.xt", s._tirerr_st._xt);
    out("last.lr.xs", s._suslr_st._xs);
    out("last.rf.fzs", s._susrf_st._fzs);
    return 0;
}

// demo_hmmwv_controlsFunctor_18gpu.cu's functor, callable on the host as well
struct StepThrottle {
    void operator()(double t, DriverInput* controls) const {
        controls->m_steering = t < 0.7 ? 0.0 : 0.05;
        controls->m_throttle = t < 0.5 ? 0.0 : 0.5;
        controls->m_braking = 0.0;
    }
};

static int step18(const char* veh, const char* tire, unsigned n) {
    d18SolverHalfImplicitGPU solver(n);
    solver.Construct(veh, tire, n);
    solver.SetTimeStep(1e-3);
    solver.SetKernelSimTime(0.5);
    d18GPU::VehicleState veh_st;
    veh_st._u = 5.0;
    d18GPU::TMeasyState tirelf_st, tirerf_st, tirelr_st, tirerr_st;
    tirelf_st._omega = tirerf_st._omega = tirelr_st._omega = tirerr_st._omega = 5.0 / 0.47;
    solver.Initialize(veh_st, tirelf_st, tirerf_st, tirelr_st, tirerr_st, n);
    double t = 0.0;
    t = solver.SolveStep(t, 0.1, 0.4, 0.0);
    t = solver.SolveStep(t, 0.0, 0.2, 0.1);
    t = solver.SolveStep(t, StepThrottle());
    t = solver.SolveStep(t, StepThrottle());
    out("t", t);
    print18("last", solver.GetSimState(n - 1));
    // errors print and the program carries on, as against the reference
    solver.Initialize(veh_st, tirelf_st, tirerf_st, tirelr_st, tirerr_st, 1);
    out("after_error", 1.0);
    return 0;
}

// The extension GetRhsJacobians after one SolveStep window: every entry of the last vehicle's
// matrices, by the reference's difference scheme and exactly.
static int jac18(const char* veh, const char* tire, unsigned n) {
    d18SolverHalfImplicitGPU solver(n);
    solver.Construct(veh, tire, n);
    solver.SetTimeStep(1e-3);
    solver.SetKernelSimTime(0.2);
    d18GPU::VehicleState veh_st;
    veh_st._u = 8.0;
    d18GPU::TMeasyState tirelf_st, tirerf_st, tirelr_st, tirerr_st;
    tirelf_st._omega = tirerf_st._omega = tirelr_st._omega = tirerr_st._omega = 8.0 / 0.47;
    solver.Initialize(veh_st, tirelf_st, tirerf_st, tirelr_st, tirerr_st, n);
    solver.SolveStep(0.0, 0.1, 0.5, 0.0);
    std::vector<double> st(n), th(n), br(n, 0.0);
    for (unsigned i = 0; i < n; ++i) {
        st[i] = 0.05 * i;
        th[i] = 0.3;
    }
    std::vector<std::vector<std::vector<double>>> js, ju;
    for (int exact = 0; exact < 2; ++exact) {
        const int ny = solver.GetRhsJacobians(st, th, br, js, ju, exact != 0);
        const char* tag = exact ? "exact" : "fd";
        out((std::string(tag) + ".ny").c_str(), ny);
        for (int r = 0; r < ny; ++r) {
            for (int c = 0; c < ny; ++c)
                out((std::string(tag) + ".s." + std::to_string(r) + "." + std::to_string(c)).c_str(), js[n - 1][r][c]);
            out((std::string(tag) + ".u." + std::to_string(r) + ".0").c_str(), ju[n - 1][r][0]);
            out((std::string(tag) + ".u." + std::to_string(r) + ".1").c_str(), ju[n - 1][r][1]);
        }
    }
    // a control vector of the wrong length is reported and nothing is computed
    out("bad_size", solver.GetRhsJacobians(std::vector<double>(1), th, br, js, ju));
    return 0;
}

int main(int argc, char** argv) {
    if (argc >= 9 && std::string(argv[1]) == "solve") {
        const int model = std::atoi(argv[2]);
        const unsigned n = (unsigned)std::strtoul(argv[7], nullptr, 10);
        const double tend = std::strtod(argv[8], nullptr);
        if (model == 18) return solve18(argv[3], argv[4], argv[6], n, tend);
        if (model == 11) return solve11(argv[3], argv[4], argv[6], n, tend);
        if (model == 24) return solve24(argv[3], argv[4], argv[5], argv[6], n, tend);
    }
    if (argc >= 5 && std::string(argv[1]) == "step") return step18(argv[2], argv[3], (unsigned)std::atoi(argv[4]));
    if (argc >= 5 && std::string(argv[1]) == "jac") return jac18(argv[2], argv[3], (unsigned)std::atoi(argv[4]));
    std::fprintf(stderr, "usage: see the header of dropin_demo.cpp\n");
    return 2;
}
