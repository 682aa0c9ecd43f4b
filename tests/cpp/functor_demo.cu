// The pattern of the reference's demo_hmmwv_controlsFunctor_18gpu.cu (18dof-gpu/demos/HMMWV:20-110):
// a functor with a __device__ operator()(double t, DriverInput* controls) drives SolveStep, compiled
// with nvcc against the C++ drop-in headers of include/lfdm (which then step the vehicles in a kernel
// instantiated for the functor, calling it on the device at every step). Also a functor that reads
// device memory, which only a device-side call can serve, and the 11- and 24-DOF solvers.
//
// usage: functor_demo 18 <veh.json> <tire.json> <n>
//        functor_demo 11 <veh.json> <tire.json> <n>
//        functor_demo 24 <veh.json> <tire.json> <sus.json> <n>
// Prints "t <value>" and "s.<field> <value>" for the flat state (lfdm.h layout) of the last vehicle,
// 17 significant digits.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "dof11_halfImplicit_gpu.cuh"
#include "dof18_halfImplicit_gpu.cuh"
#include "dof24_halfImplicit_gpu.cuh"

using namespace d18GPU;

// as in the reference demo: throttle 0 for the first second, then 0.5
struct MyFunctor {
    __device__ void operator()(double t, DriverInput* controls) {
        if (t < 1) {
            controls->m_steering = 0.0;
            controls->m_throttle = 0.0;
            controls->m_braking = 0.0;
        } else {
            controls->m_steering = 0.0;
            controls->m_throttle = 0.5;
            controls->m_braking = 0.0;
        }
    }
};

// controls from a table in device memory, one row {steering, throttle, braking} per 0.1 s from t0
struct DeviceTable {
    const double* rows;
    int nrows;
    double t0;
    __device__ void operator()(double t, DriverInput* controls) const {
        int r = (int)((t - t0) * 10.0);
        r = r < 0 ? 0 : (r >= nrows ? nrows - 1 : r);
        controls->m_steering = rows[3 * r];
        controls->m_throttle = rows[3 * r + 1];
        controls->m_braking = rows[3 * r + 2];
    }
};

static void print_state(lfdm_solver* h, unsigned i, std::size_t count, double t) {
    std::vector<double> s(count, 0.0);
    if (lfdm_get_sim_state(h, i, s.data()) != LFDM_OK) {
        std::fprintf(stderr, "GetSimState failed\n");
        std::exit(1);
    }
    std::printf("t %.17g\n", t);
    for (std::size_t k = 0; k < count; ++k) std::printf("s.%zu %.17g\n", k, s[k]);
}

// the table the DeviceTable functor reads: 10 rows, a steering ramp with a brake tap
static std::vector<double> table_rows() {
    std::vector<double> rows;
    for (int r = 0; r < 10; ++r) {
        rows.push_back(0.02 * r);
        rows.push_back(r < 6 ? 0.6 : 0.2);
        rows.push_back(r == 7 ? 0.3 : 0.0);
    }
    return rows;
}

template <typename Solver>
static double drive(Solver& solver) {
    double t = 0.0;
    const double endTime = 2.0, timeStep = solver.GetStep();
    while (t < (endTime - timeStep / 10.)) t = solver.SolveStep(t, MyFunctor());
    // one more second from a table in device memory
    const std::vector<double> rows = table_rows();
    double* d_rows = nullptr;
    if (cudaMalloc(&d_rows, rows.size() * sizeof(double)) != cudaSuccess ||
        cudaMemcpy(d_rows, rows.data(), rows.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
        std::fprintf(stderr, "device table allocation failed\n");
        std::exit(1);
    }
    DeviceTable table{d_rows, 10, t};
    for (int k = 0; k < 10; ++k) t = solver.SolveStep(t, table);
    cudaFree(d_rows);
    return t;
}

int main(int argc, char** argv) {
    if (argc < 5) {
        std::fprintf(stderr, "usage: see the header of functor_demo.cu\n");
        return 2;
    }
    const int model = std::atoi(argv[1]);
    if (model == 18) {
        const unsigned n = (unsigned)std::strtoul(argv[4], nullptr, 10);
        d18SolverHalfImplicitGPU solver(n);
        solver.Construct(argv[2], argv[3], n);
        solver.SetTimeStep(1e-3);
        solver.SetKernelSimTime(0.1);
        VehicleState veh_st;
        veh_st._u = 5.0;
        TMeasyState tirelf_st, tirerf_st, tirelr_st, tirerr_st;
        tirelf_st._omega = tirerf_st._omega = tirelr_st._omega = tirerr_st._omega = 5.0 / 0.47;
        solver.Initialize(veh_st, tirelf_st, tirerf_st, tirelr_st, tirerr_st, n);
        const double t = drive(solver);
        print_state(solver.handle(), n - 1, LFDM_S_COUNT, t);
        return 0;
    }
    if (model == 11) {
        const unsigned n = (unsigned)std::strtoul(argv[4], nullptr, 10);
        d11SolverHalfImplicitGPU solver(n);
        solver.Construct(argv[2], argv[3], n);
        solver.SetTimeStep(1e-3);
        solver.SetKernelSimTime(0.1);
        d11GPU::VehicleState veh_st;
        veh_st._u = 5.0;
        d11GPU::TMeasyState tiref_st, tirer_st;
        tiref_st._omega = tirer_st._omega = 5.0 / 0.47;
        solver.Initialize(veh_st, tiref_st, tirer_st, n);
        const double t = drive(solver);
        print_state(solver.handle(), n - 1, LFDM11_S_COUNT, t);
        return 0;
    }
    if (model == 24 && argc >= 6) {
        const unsigned n = (unsigned)std::strtoul(argv[5], nullptr, 10);
        d24SolverHalfImplicitGPU solver(n);
        solver.Construct(argv[2], argv[3], argv[4], n);
        solver.SetTimeStep(1e-3);
        solver.SetKernelSimTime(0.1);
        d24GPU::VehicleState veh_st;
        d24GPU::TMeasyState t_lf, t_rf, t_lr, t_rr;
        d24GPU::SuspensionState s_lf, s_rf, s_lr, s_rr;
        solver.Initialize(veh_st, t_lf, t_rf, t_lr, t_rr, s_lf, s_rf, s_lr, s_rr, n);
        const double t = drive(solver);
        print_state(solver.handle(), n - 1, LFDM24_S_COUNT, t);
        return 0;
    }
    std::fprintf(stderr, "usage: see the header of functor_demo.cu\n");
    return 2;
}
