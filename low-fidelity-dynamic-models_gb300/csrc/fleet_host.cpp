// Host side of the mixed-DOF fleet (lfdm_fleet_* in include/lfdm.h): schedule, vehicle ordering,
// tiles, device buffers, the CUDA graph of a solve, and the launch-configuration autotuner.
//
// No counterpart class exists in the reference: it solves one model with one end time per solver
// (d18SolverHalfImplicitGPU / d24SolverHalfImplicitGPU). A fleet holds 18-DOF and 24-DOF vehicles of
// any number of parameter classes, each with its own end time, and reproduces for every vehicle
// what the reference's Solve() computes for it with m_tend = that vehicle's end time and the
// fleet's kernel_sim_time (dof18_halfImplicit_gpu.cu:404-494, dof24_halfImplicit_gpu.cu).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/lfdm.h"
#include "fleet.h"
#include "kernels.h"

using namespace lfdm;

namespace {

thread_local std::string g_fleet_create_error;

template <typename T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaError_t ensure(size_t count) {
        if (count <= n && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        if (count == 0) return cudaSuccess;
        cudaError_t e = cudaMalloc((void**)&p, count * sizeof(T));
        if (e == cudaSuccess) n = count;
        return e;
    }
    ~DBuf() {
        if (p) cudaFree(p);
    }
};

// One model's vehicles: host data in add order, device data in step-count order.
struct ModelGroup {
    int model = 0;
    int ns = 0, nch = 0;
    std::vector<lfdm_class18> classes;
    std::vector<int32_t> class_of;   // add order
    std::vector<double> params;      // [n][P]
    std::vector<double> states;      // [n][ns] host mirror (add order)
    std::vector<double> horizon;     // [n]
    std::vector<int64_t> row_off;    // [n] into the fleet's rows
    std::vector<int32_t> row_len;    // [n]
    // derived (prepare)
    std::vector<int32_t> perm;       // sorted position -> add index
    std::vector<int32_t> nsteps;     // add order
    int npad = 0;
    DBuf<double> d_params, d_K, d_S, d_aos, d_resp, d_S_backup;
    DBuf<int32_t> d_class_of, d_row_len, d_nsteps;
    DBuf<int64_t> d_row_off;
    DBuf<unsigned char> d_classes;
    DBuf<uint32_t> d_status;
    unsigned n() const { return (unsigned)class_of.size(); }
};

}  // namespace

struct lfdm_fleet {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    ModelGroup g18, g24;
    std::vector<double> rows;  // concatenated driver rows
    double dt = 1e-3, ksim = 2.0, dtout = 0.0;
    // launch configuration (0 = automatic)
    unsigned threads = 128, blocks_per_sm = 0, steps_per_launch = 0;
    // schedule
    std::vector<double> step_t;
    std::vector<int32_t> step_sample;
    std::vector<int32_t> window_end;  // cumulative steps at the end of each window
    int spw = 0, nsamples = 0, total_steps = 0;
    std::vector<FleetTile> tiles;   // the 18-DOF tiles [0, ntiles18), then the 24-DOF tiles
    std::vector<FleetTile> merged;  // all tiles in one list by estimated cost
    int ntiles18 = 0;
    double frac18 = 1.0;            // 18-DOF share of the estimated work (steps x per-step cost)
    bool affinity = false;          // split the SMs between the two models' tile lists
    int precision = LFDM_PREC_FP64;  // or LFDM_PREC_MIXED_TIRE
    bool f32() const { return precision == LFDM_PREC_MIXED_TIRE; }
    DBuf<double> d_rows, d_step_t;
    DBuf<int32_t> d_step_sample;
    DBuf<FleetTile> d_tiles;
    DBuf<int> d_queue;
    bool dirty = true;         // inputs changed: prepare again
    bool states_dirty = true;  // host states newer than device
    bool device_newer = false; // device states newer than host
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    unsigned graph_launches = 0;
    double last_ms = 0;
    unsigned last_launches = 0;
    double tune_ms = 0;
    std::string err;

    int fail(int code, const char* fmt, ...) {
        char buf[1024];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        err = buf;
        return code;
    }
    int cuda_fail(cudaError_t e, const char* what) { return fail(LFDM_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e)); }
    void drop_graph() {
        if (graph_exec) cudaGraphExecDestroy(graph_exec);
        if (graph) cudaGraphDestroy(graph);
        graph_exec = nullptr;
        graph = nullptr;
    }
    ModelGroup* group(int model) { return model == LFDM_MODEL_18 ? &g18 : model == LFDM_MODEL_24 ? &g24 : nullptr; }
};

#define FCK(expr)                                                \
    do {                                                         \
        cudaError_t e_ = (expr);                                 \
        if (e_ != cudaSuccess) return f->cuda_fail(e_, #expr);   \
    } while (0)

namespace {

// The reference's Solve loop on the host (dof18_halfImplicit_gpu.cu:438-463 with the device loop
// :893-975): windows of ksim from current_time = 0 (accumulated in FP64) while current_time < tend;
// in each window t restarts at the window start and steps while t < (start + ksim) - dt/10; a
// sample is taken when |kernel_time - (stored + 1) * dtout| < 1e-7, at most spw per window.
void replay_schedule(lfdm_fleet* f, double tend_max) {
    f->step_t.clear();
    f->step_sample.clear();
    f->window_end.clear();
    f->spw = f->dtout > 0 ? (int)std::ceil(f->ksim / f->dtout - 1e-9) : 0;
    double current_time = 0;
    int w = 0;
    while (current_time < tend_max) {
        double t = current_time, kt = 0;
        const double end_time = (t + f->ksim) - f->dt / 10.;
        int stored = 0;
        while (t < end_time) {
            f->step_t.push_back(t);
            t += f->dt;
            kt += f->dt;
            int sample = -1;
            if (f->dtout > 0 && std::fabs(kt - (stored + 1) * f->dtout) < 1e-7) {
                if (stored < f->spw) sample = w * f->spw + stored;
                ++stored;
            }
            f->step_sample.push_back(sample);
        }
        f->window_end.push_back((int32_t)f->step_t.size());
        current_time = current_time + f->ksim;
        ++w;
    }
    f->total_steps = (int)f->step_t.size();
    f->nsamples = w * f->spw;
}

// Steps of a vehicle whose end time is tend: the steps of the windows that start before tend.
int32_t steps_for(const lfdm_fleet* f, double tend) {
    double current_time = 0;
    int w = 0;
    while (current_time < tend && w < (int)f->window_end.size()) {
        current_time = current_time + f->ksim;
        ++w;
    }
    return w == 0 ? 0 : f->window_end[w - 1];
}

int prepare_group(lfdm_fleet* f, ModelGroup& g) {
    const unsigned n = g.n();
    g.nsteps.resize(n);
    for (unsigned i = 0; i < n; ++i) g.nsteps[i] = steps_for(f, g.horizon[i]);
    g.perm.resize(n);
    std::iota(g.perm.begin(), g.perm.end(), 0);
    std::stable_sort(g.perm.begin(), g.perm.end(), [&](int a, int b) { return g.nsteps[a] > g.nsteps[b]; });
    if (n == 0) return LFDM_OK;
    g.npad = (int)((n + 31) / 32 * 32);
    std::vector<double> p(n * (size_t)LFDM_P_COUNT);
    std::vector<int32_t> cls(n), len(n), nst(n);
    std::vector<int64_t> off(n);
    for (unsigned k = 0; k < n; ++k) {
        const int i = g.perm[k];
        std::memcpy(&p[(size_t)k * LFDM_P_COUNT], &g.params[(size_t)i * LFDM_P_COUNT], LFDM_P_COUNT * sizeof(double));
        cls[k] = g.class_of[i];
        off[k] = g.row_off[i];
        len[k] = g.row_len[i];
        nst[k] = g.nsteps[i];
    }
    const size_t cs = class_dev18_size();
    std::vector<unsigned char> cbuf(cs * g.classes.size());
    for (size_t c = 0; c < g.classes.size(); ++c)
        build_class_dev18(g.classes[c], reinterpret_cast<ClassDev18*>(cbuf.data() + c * cs));
    const int kcount = g.model == LFDM_MODEL_24 ? k24_count() : k18_count();
    FCK(g.d_params.ensure(p.size()));
    FCK(g.d_K.ensure((size_t)kcount * g.npad));
    FCK(g.d_S.ensure((size_t)g.ns * g.npad));
    FCK(g.d_aos.ensure((size_t)g.ns * n));
    FCK(g.d_class_of.ensure(n));
    FCK(g.d_row_off.ensure(n));
    FCK(g.d_row_len.ensure(n));
    FCK(g.d_nsteps.ensure(n));
    FCK(g.d_classes.ensure(cbuf.size()));
    FCK(g.d_status.ensure(n));
    cudaStream_t st = f->stream;
    FCK(cudaMemcpyAsync(g.d_params.p, p.data(), p.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    FCK(cudaMemcpyAsync(g.d_class_of.p, cls.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    FCK(cudaMemcpyAsync(g.d_row_off.p, off.data(), n * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    FCK(cudaMemcpyAsync(g.d_row_len.p, len.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    FCK(cudaMemcpyAsync(g.d_nsteps.p, nst.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    FCK(cudaMemcpyAsync(g.d_classes.p, cbuf.data(), cbuf.size(), cudaMemcpyHostToDevice, st));
    FCK(cudaMemsetAsync(g.d_status.p, 0, n * sizeof(uint32_t), st));
    FCK(g.model == LFDM_MODEL_24 ? launch_prepare24(g.d_params.p, (int)n, g.npad, g.d_K.p, st)
                                 : launch_prepare18(g.d_params.p, (int)n, g.npad, g.d_K.p, st));
    if (f->nsamples > 0) {
        FCK(g.d_resp.ensure((size_t)f->nsamples * g.nch * n));
        FCK(cudaMemsetAsync(g.d_resp.p, 0, (size_t)f->nsamples * g.nch * n * sizeof(double), st));
    }
    FCK(cudaStreamSynchronize(st));
    return LFDM_OK;
}

int upload_states(lfdm_fleet* f, ModelGroup& g) {
    const unsigned n = g.n();
    if (n == 0) return LFDM_OK;
    std::vector<double> s((size_t)g.ns * n);
    for (unsigned k = 0; k < n; ++k)
        std::memcpy(&s[(size_t)k * g.ns], &g.states[(size_t)g.perm[k] * g.ns], g.ns * sizeof(double));
    FCK(cudaMemcpyAsync(g.d_aos.p, s.data(), s.size() * sizeof(double), cudaMemcpyHostToDevice, f->stream));
    FCK(launch_states_to_soa(g.d_aos.p, (int)n, g.ns, g.npad, g.d_S.p, f->stream));
    FCK(cudaStreamSynchronize(f->stream));
    return LFDM_OK;
}

int download_states(lfdm_fleet* f, ModelGroup& g) {
    const unsigned n = g.n();
    if (n == 0) return LFDM_OK;
    std::vector<double> s((size_t)g.ns * n);
    FCK(launch_states_to_aos(g.d_S.p, (int)n, g.ns, g.npad, g.d_aos.p, f->stream));
    FCK(cudaMemcpyAsync(s.data(), g.d_aos.p, s.size() * sizeof(double), cudaMemcpyDeviceToHost, f->stream));
    FCK(cudaStreamSynchronize(f->stream));
    for (unsigned k = 0; k < n; ++k)
        std::memcpy(&g.states[(size_t)g.perm[k] * g.ns], &s[(size_t)k * g.ns], g.ns * sizeof(double));
    return LFDM_OK;
}

// Relative per-step cost of the two models (source-level FP64 operations per step of the
// reference algorithm, 1391 and 1941), used to order tiles.
constexpr double kCost18 = 1391, kCost24 = 1941;

int prepare(lfdm_fleet* f) {
    if (!f->dirty) return LFDM_OK;
    if (f->g18.n() + f->g24.n() == 0) return f->fail(LFDM_ERR_STATE, "the fleet has no vehicles");
    FCK(cudaSetDevice(f->device));
    double tend_max = 0;
    for (ModelGroup* g : {&f->g18, &f->g24})
        for (double h : g->horizon) tend_max = std::max(tend_max, h);
    replay_schedule(f, tend_max);
    if (f->total_steps == 0) return f->fail(LFDM_ERR_STATE, "no vehicle has a positive end time");
    for (ModelGroup* g : {&f->g18, &f->g24}) {
        int rc = prepare_group(f, *g);
        if (rc) return rc;
    }
    // tiles of 32 vehicles in step-count order: the 18-DOF list, then the 24-DOF list, each largest
    // estimated cost first; the share of the estimated work that is 18-DOF sets the SM split
    f->tiles.clear();
    double work[2] = {0, 0};
    for (ModelGroup* g : {&f->g18, &f->g24}) {
        const size_t start = f->tiles.size();
        const unsigned n = g->n();
        const bool m24 = g->model == LFDM_MODEL_24;
        for (unsigned first = 0; first < n; first += 32) {
            FleetTile t;
            t.model = g->model;
            t.first = (int)first;
            t.count = (int)std::min<unsigned>(32, n - first);
            t.nsteps_max = g->nsteps[g->perm[first]];
            if (t.nsteps_max > 0) f->tiles.push_back(t);
        }
        for (unsigned k = 0; k < n; ++k) work[m24] += (double)g->nsteps[k] * (m24 ? kCost24 : kCost18);
        std::stable_sort(f->tiles.begin() + start, f->tiles.end(), [](const FleetTile& a, const FleetTile& b) {
            return (double)a.nsteps_max * a.count > (double)b.nsteps_max * b.count;
        });
        if (!m24) f->ntiles18 = (int)f->tiles.size();
    }
    f->frac18 = work[0] + work[1] > 0 ? work[0] / (work[0] + work[1]) : 1.0;
    f->merged = f->tiles;
    std::stable_sort(f->merged.begin(), f->merged.end(), [](const FleetTile& a, const FleetTile& b) {
        const double ca = (double)a.nsteps_max * (a.model == LFDM_MODEL_24 ? kCost24 : kCost18) * a.count;
        const double cb = (double)b.nsteps_max * (b.model == LFDM_MODEL_24 ? kCost24 : kCost18) * b.count;
        return ca > cb;
    });
    FCK(f->d_rows.ensure(std::max<size_t>(4, f->rows.size())));
    FCK(cudaMemcpyAsync(f->d_rows.p, f->rows.data(), f->rows.size() * sizeof(double), cudaMemcpyHostToDevice,
                        f->stream));
    FCK(f->d_step_t.ensure(f->total_steps));
    FCK(f->d_step_sample.ensure(f->total_steps));
    FCK(cudaMemcpyAsync(f->d_step_t.p, f->step_t.data(), f->total_steps * sizeof(double), cudaMemcpyHostToDevice,
                        f->stream));
    FCK(cudaMemcpyAsync(f->d_step_sample.p, f->step_sample.data(), f->total_steps * sizeof(int32_t),
                        cudaMemcpyHostToDevice, f->stream));
    FCK(f->d_tiles.ensure(std::max<size_t>(2, 2 * f->tiles.size())));
    FCK(cudaMemcpyAsync(f->d_tiles.p, f->tiles.data(), f->tiles.size() * sizeof(FleetTile), cudaMemcpyHostToDevice,
                        f->stream));
    FCK(cudaMemcpyAsync(f->d_tiles.p + f->tiles.size(), f->merged.data(), f->merged.size() * sizeof(FleetTile),
                        cudaMemcpyHostToDevice, f->stream));
    FCK(cudaStreamSynchronize(f->stream));
    f->drop_graph();
    f->dirty = false;
    f->states_dirty = true;
    return LFDM_OK;
}

FleetModelDev model_dev(const lfdm_fleet* f, const ModelGroup& g) {
    FleetModelDev m;
    m.n = (int)g.n();
    m.npad = g.npad;
    m.K = g.d_K.p;
    m.S = g.d_S.p;
    m.class_of = g.d_class_of.p;
    m.classes = reinterpret_cast<const ClassDev18*>(g.d_classes.p);
    m.row_off = g.d_row_off.p;
    m.row_len = g.d_row_len.p;
    m.nsteps = g.d_nsteps.p;
    m.resp = f->nsamples > 0 ? g.d_resp.p : nullptr;
    m.status = g.d_status.p;
    return m;
}

// Launch plan for global steps [0, steps): grid size and chunking, with the buffers it needs
// allocated (outside any stream capture).
struct Plan {
    int blocks = 0, chunk = 0, nl = 0;
    unsigned threads = 128;
};

int plan(lfdm_fleet* f, int steps, unsigned threads, unsigned bps, unsigned spl, Plan* p) {
    int dev_sms = 0;
    FCK(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, f->device));
    FCK(fleet_kernel_setup());
    int occ = 0;
    FCK(fleet_occupancy((int)threads, f->f32(), &occ));
    if (occ < 1) return f->fail(LFDM_ERR_CUDA, "the fleet kernel does not fit with %u threads per block", threads);
    const int per_sm = bps ? std::min<int>((int)bps, occ) : occ;
    p->blocks = dev_sms * per_sm;
    p->chunk = spl ? (int)std::min<unsigned>(spl, (unsigned)steps) : steps;
    p->nl = (steps + p->chunk - 1) / p->chunk;
    p->threads = threads;
    FCK(f->d_queue.ensure(2 * std::max(1, p->nl)));
    return LFDM_OK;
}

// Enqueue (or record into a capture) the launches of a plan.
int enqueue(lfdm_fleet* f, int steps, const Plan& p) {
    FCK(cudaMemsetAsync(f->d_queue.p, 0, 2 * p.nl * sizeof(int), f->stream));
    for (int c = 0; c < p.nl; ++c) {
        FleetLaunch L;
        L.m18 = model_dev(f, f->g18);
        L.m24 = model_dev(f, f->g24);
        L.rows = f->d_rows.p;
        L.tiles = f->d_tiles.p;
        L.ntiles = (int)f->tiles.size();
        L.merged = f->d_tiles.p + f->tiles.size();
        L.ntiles18 = f->ntiles18;
        L.queue = f->d_queue.p + 2 * c;
        L.affinity = f->affinity ? 1 : 0;
        L.home18 = (float)f->frac18;
        L.step_t = f->d_step_t.p;
        L.step_sample = f->d_step_sample.p;
        L.s_begin = c * p.chunk;
        L.s_end = std::min(steps, (c + 1) * p.chunk);
        L.dt = f->dt;
        L.nsamples = f->nsamples;
        FCK(launch_fleet(L, p.blocks, (int)p.threads, f->f32(), f->stream));
    }
    return LFDM_OK;
}

int build_graph(lfdm_fleet* f) {
    if (f->graph_exec) return LFDM_OK;
    Plan p;
    int rc = plan(f, f->total_steps, f->threads, f->blocks_per_sm, f->steps_per_launch, &p);
    if (rc) return rc;
    FCK(cudaStreamBeginCapture(f->stream, cudaStreamCaptureModeThreadLocal));
    rc = enqueue(f, f->total_steps, p);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(f->stream, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return f->cuda_fail(e, "cudaStreamEndCapture");
    f->graph = g;
    FCK(cudaGraphInstantiate(&f->graph_exec, f->graph, 0));
    f->graph_launches = (unsigned)p.nl;
    return LFDM_OK;
}

}  // namespace

extern "C" {

int lfdm_fleet_create(int device, lfdm_fleet** out) {
    if (!out) return LFDM_ERR_ARG;
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        g_fleet_create_error = std::string("no CUDA device: ") + cudaGetErrorString(e);
        return LFDM_ERR_NODEVICE;
    }
    if (device < 0 || device >= ndev) {
        g_fleet_create_error = "device index out of range";
        return LFDM_ERR_ARG;
    }
    std::unique_ptr<lfdm_fleet> f(new lfdm_fleet());
    f->device = device;
    f->g18.model = LFDM_MODEL_18;
    f->g18.ns = LFDM_S_COUNT;
    f->g18.nch = LFDM18_RESP_CHANNELS;
    f->g24.model = LFDM_MODEL_24;
    f->g24.ns = LFDM24_S_COUNT;
    f->g24.nch = LFDM24_RESP_CHANNELS;
    if ((e = cudaSetDevice(device)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&f->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreate(&f->ev0)) != cudaSuccess || (e = cudaEventCreate(&f->ev1)) != cudaSuccess) {
        g_fleet_create_error = std::string("CUDA set-up failed: ") + cudaGetErrorString(e);
        return LFDM_ERR_CUDA;
    }
    *out = f.release();
    return LFDM_OK;
}

int lfdm_fleet_destroy(lfdm_fleet* f) {
    if (!f) return LFDM_OK;
    cudaSetDevice(f->device);
    f->drop_graph();
    if (f->ev0) cudaEventDestroy(f->ev0);
    if (f->ev1) cudaEventDestroy(f->ev1);
    if (f->stream) cudaStreamDestroy(f->stream);
    delete f;
    return LFDM_OK;
}

const char* lfdm_fleet_last_error(const lfdm_fleet* f) { return f ? f->err.c_str() : g_fleet_create_error.c_str(); }

int lfdm_fleet_add(lfdm_fleet* f, int model, const lfdm_class18* cls, unsigned n, const double* params,
                   const double* states, const double* horizons, const double* rows, size_t nrows,
                   const int64_t* row_off, const int32_t* row_len) {
    if (!f) return LFDM_ERR_ARG;
    ModelGroup* g = f->group(model);
    if (!g) return f->fail(LFDM_ERR_ARG, "the fleet holds 18-DOF and 24-DOF vehicles (model %d)", model);
    if (!cls || !params || !states || !horizons || !row_off || !row_len || n == 0 || (!rows && nrows))
        return f->fail(LFDM_ERR_ARG, "null argument or no vehicles");
    const lfdm_class18& c = *cls;
    bool ok = c.noGears >= 1 && c.noGears <= LFDM_MAX_GEARS && c.powertrainMapSize >= 1 &&
              c.powertrainMapSize <= LFDM_MAX_MAP && c.lossesMapSize >= 1 && c.lossesMapSize <= LFDM_MAX_MAP;
    if (c.tcbool) ok = ok && c.CFmapSize >= 1 && c.CFmapSize <= LFDM_MAX_MAP && c.TRmapSize >= 1 &&
                       c.TRmapSize <= LFDM_MAX_MAP;
    if (c.nonLinearSteer) ok = ok && c.steerMapSize >= 1 && c.steerMapSize <= LFDM_MAX_MAP;
    if (!ok) return f->fail(LFDM_ERR_ARG, "gear count or map sizes out of range");
    if ((size_t)g->n() + n > (1u << 30)) return f->fail(LFDM_ERR_CAPACITY, "too many vehicles");
    // rows == NULL: row_off indexes the rows the fleet already holds (lfdm_fleet_add_rows)
    const double* R = rows ? rows : f->rows.data();
    const size_t NR = rows ? nrows : f->rows.size() / 4;
    for (unsigned i = 0; i < n; ++i) {
        if (row_len[i] < 1 || row_off[i] < 0 || (size_t)row_off[i] + (size_t)row_len[i] > NR)
            return f->fail(LFDM_ERR_ARG, "vehicle %u: driver rows [%lld, +%d) outside the %zu rows given", i,
                           (long long)row_off[i], row_len[i], NR);
        if (!(horizons[i] >= 0) || !(horizons[i] < 1e6))
            return f->fail(LFDM_ERR_ARG, "vehicle %u: end time must be finite and >= 0", i);
    }
    {
        // within each vehicle's rows the times must not decrease (GetDriverInput's lower_bound needs
        // sorted times, utils/utils_gpu.cu:95-107): mark the rows that follow a row of the same range
        std::vector<int32_t> d(NR + 1, 0);
        for (unsigned i = 0; i < n; ++i) {
            d[(size_t)row_off[i] + 1] += 1;
            d[(size_t)row_off[i] + (size_t)row_len[i]] -= 1;
        }
        int32_t inside = 0;
        for (size_t r = 1; r < NR; ++r) {
            inside += d[r];
            if (inside > 0 && R[4 * r] < R[4 * (r - 1)])
                return f->fail(LFDM_ERR_PARSE, "driver table times must be non-decreasing (row %zu)", r);
        }
    }
    const int64_t base = rows ? (int64_t)(f->rows.size() / 4) : 0;
    if (rows) f->rows.insert(f->rows.end(), rows, rows + 4 * nrows);
    const int32_t ci = (int32_t)g->classes.size();
    g->classes.push_back(c);
    g->params.insert(g->params.end(), params, params + (size_t)n * LFDM_P_COUNT);
    g->states.insert(g->states.end(), states, states + (size_t)n * g->ns);
    for (unsigned i = 0; i < n; ++i) {
        g->class_of.push_back(ci);
        g->horizon.push_back(horizons[i]);
        g->row_off.push_back(base + row_off[i]);
        g->row_len.push_back(row_len[i]);
    }
    f->dirty = true;
    f->device_newer = false;
    return LFDM_OK;
}

int lfdm_fleet_add_rows(lfdm_fleet* f, const double* rows, size_t nrows, int64_t* first_row) {
    if (!f || !rows || !first_row) return f ? f->fail(LFDM_ERR_ARG, "null argument") : LFDM_ERR_ARG;
    *first_row = (int64_t)(f->rows.size() / 4);
    f->rows.insert(f->rows.end(), rows, rows + 4 * nrows);
    f->dirty = true;
    return LFDM_OK;
}

int lfdm_fleet_set_time_step(lfdm_fleet* f, double dt) {
    if (!f) return LFDM_ERR_ARG;
    if (!(dt > 0) || !(dt < 1)) return f->fail(LFDM_ERR_ARG, "time step must be in (0, 1) s");
    f->dt = dt;
    f->dirty = true;
    return LFDM_OK;
}
int lfdm_fleet_set_kernel_sim_time(lfdm_fleet* f, double ksim) {
    if (!f) return LFDM_ERR_ARG;
    if (!(ksim > 0)) return f->fail(LFDM_ERR_ARG, "kernel_sim_time must be positive");
    f->ksim = ksim;
    f->dirty = true;
    return LFDM_OK;
}
int lfdm_fleet_set_output(lfdm_fleet* f, double dtout) {
    if (!f) return LFDM_ERR_ARG;
    if (!(dtout >= 0)) return f->fail(LFDM_ERR_ARG, "output interval must be >= 0");
    f->dtout = dtout;
    f->dirty = true;
    return LFDM_OK;
}

int lfdm_fleet_set_launch(lfdm_fleet* f, unsigned threads, unsigned blocks_per_sm, unsigned steps_per_launch) {
    if (!f) return LFDM_ERR_ARG;
    if (threads == 0) threads = 128;
    if (threads > 128 || (threads & 31)) return f->fail(LFDM_ERR_ARG, "threads per block: 32, 64, 96 or 128");
    f->threads = threads;
    f->blocks_per_sm = blocks_per_sm;
    f->steps_per_launch = steps_per_launch;
    f->drop_graph();
    return LFDM_OK;
}

int lfdm_fleet_set_precision(lfdm_fleet* f, int precision) {
    if (!f) return LFDM_ERR_ARG;
    if (precision != LFDM_PREC_FP64 && precision != LFDM_PREC_MIXED_TIRE)
        return f->fail(LFDM_ERR_ARG, "the fleet steps in FP64 or with the FP32 tire core (precision %d)", precision);
    f->precision = precision;
    f->drop_graph();
    return LFDM_OK;
}

int lfdm_fleet_set_affinity(lfdm_fleet* f, int on) {
    if (!f) return LFDM_ERR_ARG;
    f->affinity = on != 0;
    f->drop_graph();
    return LFDM_OK;
}

int lfdm_fleet_get_affinity(lfdm_fleet* f, int* on, double* frac18) {
    if (!f) return LFDM_ERR_ARG;
    if (on) *on = f->affinity ? 1 : 0;
    if (frac18) *frac18 = f->frac18;
    return LFDM_OK;
}

int lfdm_fleet_get_launch(lfdm_fleet* f, unsigned* threads, unsigned* blocks_per_sm, unsigned* steps_per_launch) {
    if (!f) return LFDM_ERR_ARG;
    if (threads) *threads = f->threads;
    if (blocks_per_sm) *blocks_per_sm = f->blocks_per_sm;
    if (steps_per_launch) *steps_per_launch = f->steps_per_launch;
    return LFDM_OK;
}

int lfdm_fleet_info(lfdm_fleet* f, unsigned* n18, unsigned* n24, long long* total_steps, double* vehicle_steps,
                    unsigned* nsamples) {
    if (!f) return LFDM_ERR_ARG;
    int rc = prepare(f);
    if (rc) return rc;
    double vs = 0;
    for (ModelGroup* g : {&f->g18, &f->g24})
        for (int32_t s : g->nsteps) vs += s;
    if (n18) *n18 = f->g18.n();
    if (n24) *n24 = f->g24.n();
    if (total_steps) *total_steps = f->total_steps;
    if (vehicle_steps) *vehicle_steps = vs;
    if (nsamples) *nsamples = (unsigned)f->nsamples;
    return LFDM_OK;
}

int lfdm_fleet_solve(lfdm_fleet* f) {
    if (!f) return LFDM_ERR_ARG;
    int rc = prepare(f);
    if (rc) return rc;
    FCK(cudaSetDevice(f->device));
    if (f->states_dirty) {
        for (ModelGroup* g : {&f->g18, &f->g24}) {
            rc = upload_states(f, *g);
            if (rc) return rc;
        }
        f->states_dirty = false;
    }
    rc = build_graph(f);
    if (rc) return rc;
    FCK(cudaEventRecord(f->ev0, f->stream));
    FCK(cudaGraphLaunch(f->graph_exec, f->stream));
    FCK(cudaEventRecord(f->ev1, f->stream));
    FCK(cudaStreamSynchronize(f->stream));
    float ms = 0;
    FCK(cudaEventElapsedTime(&ms, f->ev0, f->ev1));
    f->last_ms = ms;
    f->last_launches = f->graph_launches;
    f->device_newer = true;
    return LFDM_OK;
}

// Autotuner: times each candidate launch configuration on the first pilot_steps steps of the fleet
// (from the current states, which are restored afterwards) and keeps the fastest. Candidates:
// 32/64/128 threads per block, the maximum resident blocks per SM or half of it, and the whole
// pilot in one launch or in four.
int lfdm_fleet_tune(lfdm_fleet* f, unsigned pilot_steps, double* best_ms) {
    if (!f) return LFDM_ERR_ARG;
    int rc = prepare(f);
    if (rc) return rc;
    FCK(cudaSetDevice(f->device));
    if (f->states_dirty) {
        for (ModelGroup* g : {&f->g18, &f->g24}) {
            rc = upload_states(f, *g);
            if (rc) return rc;
        }
        f->states_dirty = false;
    }
    const int steps = (int)std::min<long long>(pilot_steps ? pilot_steps : 500, f->total_steps);
    for (ModelGroup* g : {&f->g18, &f->g24}) {
        if (!g->n()) continue;
        FCK(g->d_S_backup.ensure(g->d_S.n));
        FCK(cudaMemcpyAsync(g->d_S_backup.p, g->d_S.p, g->d_S.n * sizeof(double), cudaMemcpyDeviceToDevice,
                            f->stream));
    }
    struct Cand {
        unsigned threads, bps, spl;
        bool aff;
    };
    std::vector<Cand> cands;
    FCK(fleet_kernel_setup());
    for (unsigned th : {32u, 64u, 128u}) {
        int occ = 0;
        FCK(fleet_occupancy((int)th, f->f32(), &occ));
        if (occ < 1) continue;
        std::vector<unsigned> bl = {0u};
        if (occ >= 2) bl.push_back((unsigned)occ / 2);
        for (unsigned b : bl)
            for (unsigned spl : {0u, (unsigned)std::max(1, steps / 4)})
                for (bool aff : {false, true}) cands.push_back({th, b, spl, aff});
    }
    double best = 1e300;
    Cand best_c = {f->threads, f->blocks_per_sm, f->steps_per_launch, f->affinity};
    const bool both_models = f->g18.n() > 0 && f->g24.n() > 0;
    for (const Cand& c : cands) {
        if (c.aff && !both_models) continue;  // one model: the lists coincide
        f->affinity = c.aff;
        for (ModelGroup* g : {&f->g18, &f->g24})
            if (g->n())
                FCK(cudaMemcpyAsync(g->d_S.p, g->d_S_backup.p, g->d_S.n * sizeof(double), cudaMemcpyDeviceToDevice,
                                    f->stream));
        Plan p;
        rc = plan(f, steps, c.threads, c.bps, c.spl, &p);
        if (rc) return rc;
        FCK(cudaEventRecord(f->ev0, f->stream));
        rc = enqueue(f, steps, p);
        if (rc) return rc;
        FCK(cudaEventRecord(f->ev1, f->stream));
        FCK(cudaStreamSynchronize(f->stream));
        float ms = 0;
        FCK(cudaEventElapsedTime(&ms, f->ev0, f->ev1));
        if (ms < best) {
            best = ms;
            best_c = c;
        }
    }
    for (ModelGroup* g : {&f->g18, &f->g24}) {
        if (!g->n()) continue;
        FCK(cudaMemcpyAsync(g->d_S.p, g->d_S_backup.p, g->d_S.n * sizeof(double), cudaMemcpyDeviceToDevice,
                            f->stream));
        FCK(cudaMemsetAsync(g->d_status.p, 0, g->n() * sizeof(uint32_t), f->stream));
    }
    FCK(cudaStreamSynchronize(f->stream));
    f->threads = best_c.threads;
    f->blocks_per_sm = best_c.bps;
    f->affinity = best_c.aff;
    // the pilot's chunking, scaled to the whole horizon (0 = one launch)
    f->steps_per_launch = best_c.spl ? (unsigned)std::max<long long>(1, (long long)f->total_steps / 4) : 0;
    f->tune_ms = best;
    f->drop_graph();
    if (best_ms) *best_ms = best;
    return LFDM_OK;
}

int lfdm_fleet_last_ms(lfdm_fleet* f, double* ms, unsigned* launches) {
    if (!f) return LFDM_ERR_ARG;
    if (ms) *ms = f->last_ms;
    if (launches) *launches = f->last_launches;
    return LFDM_OK;
}

int lfdm_fleet_get_states(lfdm_fleet* f, int model, unsigned first, unsigned count, double* out) {
    if (!f || !out) return f ? f->fail(LFDM_ERR_ARG, "null argument") : LFDM_ERR_ARG;
    ModelGroup* g = f->group(model);
    if (!g) return f->fail(LFDM_ERR_ARG, "model %d", model);
    if ((size_t)first + count > g->n()) return f->fail(LFDM_ERR_ARG, "vehicles [%u, %u) out of range", first, first + count);
    if (f->device_newer) {
        for (ModelGroup* m : {&f->g18, &f->g24}) {
            int rc = download_states(f, *m);
            if (rc) return rc;
        }
        f->device_newer = false;
    }
    std::memcpy(out, &g->states[(size_t)first * g->ns], (size_t)count * g->ns * sizeof(double));
    return LFDM_OK;
}

int lfdm_fleet_set_states(lfdm_fleet* f, int model, unsigned first, unsigned count, const double* states) {
    if (!f || !states) return f ? f->fail(LFDM_ERR_ARG, "null argument") : LFDM_ERR_ARG;
    ModelGroup* g = f->group(model);
    if (!g) return f->fail(LFDM_ERR_ARG, "model %d", model);
    if ((size_t)first + count > g->n()) return f->fail(LFDM_ERR_ARG, "vehicles [%u, %u) out of range", first, first + count);
    if (f->device_newer) {
        for (ModelGroup* m : {&f->g18, &f->g24}) {
            int rc = download_states(f, *m);
            if (rc) return rc;
        }
        f->device_newer = false;
    }
    std::memcpy(&g->states[(size_t)first * g->ns], states, (size_t)count * g->ns * sizeof(double));
    f->states_dirty = true;
    return LFDM_OK;
}

// Response of one model, [nsamples][channels][n] in add order (samples a vehicle's horizon does not
// reach are zero).
int lfdm_fleet_get_response(lfdm_fleet* f, int model, double* out, size_t capacity, unsigned* nsamples) {
    if (!f) return LFDM_ERR_ARG;
    ModelGroup* g = f->group(model);
    if (!g) return f->fail(LFDM_ERR_ARG, "model %d", model);
    int rc = prepare(f);
    if (rc) return rc;
    if (nsamples) *nsamples = (unsigned)f->nsamples;
    const size_t n = g->n(), need = (size_t)f->nsamples * g->nch * n;
    if (!out) return LFDM_OK;
    if (capacity < need) return f->fail(LFDM_ERR_CAPACITY, "response needs %zu doubles, %zu given", need, capacity);
    if (need == 0) return LFDM_OK;
    std::vector<double> sorted(need);
    FCK(cudaMemcpy(sorted.data(), g->d_resp.p, need * sizeof(double), cudaMemcpyDeviceToHost));
    for (size_t r = 0; r < (size_t)f->nsamples * g->nch; ++r)
        for (size_t k = 0; k < n; ++k) out[r * n + g->perm[k]] = sorted[r * n + k];
    return LFDM_OK;
}

int lfdm_fleet_get_status_words(lfdm_fleet* f, int model, uint32_t* out) {
    if (!f || !out) return LFDM_ERR_ARG;
    ModelGroup* g = f->group(model);
    if (!g) return f->fail(LFDM_ERR_ARG, "model %d", model);
    const size_t n = g->n();
    if (!n) return LFDM_OK;
    std::vector<uint32_t> sorted(n);
    FCK(cudaMemcpy(sorted.data(), g->d_status.p, n * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    for (size_t k = 0; k < n; ++k) out[g->perm[k]] = sorted[k];
    return LFDM_OK;
}

}  // extern "C"
