// Host side of the library: the solver handle behind the C ABI of include/lfdm.h.
//
// Semantics follow d18SolverHalfImplicitGPU (18dof-gpu/dof18_halfImplicit_gpu.cu/.cuh):
//   * Construct appends num_vehicles vehicles of one parameter class (:53-285);
//   * Initialize copies one state into the next num_vehicles vehicles (:290-339);
//   * Solve integrates from t = 0 in windows of kernel_sim_time until the window start reaches the
//     end time (:404-494); SolveStep runs one window with constant controls (:497-550);
//   * SetOutput writes <file>_<idx>.csv files with the reference's header, zero first row and
//     per-window rows (:342-399, :552-663).
// Differences, all deliberate: errors are returned codes instead of prints/asserts/exit(); the
// device state is SoA in HBM (not managed AoS); a driver table is stored once for all vehicles of
// a Construct call; throttleMod scales a private copy of the engine map (the reference GPU code
// scales the shared map in place, dof18_gpu.cu:18-26, which compounds every step).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <memory>
#include <numeric>
#include <random>
#include <sstream>
#include <string>
#include <new>
#include <vector>

#include "../../include/lfdm.h"
#include "adjoint18.h"
#include "jacobian18.h"
#include "jacobian_fd.h"
#include "json_loader.h"
#include "kernels.h"

using namespace lfdm;

namespace {

thread_local std::string g_create_error;

template <typename T>
struct DevBuf {
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
    ~DevBuf() {
        if (p) cudaFree(p);
    }
};

}  // namespace

struct lfdm_solver {
    int model = 18;
    int ns = LFDM_S_COUNT;            // doubles per flat state vector of this model
    int nresp = LFDM18_RESP_CHANNELS; // response channels of this model
    unsigned N = 0;
    int device = 0;
    int npad = 0;
    cudaStream_t stream = nullptr, copy_stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t win_done[2] = {nullptr, nullptr}, copy_done[2] = {nullptr, nullptr};

    // host-side authoritative data
    std::vector<lfdm_class18> classes;
    std::vector<int32_t> class_of;
    std::vector<double> params;   // [N][P_COUNT]
    std::vector<double> rows;     // concatenated driver tables
    std::vector<int64_t> row_off;  // [N]
    std::vector<int32_t> row_len;  // [N]
    std::vector<double> states;   // [N][S_COUNT] host mirror
    int tire_type = -1;
    unsigned constructed = 0, initialized = 0;

    // settings (defaults of the reference constructor, dof18_halfImplicit_gpu.cu:14-22)
    double step = 0.001, tend = 0., ksim = 2., host_dump = 10.;
    unsigned tpb_hint = 32;
    int threads = 128;
    int precision = LFDM_PREC_FP64;
    int split = -1;  // 11-DOF split-warp kernel: -1 for small fleets, 0 never, 1 always

    // CSV output (SetOutput)
    bool output = false;
    std::string out_file;
    double dtout = 0;
    bool store_all = false;
    unsigned num_outs = 0;
    std::vector<unsigned> which_outs;
    std::vector<std::ostringstream> csv;

    // response streaming
    double* resp_host = nullptr;
    size_t resp_cap = 0;
    double resp_dtout = 0;
    double* resp_dev = nullptr;
    size_t resp_dev_cap = 0;
    double resp_dev_dtout = 0;
    size_t resp_written = 0;

    // device mirrors
    DevBuf<double> d_params, d_K, d_S, d_rows, d_aos, d_ctl, d_resp, d_sched;
    DevBuf<int64_t> d_off;
    DevBuf<int32_t> d_len, d_class_of, d_samples;
    DevBuf<unsigned char> d_classes, d_classes_f;
    DevBuf<uint32_t> d_status;
    DevBuf<unsigned> d_bad;
    // differentiable rollout (lfdm_traj18_*)
    DevBuf<double> d_adj_ckpt, d_adj_tape;
    // right-hand-side Jacobians with host buffers (lfdm_rhs_jacobian_host)
    DevBuf<double> d_jac_in, d_jac_s, d_jac_u;
    unsigned adj_nsteps = 0, adj_ckpt = 0;
    bool adj_valid = false;
    double adj_fwd_ms = 0, adj_bwd_ms = 0;
    bool rows_device_only = false;  // driver rows live only in d_rows (bulk upload path)
    bool dirty_params = true, dirty_classes = true, dirty_tables = true, dirty_states = true;
    bool device_newer = false;  // device state newer than host mirror

    double last_ms = 0;
    unsigned last_launches = 0;
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
    int cuda_fail(cudaError_t e, const char* what) {
        return fail(LFDM_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    }
};

#define CK(expr)                                                     \
    do {                                                             \
        cudaError_t e_ = (expr);                                     \
        if (e_ != cudaSuccess) return h->cuda_fail(e_, #expr);       \
    } while (0)

namespace {

int set_device(lfdm_solver* h) {
    cudaError_t e = cudaSetDevice(h->device);
    if (e != cudaSuccess) return h->cuda_fail(e, "cudaSetDevice");
    return LFDM_OK;
}

// Number of steps and sample steps of a window starting at t0: the reference's device loop
// (dof18_halfImplicit_gpu.cu:893-975) simulated on the host in the same FP64 arithmetic.
void window_schedule(double t0, double ksim, double dt, double dtout, int spw, int& nsteps, std::vector<int32_t>& samp,
                     std::vector<double>* times = nullptr) {
    double t = t0, kt = 0;
    const double end_time = (t + ksim) - dt / 10.;
    int s = 0, stored = 0;
    samp.clear();
    while (t < end_time) {
        if (times) times->push_back(t);
        t += dt;
        kt += dt;
        ++s;
        if (dtout > 0 && std::fabs(kt - (stored + 1) * dtout) < 1e-7) {
            if (stored < spw) samp.push_back(s);
            ++stored;
        }
    }
    nsteps = s;
}

// initializeTireSus (24dof-gpu/dof24_gpu.cu:34-90), which the reference's Initialize applies to
// each vehicle's state (dof24_halfImplicit_gpu.cu:311-345): static tire loads and compressions,
// spring preload and strut lengths from the vehicle's parameters p; unsprung vertical speed = w.
void init_tire_sus24(const double* p, double* s) {
    const double G = 9.81;  // utils/utils_gpu.cuh
    const double a = p[LFDM_P_A], b = p[LFDM_P_B], m = p[LFDM_P_M], ks = p[LFDM_P_KS];
    const double fz_f = (m * G * b) / (2 * (a + b)) + p[LFDM_P_MUF] * G;
    const double fz_r = (m * G * a) / (2 * (a + b)) + p[LFDM_P_MUR] * G;
    const double xsi_f = (m * G * b) / (2 * (a + b) * ks);
    const double xsi_r = (m * G * a) / (2 * (a + b) * ks);
    for (int c = 0; c < 4; ++c) {
        double* t = s + LFDM24_S_TIRE0 + c * LFDM24_T_COUNT;
        double* su = s + LFDM24_S_SUS0 + c * LFDM24_SUS_COUNT;
        t[LFDM24_T_FZ] = c < 2 ? fz_f : fz_r;
        t[LFDM24_T_XT] = t[LFDM24_T_FZ] / p[LFDM_P_KT];
        su[LFDM24_SUS_XSI] = c < 2 ? xsi_f : xsi_r;
        su[LFDM24_SUS_XS] = su[LFDM24_SUS_XSI];
        su[LFDM24_SUS_LSI] = p[LFDM_P_H] - (p[LFDM_P_R0] - t[LFDM24_T_XT]);
        su[LFDM24_SUS_LS] = su[LFDM24_SUS_LSI];
        su[LFDM24_SUS_WU] = s[LFDM24_S_W];
    }
}

int sync_device(lfdm_solver* h) {
    int rc = set_device(h);
    if (rc) return rc;
    const size_t N = h->N, np = (size_t)h->npad;
    if (h->dirty_classes) {
        const size_t cs = class_dev18_size();
        std::vector<unsigned char> buf(cs * std::max<size_t>(1, h->classes.size()));
        for (size_t i = 0; i < h->classes.size(); ++i)
            build_class_dev18(h->classes[i], reinterpret_cast<ClassDev18*>(buf.data() + i * cs));
        CK(h->d_classes.ensure(buf.size()));
        CK(cudaMemcpyAsync(h->d_classes.p, buf.data(), buf.size(), cudaMemcpyHostToDevice, h->stream));
        const size_t csf = class_dev18f_size();
        std::vector<unsigned char> buff(csf * std::max<size_t>(1, h->classes.size()));
        for (size_t i = 0; i < h->classes.size(); ++i)
            build_class_dev18f(h->classes[i], reinterpret_cast<ClassDev18F*>(buff.data() + i * csf));
        CK(h->d_classes_f.ensure(buff.size()));
        CK(cudaMemcpyAsync(h->d_classes_f.p, buff.data(), buff.size(), cudaMemcpyHostToDevice, h->stream));
        CK(h->d_class_of.ensure(N));
        CK(cudaMemcpyAsync(h->d_class_of.p, h->class_of.data(), N * sizeof(int32_t), cudaMemcpyHostToDevice,
                           h->stream));
        CK(cudaStreamSynchronize(h->stream));
        h->dirty_classes = false;
    }
    if (h->dirty_params) {
        CK(h->d_params.ensure(N * LFDM_P_COUNT));
        CK(h->d_K.ensure((size_t)(h->model == LFDM_MODEL_24 ? k24_count() : k18_count()) * np));
        CK(cudaMemcpyAsync(h->d_params.p, h->params.data(), N * LFDM_P_COUNT * sizeof(double),
                           cudaMemcpyHostToDevice, h->stream));
        CK(h->model == LFDM_MODEL_24 ? launch_prepare24(h->d_params.p, (int)N, h->npad, h->d_K.p, h->stream)
                                     : launch_prepare18(h->d_params.p, (int)N, h->npad, h->d_K.p, h->stream));
        h->dirty_params = false;
    }
    if (h->dirty_tables) {
        if (!h->rows.empty() && !h->rows_device_only) {
            CK(h->d_rows.ensure(h->rows.size()));
            CK(cudaMemcpyAsync(h->d_rows.p, h->rows.data(), h->rows.size() * sizeof(double), cudaMemcpyHostToDevice,
                               h->stream));
        }
        CK(h->d_off.ensure(N));
        CK(h->d_len.ensure(N));
        CK(cudaMemcpyAsync(h->d_off.p, h->row_off.data(), N * sizeof(int64_t), cudaMemcpyHostToDevice, h->stream));
        CK(cudaMemcpyAsync(h->d_len.p, h->row_len.data(), N * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        h->dirty_tables = false;
    }
    if (h->dirty_states) {
        CK(h->d_S.ensure(h->ns * np));
        CK(h->d_aos.ensure(N * h->ns));
        CK(cudaMemcpyAsync(h->d_aos.p, h->states.data(), N * h->ns * sizeof(double), cudaMemcpyHostToDevice,
                           h->stream));
        CK(launch_states_to_soa(h->d_aos.p, (int)N, h->ns, h->npad, h->d_S.p, h->stream));
        h->dirty_states = false;
    }
    CK(h->d_status.ensure(N));
    CK(cudaStreamSynchronize(h->stream));
    return LFDM_OK;
}

int pull_states(lfdm_solver* h) {
    if (!h->device_newer) return LFDM_OK;
    int rc = set_device(h);
    if (rc) return rc;
    CK(launch_states_to_aos(h->d_S.p, (int)h->N, h->ns, h->npad, h->d_aos.p, h->stream));
    CK(cudaMemcpyAsync(h->states.data(), h->d_aos.p, (size_t)h->N * h->ns * sizeof(double),
                       cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    h->device_newer = false;
    return LFDM_OK;
}

// Bring device-only driver rows back to the host mirror (before a partial table update).
int pull_rows(lfdm_solver* h) {
    if (!h->rows_device_only) return LFDM_OK;
    int rc = set_device(h);
    if (rc) return rc;
    size_t nd = 0;
    for (unsigned i = 0; i < h->N; ++i)
        nd = std::max(nd, (size_t)(h->row_off[i] + h->row_len[i]) * 4);
    h->rows.resize(nd);
    if (nd) CK(cudaMemcpy(h->rows.data(), h->d_rows.p, nd * sizeof(double), cudaMemcpyDeviceToHost));
    h->rows_device_only = false;
    return LFDM_OK;
}

int check_ready(lfdm_solver* h, bool need_tables) {
    if (h->constructed != h->N)
        return h->fail(LFDM_ERR_STATE, "%u of %u vehicles constructed; call Construct for all vehicles", h->constructed,
                       h->N);
    if (h->initialized != h->N)
        return h->fail(LFDM_ERR_STATE, "%u of %u vehicles initialized; call Initialize for all vehicles",
                       h->initialized, h->N);
    if (need_tables) {
        for (unsigned i = 0; i < h->N; ++i)
            if (h->row_len[i] <= 0)
                return h->fail(LFDM_ERR_STATE, "vehicle %u has no driver table (Construct without a driver file)", i);
    }
    return LFDM_OK;
}

void csv_header(lfdm_solver* h) {
    // 18dof-gpu/dof18_halfImplicit_gpu.cu SolveStep header; 11dof-gpu/dof11_halfImplicit_gpu.cu:561-569
    static const char* hdr18[] = {"time", "x", "y", "vx", "vy", "roll", "yaw", "roll_rate", "yaw_rate",
                                  "wlf", "wrf", "wlr", "wrr"};
    static const char* hdr11[] = {"time", "x", "y", "vx", "vy", "yaw", "yaw_rate", "wf", "wr"};
    // 24dof-gpu/dof24_halfImplicit_gpu.cu:608-622
    static const char* hdr24[] = {"time",      "x",        "y",          "vx",  "vy",  "roll", "yaw", "pitch",
                                  "roll_rate", "yaw_rate", "pitch_rate", "wlf", "wrf", "wlr",  "wrr"};
    const char* const* hdr = h->model == LFDM_MODEL_11 ? hdr11 : h->model == LFDM_MODEL_24 ? hdr24 : hdr18;
    for (unsigned k = 0; k < h->num_outs; ++k) {
        auto& os = h->csv[k];
        for (int c = 0; c < h->nresp; ++c) os << hdr[c] << ",";
        os << std::endl;
        for (int c = 0; c < h->nresp; ++c) os << 0 << ",";
        os << std::endl;
    }
}

void csv_append(lfdm_solver* h, const double* resp, int samples) {
    const size_t N = h->N;
    for (unsigned k = 0; k < h->num_outs; ++k) {
        const unsigned idx = h->store_all ? k : h->which_outs[k];
        auto& os = h->csv[k];
        for (int s = 0; s < samples; ++s) {
            const double* r = resp + (size_t)s * h->nresp * N;
            for (int c = 0; c < h->nresp; ++c) os << r[(size_t)c * N + idx] << ",";
            os << std::endl;
        }
    }
}

int csv_write(lfdm_solver* h) {
    for (unsigned k = 0; k < h->num_outs; ++k) {
        const unsigned idx = h->store_all ? k : h->which_outs[k];
        std::string path = h->out_file + "_" + std::to_string(idx) + ".csv";
        std::ofstream f(path.c_str());
        if (!f) return h->fail(LFDM_ERR_IO, "cannot write %s", path.c_str());
        f << h->csv[k].str();
        h->csv[k].str("");
        h->csv[k].clear();
    }
    return LFDM_OK;
}

// Runs windows. solve_all: the Solve() schedule (starts 0, k, 2k, ... while start < tend), of which
// only windows starting in [t0, t_end) are run; otherwise exactly one window starting at t0.
int run_windows(lfdm_solver* h, double t0, double t_end, bool solve_all, int ctl_mode, double st, double th,
                double br, const double* ctl_dev, const double* sched_dev, unsigned sched_steps, bool csv_ok) {
    int rc = sync_device(h);
    if (rc) return rc;
    const size_t N = h->N;
    // output configuration: CSV (reference semantics), response streaming to host, or device
    const bool csv = h->output && solve_all && csv_ok;
    const bool dev_resp = h->resp_dev != nullptr && solve_all && !csv;
    const bool stream_resp = h->resp_host != nullptr && solve_all && !csv && !dev_resp;
    const double dtout = csv ? h->dtout : (stream_resp ? h->resp_dtout : (dev_resp ? h->resp_dev_dtout : 0.0));
    const int spw = dtout > 0 ? (int)std::ceil(h->ksim / dtout) : 0;
    const size_t slot = (size_t)spw * h->nresp * N;  // doubles per window buffer
    const int nbuf = stream_resp ? 2 : 1;
    if (dtout > 0 && !dev_resp) CK(h->d_resp.ensure(slot * nbuf));
    size_t dev_windows = 0;
    if (dev_resp) {
        dev_windows = spw > 0 ? h->resp_dev_cap / slot : 0;
        if (dev_windows == 0 || dev_windows * slot != h->resp_dev_cap)
            return h->fail(LFDM_ERR_CAPACITY, "device response buffer must hold a whole number of windows (%zu doubles)",
                           slot);
    }
    std::vector<double> host_window;
    if (csv) {
        host_window.resize(slot);
        csv_header(h);
    }
    CK(cudaMemsetAsync(h->d_status.p, 0, N * sizeof(uint32_t), h->stream));

    Window18 w;
    w.n = (int)N;
    w.npad = h->npad;
    w.tire_nr = h->tire_type == LFDM_TIRE_TMEASY_NR;
    w.precision = h->precision;
    w.dt = h->step;
    w.K = h->d_K.p;
    w.classes = reinterpret_cast<const ClassDev18*>(h->d_classes.p);
    w.classes_f = reinterpret_cast<const ClassDev18F*>(h->d_classes_f.p);
    if (h->precision == LFDM_PREC_MIXED && w.tire_nr)
        return h->fail(LFDM_ERR_ARG, "the FP32 right-hand-side stepper supports TMeasy tires only");
    w.nclasses = (int)h->classes.size();
    w.class_of = h->d_class_of.p;
    w.S = h->d_S.p;
    w.ctl_mode = ctl_mode;
    w.rows = h->d_rows.p;
    w.row_off = h->d_off.p;
    w.row_len = h->d_len.p;
    w.steer = st;
    w.thr = th;
    w.brk = br;
    w.ctl = ctl_dev;
    w.sched = sched_dev;
    w.status = h->d_status.p;
    w.threads = h->threads;
    w.split = h->split;

    std::vector<int32_t> samp;
    double current = solve_all ? 0.0 : t0;
    unsigned launches = 0;
    size_t widx = 0;
    float total_ms = 0;
    if (!solve_all || t0 <= 0) h->resp_written = 0;
    const size_t resp_cap_samples = stream_resp ? h->resp_cap / (h->nresp * N) : 0;
    if (stream_resp && resp_cap_samples == 0)
        return h->fail(LFDM_ERR_CAPACITY, "response buffer holds less than one sample");
    for (;;) {
        if (solve_all && !(current < h->tend && current < t_end)) break;
        if (solve_all && current < t0) {  // window before the requested range: same start times as Solve
            current = current + h->ksim;
            ++widx;
            continue;
        }
        int nsteps = 0;
        window_schedule(current, h->ksim, h->step, dtout, spw, nsteps, samp);
        if (sched_dev && (unsigned)nsteps != sched_steps)
            return h->fail(LFDM_ERR_ARG, "control schedule has %u steps, the window has %d", sched_steps, nsteps);
        const int b = (int)(widx % nbuf);
        if (dtout > 0 && !samp.empty()) {
            CK(h->d_samples.ensure((size_t)(spw + 1) * nbuf));
            // sample-step lists are tiny; copy synchronously on the compute stream
            CK(cudaMemcpyAsync(h->d_samples.p + (size_t)b * (spw + 1), samp.data(), samp.size() * sizeof(int32_t),
                               cudaMemcpyHostToDevice, h->stream));
        }
        if (stream_resp && launches >= 2) CK(cudaStreamWaitEvent(h->stream, h->copy_done[b], 0));
        w.t0 = current;
        w.nsteps = nsteps;
        w.resp = dtout > 0 ? (dev_resp ? h->resp_dev + (widx % dev_windows) * slot : h->d_resp.p + (size_t)b * slot)
                           : nullptr;
        w.nsamples = dtout > 0 ? (int)samp.size() : 0;
        w.sample_steps = dtout > 0 ? h->d_samples.p + (size_t)b * (spw + 1) : nullptr;
        CK(cudaEventRecord(h->ev0, h->stream));
        CK(h->model == LFDM_MODEL_11   ? launch_window11(w, h->stream)
           : h->model == LFDM_MODEL_24 ? launch_window24(w, h->stream)
                                       : launch_window18(w, h->stream));
        CK(cudaEventRecord(h->ev1, h->stream));
        ++launches;
        if (stream_resp) {
            CK(cudaEventRecord(h->win_done[b], h->stream));
            CK(cudaStreamWaitEvent(h->copy_stream, h->win_done[b], 0));
            // window samples k land at global sample widx*spw + k (ring over the caller's buffer);
            // one copy per contiguous run of ring slots
            const size_t per = h->nresp * N;
            for (int k = 0; k < w.nsamples;) {
                const size_t gs = widx * (size_t)spw + k;
                const size_t slot0 = gs % resp_cap_samples;
                const int run = (int)std::min<size_t>((size_t)(w.nsamples - k), resp_cap_samples - slot0);
                CK(cudaMemcpyAsync(h->resp_host + slot0 * per, w.resp + (size_t)k * per, run * per * sizeof(double),
                                   cudaMemcpyDeviceToHost, h->copy_stream));
                k += run;
            }
            CK(cudaEventRecord(h->copy_done[b], h->copy_stream));
            h->resp_written = widx * (size_t)spw + w.nsamples;
        }
        if (csv) {
            CK(cudaMemcpyAsync(host_window.data(), w.resp, slot * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
            CK(cudaStreamSynchronize(h->stream));
            csv_append(h, host_window.data(), spw);
        }
        CK(cudaEventSynchronize(h->ev1));
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
        total_ms += ms;
        current = current + h->ksim;
        ++widx;
        if (!solve_all) break;
    }
    if (stream_resp) CK(cudaStreamSynchronize(h->copy_stream));
    CK(cudaStreamSynchronize(h->stream));
    h->device_newer = true;
    h->last_ms = total_ms;
    h->last_launches = launches;
    if (csv) {
        rc = csv_write(h);
        if (rc) return rc;
    }
    // non-finite check
    std::vector<uint32_t> st_words(N);
    CK(cudaMemcpy(st_words.data(), h->d_status.p, N * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < N; ++i)
        if (st_words[i] & 1u)
            return h->fail(LFDM_ERR_NUMERIC, "vehicle %zu reached a non-finite state", i);
    return LFDM_OK;
}

int append_vehicles(lfdm_solver* h, const lfdm_class18& cls, const double* params_one, const double* params_many,
                    unsigned n, int tire_type, const std::vector<double>* table) {
    if (n == 0) return h->fail(LFDM_ERR_ARG, "num_vehicles must be > 0");
    if ((size_t)h->constructed + n > h->N)
        return h->fail(LFDM_ERR_CAPACITY,
                       "Number of vehicles added makes the vehicle count greater than the total number of vehicles "
                       "(%u + %u > %u)",
                       h->constructed, n, h->N);
    if (tire_type != LFDM_TIRE_TMEASY && tire_type != LFDM_TIRE_TMEASY_NR)
        return h->fail(LFDM_ERR_ARG, "unknown tire type %d", tire_type);
    if (h->tire_type >= 0 && h->tire_type != tire_type)
        return h->fail(LFDM_ERR_STATE, "all vehicles of a solver use one tire type");
    if (cls.noGears < 1 || cls.noGears > LFDM_MAX_GEARS) return h->fail(LFDM_ERR_ARG, "bad gear count %d", cls.noGears);
    for (int s : {cls.powertrainMapSize, cls.lossesMapSize})
        if (s < 1 || s > LFDM_MAX_MAP) return h->fail(LFDM_ERR_ARG, "engine/loss map size %d out of range", s);
    if (cls.tcbool && (cls.CFmapSize < 1 || cls.TRmapSize < 1 || cls.CFmapSize > LFDM_MAX_MAP ||
                       cls.TRmapSize > LFDM_MAX_MAP))
        return h->fail(LFDM_ERR_ARG, "torque converter maps missing or too long");
    if (cls.nonLinearSteer && (cls.steerMapSize < 1 || cls.steerMapSize > LFDM_MAX_MAP))
        return h->fail(LFDM_ERR_ARG, "steering map missing or too long");
    if (table) {
        for (size_t r = 1; r < table->size() / 4; ++r)
            if ((*table)[4 * r] < (*table)[4 * (r - 1)])
                return h->fail(LFDM_ERR_PARSE, "driver table times must be non-decreasing (row %zu)", r);
    }
    if (table) {
        int rc = pull_rows(h);
        if (rc) return rc;
    }
    h->tire_type = tire_type;
    const int ci = (int)h->classes.size();
    h->classes.push_back(cls);
    int64_t off = -1;
    int32_t len = 0;
    if (table) {
        off = (int64_t)(h->rows.size() / 4);
        len = (int32_t)(table->size() / 4);
        h->rows.insert(h->rows.end(), table->begin(), table->end());
    }
    for (unsigned k = 0; k < n; ++k) {
        const unsigned i = h->constructed + k;
        h->class_of[i] = ci;
        std::memcpy(&h->params[(size_t)i * LFDM_P_COUNT], params_many ? params_many + (size_t)k * LFDM_P_COUNT : params_one,
                    LFDM_P_COUNT * sizeof(double));
        h->row_off[i] = off < 0 ? 0 : off;
        h->row_len[i] = len;
    }
    h->constructed += n;
    h->dirty_params = h->dirty_classes = true;
    if (table) h->dirty_tables = true;
    return LFDM_OK;
}

}  // namespace

// =============================================================================================
extern "C" {

const char* lfdm_version(void) { return "lfdm-gb300 0.1 (sm_103a, FP64 + mixed)"; }

int lfdm_measure_fp64_peak(int device, double* dfma_per_s) {
    return lfdm_measure_fp64_peak_clock(device, dfma_per_s, nullptr);
}

int lfdm_measure_fp64_peak_clock(int device, double* dfma_per_s, double* sm_ghz) {
    if (!dfma_per_s) return LFDM_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return LFDM_ERR_NODEVICE;
    return measure_dfma_rate(dfma_per_s, sm_ghz) == cudaSuccess ? LFDM_OK : LFDM_ERR_CUDA;
}

int lfdm_measure_fp32_peak_clock(int device, double* ffma_per_s, double* sm_ghz) {
    if (!ffma_per_s) return LFDM_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return LFDM_ERR_NODEVICE;
    return measure_ffma_rate(ffma_per_s, sm_ghz) == cudaSuccess ? LFDM_OK : LFDM_ERR_CUDA;
}

int lfdm_create_on_device(int model, unsigned total_num_vehicles, int device, lfdm_solver** out) {
    if (!out) return LFDM_ERR_ARG;
    *out = nullptr;
    if (model != LFDM_MODEL_18 && model != LFDM_MODEL_11 && model != LFDM_MODEL_24) {
        g_create_error = "model " + std::to_string(model) + " is not one of the library's models (11, 18, 24)";
        return LFDM_ERR_ARG;
    }
    if (total_num_vehicles == 0 || total_num_vehicles > (1u << 30)) {
        g_create_error = "total_num_vehicles must be in [1, 2^30]";
        return LFDM_ERR_ARG;
    }
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        g_create_error = std::string("no CUDA device: ") + cudaGetErrorString(e);
        return LFDM_ERR_NODEVICE;
    }
    if (device < 0 || device >= ndev) {
        g_create_error = "device index out of range";
        return LFDM_ERR_ARG;
    }
    std::unique_ptr<lfdm_solver> h(new lfdm_solver());
    h->model = model;
    if (model == LFDM_MODEL_11) {
        h->ns = LFDM11_S_COUNT;
        h->nresp = LFDM11_RESP_CHANNELS;
    } else if (model == LFDM_MODEL_24) {
        h->ns = LFDM24_S_COUNT;
        h->nresp = LFDM24_RESP_CHANNELS;
    }
    h->N = total_num_vehicles;
    h->device = device;
    h->npad = (int)((total_num_vehicles + 127) / 128 * 128);
    if ((e = cudaSetDevice(device)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreate(&h->ev0)) != cudaSuccess || (e = cudaEventCreate(&h->ev1)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&h->win_done[0], cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&h->win_done[1], cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&h->copy_done[0], cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&h->copy_done[1], cudaEventDisableTiming)) != cudaSuccess) {
        g_create_error = std::string("CUDA setup failed: ") + cudaGetErrorString(e);
        return LFDM_ERR_CUDA;
    }
    h->class_of.assign(h->N, 0);
    h->params.assign((size_t)h->N * LFDM_P_COUNT, 0.0);
    h->row_off.assign(h->N, 0);
    h->row_len.assign(h->N, 0);
    h->states.assign((size_t)h->N * h->ns, 0.0);
    *out = h.release();
    return LFDM_OK;
}

int lfdm_create(int model, unsigned total_num_vehicles, lfdm_solver** out) {
    return lfdm_create_on_device(model, total_num_vehicles, 0, out);
}

int lfdm_destroy(lfdm_solver* h) {
    if (!h) return LFDM_ERR_ARG;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->copy_stream) cudaStreamSynchronize(h->copy_stream);
    for (cudaEvent_t e : {h->ev0, h->ev1, h->win_done[0], h->win_done[1], h->copy_done[0], h->copy_done[1]})
        if (e) cudaEventDestroy(e);
    if (h->stream) cudaStreamDestroy(h->stream);
    if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
    delete h;
    return LFDM_OK;
}

const char* lfdm_last_error(const lfdm_solver* h) { return h ? h->err.c_str() : g_create_error.c_str(); }

int lfdm_construct(lfdm_solver* h, const char* veh_json, const char* tire_json, const char* sus_json,
                   unsigned num_vehicles, const char* driver_file, int tire_type) {
    if (!h || !veh_json || !tire_json) return h ? h->fail(LFDM_ERR_ARG, "null path") : LFDM_ERR_ARG;
    if (h->model == LFDM_MODEL_24 && !sus_json) return h->fail(LFDM_ERR_ARG, "the 24-DOF model needs a suspension file");
    if (h->model != LFDM_MODEL_24 && sus_json)
        return h->fail(LFDM_ERR_ARG, "suspension file given for a %d-DOF solver", h->model);
    lfdm_class18 cls;
    std::vector<double> p(LFDM_P_COUNT);
    std::string err;
    if (!load_vehicle(h->model, veh_json, tire_json, sus_json ? sus_json : "", tire_type, cls, p.data(), err))
        return h->fail(err.rfind("cannot open", 0) == 0 ? LFDM_ERR_IO : LFDM_ERR_PARSE, "%s", err.c_str());
    std::vector<double> table;
    if (driver_file) {
        if (!load_driver_file(driver_file, table, err)) {
            return h->fail(err.rfind("cannot open", 0) == 0 ? LFDM_ERR_IO : LFDM_ERR_PARSE, "%s", err.c_str());
        }
    }
    return append_vehicles(h, cls, p.data(), nullptr, num_vehicles, tire_type, driver_file ? &table : nullptr);
}

int lfdm_construct_class(lfdm_solver* h, const lfdm_class18* cls, unsigned num_vehicles, const double* params,
                         int tire_type) {
    if (!h || !cls || !params) return h ? h->fail(LFDM_ERR_ARG, "null argument") : LFDM_ERR_ARG;
    return append_vehicles(h, *cls, nullptr, params, num_vehicles, tire_type, nullptr);
}

int lfdm_set_params(lfdm_solver* h, unsigned first, unsigned count, const double* params) {
    if (!h || !params) return h ? h->fail(LFDM_ERR_ARG, "null argument") : LFDM_ERR_ARG;
    if ((size_t)first + count > h->constructed)
        return h->fail(LFDM_ERR_ARG, "vehicles [%u, %u) not constructed", first, first + count);
    std::memcpy(&h->params[(size_t)first * LFDM_P_COUNT], params, (size_t)count * LFDM_P_COUNT * sizeof(double));
    h->dirty_params = true;
    return LFDM_OK;
}

int lfdm_get_params(lfdm_solver* h, unsigned first, unsigned count, double* params) {
    if (!h || !params) return h ? h->fail(LFDM_ERR_ARG, "null argument") : LFDM_ERR_ARG;
    if ((size_t)first + count > h->N) return h->fail(LFDM_ERR_ARG, "index out of range");
    std::memcpy(params, &h->params[(size_t)first * LFDM_P_COUNT], (size_t)count * LFDM_P_COUNT * sizeof(double));
    return LFDM_OK;
}

int lfdm_tire_init(double* params) {
    if (!params) return LFDM_ERR_ARG;
    tire_init(params);
    return LFDM_OK;
}

static int set_tables(lfdm_solver* h, unsigned first, unsigned count, const double* rows, unsigned nrows, bool shared) {
    if (!h || !rows || nrows == 0) return h ? h->fail(LFDM_ERR_ARG, "empty driver table") : LFDM_ERR_ARG;
    if ((size_t)first + count > h->N) return h->fail(LFDM_ERR_ARG, "vehicles [%u, %u) out of range", first, first + count);
    const unsigned ntab = shared ? 1 : count;
    const bool all = first == 0 && count == h->N;
    if (all) {
        // every table replaced: DMA straight from the caller's buffer (page-locked buffers copy at
        // full link speed), validate on the device, keep no host copy
        int rc = set_device(h);
        if (rc) return rc;
        const size_t nd = (size_t)ntab * nrows * 4;
        CK(h->d_rows.ensure(nd));
        CK(cudaMemcpyAsync(h->d_rows.p, rows, nd * sizeof(double), cudaMemcpyHostToDevice, h->stream));
        CK(h->d_bad.ensure(1));
        CK(cudaMemsetAsync(h->d_bad.p, 0, sizeof(unsigned), h->stream));
        CK(launch_check_tables(h->d_rows.p, ntab, (int)nrows, h->d_bad.p, h->stream));
        unsigned bad = 0;
        CK(cudaMemcpyAsync(&bad, h->d_bad.p, sizeof(unsigned), cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        if (bad) {
            h->dirty_tables = true;  // restore the previous tables at the next solve
            return h->fail(LFDM_ERR_PARSE, "driver tables: %u rows have a time smaller than the previous row", bad);
        }
        h->rows.clear();
        h->rows.shrink_to_fit();
        h->rows_device_only = true;
        for (unsigned k = 0; k < count; ++k) {
            h->row_off[k] = shared ? 0 : (int64_t)k * nrows;
            h->row_len[k] = (int32_t)nrows;
        }
        CK(h->d_off.ensure(h->N));
        CK(h->d_len.ensure(h->N));
        CK(cudaMemcpyAsync(h->d_off.p, h->row_off.data(), h->N * sizeof(int64_t), cudaMemcpyHostToDevice, h->stream));
        CK(cudaMemcpyAsync(h->d_len.p, h->row_len.data(), h->N * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        h->dirty_tables = false;
        return LFDM_OK;
    }
    for (unsigned k = 0; k < ntab; ++k) {
        const double* t = rows + (size_t)k * nrows * 4;
        for (unsigned r = 1; r < nrows; ++r)
            if (t[4 * r] < t[4 * (r - 1)])
                return h->fail(LFDM_ERR_PARSE, "driver table %u: times must be non-decreasing (row %u)", k, r);
    }
    int rc = pull_rows(h);
    if (rc) return rc;
    const int64_t base = (int64_t)(h->rows.size() / 4);
    const int64_t b2 = base;
    h->rows.insert(h->rows.end(), rows, rows + (size_t)ntab * nrows * 4);
    for (unsigned k = 0; k < count; ++k) {
        h->row_off[first + k] = b2 + (shared ? 0 : (int64_t)k * nrows);
        h->row_len[first + k] = (int32_t)nrows;
    }
    h->dirty_tables = true;
    return LFDM_OK;
}

int lfdm_set_driver_table(lfdm_solver* h, unsigned first, unsigned count, const double* rows, unsigned nrows) {
    return set_tables(h, first, count, rows, nrows, true);
}
int lfdm_set_driver_tables(lfdm_solver* h, unsigned first, unsigned count, const double* rows, unsigned nrows) {
    return set_tables(h, first, count, rows, nrows, false);
}

int lfdm_initialize(lfdm_solver* h, const double* state, unsigned num_vehicles) {
    if (!h || !state) return h ? h->fail(LFDM_ERR_ARG, "null argument") : LFDM_ERR_ARG;
    if ((size_t)h->initialized + num_vehicles > h->N)
        return h->fail(LFDM_ERR_CAPACITY,
                       "Number of vehicles added makes the vehicle count greater than the total number of vehicles "
                       "(%u + %u > %u)",
                       h->initialized, num_vehicles, h->N);
    if (h->model == LFDM_MODEL_24 && h->initialized + num_vehicles > h->constructed)
        return h->fail(LFDM_ERR_STATE, "24-DOF vehicles must be constructed before Initialize (initializeTireSus "
                                       "uses their parameters)");
    int rc = pull_states(h);
    if (rc) return rc;
    for (unsigned k = 0; k < num_vehicles; ++k) {
        double* dst = &h->states[(size_t)(h->initialized + k) * h->ns];
        std::memcpy(dst, state, h->ns * sizeof(double));
        if (h->model == LFDM_MODEL_24) init_tire_sus24(&h->params[(size_t)(h->initialized + k) * LFDM_P_COUNT], dst);
    }
    h->initialized += num_vehicles;
    h->dirty_states = true;
    return LFDM_OK;
}

int lfdm_set_states(lfdm_solver* h, unsigned first, unsigned count, const double* states) {
    if (!h || !states) return h ? h->fail(LFDM_ERR_ARG, "null argument") : LFDM_ERR_ARG;
    if ((size_t)first + count > h->N) return h->fail(LFDM_ERR_ARG, "vehicles [%u, %u) out of range", first, first + count);
    if (!(first == 0 && count == h->N)) {
        int rc = pull_states(h);
        if (rc) return rc;
    }
    std::memcpy(&h->states[(size_t)first * h->ns], states, (size_t)count * h->ns * sizeof(double));
    h->initialized = std::max(h->initialized, first + count);
    h->device_newer = false;
    h->dirty_states = true;
    return LFDM_OK;
}

int lfdm_get_states(lfdm_solver* h, unsigned first, unsigned count, double* states) {
    if (!h || !states) return h ? h->fail(LFDM_ERR_ARG, "null argument") : LFDM_ERR_ARG;
    if ((size_t)first + count > h->N) return h->fail(LFDM_ERR_ARG, "index out of range");
    int rc = pull_states(h);
    if (rc) return rc;
    std::memcpy(states, &h->states[(size_t)first * h->ns], (size_t)count * h->ns * sizeof(double));
    return LFDM_OK;
}

int lfdm_get_sim_state(lfdm_solver* h, unsigned i, double* state) {
    if (!h || !state) return h ? h->fail(LFDM_ERR_ARG, "null argument") : LFDM_ERR_ARG;
    if (i >= h->N) return h->fail(LFDM_ERR_ARG, "Vehicle index out of bounds (%u >= %u)", i, h->N);
    if (h->device_newer) {
        int rc = set_device(h);
        if (rc) return rc;
        CK(cudaMemcpy2D(state, sizeof(double), h->d_S.p + i, (size_t)h->npad * sizeof(double), sizeof(double),
                        h->ns, cudaMemcpyDeviceToHost));
        return LFDM_OK;
    }
    std::memcpy(state, &h->states[(size_t)i * h->ns], h->ns * sizeof(double));
    return LFDM_OK;
}

#define SETTER(name, field, cond, msg)                                   \
    int name(lfdm_solver* h, double v) {                                 \
        if (!h) return LFDM_ERR_ARG;                                     \
        if (!(cond)) return h->fail(LFDM_ERR_ARG, msg " (got %g)", v);   \
        h->field = v;                                                    \
        return LFDM_OK;                                                  \
    }
SETTER(lfdm_set_time_step, step, v > 0 && std::isfinite(v), "time step must be positive")
SETTER(lfdm_set_end_time, tend, v > 0 && std::isfinite(v), "end time must be positive")
SETTER(lfdm_set_kernel_sim_time, ksim, v > 0 && std::isfinite(v), "kernel sim time must be positive")
SETTER(lfdm_set_host_dump_time, host_dump, v > 0 && std::isfinite(v), "host dump time must be positive")
#undef SETTER

int lfdm_set_threads_per_block(lfdm_solver* h, unsigned threads) {
    if (!h) return LFDM_ERR_ARG;
    if (threads == 0 || threads > 1024) return h->fail(LFDM_ERR_ARG, "threads per block must be in [1, 1024]");
    h->tpb_hint = threads;
    // the stepping kernel runs 32..128 threads per block (multiples of a warp)
    int t = (int)((threads + 31) / 32 * 32);
    h->threads = t > 128 ? 128 : t;
    return LFDM_OK;
}

int lfdm_get_step(lfdm_solver* h, double* v) {
    if (!h || !v) return LFDM_ERR_ARG;
    *v = h->step;
    return LFDM_OK;
}
int lfdm_get_end_time(lfdm_solver* h, double* v) {
    if (!h || !v) return LFDM_ERR_ARG;
    *v = h->tend;
    return LFDM_OK;
}
int lfdm_get_tire_type(lfdm_solver* h, int* v) {
    if (!h || !v) return LFDM_ERR_ARG;
    *v = h->tire_type < 0 ? LFDM_TIRE_TMEASY : h->tire_type;
    return LFDM_OK;
}
int lfdm_get_num_vehicles(lfdm_solver* h, unsigned* total, unsigned* constructed, unsigned* initialized) {
    if (!h) return LFDM_ERR_ARG;
    if (total) *total = h->N;
    if (constructed) *constructed = h->constructed;
    if (initialized) *initialized = h->initialized;
    return LFDM_OK;
}
int lfdm_set_precision(lfdm_solver* h, int precision) {
    if (!h) return LFDM_ERR_ARG;
    if (precision != LFDM_PREC_FP64 && precision != LFDM_PREC_MIXED && precision != LFDM_PREC_MIXED_TIRE)
        return h->fail(LFDM_ERR_ARG, "unknown precision %d", precision);
    if (precision == LFDM_PREC_MIXED && h->model != LFDM_MODEL_18)
        return h->fail(LFDM_ERR_ARG, "mixed precision is built for the 18-DOF model only");
    h->precision = precision;
    return LFDM_OK;
}

int lfdm_set_output(lfdm_solver* h, const char* output_file, double output_freq, int store_all, unsigned no_outs) {
    if (!h || !output_file) return h ? h->fail(LFDM_ERR_ARG, "null output file") : LFDM_ERR_ARG;
    if (!(output_freq > 0)) return h->fail(LFDM_ERR_ARG, "output frequency must be positive");
    h->output = true;
    h->store_all = store_all != 0;
    if (!h->store_all) {
        if (no_outs > h->N) {
            std::printf(
                "Number of outputs asked is greater than the total number of vehicles, setting number of outputs to "
                "total number of vehicles\n");
            no_outs = h->N;
        }
        h->num_outs = no_outs;
        // the vehicles dumped are the first no_outs of a shuffle of 0..N-1 (dof18_halfImplicit_gpu.cu:359-369)
        float some_seed = 68;
        std::mt19937 generator(some_seed);
        std::vector<int> numbers(h->N);
        std::iota(numbers.begin(), numbers.end(), 0);
        std::shuffle(numbers.begin(), numbers.end(), generator);
        h->which_outs.assign(numbers.begin(), numbers.begin() + no_outs);
    } else {
        h->num_outs = h->N;
    }
    h->csv = std::vector<std::ostringstream>(h->num_outs);
    h->out_file = output_file;
    h->dtout = 1.0 / output_freq;
    return LFDM_OK;
}

int lfdm_set_response_buffer(lfdm_solver* h, double* dst, size_t capacity, double output_freq) {
    if (!h) return LFDM_ERR_ARG;
    if (!dst) {
        h->resp_host = nullptr;
        h->resp_cap = 0;
        return LFDM_OK;
    }
    if (!(output_freq > 0)) return h->fail(LFDM_ERR_ARG, "output frequency must be positive");
    h->resp_host = dst;
    h->resp_cap = capacity;
    h->resp_dtout = 1.0 / output_freq;
    return LFDM_OK;
}

int lfdm_response_samples(lfdm_solver* h, size_t* n) {
    if (!h || !n) return LFDM_ERR_ARG;
    *n = h->resp_written;
    return LFDM_OK;
}

int lfdm_register_host(void* ptr, size_t bytes) {
    if (!ptr || bytes == 0) return LFDM_ERR_ARG;
    return cudaHostRegister(ptr, bytes, cudaHostRegisterDefault) == cudaSuccess ? LFDM_OK : LFDM_ERR_CUDA;
}
int lfdm_unregister_host(void* ptr) {
    if (!ptr) return LFDM_ERR_ARG;
    return cudaHostUnregister(ptr) == cudaSuccess ? LFDM_OK : LFDM_ERR_CUDA;
}

int lfdm_set_response_device(lfdm_solver* h, double* dst_dev, size_t capacity, double output_freq) {
    if (!h) return LFDM_ERR_ARG;
    if (!dst_dev) {
        h->resp_dev = nullptr;
        h->resp_dev_cap = 0;
        return LFDM_OK;
    }
    if (!(output_freq > 0)) return h->fail(LFDM_ERR_ARG, "output frequency must be positive");
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, dst_dev) != cudaSuccess || at.type != cudaMemoryTypeDevice ||
        at.device != h->device) {
        cudaGetLastError();
        return h->fail(LFDM_ERR_ARG, "response buffer is not device memory of device %d", h->device);
    }
    h->resp_dev = dst_dev;
    h->resp_dev_cap = capacity;
    h->resp_dev_dtout = 1.0 / output_freq;
    return LFDM_OK;
}

int lfdm_solve_range(lfdm_solver* h, double t_begin, double t_end) {
    if (!h) return LFDM_ERR_ARG;
    if (!(h->tend > 0)) return h->fail(LFDM_ERR_STATE, "Final time not set, please use SetEndTime function");
    int rc = check_ready(h, true);
    if (rc) return rc;
    return run_windows(h, t_begin, t_end, true, CTL_TABLE, 0, 0, 0, nullptr, nullptr, 0, false);
}

static int traj_guard(lfdm_solver* h, const double* ctl, const double* ref, unsigned nsteps, unsigned ckpt) {
    if (!ctl || !ref || nsteps == 0 || ckpt == 0) return h->fail(LFDM_ERR_ARG, "null array or zero steps");
    if (h->model != LFDM_MODEL_18) return h->fail(LFDM_ERR_ARG, "the differentiable rollout is the 18-DOF model's");
    if (h->tire_type == LFDM_TIRE_TMEASY_NR) return h->fail(LFDM_ERR_ARG, "the differentiable rollout needs TMeasy");
    if (h->precision != LFDM_PREC_FP64) return h->fail(LFDM_ERR_ARG, "the differentiable rollout is FP64");
    for (const lfdm_class18& c : h->classes)
        if (c.throttleMod) return h->fail(LFDM_ERR_ARG, "throttleMod is not differentiated");
    int rc = check_ready(h, false);
    if (rc) return rc;
    return sync_device(h);
}

static AdjLaunch traj_launch(lfdm_solver* h, const double* ctl, const double* ref, unsigned nsteps, double weight_u,
                             unsigned ckpt) {
    AdjLaunch A;
    A.n = (int)h->N;
    A.npad = h->npad;
    A.nsteps = (int)nsteps;
    A.ckpt = (int)ckpt;
    A.dt = h->step;
    A.weight_u = weight_u;
    A.K = h->d_K.p;
    A.classes = reinterpret_cast<const ClassDev18*>(h->d_classes.p);
    A.nclasses = (int)h->classes.size();
    A.class_of = h->d_class_of.p;
    A.params = h->d_params.p;
    A.S0 = h->d_S.p;
    A.ctl = ctl;
    A.ref = ref;
    A.ckpts = h->d_adj_ckpt.p;
    A.tape = h->d_adj_tape.p;
    return A;
}

int lfdm_traj18_forward(lfdm_solver* h, const double* ctl, const double* ref, unsigned nsteps, double weight_u,
                        unsigned ckpt_every, double* loss) {
    if (!h) return LFDM_ERR_ARG;
    if (!loss) return h->fail(LFDM_ERR_ARG, "null loss array");
    int rc = traj_guard(h, ctl, ref, nsteps, ckpt_every);
    if (rc) return rc;
    const size_t nseg = (nsteps + ckpt_every - 1) / ckpt_every;
    CK(h->d_adj_ckpt.ensure(nseg * (size_t)traj18_ckpt_fields() * h->npad));
    CK(h->d_adj_tape.ensure((size_t)ckpt_every * traj18_tape_doubles_per_step() * h->npad));
    AdjLaunch A = traj_launch(h, ctl, ref, nsteps, weight_u, ckpt_every);
    A.loss = loss;
    CK(cudaEventRecord(h->ev0, h->stream));
    CK(launch_traj18_forward(A, h->stream));
    CK(cudaEventRecord(h->ev1, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
    h->adj_fwd_ms = ms;
    h->adj_nsteps = nsteps;
    h->adj_ckpt = ckpt_every;
    h->adj_valid = true;
    return LFDM_OK;
}

int lfdm_traj18_branch_signature(lfdm_solver* h, const double* ctl, unsigned nsteps, uint64_t* sig) {
    if (!h) return LFDM_ERR_ARG;
    if (!sig) return h->fail(LFDM_ERR_ARG, "null signature array");
    int rc = traj_guard(h, ctl, ctl, nsteps, 1);
    if (rc) return rc;
    CK(h->d_adj_tape.ensure(traj18_tape_doubles_per_step() * h->npad));
    AdjLaunch A = traj_launch(h, ctl, ctl, nsteps, 0.0, 1);
    CK(launch_traj18_signature(A, sig, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return LFDM_OK;
}

int lfdm_traj18_backward(lfdm_solver* h, const double* ctl, const double* ref, unsigned nsteps, double weight_u,
                         unsigned ckpt_every, double* grad_ctl, double* grad_params, double* grad_state0) {
    if (!h) return LFDM_ERR_ARG;
    if (!grad_ctl || !grad_params) return h->fail(LFDM_ERR_ARG, "null gradient array");
    int rc = traj_guard(h, ctl, ref, nsteps, ckpt_every);
    if (rc) return rc;
    if (!h->adj_valid || h->adj_nsteps != nsteps || h->adj_ckpt != ckpt_every)
        return h->fail(LFDM_ERR_STATE, "call lfdm_traj18_forward with the same steps and checkpoint interval first");
    CK(h->d_adj_tape.ensure((size_t)ckpt_every * traj18_tape_doubles_per_step() * h->npad));
    AdjLaunch A = traj_launch(h, ctl, ref, nsteps, weight_u, ckpt_every);
    A.grad_ctl = grad_ctl;
    A.grad_params = grad_params;
    A.grad_state0 = grad_state0;
    CK(cudaEventRecord(h->ev0, h->stream));
    CK(launch_traj18_backward(A, h->stream));
    CK(cudaEventRecord(h->ev1, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
    h->adj_bwd_ms = ms;
    return LFDM_OK;
}

// The solver configurations a right-hand-side Jacobian can be formed for (exact: every model without
// throttleMod, the 24-DOF model with TMeasy tires; either: FP64, all vehicles with or without a
// torque converter).
static int jacobian_supported(lfdm_solver* h, bool exact) {
    if (exact && h->model == LFDM_MODEL_24 && h->tire_type == LFDM_TIRE_TMEASY_NR)
        return h->fail(LFDM_ERR_ARG, "the exact 24-DOF right-hand-side Jacobian is built for TMeasy tires");
    if (h->precision != LFDM_PREC_FP64) return h->fail(LFDM_ERR_ARG, "the right-hand-side Jacobian is FP64");
    if (h->classes.empty()) return h->fail(LFDM_ERR_STATE, "no vehicles constructed");
    const int tc = h->classes[0].tcbool != 0;
    for (const lfdm_class18& c : h->classes) {
        if (exact && c.throttleMod) return h->fail(LFDM_ERR_ARG, "throttleMod is not differentiated");
        if ((c.tcbool != 0) != (tc != 0))
            return h->fail(LFDM_ERR_ARG, "all vehicles must agree on the torque converter (it sets the state count)");
    }
    return LFDM_OK;
}

int lfdm_rhs_jacobian18(lfdm_solver* h, const double* ctl, int reference_point, double* jac_state, double* jac_ctl,
                        int* ny) {
    if (!h) return LFDM_ERR_ARG;
    if (h->model != LFDM_MODEL_18) return h->fail(LFDM_ERR_ARG, "lfdm_rhs_jacobian18 needs an 18-DOF solver");
    return lfdm_rhs_jacobian_exact(h, ctl, reference_point, jac_state, jac_ctl, ny);
}

int lfdm_rhs_jacobian_exact(lfdm_solver* h, const double* ctl, int reference_point, double* jac_state,
                            double* jac_ctl, int* ny) {
    if (!h) return LFDM_ERR_ARG;
    if (!ctl || !jac_state || !jac_ctl) return h->fail(LFDM_ERR_ARG, "null array");
    int rc = jacobian_supported(h, true);
    if (rc) return rc;
    const int tc = h->classes[0].tcbool != 0;
    rc = check_ready(h, false);
    if (rc) return rc;
    rc = sync_device(h);
    if (rc) return rc;
    CK(h->d_adj_tape.ensure(std::max(traj18_tape_doubles_per_step(), jac24_tape_doubles()) * h->npad));
    JacLaunch A;
    A.n = (int)h->N;
    A.npad = h->npad;
    A.K = h->d_K.p;
    A.classes = reinterpret_cast<const ClassDev18*>(h->d_classes.p);
    A.nclasses = (int)h->classes.size();
    A.class_of = h->d_class_of.p;
    A.S = h->d_S.p;
    A.ctl = ctl;
    A.reference_point = reference_point ? 1 : 0;
    A.tire_nr = h->tire_type == LFDM_TIRE_TMEASY_NR ? 1 : 0;
    A.tape = h->d_adj_tape.p;
    A.jac_state = jac_state;
    A.jac_ctl = jac_ctl;
    CK(h->model == LFDM_MODEL_11   ? launch_rhs_jacobian11(A, h->stream)
       : h->model == LFDM_MODEL_24 ? launch_rhs_jacobian24(A, h->stream)
                                   : launch_rhs_jacobian18(A, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (ny) *ny = jac_fd_ny((int)h->model, A.tire_nr != 0, tc != 0);
    return LFDM_OK;
}

int lfdm_rhs_jacobian_fd(lfdm_solver* h, const double* ctl, int reference_point, double* jac_state, double* jac_ctl,
                         int* ny) {
    if (!h) return LFDM_ERR_ARG;
    if (!ctl || !jac_state || !jac_ctl) return h->fail(LFDM_ERR_ARG, "null array");
    int rc = jacobian_supported(h, false);
    if (rc) return rc;
    const int tc = h->classes[0].tcbool != 0;
    rc = check_ready(h, false);
    if (rc) return rc;
    rc = sync_device(h);
    if (rc) return rc;
    JacFdLaunch A;
    A.model = (int)h->model;
    A.tire_nr = h->tire_type == LFDM_TIRE_TMEASY_NR ? 1 : 0;
    A.n = (int)h->N;
    A.npad = h->npad;
    A.K = h->d_K.p;
    A.classes = reinterpret_cast<const ClassDev18*>(h->d_classes.p);
    A.nclasses = (int)h->classes.size();
    A.class_of = h->d_class_of.p;
    A.S = h->d_S.p;
    A.ctl = ctl;
    A.reference_point = reference_point ? 1 : 0;
    A.jac_state = jac_state;
    A.jac_ctl = jac_ctl;
    CK(launch_rhs_jacobian_fd(A, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (ny) *ny = jac_fd_ny(A.model, A.tire_nr != 0, tc != 0);
    return LFDM_OK;
}

int lfdm_rhs_jacobian_host(lfdm_solver* h, int exact, const double* ctl, int reference_point, double* jac_state,
                           double* jac_ctl, int* ny) {
    if (!h) return LFDM_ERR_ARG;
    // every check the Jacobian call makes on the configuration runs before the size query and
    // before any buffer is grown
    const int sup = jacobian_supported(h, exact != 0);
    if (sup) return sup;
    const bool nr = h->tire_type == LFDM_TIRE_TMEASY_NR;
    const int m = jac_fd_ny((int)h->model, nr, h->classes[0].tcbool != 0);
    if (ny) *ny = m;
    if (!jac_state && !jac_ctl) return LFDM_OK;  // size query
    if (!ctl || !jac_state || !jac_ctl) return h->fail(LFDM_ERR_ARG, "null array");
    const size_t n = h->N, mm = (size_t)m * m;
    CK(h->d_jac_in.ensure(3 * n));
    CK(h->d_jac_s.ensure(mm * n));
    CK(h->d_jac_u.ensure((size_t)m * 2 * n));
    CK(cudaMemcpyAsync(h->d_jac_in.p, ctl, 3 * n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    int got = 0;
    const int rc = exact ? lfdm_rhs_jacobian_exact(h, h->d_jac_in.p, reference_point, h->d_jac_s.p, h->d_jac_u.p, &got)
                         : lfdm_rhs_jacobian_fd(h, h->d_jac_in.p, reference_point, h->d_jac_s.p, h->d_jac_u.p, &got);
    if (rc) return rc;
    if (got != m) return h->fail(LFDM_ERR_STATE, "unexpected Jacobian size");
    // device [r][c][vehicle] -> host [vehicle][r][c]
    std::vector<double> s_host, u_host;
    try {
        s_host.resize(mm * n);
        u_host.resize((size_t)m * 2 * n);
    } catch (const std::bad_alloc&) {
        return h->fail(LFDM_ERR_CAPACITY, "no host memory to stage the Jacobians");
    }
    CK(cudaMemcpyAsync(s_host.data(), h->d_jac_s.p, s_host.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(u_host.data(), h->d_jac_u.p, u_host.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (size_t rc2 = 0; rc2 < mm; ++rc2)
        for (size_t i = 0; i < n; ++i) jac_state[i * mm + rc2] = s_host[rc2 * n + i];
    for (size_t rc2 = 0; rc2 < (size_t)m * 2; ++rc2)
        for (size_t i = 0; i < n; ++i) jac_ctl[i * m * 2 + rc2] = u_host[rc2 * n + i];
    return LFDM_OK;
}

int lfdm_traj18_last_ms(lfdm_solver* h, double* forward_ms, double* backward_ms) {
    if (!h) return LFDM_ERR_ARG;
    if (forward_ms) *forward_ms = h->adj_fwd_ms;
    if (backward_ms) *backward_ms = h->adj_bwd_ms;
    return LFDM_OK;
}

int lfdm_solve(lfdm_solver* h) {
    if (!h) return LFDM_ERR_ARG;
    if (!(h->tend > 0)) return h->fail(LFDM_ERR_STATE, "Final time not set, please use SetEndTime function");
    int rc = check_ready(h, true);
    if (rc) return rc;
    return run_windows(h, 0.0, h->tend, true, CTL_TABLE, 0, 0, 0, nullptr, nullptr, 0, true);
}

static int step_guard(lfdm_solver* h) {
    if (h->output)
        return h->fail(LFDM_ERR_STATE,
                       "Cannot get csv file output if SolveStep is called, please access sim_states through "
                       "GetSimSate");
    return check_ready(h, false);
}

int lfdm_solve_step(lfdm_solver* h, double t, double steering, double throttle, double braking, double* t_out) {
    if (!h) return LFDM_ERR_ARG;
    int rc = step_guard(h);
    if (rc) return rc;
    rc = run_windows(h, t, t, false, CTL_SCALAR, steering, throttle, braking, nullptr, nullptr, 0, false);
    if (rc) return rc;
    if (t_out) *t_out = t + h->ksim;
    return LFDM_OK;
}

int lfdm_solve_step_controls(lfdm_solver* h, double t, const double* steering, const double* throttle,
                             const double* braking, double* t_out) {
    if (!h || !steering || !throttle || !braking) return h ? h->fail(LFDM_ERR_ARG, "null control array") : LFDM_ERR_ARG;
    int rc = step_guard(h);
    if (rc) return rc;
    rc = set_device(h);
    if (rc) return rc;
    const size_t np = (size_t)h->npad;
    CK(h->d_ctl.ensure(3 * np));
    CK(cudaMemcpyAsync(h->d_ctl.p, steering, h->N * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->d_ctl.p + np, throttle, h->N * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->d_ctl.p + 2 * np, braking, h->N * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    rc = run_windows(h, t, t, false, CTL_ARRAY, 0, 0, 0, h->d_ctl.p, nullptr, 0, false);
    if (rc) return rc;
    if (t_out) *t_out = t + h->ksim;
    return LFDM_OK;
}

int lfdm_window_steps(lfdm_solver* h, double t, unsigned* nsteps, double* times, unsigned capacity) {
    if (!h || !nsteps) return LFDM_ERR_ARG;
    std::vector<int32_t> samp;
    std::vector<double> ts;
    int n = 0;
    window_schedule(t, h->ksim, h->step, 0.0, 0, n, samp, &ts);
    *nsteps = (unsigned)n;
    if (times) {
        if (capacity < (unsigned)n) return h->fail(LFDM_ERR_CAPACITY, "times buffer holds %u < %d steps", capacity, n);
        std::memcpy(times, ts.data(), ts.size() * sizeof(double));
    }
    return LFDM_OK;
}

int lfdm_solve_step_schedule(lfdm_solver* h, double t, const double* ctl, unsigned nsteps, int ctl_on_device,
                             double* t_out) {
    if (!h || !ctl) return h ? h->fail(LFDM_ERR_ARG, "null schedule") : LFDM_ERR_ARG;
    int rc = step_guard(h);
    if (rc) return rc;
    rc = set_device(h);
    if (rc) return rc;
    const double* sched = ctl;
    if (!ctl_on_device) {
        CK(h->d_sched.ensure((size_t)nsteps * 3));
        CK(cudaMemcpyAsync(h->d_sched.p, ctl, (size_t)nsteps * 3 * sizeof(double), cudaMemcpyHostToDevice, h->stream));
        sched = h->d_sched.p;
    }
    rc = run_windows(h, t, t, false, CTL_SCHEDULE, 0, 0, 0, nullptr, sched, nsteps, false);
    if (rc) return rc;
    if (t_out) *t_out = t + h->ksim;
    return LFDM_OK;
}

int lfdm_device_window_begin(lfdm_solver* h, double t, lfdm_device_window* view) {
    if (!h || !view) return h ? h->fail(LFDM_ERR_ARG, "null view") : LFDM_ERR_ARG;
    int rc = step_guard(h);
    if (rc) return rc;
    if (h->precision != LFDM_PREC_FP64) return h->fail(LFDM_ERR_ARG, "a device-functor window steps in FP64");
    rc = sync_device(h);
    if (rc) return rc;
    std::vector<int32_t> samp;
    int nsteps = 0;
    window_schedule(t, h->ksim, h->step, 0.0, 0, nsteps, samp);
    CK(cudaMemsetAsync(h->d_status.p, 0, h->N * sizeof(uint32_t), h->stream));
    CK(cudaStreamSynchronize(h->stream));
    std::memset(view, 0, sizeof(*view));
    view->model = h->model;
    view->tire_type = h->tire_type;
    view->n = (int32_t)h->N;
    view->npad = h->npad;
    view->nclasses = (int32_t)h->classes.size();
    view->nsteps = nsteps;
    view->kcount = h->model == LFDM_MODEL_24 ? k24_count() : k18_count();
    view->t0 = t;
    view->dt = h->step;
    view->K = h->d_K.p;
    view->classes = h->d_classes.p;
    view->class_of = h->d_class_of.p;
    view->S = h->d_S.p;
    view->status = h->d_status.p;
    view->stream = h->stream;
    h->device_newer = true;  // the caller's kernel steps the device states
    return LFDM_OK;
}

int lfdm_device_window_end(lfdm_solver* h, double t, double* t_out) {
    if (!h) return LFDM_ERR_ARG;
    int rc = set_device(h);
    if (rc) return rc;
    CK(cudaStreamSynchronize(h->stream));
    h->device_newer = true;
    h->last_launches = 1;
    std::vector<uint32_t> st_words(h->N);
    CK(cudaMemcpy(st_words.data(), h->d_status.p, h->N * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    if (t_out) *t_out = t + h->ksim;
    for (size_t i = 0; i < h->N; ++i)
        if (st_words[i] & 1u) return h->fail(LFDM_ERR_NUMERIC, "vehicle %zu reached a non-finite state", i);
    return LFDM_OK;
}

int lfdm_set_split_warps(lfdm_solver* h, int mode) {
    if (!h) return LFDM_ERR_ARG;
    if (mode < -1 || mode > 1) return h->fail(LFDM_ERR_ARG, "split-warp mode must be -1, 0 or 1");
    h->split = mode;
    return LFDM_OK;
}

int lfdm_get_status_words(lfdm_solver* h, unsigned first, unsigned count, uint32_t* words) {
    if (!h || !words) return LFDM_ERR_ARG;
    if ((size_t)first + count > h->N) return h->fail(LFDM_ERR_ARG, "index out of range");
    if (!h->d_status.p) {
        std::memset(words, 0, count * sizeof(uint32_t));
        return LFDM_OK;
    }
    int rc = set_device(h);
    if (rc) return rc;
    CK(cudaMemcpy(words, h->d_status.p + first, count * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    return LFDM_OK;
}

int lfdm_last_kernel_ms(lfdm_solver* h, double* ms, unsigned* launches) {
    if (!h) return LFDM_ERR_ARG;
    if (ms) *ms = h->last_ms;
    if (launches) *launches = h->last_launches;
    return LFDM_OK;
}

int lfdm_parse_vehicle18(const char* veh_json, const char* tire_json, int tire_type, lfdm_class18* cls,
                         double* params, char* err, size_t err_len) {
    if (!veh_json || !tire_json || !cls || !params) return LFDM_ERR_ARG;
    std::string e;
    if (!load_vehicle(LFDM_MODEL_18, veh_json, tire_json, "", tire_type, *cls, params, e)) {
        if (err && err_len) std::snprintf(err, err_len, "%s", e.c_str());
        return e.rfind("cannot open", 0) == 0 ? LFDM_ERR_IO : LFDM_ERR_PARSE;
    }
    return LFDM_OK;
}

int lfdm_parse_vehicle(int model, const char* veh_json, const char* tire_json, const char* sus_json, int tire_type,
                       lfdm_class18* cls, double* params, char* err, size_t err_len) {
    if (!veh_json || !tire_json || !cls || !params) return LFDM_ERR_ARG;
    if (model != LFDM_MODEL_11 && model != LFDM_MODEL_18 && model != LFDM_MODEL_24) return LFDM_ERR_ARG;
    std::string e;
    if (!load_vehicle(model, veh_json, tire_json, sus_json ? sus_json : "", tire_type, *cls, params, e)) {
        if (err && err_len) std::snprintf(err, err_len, "%s", e.c_str());
        return e.rfind("cannot open", 0) == 0 ? LFDM_ERR_IO : LFDM_ERR_PARSE;
    }
    return LFDM_OK;
}

int lfdm_load_driver_file(const char* path, double* rows, unsigned capacity_rows, unsigned* nrows, char* err,
                          size_t err_len) {
    if (!path || !nrows) return LFDM_ERR_ARG;
    std::vector<double> r;
    std::string e;
    if (!load_driver_file(path, r, e)) {
        if (err && err_len) std::snprintf(err, err_len, "%s", e.c_str());
        return e.rfind("cannot open", 0) == 0 ? LFDM_ERR_IO : LFDM_ERR_PARSE;
    }
    *nrows = (unsigned)(r.size() / 4);
    if (rows) {
        if (capacity_rows < *nrows) return LFDM_ERR_CAPACITY;
        std::memcpy(rows, r.data(), r.size() * sizeof(double));
    }
    return LFDM_OK;
}

}  // extern "C"
