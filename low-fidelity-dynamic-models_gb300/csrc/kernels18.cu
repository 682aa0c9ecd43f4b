// CUDA kernels of the 18-DOF stepper: derived constants, state layout transposes and the window
// stepping kernel (the GB300 counterpart of the reference's Integrate kernels,
// 18dof-gpu/dof18_halfImplicit_gpu.cu:882-1250 and .cuh:454-640).
//
// Layout in HBM (n vehicles, npad = row stride):
//   K  [K18_COUNT][npad] FP64 derived per-vehicle constants (prepare18_kernel)
//   S  [LFDM_S_COUNT][npad] FP64 state, one coalesced row per field
//   rows  per-vehicle driver tables, {t, steering, throttle, braking} rows, 32-byte aligned
//   resp  [sample][13][n] FP64 response of one window (the reference's device response layout)
// Each thread integrates one vehicle over a whole window with the carried state in registers;
// per-block copies of the class tables and of the block's derived constants live in shared
// memory.
#include <cuda_runtime.h>

#include <vector>

#include <cmath>
#include <cstring>

#include "../../include/lfdm/device/dof18_device.cuh"
#include "dof18_mixed.cuh"
#include "kernels.h"
#include "window_common.cuh"

namespace lfdm {

static_assert(sizeof(ClassDev18) % 16 == 0, "ClassDev18 must be a multiple of 16 bytes");
static_assert(sizeof(ClassDev18F) % 16 == 0, "ClassDev18F must be a multiple of 16 bytes");

int k18_count() { return K18_COUNT; }
size_t class_dev18_size() { return sizeof(ClassDev18); }

// ---------------------------------------------------------------------------------------------
// derived constants

__global__ void prepare18_kernel(const double* __restrict__ P, int n, int npad, double* __restrict__ K) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* p = P + (size_t)i * LFDM_P_COUNT;
    auto put = [&](int k, double v) { K[(size_t)k * npad + i] = v; };
    prepare_shared_k(p, put);
    const double a = p[LFDM_P_A], b = p[LFDM_P_B], h = p[LFDM_P_H], m = p[LFDM_P_M];
    const double jz = p[LFDM_P_JZ], jx = p[LFDM_P_JX], jxz = p[LFDM_P_JXZ];
    const double cf = p[LFDM_P_CF], cr = p[LFDM_P_CR], muf = p[LFDM_P_MUF], mur = p[LFDM_P_MUR];
    const double hrcf = p[LFDM_P_HRCF], hrcr = p[LFDM_P_HRCR];
    const double krof = p[LFDM_P_KROF], kror = p[LFDM_P_KROR], brof = p[LFDM_P_BROF], bror = p[LFDM_P_BROR];
    const double r0 = p[LFDM_P_R0];
    put(K_A, a);
    put(K_B, b);
    put(K_CF2, cf / 2.);
    put(K_CR2, cr / 2.);
    // computeTireLoads (dof18_gpu.cu:305-340), huf = hur = r0
    const double huf = r0, hur = r0;
    put(K_Z1F, (m * kG * b) / (2. * (a + b)) + (muf * kG) / 2.);
    put(K_Z2F, (muf * huf) / cf + m * b * (h - hrcf) / (cf * (a + b)));
    put(K_Z3FK, krof / cf);
    put(K_Z3FB, brof / cf);
    put(K_Z4, (m * h + muf * huf + mur * hur) / (2. * (a + b)));
    put(K_Z1R, (m * kG * a) / (2. * (a + b)) + (mur * kG) / 2.);
    put(K_Z2R, (mur * hur) / cr + m * a * (h - hrcr) / (cr * (a + b)));
    put(K_Z3RK, kror / cr);
    put(K_Z3RB, bror / cr);
    // computeVehRHS (dof18_gpu.cu:1017-1068): the 3x3 solve as coefficients of E1, E2, E3
    const double mt = m + 2 * (muf + mur);
    const double hrc = (hrcf * b + hrcr * a) / (a + b);
    const double A1 = mur * b - muf * a;
    const double A2 = jx + m * hrc * hrc;
    const double A3 = hrc * m;
    const double denom = A2 * A1 * A1 - 2. * A1 * A3 * jxz + jz * A3 * A3 + mt * jxz * jxz - A2 * jz * mt;
    put(K_MT, mt);
    put(K_INVMT, 1 / mt);
    put(K_E2WU, -muf * a + mur * b);
    put(K_E3PHI, m * kG * hrc - (krof + kror));
    put(K_E3WX, -(brof + bror));
    put(K_E3WU, hrc * m);
    put(K_UWZ2, -mur * b + muf * a);
    put(K_UWZWX, 2. * hrc * m);
    put(K_CV1, (jxz * jxz - A2 * jz) / denom);
    put(K_CV2, (A3 * jxz - A1 * A2) / denom);
    put(K_CV3, (A1 * jxz - A3 * jz) / denom);
    put(K_CX2, (jxz * mt - A1 * A3) / denom);
    put(K_CX3, (A1 * A1 - jz * mt) / denom);
    put(K_CZ2, (A3 * A3 - A2 * mt) / denom);
    put(K_INVJZ, 1. / jz);
}

cudaError_t launch_prepare18(const double* params_dev, int n, int npad, double* K_dev, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    prepare18_kernel<<<(n + 127) / 128, 128, 0, stream>>>(params_dev, n, npad, K_dev);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// state transposes

__global__ void aos_to_soa_kernel(const double* __restrict__ aos, int n, int ns, int npad, double* __restrict__ soa) {
    const size_t total = (size_t)n * ns;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const size_t v = i / ns, f = i % ns;
        soa[f * npad + v] = aos[i];
    }
}
__global__ void soa_to_aos_kernel(const double* __restrict__ soa, int n, int ns, int npad, double* __restrict__ aos) {
    const size_t total = (size_t)n * ns;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const size_t v = i / ns, f = i % ns;
        aos[i] = soa[f * npad + v];
    }
}
static int grid_for(size_t total) {
    size_t g = (total + 255) / 256;
    return (int)(g > 152 * 32 ? 152 * 32 : (g == 0 ? 1 : g));
}
cudaError_t launch_states_to_soa(const double* aos, int n, int ns, int npad, double* soa, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    aos_to_soa_kernel<<<grid_for((size_t)n * ns), 256, 0, stream>>>(aos, n, ns, npad, soa);
    return cudaGetLastError();
}
cudaError_t launch_states_to_aos(const double* soa, int n, int ns, int npad, double* aos, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    soa_to_aos_kernel<<<grid_for((size_t)n * ns), 256, 0, stream>>>(soa, n, ns, npad, aos);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// driver-table validation and the FP64 peak probe

__global__ void check_tables_kernel(const double* __restrict__ rows, long long ntables, int nrows, unsigned* bad) {
    const long long total = ntables * (long long)nrows;
    unsigned local = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        if (i % nrows == 0) continue;
        if (rows[4 * i] < rows[4 * (i - 1)]) ++local;
    }
    if (local) atomicAdd(bad, local);
}

cudaError_t launch_check_tables(const double* rows, long long ntables, int nrows, unsigned* bad_dev,
                                cudaStream_t stream) {
    if (ntables <= 0 || nrows <= 1) return cudaSuccess;
    check_tables_kernel<<<152 * 8, 256, 0, stream>>>(rows, ntables, nrows, bad_dev);
    return cudaGetLastError();
}

// FMA pipe probes. FP64: every thread runs 8 independent DFMA chains (enough to keep a
// sub-partition's FP64 unit busy: on GB300 it accepts one warp-wide DFMA every 64 cycles whatever
// the number of active lanes, so the rate is set by warp instructions, not by latency), 8 warps per
// sub-partition. FP32: the same kernel on FFMA chains, 64 times as many iterations (the FP32 pipes
// retire 64 times as many lane operations per clock). Thread 0 of every block reads the SM clock
// counter and the global nanosecond timer at its start and end, which gives the SM clock the probe
// ran at.
constexpr int kProbeIter = 4096;
template <typename T>
__global__ void __launch_bounds__(1024) fma_probe_kernel(T* out, long long* clk, T seed, int iters) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    long long c0 = 0, t0 = 0;
    if (threadIdx.x == 0) {
        c0 = clock64();
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    }
    T a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = seed + (T)(tid * 1e-9) + (T)(k * 0.1);
    const T m = (T)0.999999, c = (T)1e-7;
#pragma unroll 4
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = fma(a[k], m, c);
    }
    T s = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += a[k];
    out[tid] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long t1 = 0;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
        clk[2 * blockIdx.x] = clock64() - c0;
        clk[2 * blockIdx.x + 1] = t1 - t0;
    }
}

// Best of 5 timed launches (after one warm-up) of the probe on every SM: lane FMA per second and the
// SM clock (GHz) of the fastest launch.
template <typename T>
static cudaError_t measure_fma_rate(double* rate, double* sm_ghz, int iters) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const int threads = 1024, blocks = sms;  // 32 warps per SM, 8 per sub-partition
    T* out = nullptr;
    long long* clk = nullptr;
    if ((e = cudaMalloc(&out, sizeof(T) * threads * blocks)) != cudaSuccess) return e;
    if ((e = cudaMalloc(&clk, sizeof(long long) * 2 * blocks)) != cudaSuccess) {
        cudaFree(out);
        return e;
    }
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    fma_probe_kernel<T><<<blocks, threads>>>(out, clk, (T)0.5, iters);
    float best = 1e30f;
    double ghz = 0;
    std::vector<long long> h(2 * (size_t)blocks);
    for (int r = 0; r < 5; ++r) {
        cudaEventRecord(a);
        fma_probe_kernel<T><<<blocks, threads>>>(out, clk, (T)0.5, iters);
        cudaEventRecord(b);
        cudaEventSynchronize(b);
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        if (ms < best) {
            best = ms;
            if (cudaMemcpy(h.data(), clk, h.size() * sizeof(long long), cudaMemcpyDeviceToHost) == cudaSuccess) {
                double cyc = 0, ns = 0;
                for (int k = 0; k < blocks; ++k) {
                    cyc += (double)h[2 * k];
                    ns += (double)h[2 * k + 1];
                }
                ghz = ns > 0 ? cyc / ns : 0;
            }
        }
    }
    e = cudaGetLastError();
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    cudaFree(clk);
    *rate = (double)threads * blocks * iters * 8 / (best * 1e-3);
    if (sm_ghz) *sm_ghz = ghz;
    return e;
}

cudaError_t measure_dfma_rate(double* rate, double* sm_ghz) { return measure_fma_rate<double>(rate, sm_ghz, kProbeIter); }
cudaError_t measure_ffma_rate(double* rate, double* sm_ghz) {
    return measure_fma_rate<float>(rate, sm_ghz, 64 * kProbeIter);
}

// ---------------------------------------------------------------------------------------------
// class tables

// okey (dof18_device.cuh) on the host: an int64 ordered as the double values, both zeros at 0
static long long order_key(double x) {
    long long b;
    std::memcpy(&b, &x, sizeof b);
    return b >= 0 ? b : -(b & 0x7FFFFFFFFFFFFFFFLL);
}

static void build_map(const double (*pts)[2], int n, MapDev& m) {
    std::memset(&m, 0, sizeof(m));
    m.n = n;
    for (int k = 0; k < n; ++k) {
        m.x[k] = pts[k][0];
        m.y[k] = pts[k][1];
    }
    for (int k = 0; k + 1 < n; ++k) {
        m.dx[k] = m.x[k + 1] - m.x[k];
        m.dy[k] = m.y[k + 1] - m.y[k];
        m.idx[k] = 1.0 / m.dx[k];
    }
    for (int k = 0; k < n; ++k) m.kx[k] = order_key(m.x[k]);
}

void build_class_dev18(const lfdm_class18& c, ClassDev18* out) {
    std::memset(out, 0, sizeof(*out));
    out->nonLinearSteer = c.nonLinearSteer;
    out->tcbool = c.tcbool;
    out->throttleMod = c.throttleMod;
    out->driveType = c.driveType;
    out->whichWheels = c.whichWheels;
    out->noGears = c.noGears;
    for (int g = 0; g < c.noGears && g < LFDM_MAX_GEARS; ++g) {
        out->gear[g] = c.gearRatios[g];
        out->invgear[g] = 1.0 / c.gearRatios[g];
        out->down[g] = c.shiftMap[g][0];
        out->up[g] = c.shiftMap[g][1];
    }
    build_map(c.steerMap, c.steerMapSize, out->steer);
    build_map(c.powertrainMap, c.powertrainMapSize, out->pt);
    build_map(c.lossesMap, c.lossesMapSize, out->loss);
    build_map(c.CFmap, c.CFmapSize, out->cf);
    build_map(c.TRmap, c.TRmapSize, out->tr);
}

// ---------------------------------------------------------------------------------------------
// window kernel


size_t window18_smem(int threads, int nclasses, bool f32) {
    const size_t cls = nclasses <= kMaxSmemClasses ? (size_t)nclasses * sizeof(ClassDev18) : 0;
    return cls + (size_t)K18_COUNT * threads * (sizeof(double) + (f32 ? sizeof(float) : 0));
}

// kF32: the TMeasy tire core in FP32 (precision LFDM_PREC_MIXED_TIRE), on FP32 copies of the
// derived constants staged beside the FP64 ones.
// Resident 128-thread blocks per SM the compiler budgets registers for. 1 (up to 255 registers, 8
// warps per SM) for the FP64 kernels, which are FP64-pipe bound and fastest with every register, and
// for the FP32-tire-core kernels (measured: 2 and 3 blocks were 3 % and 8 % slower). 4 (128
// registers, 16 warps per SM) for the FP32 right-hand-side kernel, whose mostly short-latency FP32
// chains need more warps in flight: 4.50e9 against 3.58e9 vehicle-steps/s at 1 block, 3.97e9 at 5
// and 3.88e9 at 6 (300,000 vehicles; bit-identical results).
#ifndef LFDM_TF_MIN_BLOCKS
#define LFDM_TF_MIN_BLOCKS 1
#endif
#ifndef LFDM_MIXED_MIN_BLOCKS
#define LFDM_MIXED_MIN_BLOCKS 4
#endif

template <bool kNr, int kCtl, bool kOut, bool kF32>
__global__ void __launch_bounds__(128, kF32 ? LFDM_TF_MIN_BLOCKS : 1) window18_kernel(const Window18 w) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int tid = threadIdx.x;
    const bool cls_smem = w.nclasses <= kMaxSmemClasses;
    ClassDev18* cls = reinterpret_cast<ClassDev18*>(smem);
    double* ks = reinterpret_cast<double*>(smem + (cls_smem ? (size_t)w.nclasses * sizeof(ClassDev18) : 0));
    float* fks = reinterpret_cast<float*>(ks + (size_t)K18_COUNT * blockDim.x);
    if (cls_smem) {
        const int4* src = reinterpret_cast<const int4*>(w.classes);
        int4* dst = reinterpret_cast<int4*>(smem);
        const int words = (int)(w.nclasses * sizeof(ClassDev18) / 16);
        for (int i = tid; i < words; i += blockDim.x) dst[i] = __ldg(src + i);
    }
    const int vid = blockIdx.x * blockDim.x + tid;
    const bool active = vid < w.n;
    if (active) {
#pragma unroll 4
        for (int k = 0; k < K18_COUNT; ++k) {
            const double x = __ldg(w.K + (size_t)k * w.npad + vid);
            ks[k * blockDim.x + tid] = x;
            if (kF32) fks[k * blockDim.x + tid] = (float)x;
        }
    }
    __syncthreads();
    if (!active) return;

    const KView K{ks + tid, (int)blockDim.x, kF32 ? fks + tid : nullptr};
    const int ci = __ldg(w.class_of + vid);
    const ClassDev18& C = cls_smem ? cls[ci] : w.classes[ci];
    const size_t np = (size_t)w.npad;
    double* S = w.S + vid;

    VehC v;
    VehAux va;
    TireC ts[4];
    TireAux ta[4];
    load_state18(S, np, v, va, ts, ta);

    DriverCursor cur;
    double steer = w.steer, thr = w.thr, brk = w.brk;
    if (kCtl == CTL_TABLE) {
        driver_begin(cur, w.rows + 4 * __ldg(w.row_off + vid), __ldg(w.row_len + vid), w.t0);
    } else if (kCtl == CTL_ARRAY) {
        steer = __ldg(w.ctl + vid);
        thr = __ldg(w.ctl + np + vid);
        brk = __ldg(w.ctl + 2 * np + vid);
    }
    int next_k = 0;
    int next_step = (kOut && w.nsamples > 0) ? __ldg(w.sample_steps) : -1;

    double t = w.t0;
    const double dt = w.dt;
    for (int s = 0; s < w.nsteps; ++s) {
        if (kCtl == CTL_TABLE) {
            driver_at(cur, t, steer, thr, brk);
        } else if (kCtl == CTL_SCHEDULE) {
            steer = __ldg(w.sched + 3 * s);
            thr = __ldg(w.sched + 3 * s + 1);
            brk = __ldg(w.sched + 3 * s + 2);
        }
        step18<kNr, kF32>(v, va, ts, ta, K, C, steer, thr, brk, dt);
        t += dt;
        if (kOut && s + 1 == next_step) {
            double* r = w.resp + (size_t)next_k * LFDM18_RESP_CHANNELS * w.n + vid;
            const size_t n = (size_t)w.n;
            r[0 * n] = t;
            r[1 * n] = v.x;
            r[2 * n] = v.y;
            r[3 * n] = v.u;
            r[4 * n] = v.v;
            r[5 * n] = v.phi;
            r[6 * n] = v.psi;
            r[7 * n] = v.wx;
            r[8 * n] = v.wz;
            r[9 * n] = ts[0].omega;
            r[10 * n] = ts[1].omega;
            r[11 * n] = ts[2].omega;
            r[12 * n] = ts[3].omega;
            ++next_k;
            next_step = next_k < w.nsamples ? __ldg(w.sample_steps + next_k) : -1;
        }
    }

    store_state18(S, np, v, va, ts, ta);
    if (w.status && !state18_finite(v, ts)) w.status[vid] |= 1u;
}

// ---------------------------------------------------------------------------------------------
// mixed-precision window kernel (TMeasy)

size_t window18_mixed_smem(int threads, int nclasses) {
    const size_t cls = nclasses <= kMaxSmemClasses ? (size_t)nclasses * sizeof(ClassDev18F) : 0;
    return cls + (size_t)K18_COUNT * threads * sizeof(float);
}

// Driver input with the current table segment cached in FP32 (reloaded when the cursor moves):
// the step costs one FP64 subtraction and one conversion.
struct DriverCursorF {
    DriverCursor c;
    int seg;       // cursor value the cache was built for (-1: none)
    double tL;
    float inv, sL, dS, hL, dH, bL, dB;
};

__device__ __forceinline__ void driver_at_f(DriverCursorF& d, double t, float& st, float& th, float& br) {
    DriverCursor& c = d.c;
    const long long kt = okey(t);
    if (kt <= c.kfirst) {
        st = (float)__ldg(c.rows + 1);
        th = (float)__ldg(c.rows + 2);
        br = (float)__ldg(c.rows + 3);
        return;
    }
    if (kt >= c.klast) {
        const double* L = c.rows + 4 * (c.len - 1);
        st = (float)__ldg(L + 1);
        th = (float)__ldg(L + 2);
        br = (float)__ldg(L + 3);
        return;
    }
    while (okey(__ldg(c.rows + 4 * c.r)) < kt) ++c.r;
    while (c.r > 1 && okey(__ldg(c.rows + 4 * (c.r - 1))) >= kt) --c.r;
    if (d.seg != c.r) {
        const double2* L = reinterpret_cast<const double2*>(c.rows + 4 * (c.r - 1));
        const double2 L01 = __ldg(L), L23 = __ldg(L + 1), R01 = __ldg(L + 2), R23 = __ldg(L + 3);
        d.tL = L01.x;
        d.inv = (float)(1.0 / (R01.x - L01.x));
        d.sL = (float)L01.y;
        d.dS = (float)(R01.y - L01.y);
        d.hL = (float)L23.x;
        d.dH = (float)(R23.x - L23.x);
        d.bL = (float)L23.y;
        d.dB = (float)(R23.y - L23.y);
        d.seg = c.r;
    }
    const float tbar = (float)(t - d.tL) * d.inv;
    st = fmaf(tbar, d.dS, d.sL);
    th = fmaf(tbar, d.dH, d.hL);
    br = fmaf(tbar, d.dB, d.bL);
}

template <int kCtl, bool kOut>
__global__ void __launch_bounds__(128, LFDM_MIXED_MIN_BLOCKS) window18_mixed_kernel(const Window18 w) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int tid = threadIdx.x;
    const bool cls_smem = w.nclasses <= kMaxSmemClasses;
    const ClassDev18F* gcls = reinterpret_cast<const ClassDev18F*>(w.classes_f);
    float* ks = reinterpret_cast<float*>(smem + (cls_smem ? (size_t)w.nclasses * sizeof(ClassDev18F) : 0));
    if (cls_smem) {
        const int4* src = reinterpret_cast<const int4*>(gcls);
        int4* dst = reinterpret_cast<int4*>(smem);
        const int words = (int)(w.nclasses * sizeof(ClassDev18F) / 16);
        for (int i = tid; i < words; i += blockDim.x) dst[i] = __ldg(src + i);
    }
    const int vid = blockIdx.x * blockDim.x + tid;
    const bool active = vid < w.n;
    if (active) {
#pragma unroll 4
        for (int k = 0; k < K18_COUNT; ++k) ks[k * blockDim.x + tid] = (float)__ldg(w.K + (size_t)k * w.npad + vid);
    }
    __syncthreads();
    if (!active) return;
    const KViewF K{ks + tid, (int)blockDim.x};
    const int ci = __ldg(w.class_of + vid);
    const ClassDev18F& C = cls_smem ? reinterpret_cast<const ClassDev18F*>(smem)[ci] : gcls[ci];
    const size_t np = (size_t)w.npad;
    double* S = w.S + vid;

    VehM v;
    VehAux va;
    TireM ts[4];
    TireAuxF ta[4];
    v.x = S[LFDM_S_X * np];
    v.y = S[LFDM_S_Y * np];
    v.u = S[LFDM_S_U * np];
    v.v = S[LFDM_S_V * np];
    v.psi = S[LFDM_S_PSI * np];
    v.wz = S[LFDM_S_WZ * np];
    v.phi = S[LFDM_S_PHI * np];
    v.wx = S[LFDM_S_WX * np];
    v.udot = (float)S[LFDM_S_UDOT * np];
    v.vdot = (float)S[LFDM_S_VDOT * np];
    v.crank = S[LFDM_S_CRANKOMEGA * np];
    v.gear = (int)S[LFDM_S_CURRENT_GR * np];
    va.wxdot = S[LFDM_S_WXDOT * np];
    va.wzdot = S[LFDM_S_WZDOT * np];
    va.dOmega_crank = S[LFDM_S_DOMEGA_CRANK * np];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const size_t b = (size_t)(LFDM_S_TIRE0 + k * LFDM_S_TIRE_STRIDE) * np;
        ts[k].xe = (float)S[b + LFDM_T_XE * np];
        ts[k].ye = (float)S[b + LFDM_T_YE * np];
        ts[k].xedot = (float)S[b + LFDM_T_XEDOT * np];
        ts[k].yedot = (float)S[b + LFDM_T_YEDOT * np];
        ts[k].omega = S[b + LFDM_T_OMEGA * np];
        ta[k].dOmega = (float)S[b + LFDM_T_DOMEGA * np];
        ta[k].xt = (float)S[b + LFDM_T_XT * np];
        ta[k].rStat = (float)S[b + LFDM_T_RSTAT * np];
        ta[k].fx = (float)S[b + LFDM_T_FX * np];
        ta[k].fy = (float)S[b + LFDM_T_FY * np];
        ta[k].fz = (float)S[b + LFDM_T_FZ * np];
        ta[k].vsx = (float)S[b + LFDM_T_VSX * np];
        ta[k].vsy = (float)S[b + LFDM_T_VSY * np];
        ta[k].My = (float)S[b + LFDM_T_MY * np];
        ta[k].engTor = (float)S[b + LFDM_T_ENGTOR * np];
    }
    DriverCursorF cur;
    float steer = (float)w.steer, thr = (float)w.thr, brk = (float)w.brk;
    if (kCtl == CTL_TABLE) {
        driver_begin(cur.c, w.rows + 4 * __ldg(w.row_off + vid), __ldg(w.row_len + vid), w.t0);
        cur.seg = -1;
    } else if (kCtl == CTL_ARRAY) {
        steer = (float)__ldg(w.ctl + vid);
        thr = (float)__ldg(w.ctl + np + vid);
        brk = (float)__ldg(w.ctl + 2 * np + vid);
    }
    int next_k = 0;
    int next_step = (kOut && w.nsamples > 0) ? __ldg(w.sample_steps) : -1;
    double t = w.t0;
    const double dt = w.dt;
    for (int s = 0; s < w.nsteps; ++s) {
        if (kCtl == CTL_TABLE) {
            driver_at_f(cur, t, steer, thr, brk);
        } else if (kCtl == CTL_SCHEDULE) {
            steer = (float)__ldg(w.sched + 3 * s);
            thr = (float)__ldg(w.sched + 3 * s + 1);
            brk = (float)__ldg(w.sched + 3 * s + 2);
        }
        step18_mixed(v, va, ts, ta, K, C, steer, thr, brk, dt);
        t += dt;
        if (kOut && s + 1 == next_step) {
            double* r = w.resp + (size_t)next_k * LFDM18_RESP_CHANNELS * w.n + vid;
            const size_t n = (size_t)w.n;
            r[0 * n] = t;
            r[1 * n] = v.x;
            r[2 * n] = v.y;
            r[3 * n] = v.u;
            r[4 * n] = v.v;
            r[5 * n] = v.phi;
            r[6 * n] = v.psi;
            r[7 * n] = v.wx;
            r[8 * n] = v.wz;
            r[9 * n] = ts[0].omega;
            r[10 * n] = ts[1].omega;
            r[11 * n] = ts[2].omega;
            r[12 * n] = ts[3].omega;
            ++next_k;
            next_step = next_k < w.nsamples ? __ldg(w.sample_steps + next_k) : -1;
        }
    }
    S[LFDM_S_X * np] = v.x;
    S[LFDM_S_Y * np] = v.y;
    S[LFDM_S_U * np] = v.u;
    S[LFDM_S_V * np] = v.v;
    S[LFDM_S_PSI * np] = v.psi;
    S[LFDM_S_WZ * np] = v.wz;
    S[LFDM_S_PHI * np] = v.phi;
    S[LFDM_S_WX * np] = v.wx;
    S[LFDM_S_UDOT * np] = v.udot;
    S[LFDM_S_VDOT * np] = v.vdot;
    S[LFDM_S_WXDOT * np] = va.wxdot;
    S[LFDM_S_WZDOT * np] = va.wzdot;
    S[LFDM_S_CRANKOMEGA * np] = v.crank;
    S[LFDM_S_DOMEGA_CRANK * np] = va.dOmega_crank;
    S[LFDM_S_CURRENT_GR * np] = (double)v.gear;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const size_t b = (size_t)(LFDM_S_TIRE0 + k * LFDM_S_TIRE_STRIDE) * np;
        S[b + LFDM_T_XE * np] = ts[k].xe;
        S[b + LFDM_T_YE * np] = ts[k].ye;
        S[b + LFDM_T_XEDOT * np] = ts[k].xedot;
        S[b + LFDM_T_YEDOT * np] = ts[k].yedot;
        S[b + LFDM_T_OMEGA * np] = ts[k].omega;
        S[b + LFDM_T_DOMEGA * np] = ta[k].dOmega;
        S[b + LFDM_T_XT * np] = ta[k].xt;
        S[b + LFDM_T_RSTAT * np] = ta[k].rStat;
        S[b + LFDM_T_FX * np] = ta[k].fx;
        S[b + LFDM_T_FY * np] = ta[k].fy;
        S[b + LFDM_T_FZ * np] = ta[k].fz;
        S[b + LFDM_T_VSX * np] = ta[k].vsx;
        S[b + LFDM_T_VSY * np] = ta[k].vsy;
        S[b + LFDM_T_MY * np] = ta[k].My;
        S[b + LFDM_T_ENGTOR * np] = ta[k].engTor;
    }
    if (w.status) {
        const bool bad = !(isfinite(v.x) && isfinite(v.y) && isfinite(v.u) && isfinite(v.v) && isfinite(v.psi) &&
                           isfinite(v.wz) && isfinite(ts[0].omega) && isfinite(ts[1].omega) &&
                           isfinite(ts[2].omega) && isfinite(ts[3].omega));
        if (bad) w.status[vid] |= 1u;
    }
}

template <int kCtl, bool kOut>
static cudaError_t launch_mixed_t(const Window18& w, cudaStream_t stream) {
    const int threads = w.threads;
    const size_t smem = window18_mixed_smem(threads, w.nclasses);
    auto kern = window18_mixed_kernel<kCtl, kOut>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<(w.n + threads - 1) / threads, threads, smem, stream>>>(w);
    return cudaGetLastError();
}

template <int kCtl>
static cudaError_t launch_mixed_o(const Window18& w, cudaStream_t s) {
    return (w.resp && w.nsamples > 0) ? launch_mixed_t<kCtl, true>(w, s) : launch_mixed_t<kCtl, false>(w, s);
}

static cudaError_t launch_mixed(const Window18& w, cudaStream_t s) {
    switch (w.ctl_mode) {
        case CTL_TABLE: return launch_mixed_o<CTL_TABLE>(w, s);
        case CTL_SCALAR: return launch_mixed_o<CTL_SCALAR>(w, s);
        case CTL_SCHEDULE: return launch_mixed_o<CTL_SCHEDULE>(w, s);
        default: return launch_mixed_o<CTL_ARRAY>(w, s);
    }
}

void build_class_dev18f(const lfdm_class18& c, ClassDev18F* out) {
    std::memset(out, 0, sizeof(*out));
    out->nonLinearSteer = c.nonLinearSteer;
    out->tcbool = c.tcbool;
    out->throttleMod = c.throttleMod;
    out->driveType = c.driveType;
    out->whichWheels = c.whichWheels;
    out->noGears = c.noGears;
    for (int g = 0; g < c.noGears && g < LFDM_MAX_GEARS; ++g) {
        out->gear[g] = (float)c.gearRatios[g];
        out->down[g] = (float)c.shiftMap[g][0];
        out->up[g] = (float)c.shiftMap[g][1];
    }
    auto mapf = [](const double (*pts)[2], int n, MapF& m) {
        m.n = n;
        for (int k = 0; k < n; ++k) {
            m.x[k] = (float)pts[k][0];
            m.y[k] = (float)pts[k][1];
        }
        for (int k = 0; k + 1 < n; ++k) {
            m.dx[k] = m.x[k + 1] - m.x[k];
            m.dy[k] = m.y[k + 1] - m.y[k];
        }
    };
    mapf(c.steerMap, c.steerMapSize, out->steer);
    mapf(c.powertrainMap, c.powertrainMapSize, out->pt);
    mapf(c.lossesMap, c.lossesMapSize, out->loss);
    mapf(c.CFmap, c.CFmapSize, out->cf);
    mapf(c.TRmap, c.TRmapSize, out->tr);
}
size_t class_dev18f_size() { return sizeof(ClassDev18F); }

template <bool kNr, int kCtl, bool kOut, bool kF32>
static cudaError_t launch_t(const Window18& w, cudaStream_t stream) {
    const int threads = w.threads;
    const size_t smem = window18_smem(threads, w.nclasses, kF32);
    auto kern = window18_kernel<kNr, kCtl, kOut, kF32>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int blocks = (w.n + threads - 1) / threads;
    kern<<<blocks, threads, smem, stream>>>(w);
    return cudaGetLastError();
}

template <bool kNr, int kCtl, bool kF32>
static cudaError_t launch_o(const Window18& w, cudaStream_t s) {
    return (w.resp && w.nsamples > 0) ? launch_t<kNr, kCtl, true, kF32>(w, s) : launch_t<kNr, kCtl, false, kF32>(w, s);
}
template <bool kNr, bool kF32 = false>
static cudaError_t launch_c(const Window18& w, cudaStream_t s) {
    switch (w.ctl_mode) {
        case CTL_TABLE: return launch_o<kNr, CTL_TABLE, kF32>(w, s);
        case CTL_SCALAR: return launch_o<kNr, CTL_SCALAR, kF32>(w, s);
        case CTL_SCHEDULE: return launch_o<kNr, CTL_SCHEDULE, kF32>(w, s);
        default: return launch_o<kNr, CTL_ARRAY, kF32>(w, s);
    }
}

cudaError_t launch_window18(const Window18& w, cudaStream_t stream) {
    if (w.n <= 0 || w.nsteps <= 0) return cudaSuccess;
    if (w.threads <= 0 || w.threads > 128 || (w.threads & 31)) return cudaErrorInvalidValue;
    if (w.precision == LFDM_PREC_MIXED) {
        if (w.tire_nr || !w.classes_f) return cudaErrorInvalidValue;
        return launch_mixed(w, stream);
    }
    if (w.precision == LFDM_PREC_MIXED_TIRE)
        return w.tire_nr ? launch_c<true, true>(w, stream) : launch_c<false, true>(w, stream);
    if (w.precision != LFDM_PREC_FP64) return cudaErrorInvalidValue;
    return w.tire_nr ? launch_c<true>(w, stream) : launch_c<false>(w, stream);
}

}  // namespace lfdm
