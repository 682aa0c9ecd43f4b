// Differentiable 18-DOF rollout: forward kernel (loss, checkpoints) and backward kernel (adjoint
// through the half-implicit steps with checkpointing and per-segment recomputation).
//
// Rollout: nsteps steps of step18<false> from the solver's current states with per-step controls
// ctl[k][3][n] = {steering, throttle, braking}. Loss per vehicle (after every step k):
//   e_lat = -(x - xr) sin(psir) + (y - yr) cos(psir), e_head = psi - psir,
//   L += e_lat^2 + e_head^2 + w (steering^2 + throttle^2 + braking^2),
// with the reference path ref[k][3][n] = {xr, yr, psir} at the end of step k.
// Backward: the forward stores the state every `ckpt` steps and runs the last segment with
// fwd18_tape, leaving that segment's tape in HBM. The backward runs the segments last to first: it
// recomputes each earlier segment from its checkpoint with fwd18_tape (dof18_adjoint.cuh), storing
// each step's tape in HBM, then sweeps the segment backwards with rev18, writing the control
// gradients and accumulating the adjoints of the parameter-dependent constants; at the end those
// are contracted with dK/dp (forward-mode dual numbers through the prepare formulas) for the
// parameter gradients: mass, Jz, CG-to-front distance a (b held), tire friction scale (a common
// factor on the peak and sliding forces fxmPn..fysP2n, derivative at scale 1), tire vertical
// stiffness kt.
#include <cuda_runtime.h>

#include "adjoint18.h"
#include "dof18_adjoint.cuh"
#include "window_common.cuh"

namespace lfdm {

constexpr int kCkptFields = 32;  // VehC (11 doubles + gear) and 4 x TireC (5 doubles)

__device__ __forceinline__ void store_ckpt(double* P, size_t np, const VehC& v, const TireC* ts) {
    const double vals[12] = {v.x, v.y, v.u, v.v, v.psi, v.wz, v.phi, v.wx, v.udot, v.vdot, v.crank, (double)v.gear};
#pragma unroll
    for (int f = 0; f < 12; ++f) P[f * np] = vals[f];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        P[(12 + 5 * k) * np] = ts[k].xe;
        P[(13 + 5 * k) * np] = ts[k].ye;
        P[(14 + 5 * k) * np] = ts[k].xedot;
        P[(15 + 5 * k) * np] = ts[k].yedot;
        P[(16 + 5 * k) * np] = ts[k].omega;
    }
}
__device__ __forceinline__ void load_ckpt(const double* P, size_t np, VehC& v, TireC* ts) {
    v.x = P[0];
    v.y = P[1 * np];
    v.u = P[2 * np];
    v.v = P[3 * np];
    v.psi = P[4 * np];
    v.wz = P[5 * np];
    v.phi = P[6 * np];
    v.wx = P[7 * np];
    v.udot = P[8 * np];
    v.vdot = P[9 * np];
    v.crank = P[10 * np];
    v.gear = (int)P[11 * np];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        ts[k].xe = P[(12 + 5 * k) * np];
        ts[k].ye = P[(13 + 5 * k) * np];
        ts[k].xedot = P[(14 + 5 * k) * np];
        ts[k].yedot = P[(15 + 5 * k) * np];
        ts[k].omega = P[(16 + 5 * k) * np];
    }
}

__device__ __forceinline__ double step_loss(const AdjLaunch& A, int k, int vid, double x, double y, double psi,
                                            double st, double th, double br) {
    const size_t nu = (size_t)A.n;
    const double* R = A.ref + (size_t)k * 3 * nu + vid;
    const double xr = __ldg(R), yr = __ldg(R + nu), pr = __ldg(R + 2 * nu);
    double sr, cr;
    sincos(pr, &sr, &cr);
    const double el = fma(-(x - xr), sr, (y - yr) * cr);
    const double eh = psi - pr;
    return fma(el, el, eh * eh) + A.weight_u * fma(st, st, fma(th, th, br * br));
}

// Shared memory of the rollout kernels: the classes (when cls_smem), the derived constants of the
// block's vehicles [K18_COUNT][blockDim] and, for the backward kernel, the adjoints of the
// parameter-dependent constants [KB_COUNT][blockDim]. Every access of the inner step then stays in
// shared memory instead of interleaving with the tape's HBM stores and loads. Both kernels are
// register-bound to two 128-thread blocks per SM; the classes are staged only while two blocks
// still fit in the SM's 228 KB (1 KB of it reserved per block).
size_t traj18_smem(int threads, int nclasses, bool backward, bool* cls_smem) {
    const size_t base = (size_t)(K18_COUNT + (backward ? KB_COUNT : 0)) * threads * sizeof(double);
    const size_t cls = (size_t)nclasses * sizeof(ClassDev18);
    const bool in = nclasses <= kMaxSmemClasses && 2 * (base + cls + 1024) <= 228 * 1024;
    if (cls_smem) *cls_smem = in;
    return base + (in ? cls : 0);
}

struct RolloutSmem {
    const ClassDev18* cls;  // classes (shared or global)
    double* ks;             // [K18_COUNT][blockDim]
    double* kb;             // [KB_COUNT][blockDim] (backward)
};

__device__ __forceinline__ RolloutSmem stage_rollout(const AdjLaunch& A, unsigned char* smem, int vid) {
    const int tid = threadIdx.x;
    RolloutSmem r;
    r.cls = A.cls_smem ? reinterpret_cast<const ClassDev18*>(smem) : A.classes;
    r.ks = reinterpret_cast<double*>(smem + (A.cls_smem ? (size_t)A.nclasses * sizeof(ClassDev18) : 0));
    r.kb = r.ks + (size_t)K18_COUNT * blockDim.x;
    if (A.cls_smem) {
        const int4* src = reinterpret_cast<const int4*>(A.classes);
        int4* dst = reinterpret_cast<int4*>(smem);
        const int words = (int)(A.nclasses * sizeof(ClassDev18) / 16);
        for (int i = tid; i < words; i += blockDim.x) dst[i] = __ldg(src + i);
    }
    if (vid < A.n) {
#pragma unroll 4
        for (int k = 0; k < K18_COUNT; ++k) r.ks[k * blockDim.x + tid] = __ldg(A.K + (size_t)k * A.npad + vid);
    }
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(128) traj18_forward_kernel(const AdjLaunch A) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int vid = blockIdx.x * blockDim.x + threadIdx.x;
    const RolloutSmem sm = stage_rollout(A, smem, vid);
    if (vid >= A.n) return;
    const size_t np = (size_t)A.npad;
    const KView K{sm.ks + threadIdx.x, (int)blockDim.x};
    const ClassDev18& C = sm.cls[__ldg(A.class_of + vid)];
    VehC v;
    VehAux va;
    TireC ts[4];
    TireAux ta[4];
    load_state18(A.S0 + vid, np, v, va, ts, ta);
    const size_t nu = (size_t)A.n;
    double loss = 0;
    // the last segment runs with its tape (the backward starts there and then needs no recompute);
    // fwd18_tape and step18 round identically, so the states do not depend on which one ran
    const int klast = ((A.nsteps - 1) / A.ckpt) * A.ckpt;
    for (int k = 0; k < A.nsteps; ++k) {
        if (k % A.ckpt == 0) store_ckpt(A.ckpts + (size_t)(k / A.ckpt) * kCkptFields * np + vid, np, v, ts);
        const double* U = A.ctl + (size_t)k * 3 * nu + vid;
        const double st = __ldg(U), th = __ldg(U + nu), br = __ldg(U + 2 * nu);
        if (k < klast) {
            step18<false>(v, va, ts, ta, K, C, st, th, br, A.dt);
        } else {
            const TapeRef T{A.tape + (size_t)(k - klast) * kStepTapeDoubles * np + vid, np};
            fwd18_tape(v, va, ts, ta, T, K, C, st, th, br, A.dt);
        }
        loss += step_loss(A, k, vid, v.x, v.y, v.psi, st, th, br);
    }
    A.loss[vid] = loss;
}

// dual number for the parameter derivatives of the derived constants
struct Dual {
    double v, d;
};
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
__device__ __forceinline__ Dual operator/(Dual a, Dual b) { return {a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)}; }
__device__ __forceinline__ Dual cst(double v) { return {v, 0.0}; }

// d K_kb / d parameter `which` (0 m, 1 jz, 2 a with b held, 3 friction scale, 4 kt) for the
// constants with an adjoint (the prepare formulas of prepare18_kernel and prepare_shared_k).
__device__ void dK_dparam(const double* p, int which, double* out) {
    const Dual G = cst(kG);
    const Dual m = {p[LFDM_P_M], which == 0 ? 1.0 : 0.0};
    const Dual jz = {p[LFDM_P_JZ], which == 1 ? 1.0 : 0.0};
    const Dual a = {p[LFDM_P_A], which == 2 ? 1.0 : 0.0};
    const Dual b = cst(p[LFDM_P_B]), h = cst(p[LFDM_P_H]), jx = cst(p[LFDM_P_JX]), jxz = cst(p[LFDM_P_JXZ]);
    const Dual cf = cst(p[LFDM_P_CF]), cr = cst(p[LFDM_P_CR]), muf = cst(p[LFDM_P_MUF]), mur = cst(p[LFDM_P_MUR]);
    const Dual hrcf = cst(p[LFDM_P_HRCF]), hrcr = cst(p[LFDM_P_HRCR]);
    const Dual kr = cst(p[LFDM_P_KROF] + p[LFDM_P_KROR]);
    const Dual r0 = cst(p[LFDM_P_R0]);
    const Dual two = cst(2.0), half = cst(0.5);
    auto fr = [&](int idx) { return Dual{p[idx], which == 3 ? p[idx] : 0.0}; };  // friction-scaled field
    const Dual kt = {p[LFDM_P_KT], which == 4 ? 1.0 : 0.0};
    const Dual ab = a + b;
    const Dual huf = r0, hur = r0;
    out[KB_Z1F] = (m * G * b / (two * ab) + muf * G / two).d;
    out[KB_Z2F] = (muf * huf / cf + m * b * (h - hrcf) / (cf * ab)).d;
    out[KB_Z4] = ((m * h + muf * huf + mur * hur) / (two * ab)).d;
    out[KB_Z1R] = (m * G * a / (two * ab) + mur * G / two).d;
    out[KB_Z2R] = (mur * hur / cr + m * a * (h - hrcr) / (cr * ab)).d;
    const Dual mt = m + two * (muf + mur);
    const Dual hrc = (hrcf * b + hrcr * a) / ab;
    const Dual A1 = mur * b - muf * a;
    const Dual A2 = jx + m * hrc * hrc;
    const Dual A3 = hrc * m;
    const Dual den = A2 * A1 * A1 - two * A1 * A3 * jxz + jz * A3 * A3 + mt * jxz * jxz - A2 * jz * mt;
    out[KB_MT] = mt.d;
    out[KB_INVMT] = (cst(1.0) / mt).d;
    out[KB_E2WU] = (cst(0.0) - muf * a + mur * b).d;
    out[KB_E3PHI] = (m * G * hrc - kr).d;
    out[KB_E3WU] = (hrc * m).d;
    out[KB_UWZ2] = (cst(0.0) - mur * b + muf * a).d;
    out[KB_UWZWX] = (two * hrc * m).d;
    out[KB_CV1] = ((jxz * jxz - A2 * jz) / den).d;
    out[KB_CV2] = ((A3 * jxz - A1 * A2) / den).d;
    out[KB_CV3] = ((A1 * jxz - A3 * jz) / den).d;
    out[KB_CX2] = ((jxz * mt - A1 * A3) / den).d;
    out[KB_CX3] = ((A1 * A1 - jz * mt) / den).d;
    out[KB_CZ2] = ((A3 * A3 - A2 * mt) / den).d;
    out[KB_A] = a.d;
    auto q1 = [&](int i1, int i2) { return (two * fr(i1) - half * fr(i2)).d; };
    auto q2 = [&](int i1, int i2) { return (fr(i1) - half * fr(i2)).d; };
    out[KB_Q1FXM] = q1(LFDM_P_FXMPN, LFDM_P_FXMP2N);
    out[KB_Q2FXM] = q2(LFDM_P_FXMPN, LFDM_P_FXMP2N);
    out[KB_Q1FYM] = q1(LFDM_P_FYMPN, LFDM_P_FYMP2N);
    out[KB_Q2FYM] = q2(LFDM_P_FYMPN, LFDM_P_FYMP2N);
    out[KB_Q1FXS] = q1(LFDM_P_FXSPN, LFDM_P_FXSP2N);
    out[KB_Q2FXS] = q2(LFDM_P_FXSPN, LFDM_P_FXSP2N);
    out[KB_Q1FYS] = q1(LFDM_P_FYSPN, LFDM_P_FYSP2N);
    out[KB_Q2FYS] = q2(LFDM_P_FYSPN, LFDM_P_FYSP2N);
    out[KB_FXMP2N] = fr(LFDM_P_FXMP2N).d;
    out[KB_FYMP2N] = fr(LFDM_P_FYMP2N).d;
    out[KB_INVKT] = (cst(1.0) / kt).d;
}

__global__ void __launch_bounds__(128) traj18_backward_kernel(const AdjLaunch A) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int vid = blockIdx.x * blockDim.x + threadIdx.x;
    const RolloutSmem sm = stage_rollout(A, smem, vid);
    if (vid >= A.n) return;
    const size_t np = (size_t)A.npad, nu = (size_t)A.n;
    const KView K{sm.ks + threadIdx.x, (int)blockDim.x};
    const ClassDev18& C = sm.cls[__ldg(A.class_of + vid)];
    const KBar kb{sm.kb + threadIdx.x, (int)blockDim.x};
#pragma unroll 1
    for (int i = 0; i < KB_COUNT; ++i) kb.base[i * blockDim.x] = 0.0;
    Adj18 L = {};
    const int nseg = (A.nsteps + A.ckpt - 1) / A.ckpt;
    for (int seg = nseg - 1; seg >= 0; --seg) {
        const int k0 = seg * A.ckpt, k1 = min(A.nsteps, k0 + A.ckpt);
        if (seg < nseg - 1) {  // the forward left the last segment's tape in place
            VehC v;
            VehAux va = {};
            TireC ts[4];
            TireAux ta[4] = {};
            load_ckpt(A.ckpts + (size_t)seg * kCkptFields * np + vid, np, v, ts);
            for (int k = k0; k < k1; ++k) {
                const double* U = A.ctl + (size_t)k * 3 * nu + vid;
                const TapeRef T{A.tape + (size_t)(k - k0) * kStepTapeDoubles * np + vid, np};
                fwd18_tape(v, va, ts, ta, T, K, C, __ldg(U), __ldg(U + nu), __ldg(U + 2 * nu), A.dt);
            }
        }
        for (int k = k1 - 1; k >= k0; --k) {
            const TapeRef T{A.tape + (size_t)(k - k0) * kStepTapeDoubles * np + vid, np};
            // loss of step k on the state after it
            {
                const double* R = A.ref + (size_t)k * 3 * nu + vid;
                const double xr = __ldg(R), yr = __ldg(R + nu), pr = __ldg(R + 2 * nu);
                double sr, cr;
                sincos(pr, &sr, &cr);
                const double el = fma(-(T.at(TS_(x1)) - xr), sr, (T.at(TS_(y1)) - yr) * cr);
                L.x += -2.0 * el * sr;
                L.y += 2.0 * el * cr;
                L.psi += 2.0 * (T.at(TS_(psi1)) - pr);
            }
            double sb = 2.0 * A.weight_u * T.at(TS_(steer)), tb = 2.0 * A.weight_u * T.at(TS_(thr)),
                   bb = 2.0 * A.weight_u * T.at(TS_(brk));
            rev18(T, K, C, kb, A.dt, L, sb, tb, bb);
            double* G = A.grad_ctl + (size_t)k * 3 * nu + vid;
            G[0] = sb;
            G[nu] = tb;
            G[2 * nu] = bb;
        }
    }
    if (A.grad_state0) {
        // fully unrolled so that L stays in registers (a runtime index would put it on the stack)
        const double* l = &L.x;
#pragma unroll
        for (int f = 0; f < kAdj18Count; ++f) A.grad_state0[f * nu + vid] = l[f];
    }
    // parameter gradients
    const double* p = A.params + (size_t)vid * LFDM_P_COUNT;
#pragma unroll 1
    for (int j = 0; j < 5; ++j) {
        double d[KB_COUNT];
        dK_dparam(p, j, d);
        double gsum = 0;
#pragma unroll 1
        for (int i = 0; i < KB_COUNT; ++i) gsum = fma(kb.base[i * blockDim.x], d[i], gsum);
        A.grad_params[j * nu + vid] = gsum;
    }
}

static cudaError_t launch_rollout(void (*kern)(const AdjLaunch), const AdjLaunch& A, bool backward,
                                  cudaStream_t stream) {
    if (A.n <= 0 || A.nsteps <= 0) return cudaSuccess;
    constexpr int threads = 128;
    AdjLaunch L = A;
    const size_t smem = traj18_smem(threads, A.nclasses, backward, &L.cls_smem);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<(A.n + threads - 1) / threads, threads, smem, stream>>>(L);
    return cudaGetLastError();
}
// ---------------------------------------------------------------------------------------------
// Branch signature of a rollout: a 64-bit hash of every discrete decision the steps take (per tire:
// wheel on the ground, dynamic-radius band, load clamp, zero combined slip, tmxy_combined regime,
// structural-force clamps, sineStep bands of the force blend, sign of the wheel speed; per vehicle:
// the segments of the steering, engine and loss maps, converter speed-ratio mode, flow direction
// and map segments, drive-torque clip, gear, differential bias bands and slower wheels). Two rollouts
// with equal signatures took the same branch at every step, so the loss is smooth between them.

__device__ __forceinline__ uint64_t sig_mix(uint64_t h, uint64_t w) {
    // FNV-1a over the 8 bytes of w
#pragma unroll
    for (int b = 0; b < 8; ++b) {
        h ^= (w >> (8 * b)) & 0xffu;
        h *= 0x100000001b3ull;
    }
    return h;
}
__device__ __forceinline__ uint64_t sig_d(uint64_t h, double x) { return sig_mix(h, (uint64_t)__double_as_longlong(x)); }
// 0 below the sineStep band, 1 inside, 2 above (weight 1, between, 0)
__device__ __forceinline__ double band(double w, double dw) {
    return (dw != 0.0) ? 1.0 : (w == 1.0 ? 0.0 : (w == 0.0 ? 2.0 : 1.0));
}
__device__ __forceinline__ double seg(const MapDev& m, double x) {
    if (x <= m.x[0]) return -1.0;
    if (x >= m.x[m.n - 1]) return (double)m.n;
    return (double)lower_bound_x(m.x, m.n, x);
}

__device__ uint64_t step_signature(uint64_t h, const TapeRef& T, const ClassDev18& C) {
    h = sig_d(h, T.at(TS_(gear)));
    h = sig_d(h, C.nonLinearSteer ? seg(C.steer, T.at(TS_(steer))) : 0.0);
    const double crank_used = C.tcbool ? T.at(TS_(crank)) : T.at(TS_(omega_in));
    h = sig_d(h, seg(C.pt, crank_used));
    h = sig_d(h, seg(C.loss, crank_used));
    if (C.tcbool) {
        h = sig_d(h, T.at(TS_(srmode)));
        h = sig_d(h, T.at(TS_(rev)));
        h = sig_d(h, seg(C.cf, T.at(TS_(sr))));
        h = sig_d(h, seg(C.tr, T.at(TS_(sr))));
    }
    h = sig_d(h, T.at(TS_(tclip)));
    // bias band of each axle's differential; which wheel gets the larger share matters only with a bias
    const double bf = T.at(TS_(dalf)) != 0.0 ? 1.0 : (T.at(TS_(alf)) == 0.5 ? 0.0 : 2.0);
    const double br = T.at(TS_(dalr)) != 0.0 ? 1.0 : (T.at(TS_(alr)) == 0.5 ? 0.0 : 2.0);
    h = sig_d(h, bf);
    h = sig_d(h, br);
    if (bf != 0.0) h = sig_d(h, T.at(TS_(slowf)));
    if (br != 0.0) h = sig_d(h, T.at(TS_(slowr)));
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const TapeRef R = tire_ref(T, k);
        const double on = R.at(TT_(on));
        h = sig_d(h, on);
        if (on == 0.0) continue;
        h = sig_d(h, R.at(TT_(fzrd)));
        h = sig_d(h, R.at(TT_(fzcl)));
        h = sig_d(h, R.at(TT_(qpos)));
        h = sig_d(h, R.at(TT_(reg)));
        h = sig_d(h, R.at(TT_(clx)));
        h = sig_d(h, R.at(TT_(cly)));
        h = sig_d(h, band(R.at(TT_(wxw)), R.at(TT_(dwx))));
        h = sig_d(h, band(R.at(TT_(wyw)), R.at(TT_(dwy))));
        h = sig_d(h, R.at(TT_(sgn)));
    }
    return h;
}

// The rollout of traj18_forward_kernel (the same arithmetic: fwd18_tape rounds as step18) with a
// one-step tape per vehicle, hashing each step's decisions.
__global__ void __launch_bounds__(128) traj18_signature_kernel(const AdjLaunch A, uint64_t* sig) {
    const int vid = blockIdx.x * blockDim.x + threadIdx.x;
    if (vid >= A.n) return;
    const size_t np = (size_t)A.npad;
    const KView K{A.K + vid, A.npad};
    const ClassDev18& C = A.classes[__ldg(A.class_of + vid)];
    VehC v;
    VehAux va;
    TireC ts[4];
    TireAux ta[4];
    load_state18(A.S0 + vid, np, v, va, ts, ta);
    const size_t nu = (size_t)A.n;
    const TapeRef T{A.tape + vid, np};
    uint64_t h = 0xcbf29ce484222325ull;
    for (int k = 0; k < A.nsteps; ++k) {
        const double* U = A.ctl + (size_t)k * 3 * nu + vid;
        fwd18_tape(v, va, ts, ta, T, K, C, __ldg(U), __ldg(U + nu), __ldg(U + 2 * nu), A.dt);
        h = step_signature(h, T, C);
    }
    sig[vid] = h;
}

cudaError_t launch_traj18_signature(const AdjLaunch& A, uint64_t* sig, cudaStream_t stream) {
    traj18_signature_kernel<<<(A.n + 127) / 128, 128, 0, stream>>>(A, sig);
    return cudaGetLastError();
}

cudaError_t launch_traj18_forward(const AdjLaunch& A, cudaStream_t stream) {
    return launch_rollout(traj18_forward_kernel, A, false, stream);
}
cudaError_t launch_traj18_backward(const AdjLaunch& A, cudaStream_t stream) {
    return launch_rollout(traj18_backward_kernel, A, true, stream);
}
size_t traj18_tape_doubles_per_step() { return (size_t)kStepTapeDoubles; }
int traj18_ckpt_fields() { return kCkptFields; }
int traj18_state_adjoints() { return kAdj18Count; }

}  // namespace lfdm
