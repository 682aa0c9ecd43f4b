"""Throughput of the batched half-implicit 18-DOF stepper on GB300 (vehicle-steps/s).

Workload (default): the seeded synthetic SUV fleet, 18-DOF with TMeasy tires, FP64, dt = 1e-3 s,
300,000 vehicles with mass, Jz, CG position, tire vertical stiffness and peak friction jittered
+/-10%, per-vehicle driver tables sampled every 10 ms (sine steering, throttle ramp, brake
pulse), outputs (13 channels) sampled every 10 ms. A bench "step" is one stepping window of
kernel_sim_time = 1 s (1,000 integration steps) over all vehicles, continuing the trajectory;
W warm-up windows then K timed windows (defaults 3 + 7 = the 10 s horizon).

value: device time (CUDA events on the solver's stream around each window kernel) with inputs
       resident in HBM and the response written into HBM.
e2e:   the same windows through the C ABI with host buffers: each step uploads that window's
       driver-table rows from page-locked host memory and streams the window's response back to
       page-locked host memory; wall-clock time.
--impl reference: the reference's CPU algorithm (the oracle restatement, oracle/lfdm_oracle.c) on
       all host cores over a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
PKG = "low-fidelity-dynamic-models_gb300"
SEED = 20261203
W_ALG_18 = 1391  # FP64 source-level operations per 18-DOF vehicle-step of the reference algorithm
W_ALG = {11: 675, 18: 1391, 24: 1941}  # the same count for the three models
# FP64 instructions the 18-DOF window kernel executes per vehicle-step (ncu, one window launch on
# 32,768 vehicles of the seeded fleet, the fourth 1 s window): DFMA + DMUL + DADD of active lanes
# (sm__sass_thread_inst_executed_op_{dfma,dmul,dadd}_pred_on.sum), and everything the FP64 pipe
# issued in lanes (sm__inst_executed_pipe_fp64.sum x 32: also compares, min/max and conversions, and
# the inactive lanes of divergent warps, which occupy the pipe alike)
FP64_INST_PER_VSTEP_18 = 1092
FP64_PIPE_PER_VSTEP_18 = 1227
# The mixed-precision forms of the 18-DOF stepper: (precision enum, key, arithmetic)
MIXED_FORMS = ((1, "mixed", "f32 RHS and tire math; f64 states, X/Y/yaw accumulation, slip and transport velocities"),
               (2, "mixed_tire", "f32 TMeasy tire core; f64 everything else"))
# Lane instructions per vehicle-step the two pipes of the mixed window kernels issue, (FMA pipe,
# FP64 pipe): ncu sm__inst_executed_pipe_fma.sum and sm__inst_executed_pipe_fp64.sum x 32 of one
# window launch on 32,768 vehicles of the seeded fleet (the fourth 1 s window), per vehicle-step.
# Of the FP64 pipe's 101 (MIXED) and 384 (MIXED_TIRE), 69 and 52 are float/double conversions.
MIXED_INST_PER_VSTEP = {1: (1320, 101), 2: (1005, 384)}
METRIC = "18-DOF vehicle-steps/s on 1 GB300: FP64 plain vs mixed at stated error; adjoint/fwd"


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=7)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--vehicles", type=int, default=300_000)
    ap.add_argument("--ksim", type=float, default=1.0)
    ap.add_argument("--threads", type=int, default=0, help="threads per block (0: library default)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-models", action="store_true", help="skip the 11/24-DOF throughput lines")
    ap.add_argument("--no-fleet", action="store_true", help="skip the mixed-DOF fleet line")
    ap.add_argument("--no-reference-gpu", action="store_true", help="skip timing the reference's own GPU solver")
    ap.add_argument("--fleet-vehicles", type=int, default=250_000)
    ap.add_argument("--no-adjoint", action="store_true", help="skip the differentiable-rollout line")
    ap.add_argument("--adjoint-vehicles", type=int, default=65_536)
    ap.add_argument("--no-jacobian", action="store_true", help="skip the right-hand-side Jacobian line")
    ap.add_argument("--jacobian-vehicles", type=int, default=65_536)
    ap.add_argument("--error-vehicles", type=int, default=1_000_000,
                    help="vehicles of the mixed-precision error run (the precision config's 1,000,000)")
    ap.add_argument("--error-horizon", type=float, default=20.0)
    ap.add_argument("--ceiling-vehicles", type=int, default=65536,
                    help="vehicles of the FP64-sensitivity runs that bound what any FP32-based form can hold")
    ap.add_argument("--cpu-sample", type=int, default=32768, help="vehicles in the CPU-baseline sample")
    return ap.parse_args()


class Dist:
    def __init__(self, n):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


class CpuTrajectory:
    """The reference's CPU algorithm (the oracle restatement, oracle/lfdm_oracle.c, built with the
    reference's Release flags -O3) on the host cores over the first `nveh` vehicles of a fleet:
    window() advances their trajectories by one stepping window of ksim seconds (the GPU solver's
    schedule), continuing from where the previous call ended, and returns its wall time."""

    def __init__(self, f, nveh: int, ksim: float, threads: int, model: int = 18):
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import oracle_lib
        self.O = oracle_lib
        sl = slice(0, nveh)
        self.cls, self.class_of, self.params = f["cls"], f["class_of"][sl], f["params"][sl]
        self.tables = f["tables"][sl]
        self.states = np.array(f["states"][sl], copy=True)
        self.nveh, self.ksim, self.threads, self.model = nveh, ksim, threads, model
        self.k = 0

    def window(self) -> float:
        t0 = time.perf_counter()
        self.states, _ = self.O.run18(self.cls, self.class_of, self.params, self.states, self.tables,
                                      t0=self.k * self.ksim, tend=(self.k + 1) * self.ksim, ksim=self.ksim, schedule=1,
                                      nthreads=self.threads, model=self.model, timing=True)
        self.k += 1
        return time.perf_counter() - t0


def run_reference(a, dist: Dist):
    if dist.rank != 0:
        return
    fleet = importlib.import_module(PKG + ".fleet")
    cores = os.cpu_count() or 1
    n = a.cpu_sample
    f = fleet.fleet18(n, seed=SEED, horizon=(a.warmup + a.steps) * a.ksim)
    cpu = CpuTrajectory(f, n, a.ksim, cores)
    for _ in range(a.warmup):
        cpu.window()
    times = [cpu.window() for _ in range(a.steps)]
    steps = int(round(a.ksim / 1e-3))
    v = n * steps * a.steps / sum(times)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "vehicle-steps/s", "n_gpus": a.gpus,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * sum(times) / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded SUV fleet)",
        "config": _config(a, n_override=n),
        "cpu_baseline": {"value": v, "unit": "vehicle-steps/s", "cores": cores, "kind": "port",
                         "sample": f"{n} vehicles x {steps} steps per step (bounded sample of the fleet), the "
                                   "trajectories continued window after window, "
                                   f"{cores} host threads; the reference's CPU algorithm as restated in "
                                   "oracle/lfdm_oracle.c, built with the reference's Release flags (-O3); "
                                   "the reference checkout is not on this host"},
        "e2e": {"value": v, "unit": "vehicle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _config(a, n_override=None):
    return {"workload": "18-DOF TMeasy SUV fleet, FP64, dt 1e-3 s, 10 ms driver tables and outputs, "
                        f"{n_override or a.vehicles} vehicles, windows of {a.ksim:g} s",
            "vehicles": n_override or a.vehicles, "dt": 1e-3, "kernel_sim_time": a.ksim, "output_hz": 100,
            "model": "18dof-tmeasy", "seed": SEED,
            "l2": "inputs larger than L2 (driver tables ~32 KB/vehicle, state 600 B, constants 560 B)"}


def _error_runs(lfdm, dev, f, horizon, runs):
    """Final states of the seeded fleet `f` after `horizon` seconds for each (key, precision, eps):
    the initial speeds scaled by (1 + eps)."""
    S = lfdm.S
    out = {}
    for key, prec, eps in runs:
        s = lfdm.d18SolverHalfImplicitGPU(f["params"].shape[0], device=dev)
        s.construct_class(f["cls"][0], f["params"])
        s.set_driver_tables(f["tables"])
        st0 = np.array(f["states"], copy=True)
        st0[:, S["u"]] *= 1.0 + eps
        s.set_states(st0)
        s.SetKernelSimTime(1.0)
        s.SetEndTime(horizon)
        s.set_precision(prec)
        s.Solve()
        out[key] = s.get_states()
        s.close()
    return out


def _dpos(S, x, y):
    return np.hypot(y[:, S["x"]] - x[:, S["x"]], y[:, S["y"]] - x[:, S["y"]])


def _stats(e):
    return {"max": float(e.max()), "p99": float(np.quantile(e, 0.99)), "p50": float(np.median(e))}


def _mixed_error(lfdm, fleet, dev, n, horizon):
    """End-of-horizon position, yaw and speed error of each mixed form against the FP64 form (max,
    p99, p50 over vehicles, and the fraction within 1 cm): the seeded fleet at n vehicles with
    initial speeds U[0.5, 30] m/s (near-standstill starts stress the low-speed slip path) and driver
    tables sampled every 50 ms (the 10 ms tables of 1,000,000 vehicles over 20 s would take 64 GB)."""
    f = fleet.fleet18(n, seed=SEED + 7, horizon=horizon, table_dt=0.05, u0_range=(0.5, 30.0))
    runs = [("fp64", 0, 0.0)] + [(key, prec, 0.0) for prec, key, _ in MIXED_FORMS]
    out = _error_runs(lfdm, dev, f, horizon, runs)
    del f
    S = lfdm.S
    a = out["fp64"]
    res = {"vehicles": n, "horizon_s": horizon, "u0_range": [0.5, 30.0], "table_dt_s": 0.05}
    for _, key, _ in MIXED_FORMS:
        b = out[key]
        pos = _dpos(S, a, b)
        yaw = np.abs(b[:, S["psi"]] - a[:, S["psi"]])
        spd = np.abs(np.hypot(b[:, S["u"]], b[:, S["v"]]) - np.hypot(a[:, S["u"]], a[:, S["v"]]))
        res[key] = {"position_m": _stats(pos), "yaw_rad": _stats(yaw), "speed_mps": _stats(spd),
                    "frac_position_within_1cm": float((pos <= 0.01).mean()),
                    "finite": bool(np.isfinite(b[:, :15]).all())}
    return res


def _mixed_retention(lfdm, fleet, dev, n, horizon):
    """What FP32-level rounding costs beyond the fleet's own sensitivity. The FP64 form is rerun from
    initial speeds u (1 + 1e-15) (FP64 rounding level) and u (1 + 1e-7) (FP32 rounding level, applied
    once). Vehicles the 1e-7 run leaves within 1 cm of FP64 are insensitive at FP32 level; the
    retention of a form is the fraction of those that it also ends within 1 cm of FP64. The 1e-15
    run's own retention is the ceiling: vehicles that even an FP64-level perturbation moves past
    1 cm are lost to rounding-level chaos whatever the arithmetic."""
    f = fleet.fleet18(n, seed=SEED + 7, horizon=horizon, table_dt=0.05, u0_range=(0.5, 30.0))
    runs = [("fp64", 0, 0.0), ("fp64_1e-15", 0, 1e-15), ("fp64_1e-7", 0, 1e-7)]
    runs += [(key, prec, 0.0) for prec, key, _ in MIXED_FORMS]
    out = _error_runs(lfdm, dev, f, horizon, runs)
    S = lfdm.S
    a = out["fp64"]
    d = {k: _dpos(S, a, v) for k, v in out.items() if k != "fp64"}
    stable = d["fp64_1e-7"] <= 0.01
    res = {"vehicles": n, "horizon_s": horizon, "insensitive_at_1e-7": float(stable.mean()),
           "fp64_1e-15_within_1cm": float((d["fp64_1e-15"] <= 0.01).mean()),
           "ceiling_fp64_1e-15_retention": float((d["fp64_1e-15"][stable] <= 0.01).mean())}
    for _, key, _ in MIXED_FORMS:
        res[key + "_retention"] = float((d[key][stable] <= 0.01).mean())
        res[key + "_within_1cm"] = float((d[key] <= 0.01).mean())
    return res


def _model_rate(lfdm, fleet, dev, model: int, n: int, windows: int, ksim: float, peak_tflops: float) -> dict:
    """FP64 vehicle-steps/s of one model's window kernel on its seeded SUV fleet: `windows` timed
    windows of ksim seconds after one warm-up window (device time, CUDA events); then the same with
    the FP32 tire core (LFDM_PREC_MIXED_TIRE) and its end-of-horizon error against FP64."""
    gen = {11: fleet.fleet11, 18: fleet.fleet18, 24: fleet.fleet24}[model]
    cls_ = {11: lfdm.d11SolverHalfImplicitGPU, 18: lfdm.d18SolverHalfImplicitGPU, 24: lfdm.d24SolverHalfImplicitGPU}
    lay = {11: lfdm.S11, 18: lfdm.S, 24: lfdm.S24}[model]
    horizon = (windows + 1) * ksim
    f = gen(n, seed=SEED + model, horizon=horizon)
    out = {}
    for prec in (0, 2):
        sol = cls_[model](n, device=dev)
        sol.construct_class(f["cls"][0], f["params"])
        sol.set_driver_tables(f["tables"])
        sol.set_states(f["states"])
        sol.SetKernelSimTime(ksim)
        sol.SetEndTime(horizon)
        sol.set_precision(prec)
        sol.solve_range(-0.5 * ksim, 0.5 * ksim)
        sol.solve_range(0.5 * ksim, (windows + 0.5) * ksim)
        ms, launches = sol.last_kernel_ms()
        out[prec] = (ms, launches, sol.get_states())
        sol.close()
    ms, launches, st = out[0]
    finite = bool(np.isfinite(st[:, :8]).all())
    vsteps = n * int(round(ksim / 1e-3)) * windows
    rate = vsteps / (ms * 1e-3)
    achieved = W_ALG[model] * rate / 1e12
    tf_ms, _, tf_st = out[2]
    d = _dpos(lay, st, tf_st)
    return {"model": f"{model}dof-tmeasy", "vehicles": n, "value": rate, "unit": "vehicle-steps/s",
            "ms_per_window": ms / windows, "gpu_launches": launches, "finite_states": finite,
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak_tflops, "unit": "TFLOP/s",
                         "frac": achieved / peak_tflops,
                         "algorithmic": f"{W_ALG[model]} FP64 ops per vehicle-step (reference op count)"},
            "mixed_tire": {"value": vsteps / (tf_ms * 1e-3), "speedup_vs_fp64": ms / tf_ms,
                           "dtype": "f32 TMeasy tire core; f64 everything else",
                           "error_vs_fp64": {"horizon_s": horizon, "position_m": _stats(d),
                                             "frac_position_within_1cm": float((d <= 0.01).mean())}}}


def _fleet_bench(lfdm, fleet, dev, n: int, torch) -> dict:
    """The mixed-DOF fleet config: 60% 18-DOF / 40% 24-DOF, four mass classes +/-10%, end times
    log-uniform in [2, 20] s, dt 1e-3, kernel_sim_time 1 s, outputs every 0.1 s, one persistent
    launch (CUDA graph) with the autotuned configuration; against the same fleet solved the
    reference's way: one solver per (model, class, end-time window count) group, each launched
    window by window (the reference's m_tend is global to a solver)."""
    ksim, dtout = 1.0, 0.1
    mf = fleet.mixed_fleet(n, seed=SEED + 99, frac24=0.4, horizon_range=(2.0, 20.0), n_tables=4096)
    f = lfdm.Fleet(device=dev, dt=1e-3, kernel_sim_time=ksim, output_dt=dtout)
    base = f.add_rows(mf["rows"])
    for g in mf["groups"]:
        f.add(g["model"], g["cls"], g["params"], g["states"], g["horizons"], None, base + g["row_off"], g["row_len"])
    info = f.info()
    t0 = time.perf_counter()
    pilot_ms = f.tune(500)
    tune_s = time.perf_counter() - t0
    threads, bps, spl = f.get_launch()
    f.solve()
    ms, launches = f.last_ms()
    fp64_states = {m: f.get_states(m) for m in (18, 24)}
    finite = {m: bool(np.isfinite(fp64_states[m][:, :8]).all()) for m in (18, 24)}
    # the same solve from the same states with the other tile order than the tuner chose (model
    # affinity on or off)
    for m in (18, 24):
        f.set_states(m, np.concatenate([g["states"] for g in mf["groups"] if g["model"] == m]))
    tuned_aff, frac18 = f.get_affinity()
    f.set_affinity(not tuned_aff)
    f.solve()
    ms_other, _ = f.last_ms()
    f.close()
    ms_aff, ms_noaff = (ms, ms_other) if tuned_aff else (ms_other, ms)
    # the same fleet without response outputs: what the 0.1 s output schedule costs the launch
    f = lfdm.Fleet(device=dev, dt=1e-3, kernel_sim_time=ksim, output_dt=0.0)
    base = f.add_rows(mf["rows"])
    for g in mf["groups"]:
        f.add(g["model"], g["cls"], g["params"], g["states"], g["horizons"], None, base + g["row_off"], g["row_len"])
    f.set_launch(threads, bps, spl)
    f.set_affinity(tuned_aff)
    f.solve()
    ms_noout, _ = f.last_ms()
    f.close()
    # the same fleet and launch configuration with the FP32 tire core, against the FP64 solve
    f = lfdm.Fleet(device=dev, dt=1e-3, kernel_sim_time=ksim, output_dt=dtout)
    base = f.add_rows(mf["rows"])
    for g in mf["groups"]:
        f.add(g["model"], g["cls"], g["params"], g["states"], g["horizons"], None, base + g["row_off"], g["row_len"])
    f.set_launch(threads, bps, spl)
    f.set_affinity(tuned_aff)
    f.set_precision(2)
    f.solve()
    ms_tf, _ = f.last_ms()
    tf_err = {}
    for m in (18, 24):
        lay = lfdm.S if m == 18 else lfdm.S24
        d = _dpos(lay, fp64_states[m], f.get_states(m))
        tf_err[f"{m}dof_position_m"] = _stats(d)
        tf_err[f"{m}dof_frac_within_1cm"] = float((d <= 0.01).mean())
    f.close()
    vs = info["vehicle_steps"]
    # baseline: per-group solvers, kernel time summed over the groups
    base_ms, base_launches, groups = 0.0, 0, 0
    for g in mf["groups"]:
        m = g["model"]
        cls_ = lfdm.d18SolverHalfImplicitGPU if m == 18 else lfdm.d24SolverHalfImplicitGPU
        nch = lfdm.RESP18 if m == 18 else lfdm.RESP24
        wins = np.ceil(g["horizons"] / ksim - 1e-12).astype(int)
        for w in np.unique(wins):
            idx = np.nonzero(wins == w)[0]
            rows_w = int(round(w * ksim / 0.01)) + 1
            tabs = np.stack([mf["rows"][g["row_off"][i]: g["row_off"][i] + rows_w] for i in idx])
            sol = cls_(len(idx), device=dev)
            sol.construct_class(g["cls"], g["params"][idx])
            sol.set_driver_tables(tabs)
            sol.set_states(g["states"][idx])
            sol.SetKernelSimTime(ksim)
            sol.SetEndTime(w * ksim - 1e-9)
            spw = int(round(ksim / dtout))
            dbuf = torch.empty(2 * spw * nch * len(idx), dtype=torch.float64, device=f"cuda:{dev}")
            sol.set_response_device(dbuf.data_ptr(), dbuf.numel(), 1.0 / dtout)
            sol.Solve()
            gms, gl = sol.last_kernel_ms()
            base_ms += gms
            base_launches += gl
            groups += 1
            sol.close()
            del dbuf
    value = vs / (ms * 1e-3)
    base_value = vs / (base_ms * 1e-3)
    return {"config": "mixed fleet: 60% 18-DOF / 40% 24-DOF (ks 4e4 N/m, bs 4e3 N s/m), classes 1300/1700/2100/"
                      "2800 kg +/-10%, end times log-uniform [2, 20] s, dt 1e-3 s, kernel_sim_time 1 s, outputs "
                      "every 0.1 s to device memory, 4,096 shared seeded driver tables",
            "vehicles": n, "n18": info["n18"], "n24": info["n24"], "vehicle_steps": vs, "dtype": "f64",
            "value": value, "unit": "vehicle-steps/s", "ms": ms, "gpu_launches": launches,
            "launch": {"threads": threads, "blocks_per_sm": bps or "max", "steps_per_launch": spl or "all",
                       "tuned_on": "first 500 steps", "pilot_ms": pilot_ms, "tune_wall_s": tune_s},
            "baseline_per_group": {"value": base_value, "unit": "vehicle-steps/s", "ms": base_ms,
                                   "solver_runs": groups, "gpu_launches": base_launches,
                                   "what": "one window-kernel solver per (model, class, window count), "
                                           "kernel time summed"},
            "speedup_vs_per_group": value / base_value, "finite_states": finite,
            "model_affinity": {"tuned": bool(tuned_aff), "frac18_of_work": frac18, "ms_with": ms_aff,
                               "ms_without": ms_noaff, "speedup": ms_noaff / ms_aff,
                               "what": "SMs split between the 18-DOF and 24-DOF tile lists in proportion to their "
                                       "estimated work, against one list of both models' tiles by estimated cost"},
            "mixed_tire": {"value": vs / (ms_tf * 1e-3), "unit": "vehicle-steps/s", "ms": ms_tf,
                           "speedup_vs_fp64": ms / ms_tf, "error_vs_fp64_end_of_horizon": tf_err,
                           "dtype": "f32 TMeasy tire core; f64 everything else"},
            "outputs": {"ms_with_0.1s_outputs": ms, "ms_without_outputs": ms_noout, "cost_frac": ms / ms_noout - 1.0,
                        "what": "the same fleet and launch configuration with no response buffer"}}


def _adjoint_bench(lfdm, fleet, dev, n: int, nsteps: int, torch) -> dict:
    """The differentiable-rollout config: 18-DOF FP64, n vehicles, nsteps steps of 1e-3 s, a
    checkpoint every 100 steps, seeded clothoid reference paths (curvature U[-0.05, 0.05] 1/m, speed
    U[5, 25] m/s), loss = squared lateral + heading error + 1e-3 |u|^2; gradients with respect to
    the per-step controls and 5 parameters; one forward and one backward, CUDA-event timed."""
    rng = np.random.default_rng(SEED + 4)
    dt = 1e-3
    cls, base = fleet.suv18()
    params = fleet.jitter_params(base, n, rng)
    ref, v = fleet.clothoid_refs(n, nsteps, dt, rng)
    sol = lfdm.d18SolverHalfImplicitGPU(n, device=dev)
    sol.construct_class(cls, params)
    sol.set_states(fleet.states_at_speed(cls, params, v))
    sol.SetTimeStep(dt)
    gdev = torch.device("cuda", dev)
    t = np.arange(nsteps) * dt
    ctl = np.zeros((nsteps, 3, n))
    ctl[:, 0, :] = rng.uniform(-0.08, 0.08, n)[None, :] * np.sin(2 * np.pi * rng.uniform(0.5, 2.0, n)[None, :]
                                                                 * t[:, None])
    ctl[:, 1, :] = rng.uniform(0.2, 0.5, n)[None, :]
    c = torch.tensor(ctl, dtype=torch.float64, device=gdev)
    r = torch.tensor(ref, dtype=torch.float64, device=gdev)
    del ctl, ref
    ro = lfdm.Rollout18(sol, nsteps, ckpt_every=100)
    loss = torch.empty(n, dtype=torch.float64, device=gdev)
    gc = torch.empty_like(c)
    gp = torch.empty(5, n, dtype=torch.float64, device=gdev)
    # one untimed pass (module load, buffer allocation), then the measured pass
    for _ in range(2):
        ro.forward_raw(c, r, loss)
        ro.backward_raw(c, r, gc, gp)
    fwd, bwd = ro.last_ms()
    finite = bool(torch.isfinite(gc).all().item() and torch.isfinite(gp).all().item())
    sol.close()
    vs = n * nsteps
    return {"config": f"18-DOF FP64 adjoint, {n} vehicles, {nsteps} steps (dt 1e-3 s), checkpoint every 100 "
                      "steps, clothoid reference paths, gradients for 3 x nsteps controls and 5 parameters",
            "forward_ms": fwd, "backward_ms": bwd, "backward_over_forward": bwd / fwd,
            "forward_vehicle_steps_per_s": vs / (fwd * 1e-3), "gradients_finite": finite,
            "checked": "tests/test_gpu_adjoint18.py: central differences h=1e-6 of the GPU rollout and of the "
                       "reference algorithm (oracle)"}


def _jacobian_bench(lfdm, fleet, dev, n: int, cpu_sample: int, torch) -> dict:
    """Right-hand-side Jacobians of every vehicle of the seeded 11/18/24-DOF SUV fleets after 1 s of
    their drivers (TMeasy, torque converter): the reference's difference scheme
    (lfdm_rhs_jacobian_fd; 2 ny + 4 right-hand sides per vehicle) and the exact Jacobian
    (lfdm_rhs_jacobian_exact). Each figure is the host wall time of the C-ABI call (it
    returns after its stream synchronizes), best of 3 after one untimed call. Beside them, the same
    scheme on all host cores over the same vehicles: the oracle's restatement of
    IntegrateStepWithJacobian's Jacobian block, pinned bit for bit to the reference's CPU solvers."""
    import ctypes

    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    gdev = torch.device("cuda", dev)
    rng = np.random.default_rng(SEED + 5)
    out = {"config": f"{n} vehicles per model, seeded SUV fleets after 1 s of their drivers, controls "
                     "steering U[-0.3, 0.3], throttle U[0, 1], braking 0; reference point (fresh state)",
           "timing": "host wall time of the C-ABI call (returns after its stream synchronizes), best of 3"}
    cores = os.cpu_count() or 1
    for model, make in ((11, fleet.fleet11), (18, fleet.fleet18), (24, fleet.fleet24)):
        f = make(n, seed=SEED + 5, horizon=2.0)
        sol = getattr(lfdm, f"d{model}SolverHalfImplicitGPU")(n, device=dev)
        sol.construct_class(f["cls"][0], f["params"])
        sol.set_driver_tables(f["tables"])
        sol.set_states(f["states"])
        sol.SetKernelSimTime(1.0)
        sol.SetEndTime(1.0)
        sol.Solve()
        ctl_h = np.stack([rng.uniform(-0.3, 0.3, n), rng.uniform(0.0, 1.0, n), np.zeros(n)])
        ctl = torch.tensor(ctl_h, dtype=torch.float64, device=gdev)
        js = torch.empty(36 * 36 * n, dtype=torch.float64, device=gdev)
        ju = torch.empty(36 * 2 * n, dtype=torch.float64, device=gdev)
        ny = ctypes.c_int()
        fns = [("fd", sol._L.lfdm_rhs_jacobian_fd), ("exact", sol._L.lfdm_rhs_jacobian_exact)]
        for name, fn in fns:
            def call():
                t0 = time.perf_counter()
                rc = fn(sol._h, ctypes.c_void_p(ctl.data_ptr()), 1, ctypes.c_void_p(js.data_ptr()),
                        ctypes.c_void_p(ju.data_ptr()), ctypes.byref(ny))
                if rc:
                    raise RuntimeError(f"{name} Jacobian failed: {rc}")
                return time.perf_counter() - t0
            call()
            best = min(call() for _ in range(3))
            out[f"{model}dof_{name}"] = {"ms": best * 1e3, "jacobians_per_s": n / best, "ny": ny.value,
                                         "finite": bool(torch.isfinite(js[: ny.value ** 2 * n]).all().item())}
        # the reference's scheme on the host cores (a bounded sample)
        m = min(cpu_sample, n)
        states = sol.get_states(0, m)
        sol.close()
        t0 = time.perf_counter()
        oracle_lib.jacobian_fd_batch(model, 0, f["cls"][0], f["params"][:m], states, ctl_h[:, :m], nthreads=cores)
        secs = time.perf_counter() - t0
        out[f"{model}dof_fd"]["cpu_reference_scheme"] = {
            "jacobians_per_s": m / secs, "cores": cores, "kind": "port",
            "sample": f"{m} vehicles ({secs:.2f} s wall), oracle_jacobian_fd_batch (oracle/lfdm_oracle.c) on "
                      "all host cores"}
        out[f"{model}dof_fd"]["speedup_vs_cpu"] = out[f"{model}dof_fd"]["jacobians_per_s"] / (m / secs)
    return out


def _reference_gpu_bench(fleet, model: int, n: int, windows: int, ksim: float, ours: float) -> dict:
    """The reference's OWN GPU solver (its Integrate kernel compiled from the reference sources into
    oracle/_ref/ref<model>.cubin, driven window by window as its Solve() does, with its managed AoS
    records) on the seeded SUV fleet of the model with outputs every 10 ms: windows 2..windows timed
    with CUDA events, at 16 and 32 threads per block (its best counts). ratio = ours / best."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import refgpu_lib
    if not refgpu_lib.available(model):
        return {"unavailable": f"oracle/_ref/ref{model}.cubin was not built (it is built where the reference "
                               "checkout exists)"}
    refgpu_lib.build_launcher()
    gen = {11: fleet.fleet11, 18: fleet.fleet18, 24: fleet.fleet24}[model]
    f = gen(n, seed=SEED + model, horizon=windows * ksim)
    out = {"vehicles": n, "windows_timed": windows - 1, "window_s": ksim, "output_hz": 100}
    best = 0.0
    for tpb in (16, 32):
        _, ms = refgpu_lib.run(f["cls"][0], f["params"], f["tables"], f["states"], model=model, ksim=ksim,
                               tend=windows * ksim, dtout=0.01, tpb=tpb)
        rate = n * int(round(ksim / 1e-3)) * (windows - 1) / (sum(ms[1:]) * 1e-3)
        out[f"tpb{tpb}"] = {"value": rate, "unit": "vehicle-steps/s", "ms_per_window": sum(ms[1:]) / (windows - 1)}
        best = max(best, rate)
    out["best"] = best
    out["ours"] = ours
    out["ratio"] = ours / best
    return out


def run_ours(a, dist: Dist):
    import torch

    lfdm = importlib.import_module(PKG)
    fleet = importlib.import_module(PKG + ".fleet")
    dev = dist.local if torch.cuda.device_count() > dist.local else 0
    torch.cuda.set_device(dev)
    n, K, W, ksim = a.vehicles, a.steps, a.warmup, a.ksim
    horizon = (W + K) * ksim
    steps_per_window = int(round(ksim / 1e-3))
    f = fleet.fleet18(n, seed=SEED + dist.rank, horizon=horizon)

    sol = lfdm.d18SolverHalfImplicitGPU(n, device=dev)
    sol.construct_class(f["cls"][0], f["params"])
    sol.set_driver_tables(f["tables"])
    sol.set_states(f["states"])
    sol.SetKernelSimTime(ksim)
    sol.SetEndTime(horizon)
    if a.threads:
        sol.SetThreadsPerBlock(a.threads)
    spw = int(np.ceil(ksim * 100.0 - 1e-9))
    per_window = spw * lfdm.RESP18 * n
    dresp = torch.empty(2 * per_window, dtype=torch.float64, device=f"cuda:{dev}")
    sol.set_response_device(dresp.data_ptr(), dresp.numel(), 100.0)

    # warm-up windows, then K timed windows (device time of the window kernels, CUDA events)
    sol.solve_range(-0.5 * ksim, (W - 0.5) * ksim)
    torch.cuda.synchronize()
    dist.barrier()
    clk = ClockSampler(dev)
    clk.start()
    wall0 = time.perf_counter()
    sol.solve_range((W - 0.5) * ksim, (W + K - 0.5) * ksim)
    wall = time.perf_counter() - wall0
    kms, launches = sol.last_kernel_ms()
    clocks = clk.stop()
    torch.cuda.synchronize()
    dist.barrier()
    kms_max = dist.max(kms)
    vsteps_rank = n * steps_per_window * K
    total_vsteps = dist.sum(vsteps_rank)
    value = total_vsteps / (kms_max * 1e-3)
    final = sol.get_states()
    finite = bool(np.isfinite(final[:, :15]).all())

    # e2e through the C ABI with host buffers: per step, H2D of that window's table rows from
    # page-locked memory and D2H of the window's response into page-locked memory
    e2e = None
    if not a.no_e2e:
        rows_pw = int(round(ksim / 0.01)) + 1
        win_tabs = np.empty((W + K, n, rows_pw, 4))
        for w in range(W + K):
            win_tabs[w] = f["tables"][:, w * (rows_pw - 1): w * (rows_pw - 1) + rows_pw, :]
        host_resp = np.empty(2 * per_window)
        lfdm.register_host(win_tabs)
        lfdm.register_host(host_resp)
        sol.set_response_device(None)
        sol.set_states(f["states"])
        sol.set_response_buffer(host_resp, 100.0)
        for w in range(W):
            sol.set_driver_tables(win_tabs[w])
            sol.solve_range((w - 0.5) * ksim, (w + 0.5) * ksim)
        dist.barrier()
        t0 = time.perf_counter()
        for w in range(W, W + K):
            sol.set_driver_tables(win_tabs[w])
            sol.solve_range((w - 0.5) * ksim, (w + 0.5) * ksim)
        e2e_wall = dist.max(time.perf_counter() - t0)
        lfdm.unregister_host(win_tabs)
        lfdm.unregister_host(host_resp)
        e2e = {"value": total_vsteps / e2e_wall, "unit": "vehicle-steps/s",
               "h2d_bytes_per_step": int(win_tabs[0].nbytes), "d2h_bytes_per_step": int(per_window * 8),
               "ms_per_step": 1e3 * e2e_wall / K}

    # mixed precision: throughput of both forms on the same fleet and windows, accuracy against the
    # FP64 path (the precision config at 1,000,000 vehicles) and against the fleet's own sensitivity
    mixed = None
    peak_ffma, probe32_ghz = (lfdm.measure_fp32_peak_clock(dev) if not a.no_mixed else (None, None))
    if not a.no_mixed:
        mixed = {}
        for prec, key, arith in MIXED_FORMS:
            solm = lfdm.d18SolverHalfImplicitGPU(n, device=dev)
            solm.construct_class(f["cls"][0], f["params"])
            solm.set_driver_tables(f["tables"])
            solm.set_states(f["states"])
            solm.SetKernelSimTime(ksim)
            solm.SetEndTime(horizon)
            solm.set_precision(prec)
            if a.threads:
                solm.SetThreadsPerBlock(a.threads)
            solm.set_response_device(dresp.data_ptr(), dresp.numel(), 100.0)
            solm.solve_range(-0.5 * ksim, (W - 0.5) * ksim)
            torch.cuda.synchronize()
            solm.solve_range((W - 0.5) * ksim, (W + K - 0.5) * ksim)
            mms, mlaunch = solm.last_kernel_ms()
            solm.close()
            mvalue = dist.sum(vsteps_rank) / (dist.max(mms) * 1e-3)
            mixed[key] = {"precision": prec, "value": mvalue, "unit": "vehicle-steps/s",
                          "speedup_vs_fp64": mvalue / value, "ms_per_step": mms / K, "gpu_launches": mlaunch,
                          "dtype": arith}
        if a.error_vehicles > 0:
            mixed["error_vs_fp64"] = _mixed_error(lfdm, fleet, dev, a.error_vehicles, a.error_horizon)
        if a.ceiling_vehicles > 0:
            mixed["retention"] = _mixed_retention(lfdm, fleet, dev, a.ceiling_vehicles, a.error_horizon)
    peak_dfma, probe_ghz = lfdm.measure_fp64_peak_clock(dev)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    max_ghz = (clocks.get("sm_max_mhz") or 2070.0) / 1e3
    if mixed:
        # issue roofline of each mixed form: its FP32 and FP64 thread-instructions per second against
        # the FFMA and DFMA probes (separate pipes, so the larger fraction is the bound)
        for prec, key, _ in MIXED_FORMS:
            m, inst = mixed[key], MIXED_INST_PER_VSTEP.get(prec)
            if inst is None:
                m["roofline"] = None
                continue
            f32, f64 = inst[0] * m["value"] / peak_ffma, inst[1] * m["value"] / peak_dfma
            fp32_bound = f32 >= f64
            m["roofline"] = {
                "bound": "fp32 issue" if fp32_bound else "fp64 issue",
                "achieved": (inst[0] if fp32_bound else inst[1]) * m["value"],
                "peak": peak_ffma if fp32_bound else peak_dfma, "unit": "thread-instructions/s",
                "frac": max(f32, f64), "fp32_frac": f32, "fp64_frac": f64,
                "inst_per_vehicle_step": {"fp32": inst[0], "fp64": inst[1]},
                "peak_source": "measured live: FFMA and DFMA throughput kernels (lfdm_measure_fp32_peak_clock, "
                               "lfdm_measure_fp64_peak_clock)",
                "probe_fp32_sm_ghz": probe32_ghz, "probe_fp64_sm_ghz": probe_ghz,
                "inst_source": "ncu sm__inst_executed_pipe_fma.sum and sm__inst_executed_pipe_fp64.sum x 32 of "
                               "one window launch on 32,768 vehicles, per vehicle-step",
                "peak_nominal_fp64_per_s": 2 * sms * max_ghz * 1e9,
                "fp64_frac_nominal": inst[1] * m["value"] / (2 * sms * max_ghz * 1e9)}
    # nominal FP64 rate: one warp-wide DFMA per 64 cycles per SM sub-partition = 2 DFMA/clock/SM
    peak_nominal = 2 * 2.0 * sms * max_ghz * 1e9 / 1e12
    launch_ms = kms / launches
    alg_flop = W_ALG_18 * n * steps_per_window
    achieved = alg_flop / (launch_ms * 1e-3) / 1e12
    peak = 2 * peak_dfma / 1e12
    # HBM view of the same kernel: algorithmic bytes per window (state in/out, constants, the
    # window's table rows, the response written)
    alg_bytes = n * (2 * 75 * 8 + 70 * 8 + (rows_w := int(round(ksim / 0.01)) + 1) * 32 + spw * 13 * 8)
    # DRAM bytes of one window launch (dram__bytes_read.sum + dram__bytes_write.sum) from one ncu
    # capture of this default configuration (300,000 vehicles, 1 s windows, 100 Hz outputs); other
    # configurations have no capture and report null
    traffic = 1687990272 + 3257568768 if (n == 300_000 and ksim == 1.0 and spw == 100) else None
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            peaks = json.load(fh)
    except OSError:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)

    # the other two models: the 11-DOF small config (1,024 vehicles, 10 s) and 11/24-DOF at scale
    models = None
    if not a.no_models:
        c0 = _model_rate(lfdm, fleet, dev, 11, 1024, 9, 1.0, peak)
        c0["config"] = "11-DOF SUV, one parameter set, 1,024 vehicles, 10 s (1 warm-up + 9 timed 1 s windows)"
        models = {"11dof_1024": c0,
                  "11dof_scale": _model_rate(lfdm, fleet, dev, 11, n, 2, ksim, peak),
                  "24dof_scale": _model_rate(lfdm, fleet, dev, 24, n, 2, ksim, peak)}
        models["24dof_scale"]["config"] = "24-DOF SUV fleet (ks 4e4 N/m, bs 4e3 N s/m), jittered as the 18-DOF fleet"
    # the reference's own GPU solver on this GPU: 18-DOF on the bench fleet's size, and the 11-DOF
    # small config and the 24-DOF model at scale beside this library's lines above
    ref_gpu = None
    if not a.no_reference_gpu and dist.rank == 0:
        ref_gpu = {"18dof": _reference_gpu_bench(fleet, 18, n, 3, ksim, value)}
        if models:
            ref_gpu["11dof_1024"] = _reference_gpu_bench(fleet, 11, 1024, 10, 1.0, models["11dof_1024"]["value"])
            ref_gpu["24dof_scale"] = _reference_gpu_bench(fleet, 24, n, 3, ksim, models["24dof_scale"]["value"])
    fleet_line = None
    if not a.no_fleet:
        fleet_line = _fleet_bench(lfdm, fleet, dev, a.fleet_vehicles, torch)
    adjoint_line = None
    if not a.no_adjoint:
        adjoint_line = _adjoint_bench(lfdm, fleet, dev, a.adjoint_vehicles, 2000, torch)
    jacobian_line = None
    if not a.no_jacobian and dist.rank == 0:
        jacobian_line = _jacobian_bench(lfdm, fleet, dev, a.jacobian_vehicles, a.jacobian_vehicles, torch)

    cpu = None
    if dist.rank == 0 and a.cpu_sample > 0:
        cores = os.cpu_count() or 1
        m = min(a.cpu_sample, n)
        traj = CpuTrajectory(f, m, ksim, cores)
        traj.window()  # warm-up: window 0
        secs = sum(traj.window() for _ in range(3))
        rate = m * steps_per_window * 3 / secs
        cpu = {"value": rate, "unit": "vehicle-steps/s", "cores": cores, "kind": "port",
               "sample": f"{m} vehicles of the fleet x windows 1-3 ({3 * steps_per_window} steps, {secs:.1f} s "
                         "wall) after window 0, trajectories continued; oracle/lfdm_oracle.c (the reference's CPU "
                         "algorithm restated) built with the reference's Release flags (-O3), all host cores"}
        if models:
            f11 = fleet.fleet11(1024, seed=SEED + 11, horizon=10.0)
            t11 = CpuTrajectory(f11, 1024, 1.0, cores, model=11)
            secs11 = sum(t11.window() for _ in range(10))
            models["11dof_1024"]["cpu_baseline"] = {
                "value": 1024 * 10000 / secs11, "unit": "vehicle-steps/s", "cores": cores, "kind": "port",
                "sample": f"the whole config: 1,024 vehicles x 10 s ({secs11:.2f} s wall), the 11-DOF oracle "
                          "restatement (-O3), all host cores"}
            models["11dof_1024"]["speedup_vs_cpu"] = models["11dof_1024"]["value"] / models["11dof_1024"]["cpu_baseline"]["value"]
    if dist.rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "vehicle-steps/s", "n_gpus": dist.world, "steps": K,
            "warmup": W, "ms_per_step": kms_max / K, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded SUV fleet; see config)",
            "config": dict(_config(a), parallelism=f"replicas x{dist.world}" if dist.world > 1 else "1 GPU"),
            "rtf": (kms_max * 1e-3) / (K * ksim),
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "traffic_source": "constant: one ncu capture of this configuration (dram__bytes_read.sum "
                                           "+ dram__bytes_write.sum of one window launch), not measured in this run",
                         "peak_source": "measured live: DFMA throughput kernel (lfdm_measure_fp64_peak_clock), "
                                        "x2 flop/FMA; MEASURED_PEAKS.json has no FP64 figure",
                         "probe_sm_ghz": probe_ghz,
                         "probe_dfma_per_clk_per_sm": peak_dfma / (sms * probe_ghz * 1e9) if probe_ghz else None,
                         "peak_nominal": peak_nominal, "frac_nominal": achieved / peak_nominal,
                         "peak_nominal_source": f"2 DFMA/clock/SM x {sms} SMs x {max_ghz:.3f} GHz (max SM clock) x 2",
                         "issue_view": {
                             "fp64_arith_inst_per_vehicle_step": FP64_INST_PER_VSTEP_18,
                             "fp64_pipe_inst_per_vehicle_step": FP64_PIPE_PER_VSTEP_18,
                             "source": "ncu sm__sass_thread_inst_executed_op_{dfma,dmul,dadd}_pred_on.sum and "
                                       "sm__inst_executed_pipe_fp64.sum x 32 per vehicle-step of one window launch "
                                       "(32,768 vehicles), one capture",
                             "frac": FP64_PIPE_PER_VSTEP_18 * value / peak_dfma,
                             "frac_nominal": FP64_PIPE_PER_VSTEP_18 * value / (peak_nominal * 1e12 / 2),
                             "arith_frac_nominal": FP64_INST_PER_VSTEP_18 * value / (peak_nominal * 1e12 / 2)},
                         "algorithmic": f"{W_ALG_18} FP64 ops per vehicle-step (reference op count) x "
                                        f"{n * steps_per_window} vehicle-steps per launch"},
            "roofline_hbm": {"bound": "hbm", "achieved": alg_bytes / (launch_ms * 1e-3) / 1e9, "peak": hbm_peak,
                             "unit": "GB/s", "frac": alg_bytes / (launch_ms * 1e-3) / 1e9 / hbm_peak,
                             "traffic": traffic, "algorithmic_bytes": alg_bytes,
                             "peak_source": "MEASURED_PEAKS.json hbm_gbs"},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "mixed": mixed,
            "models": models,
            "reference_gpu": ref_gpu,
            "fleet": fleet_line,
            "adjoint": adjoint_line,
            "jacobian": jacobian_line,
            "gpu_launches": launches,
            "clocks": clocks,
            "wall_s_timed": wall,
            "finite_states": finite,
        }
        print(json.dumps(line), flush=True)
    sol.close()


def main():
    a = _args()
    dist = Dist(a.gpus)
    if a.impl == "reference":
        run_reference(a, dist)
    else:
        run_ours(a, dist)
    if dist.pg:
        dist.pg.destroy_process_group()


if __name__ == "__main__":
    main()
