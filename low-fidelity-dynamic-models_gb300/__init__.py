"""GB300-native batched half-implicit stepper for the 11/18/24-DOF wheeled-vehicle models.

Python binding of the C ABI in include/lfdm.h (library: _build/liblfdm.so, built by build.py).
`d18SolverHalfImplicitGPU` mirrors the reference class of the same name
(18dof-gpu/dof18_halfImplicit_gpu.cuh:15-343): Construct, Initialize, SetTimeStep, SetEndTime,
SetKernelSimTime, SetHostDumpTime, SetThreadsPerBlock, SetOutput, Solve, SolveStep, GetSimState.
The extensions take numpy arrays: per-vehicle parameters, driver tables and states, per-vehicle
SolveStep controls, and a streamed SoA response buffer.

There is no CPU fallback: loading the library or creating a solver without a CUDA device raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _abi
from ._abi import (Class18, P, P_COUNT, S, S_COUNT, T, S_TIRE0, S_TIRE_STRIDE, RESP18, S11, S11_COUNT, S11_TIRE0,
                   RESP11, S24, S24_COUNT, RESP24)

__all__ = ["lib", "LfdmError", "d18SolverHalfImplicitGPU", "d11SolverHalfImplicitGPU", "TireType", "Class18", "P",
           "S", "T", "S_COUNT", "P_COUNT", "RESP18", "S_TIRE0", "S_TIRE_STRIDE", "S11", "S11_COUNT", "S11_TIRE0",
           "RESP11", "d24SolverHalfImplicitGPU", "S24", "S24_COUNT", "RESP24", "Fleet", "Rollout18",
           "ROLLOUT_PARAMS"]

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "liblfdm.so")


class LfdmError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{_abi.STATUS.get(code, code)}: {msg}")
        self.code = code


class TireType:
    TMeasy = _abi.TIRE_TMEASY
    TMeasyNr = _abi.TIRE_TMEASY_NR


_lib = None
_c_dp = ctypes.POINTER(ctypes.c_double)


def _sig(lib):
    vp, u, i, d, dp, sz = ctypes.c_void_p, ctypes.c_uint, ctypes.c_int, ctypes.c_double, ctypes.c_void_p, ctypes.c_size_t
    cp = ctypes.c_char_p
    table = {
        "lfdm_create": ([i, u, ctypes.POINTER(vp)], i),
        "lfdm_create_on_device": ([i, u, i, ctypes.POINTER(vp)], i),
        "lfdm_destroy": ([vp], i),
        "lfdm_last_error": ([vp], cp),
        "lfdm_construct": ([vp, cp, cp, cp, u, cp, i], i),
        "lfdm_construct_class": ([vp, vp, u, dp, i], i),
        "lfdm_set_params": ([vp, u, u, dp], i),
        "lfdm_get_params": ([vp, u, u, dp], i),
        "lfdm_tire_init": ([dp], i),
        "lfdm_set_driver_table": ([vp, u, u, dp, u], i),
        "lfdm_set_driver_tables": ([vp, u, u, dp, u], i),
        "lfdm_initialize": ([vp, dp, u], i),
        "lfdm_set_states": ([vp, u, u, dp], i),
        "lfdm_get_states": ([vp, u, u, dp], i),
        "lfdm_set_time_step": ([vp, d], i),
        "lfdm_set_end_time": ([vp, d], i),
        "lfdm_set_kernel_sim_time": ([vp, d], i),
        "lfdm_set_host_dump_time": ([vp, d], i),
        "lfdm_set_threads_per_block": ([vp, u], i),
        "lfdm_get_step": ([vp, _c_dp], i),
        "lfdm_get_end_time": ([vp, _c_dp], i),
        "lfdm_get_tire_type": ([vp, ctypes.POINTER(i)], i),
        "lfdm_get_num_vehicles": ([vp, ctypes.POINTER(u), ctypes.POINTER(u), ctypes.POINTER(u)], i),
        "lfdm_set_precision": ([vp, i], i),
        "lfdm_set_output": ([vp, cp, d, i, u], i),
        "lfdm_set_response_buffer": ([vp, dp, sz, d], i),
        "lfdm_response_samples": ([vp, ctypes.POINTER(sz)], i),
        "lfdm_register_host": ([vp, sz], i),
        "lfdm_unregister_host": ([vp], i),
        "lfdm_solve": ([vp], i),
        "lfdm_solve_step": ([vp, d, d, d, d, _c_dp], i),
        "lfdm_solve_step_controls": ([vp, d, dp, dp, dp, _c_dp], i),
        "lfdm_solve_step_schedule": ([vp, d, dp, u, i, _c_dp], i),
        "lfdm_window_steps": ([vp, d, ctypes.POINTER(u), dp, u], i),
        "lfdm_get_sim_state": ([vp, u, dp], i),
        "lfdm_get_status_words": ([vp, u, u, dp], i),
        "lfdm_last_kernel_ms": ([vp, _c_dp, ctypes.POINTER(u)], i),
        "lfdm_version": ([], cp),
        "lfdm_set_response_device": ([vp, vp, sz, d], i),
        "lfdm_solve_range": ([vp, d, d], i),
        "lfdm_measure_fp64_peak": ([i, _c_dp], i),
        "lfdm_set_split_warps": ([vp, i], i),
        "lfdm_measure_fp64_peak_clock": ([i, _c_dp, _c_dp], i),
        "lfdm_measure_fp32_peak_clock": ([i, _c_dp, _c_dp], i),
        "lfdm_parse_vehicle18": ([cp, cp, i, vp, dp, ctypes.c_char_p, sz], i),
        "lfdm_parse_vehicle": ([i, cp, cp, cp, i, vp, dp, ctypes.c_char_p, sz], i),
        "lfdm_load_driver_file": ([cp, dp, u, ctypes.POINTER(u), ctypes.c_char_p, sz], i),
        "lfdm_step18_noalloc": ([vp, i, vp, vp, vp, vp, vp, u, d, d, u, vp, ctypes.c_char_p, sz], i),
        "lfdm_traj18_forward": ([vp, vp, vp, u, d, u, vp], i),
        "lfdm_traj18_backward": ([vp, vp, vp, u, d, u, vp, vp, vp], i),
        "lfdm_traj18_last_ms": ([vp, _c_dp, _c_dp], i),
        "lfdm_traj18_branch_signature": ([vp, vp, u, vp], i),
        "lfdm_rhs_jacobian18": ([vp, vp, i, vp, vp, ctypes.POINTER(i)], i),
        "lfdm_rhs_jacobian_exact": ([vp, vp, i, vp, vp, ctypes.POINTER(i)], i),
        "lfdm_rhs_jacobian_fd": ([vp, vp, i, vp, vp, ctypes.POINTER(i)], i),
        "lfdm_rhs_jacobian_host": ([vp, i, vp, i, vp, vp, ctypes.POINTER(i)], i),
        "lfdm_fleet_create": ([i, ctypes.POINTER(vp)], i),
        "lfdm_fleet_destroy": ([vp], i),
        "lfdm_fleet_last_error": ([vp], cp),
        "lfdm_fleet_add": ([vp, i, vp, u, dp, dp, dp, dp, sz, vp, vp], i),
        "lfdm_fleet_add_rows": ([vp, dp, sz, ctypes.POINTER(ctypes.c_int64)], i),
        "lfdm_fleet_set_time_step": ([vp, d], i),
        "lfdm_fleet_set_kernel_sim_time": ([vp, d], i),
        "lfdm_fleet_set_output": ([vp, d], i),
        "lfdm_fleet_set_launch": ([vp, u, u, u], i),
        "lfdm_fleet_get_launch": ([vp, ctypes.POINTER(u), ctypes.POINTER(u), ctypes.POINTER(u)], i),
        "lfdm_fleet_set_affinity": ([vp, i], i),
        "lfdm_fleet_set_precision": ([vp, i], i),
        "lfdm_fleet_get_affinity": ([vp, ctypes.POINTER(i), _c_dp], i),
        "lfdm_fleet_tune": ([vp, u, _c_dp], i),
        "lfdm_fleet_solve": ([vp], i),
        "lfdm_fleet_last_ms": ([vp, _c_dp, ctypes.POINTER(u)], i),
        "lfdm_fleet_info": ([vp, ctypes.POINTER(u), ctypes.POINTER(u), ctypes.POINTER(ctypes.c_longlong), _c_dp,
                             ctypes.POINTER(u)], i),
        "lfdm_fleet_get_states": ([vp, i, u, u, dp], i),
        "lfdm_fleet_set_states": ([vp, i, u, u, dp], i),
        "lfdm_fleet_get_response": ([vp, i, dp, sz, ctypes.POINTER(u)], i),
        "lfdm_fleet_get_status_words": ([vp, i, dp], i),
    }
    for name, (args, res) in table.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    return lib


def lib():
    """The loaded C-ABI library. Raises when it has not been built (no silent fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; "
                               "g.build()'` (needs nvcc)")
        _lib = _sig(ctypes.CDLL(LIB_PATH))
    return _lib


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None:
        a = a.reshape(shape)
    return a


def parse_vehicle18(veh_json: str, tire_json: str, tire_type: int = TireType.TMeasy):
    """The library's own JSON loader (host only): returns (Class18, params[P_COUNT])."""
    c = Class18()
    p = np.zeros(P_COUNT)
    err = ctypes.create_string_buffer(512)
    rc = lib().lfdm_parse_vehicle18(veh_json.encode(), tire_json.encode(), tire_type, ctypes.byref(c), _ptr(p),
                                    err, 512)
    if rc:
        raise LfdmError(rc, err.value.decode())
    return c, p


def parse_vehicle(model: int, veh_json: str, tire_json: str, sus_json: str | None = None,
                  tire_type: int = TireType.TMeasy):
    """The library's loader for any model (11, 18, or 24 with its suspension JSON)."""
    c = Class18()
    p = np.zeros(P_COUNT)
    err = ctypes.create_string_buffer(512)
    rc = lib().lfdm_parse_vehicle(int(model), veh_json.encode(), tire_json.encode(),
                                  sus_json.encode() if sus_json else None, tire_type, ctypes.byref(c), _ptr(p), err, 512)
    if rc:
        raise LfdmError(rc, err.value.decode())
    return c, p


def load_driver_file(path: str) -> np.ndarray:
    n = ctypes.c_uint()
    err = ctypes.create_string_buffer(512)
    rc = lib().lfdm_load_driver_file(path.encode(), None, 0, ctypes.byref(n), err, 512)
    if rc:
        raise LfdmError(rc, err.value.decode())
    rows = np.zeros((n.value, 4))
    rc = lib().lfdm_load_driver_file(path.encode(), _ptr(rows), n.value, ctypes.byref(n), err, 512)
    if rc:
        raise LfdmError(rc, err.value.decode())
    return rows


class _SolverGPU:
    """Batched half-implicit stepper on one GPU; the model is fixed by the subclass."""

    MODEL = 18
    STATE_COUNT = S_COUNT
    RESP_CHANNELS = RESP18

    def __init__(self, total_num_vehicles: int, device: int = 0):
        self._L = lib()
        h = ctypes.c_void_p()
        rc = self._L.lfdm_create_on_device(self.MODEL, int(total_num_vehicles), int(device), ctypes.byref(h))
        if rc:
            raise LfdmError(rc, self._L.lfdm_last_error(None).decode())
        self._h = h
        self.n = int(total_num_vehicles)
        self.device = int(device)

    # -- plumbing -----------------------------------------------------------------------------
    def _ck(self, rc: int):
        if rc:
            raise LfdmError(rc, self._L.lfdm_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._L.lfdm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- reference API --------------------------------------------------------------------------
    def Construct(self, vehicle_params_file: str, tire_params_file: str, num_vehicles: int,
                  driver_inputs_file: str | None = None, type: int = TireType.TMeasy):  # noqa: A002
        self._ck(self._L.lfdm_construct(self._h, vehicle_params_file.encode(), tire_params_file.encode(), None,
                                        int(num_vehicles),
                                        driver_inputs_file.encode() if driver_inputs_file else None, int(type)))

    def Initialize(self, state: np.ndarray, num_vehicles: int):
        """Copy one flat state (STATE_COUNT doubles, include/lfdm.h order) into the next num_vehicles."""
        s = _f64(state, (self.STATE_COUNT,))
        self._ck(self._L.lfdm_initialize(self._h, _ptr(s), int(num_vehicles)))

    def SetTimeStep(self, step: float):
        self._ck(self._L.lfdm_set_time_step(self._h, float(step)))

    def SetEndTime(self, tend: float):
        self._ck(self._L.lfdm_set_end_time(self._h, float(tend)))

    def SetKernelSimTime(self, t: float):
        self._ck(self._L.lfdm_set_kernel_sim_time(self._h, float(t)))

    def SetHostDumpTime(self, t: float):
        self._ck(self._L.lfdm_set_host_dump_time(self._h, float(t)))

    def SetThreadsPerBlock(self, threads: int):
        self._ck(self._L.lfdm_set_threads_per_block(self._h, int(threads)))

    def GetStep(self) -> float:
        v = ctypes.c_double()
        self._ck(self._L.lfdm_get_step(self._h, ctypes.byref(v)))
        return v.value

    def GetEndTime(self) -> float:
        v = ctypes.c_double()
        self._ck(self._L.lfdm_get_end_time(self._h, ctypes.byref(v)))
        return v.value

    def GetTireType(self) -> int:
        v = ctypes.c_int()
        self._ck(self._L.lfdm_get_tire_type(self._h, ctypes.byref(v)))
        return v.value

    def SetOutput(self, output_file: str, output_freq: float, store_all: bool = False, no_outs: int = 50):
        self._ck(self._L.lfdm_set_output(self._h, output_file.encode(), float(output_freq), int(bool(store_all)),
                                         int(no_outs)))

    def Solve(self):
        self._ck(self._L.lfdm_solve(self._h))

    def SolveStep(self, t: float, steering=None, throttle=None, braking=None, schedule=None) -> float:
        """SolveStep(t, steering, throttle, braking) with scalars (reference :497-550), per-vehicle
        arrays (extension), or schedule=callable(t)->(steering, throttle, braking) evaluated at every
        step time of the window (the reference's functor SolveStep, .cuh:234-287)."""
        out = ctypes.c_double()
        if schedule is not None:
            times = self.window_times(t)
            sched = _f64([schedule(x) for x in times], (len(times), 3))
            self._ck(self._L.lfdm_solve_step_schedule(self._h, float(t), _ptr(sched), len(times), 0,
                                                      ctypes.byref(out)))
        elif np.ndim(steering) == 0 and np.ndim(throttle) == 0 and np.ndim(braking) == 0:
            self._ck(self._L.lfdm_solve_step(self._h, float(t), float(steering), float(throttle), float(braking),
                                             ctypes.byref(out)))
        else:
            st = _f64(np.broadcast_to(steering, (self.n,)))
            th = _f64(np.broadcast_to(throttle, (self.n,)))
            br = _f64(np.broadcast_to(braking, (self.n,)))
            self._ck(self._L.lfdm_solve_step_controls(self._h, float(t), _ptr(st), _ptr(th), _ptr(br),
                                                      ctypes.byref(out)))
        return out.value

    def GetSimState(self, vehicle_index: int) -> np.ndarray:
        s = np.zeros(self.STATE_COUNT)
        self._ck(self._L.lfdm_get_sim_state(self._h, int(vehicle_index), _ptr(s)))
        return s

    # -- extensions ---------------------------------------------------------------------------
    def construct_class(self, cls: Class18, params: np.ndarray, tire_type: int = TireType.TMeasy):
        p = _f64(params).reshape(-1, P_COUNT)
        self._ck(self._L.lfdm_construct_class(self._h, ctypes.byref(cls), p.shape[0], _ptr(p), int(tire_type)))

    def set_params(self, params: np.ndarray, first: int = 0):
        p = _f64(params).reshape(-1, P_COUNT)
        self._ck(self._L.lfdm_set_params(self._h, int(first), p.shape[0], _ptr(p)))

    def get_params(self, first: int = 0, count: int | None = None) -> np.ndarray:
        count = self.n - first if count is None else count
        p = np.zeros((count, P_COUNT))
        self._ck(self._L.lfdm_get_params(self._h, int(first), int(count), _ptr(p)))
        return p

    def set_driver_tables(self, tables: np.ndarray, first: int = 0):
        """tables: [rows][4] shared by all vehicles from `first`, or [count][rows][4] per vehicle."""
        t = _f64(tables)
        if t.ndim == 2:
            self._ck(self._L.lfdm_set_driver_table(self._h, int(first), self.n - first, _ptr(t), t.shape[0]))
        else:
            self._ck(self._L.lfdm_set_driver_tables(self._h, int(first), t.shape[0], _ptr(t), t.shape[1]))

    def set_states(self, states: np.ndarray, first: int = 0):
        s = _f64(states).reshape(-1, self.STATE_COUNT)
        self._ck(self._L.lfdm_set_states(self._h, int(first), s.shape[0], _ptr(s)))

    def get_states(self, first: int = 0, count: int | None = None) -> np.ndarray:
        count = self.n - first if count is None else count
        s = np.zeros((count, self.STATE_COUNT))
        self._ck(self._L.lfdm_get_states(self._h, int(first), int(count), _ptr(s)))
        return s

    def set_precision(self, precision: int):
        self._ck(self._L.lfdm_set_precision(self._h, int(precision)))

    def set_split_warps(self, mode: int):
        """11-DOF split-warp window kernel: -1 for small fleets (default), 0 never, 1 always."""
        self._ck(self._L.lfdm_set_split_warps(self._h, int(mode)))

    def set_response_buffer(self, buf: np.ndarray | None, output_freq: float = 100.0):
        """Stream Solve's SoA response [sample][RESP_CHANNELS][N] into `buf` (float64, C-contiguous); samples
        beyond its capacity wrap around."""
        if buf is None:
            self._ck(self._L.lfdm_set_response_buffer(self._h, None, 0, 1.0))
            self._resp = None
            return
        if buf.dtype != np.float64 or not buf.flags.c_contiguous:
            raise ValueError("response buffer must be C-contiguous float64")
        self._resp = buf
        self._ck(self._L.lfdm_set_response_buffer(self._h, _ptr(buf), buf.size, float(output_freq)))

    def set_response_device(self, ptr: int | None, capacity: int = 0, output_freq: float = 100.0):
        """Write Solve's SoA response straight into device memory at `ptr` (e.g. a torch CUDA tensor's
        data_ptr()) holding `capacity` doubles, a whole number of windows; windows wrap around."""
        self._ck(self._L.lfdm_set_response_device(self._h, ctypes.c_void_p(ptr) if ptr else None, int(capacity),
                                                  float(output_freq)))

    def solve_range(self, t_begin: float, t_end: float):
        """The windows of Solve() that start in [t_begin, t_end)."""
        self._ck(self._L.lfdm_solve_range(self._h, float(t_begin), float(t_end)))

    def response_samples(self) -> int:
        n = ctypes.c_size_t()
        self._ck(self._L.lfdm_response_samples(self._h, ctypes.byref(n)))
        return n.value

    def window_times(self, t: float) -> np.ndarray:
        n = ctypes.c_uint()
        self._ck(self._L.lfdm_window_steps(self._h, float(t), ctypes.byref(n), None, 0))
        times = np.zeros(n.value)
        self._ck(self._L.lfdm_window_steps(self._h, float(t), ctypes.byref(n), _ptr(times), n.value))
        return times

    def last_kernel_ms(self):
        ms = ctypes.c_double()
        n = ctypes.c_uint()
        self._ck(self._L.lfdm_last_kernel_ms(self._h, ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, n.value

    def status_words(self) -> np.ndarray:
        w = np.zeros(self.n, dtype=np.uint32)
        self._ck(self._L.lfdm_get_status_words(self._h, 0, self.n, _ptr(w)))
        return w


    def _jacobian(self, fn, steering, throttle, braking, reference_point):
        import torch
        dev = torch.device("cuda", self.device)
        n = self.n
        ctl = torch.tensor(np.stack([np.broadcast_to(np.asarray(x, dtype=np.float64), (n,))
                                     for x in (steering, throttle, braking)]), dtype=torch.float64, device=dev)
        js = torch.empty(36 * 36 * n, dtype=torch.float64, device=dev)
        ju = torch.empty(36 * 2 * n, dtype=torch.float64, device=dev)
        ny = ctypes.c_int()
        self._ck(fn(self._h, ctypes.c_void_p(ctl.data_ptr()), int(bool(reference_point)), ctypes.c_void_p(js.data_ptr()),
                    ctypes.c_void_p(ju.data_ptr()), ctypes.byref(ny)))
        m = ny.value
        jac_state = js[: m * m * n].reshape(m, m, n).permute(2, 0, 1).cpu().numpy()
        jac_ctl = ju[: m * 2 * n].reshape(m, 2, n).permute(2, 0, 1).cpu().numpy()
        return jac_state, jac_ctl

    def rhs_jacobian_fd(self, steering, throttle, braking=0.0, reference_point: bool = True):
        """The reference's IntegrateStepWithJacobian Jacobians for every vehicle (lfdm_rhs_jacobian_fd):
        central differences of the right-hand side with the reference's perturbations, any model and
        tire type, at every vehicle's current state. Controls are scalars or arrays of N; braking enters
        only the state Jacobian (the control differences use braking 0, as the reference does). Returns
        (jac_state [N, ny, ny], jac_controls [N, ny, 2]) in the model's packed order (packY / packYDOT);
        reference_point differentiates where PerturbRhsFun does (the packed states in a fresh state)
        rather than on top of the full current state."""
        return self._jacobian(self._L.lfdm_rhs_jacobian_fd, steering, throttle, braking, reference_point)


class d18SolverHalfImplicitGPU(_SolverGPU):
    """18-DOF batched half-implicit stepper on one GPU (reference: 18dof-gpu/dof18_halfImplicit_gpu.cuh)."""

    MODEL = 18
    STATE_COUNT = S_COUNT
    RESP_CHANNELS = RESP18

    def rhs_jacobian(self, steering, throttle, braking=0.0, reference_point: bool = True):
        """Exact Jacobians of the right-hand side at every vehicle's current state (lfdm_rhs_jacobian18;
        the reference CPU solver's GetJacobianState / GetJacobianControls by central differences,
        18dof/dof18_halfImplicit.cpp:356-520). Controls are scalars or arrays of N. Returns
        (jac_state [N, ny, ny], jac_controls [N, ny, 2]) in the reference's packed order, ny = 21 with a
        torque converter and 20 without (13 and 12 with TMeasyNr tires, which have no deflection
        states); reference_point selects the point the reference differentiates at (previous
        accelerations 0, first gear) rather than the full current state. rhs_jacobian_fd gives the
        reference's own difference scheme for every model."""
        return self._jacobian(self._L.lfdm_rhs_jacobian18, steering, throttle, braking, reference_point)


class d11SolverHalfImplicitGPU(_SolverGPU):
    """11-DOF batched half-implicit stepper on one GPU (reference: 11dof-gpu/dof11_halfImplicit_gpu.cuh).

    States use the LFDM11_S_* layout (S11): chassis X, Y, u, v, psi, wz, their rates, crank speed,
    crank acceleration, current gear, then the front and rear TMeasy tire blocks."""

    MODEL = 11
    STATE_COUNT = S11_COUNT
    RESP_CHANNELS = RESP11

    def rhs_jacobian(self, steering, throttle, braking=0.0, reference_point: bool = True):
        """Exact Jacobians of the 11-DOF right-hand side at every vehicle's current state
        (lfdm_rhs_jacobian_exact; the reference CPU solver's GetJacobianState / GetJacobianControls
        by central differences, 11dof/dof11_halfImplicit.cpp:335-429). Returns (jac_state [N, ny, ny],
        jac_controls [N, ny, 2]) in the reference's packed order: ny = 13 with a torque converter and
        12 without (9 and 8 with TMeasyNr tires)."""
        return self._jacobian(self._L.lfdm_rhs_jacobian_exact, steering, throttle, braking, reference_point)


class d24SolverHalfImplicitGPU(_SolverGPU):
    """24-DOF batched half-implicit stepper on one GPU (reference: 24dof-gpu/dof24_halfImplicit_gpu.cuh).

    States use the LFDM24_S_* layout (S24, 212 doubles): VehicleState, 4 TMeasyState, 4
    SuspensionState. Construct takes the suspension JSON after the tire JSON, and Initialize applies
    initializeTireSus with each vehicle's parameters, as the reference does; set_states copies raw
    states. FP64, TMeasy tires."""

    MODEL = 24
    STATE_COUNT = S24_COUNT
    RESP_CHANNELS = RESP24

    def rhs_jacobian(self, steering, throttle, braking=0.0, reference_point: bool = True):
        """Exact Jacobians of the 24-DOF right-hand side (TMeasy tires) at every vehicle's current
        state (lfdm_rhs_jacobian_exact; the reference CPU solver's GetJacobianState /
        GetJacobianControls by central differences, 24dof/dof24_halfImplicit.cpp:402-494). Returns
        (jac_state [N, ny, ny], jac_controls [N, ny, 2]) in the reference's packed order: ny = 36 with
        a torque converter and 35 without."""
        return self._jacobian(self._L.lfdm_rhs_jacobian_exact, steering, throttle, braking, reference_point)

    def Construct(self, vehicle_params_file: str, tire_params_file: str, sus_params_file: str,  # noqa: N802
                  num_vehicles: int, driver_inputs_file: str | None = None, type: int = TireType.TMeasy):  # noqa: A002
        self._ck(self._L.lfdm_construct(self._h, vehicle_params_file.encode(), tire_params_file.encode(),
                                        sus_params_file.encode(), int(num_vehicles),
                                        driver_inputs_file.encode() if driver_inputs_file else None, int(type)))


def measure_fp64_peak(device: int = 0) -> float:
    """Measured FP64 FMA instruction rate (DFMA/s) of a device."""
    return measure_fp64_peak_clock(device)[0]


def measure_fp64_peak_clock(device: int = 0) -> tuple[float, float]:
    """(measured DFMA/s, SM clock in GHz the probe ran at) of a device."""
    v, g = ctypes.c_double(), ctypes.c_double()
    rc = lib().lfdm_measure_fp64_peak_clock(int(device), ctypes.byref(v), ctypes.byref(g))
    if rc:
        raise LfdmError(rc, "FP64 peak probe failed")
    return v.value, g.value


def measure_fp32_peak_clock(device: int = 0) -> tuple[float, float]:
    """(measured lane FFMA/s, SM clock in GHz the probe ran at) of a device."""
    v, g = ctypes.c_double(), ctypes.c_double()
    rc = lib().lfdm_measure_fp32_peak_clock(int(device), ctypes.byref(v), ctypes.byref(g))
    if rc:
        raise LfdmError(rc, "FP32 peak probe failed")
    return v.value, g.value


class Fleet:
    """Mixed 18/24-DOF fleet with per-vehicle end times, stepped in one persistent launch captured in
    a CUDA graph (lfdm_fleet_* in include/lfdm.h). Vehicles are added per (model, class) group with
    numpy arrays; states and responses come back in add order per model."""

    NCH = {18: RESP18, 24: RESP24}
    NS = {18: S_COUNT, 24: S24_COUNT}

    def __init__(self, device: int = 0, dt: float = 1e-3, kernel_sim_time: float = 1.0, output_dt: float = 0.0):
        self._L = lib()
        h = ctypes.c_void_p()
        rc = self._L.lfdm_fleet_create(int(device), ctypes.byref(h))
        if rc:
            raise LfdmError(rc, self._L.lfdm_fleet_last_error(None).decode())
        self._h = h
        self.count = {18: 0, 24: 0}
        self._ck(self._L.lfdm_fleet_set_time_step(h, float(dt)))
        self._ck(self._L.lfdm_fleet_set_kernel_sim_time(h, float(kernel_sim_time)))
        self._ck(self._L.lfdm_fleet_set_output(h, float(output_dt)))

    def _ck(self, rc: int):
        if rc:
            raise LfdmError(rc, self._L.lfdm_fleet_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._L.lfdm_fleet_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_rows(self, rows: np.ndarray) -> int:
        """Driver rows [nrows][4] shared by later add(..., rows=None) calls; returns their first index."""
        r = _f64(rows).reshape(-1, 4)
        first = ctypes.c_int64()
        self._ck(self._L.lfdm_fleet_add_rows(self._h, _ptr(r), r.shape[0], ctypes.byref(first)))
        return first.value

    def add(self, model: int, cls: Class18, params: np.ndarray, states: np.ndarray, horizons: np.ndarray,
            rows: np.ndarray | None, row_off: np.ndarray, row_len: np.ndarray):
        """Append vehicles: params [n][P_COUNT], states [n][states of the model], horizons [n] end times
        (s), driver rows [nrows][4] with per-vehicle first row and row count (rows None: row_off
        indexes the rows given to add_rows)."""
        if model not in self.NS:
            raise LfdmError(_abi.C["LFDM_ERR_ARG"], f"the fleet holds 18-DOF and 24-DOF vehicles (model {model})")
        p = _f64(params).reshape(-1, P_COUNT)
        n = p.shape[0]
        st = _f64(states).reshape(n, self.NS[model])
        hz = _f64(horizons).reshape(n)
        r = _f64(rows).reshape(-1, 4) if rows is not None else None
        off = np.ascontiguousarray(row_off, dtype=np.int64).reshape(n)
        ln = np.ascontiguousarray(row_len, dtype=np.int32).reshape(n)
        self._ck(self._L.lfdm_fleet_add(self._h, int(model), ctypes.byref(cls), n, _ptr(p), _ptr(st), _ptr(hz),
                                        _ptr(r), r.shape[0] if r is not None else 0, _ptr(off), _ptr(ln)))
        self.count[model] += n

    def set_launch(self, threads: int = 128, blocks_per_sm: int = 0, steps_per_launch: int = 0):
        self._ck(self._L.lfdm_fleet_set_launch(self._h, int(threads), int(blocks_per_sm), int(steps_per_launch)))

    def get_launch(self) -> tuple[int, int, int]:
        a, b, c = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_uint()
        self._ck(self._L.lfdm_fleet_get_launch(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def set_precision(self, precision: int):
        """LFDM_PREC_FP64 (0, default) or LFDM_PREC_MIXED_TIRE (2)."""
        self._ck(self._L.lfdm_fleet_set_precision(self._h, int(precision)))

    def set_affinity(self, on: bool = True):
        """Split the SMs between the 18-DOF and 24-DOF tile lists (default on)."""
        self._ck(self._L.lfdm_fleet_set_affinity(self._h, int(bool(on))))

    def get_affinity(self) -> tuple[bool, float]:
        """(affinity on, 18-DOF share of the prepared fleet's estimated work)."""
        on, fr = ctypes.c_int(), ctypes.c_double()
        self._ck(self._L.lfdm_fleet_get_affinity(self._h, ctypes.byref(on), ctypes.byref(fr)))
        return bool(on.value), fr.value

    def tune(self, pilot_steps: int = 500) -> float:
        ms = ctypes.c_double()
        self._ck(self._L.lfdm_fleet_tune(self._h, int(pilot_steps), ctypes.byref(ms)))
        return ms.value

    def solve(self):
        self._ck(self._L.lfdm_fleet_solve(self._h))

    def last_ms(self) -> tuple[float, int]:
        ms, n = ctypes.c_double(), ctypes.c_uint()
        self._ck(self._L.lfdm_fleet_last_ms(self._h, ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, n.value

    def info(self) -> dict:
        a, b, s, v, k = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_longlong(), ctypes.c_double(), ctypes.c_uint()
        self._ck(self._L.lfdm_fleet_info(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(s), ctypes.byref(v),
                                         ctypes.byref(k)))
        return {"n18": a.value, "n24": b.value, "total_steps": s.value, "vehicle_steps": v.value, "nsamples": k.value}

    def get_states(self, model: int) -> np.ndarray:
        out = np.zeros((self.count[model], self.NS[model]))
        if out.size:
            self._ck(self._L.lfdm_fleet_get_states(self._h, int(model), 0, out.shape[0], _ptr(out)))
        return out

    def set_states(self, model: int, states: np.ndarray):
        st = _f64(states).reshape(self.count[model], self.NS[model])
        self._ck(self._L.lfdm_fleet_set_states(self._h, int(model), 0, st.shape[0], _ptr(st)))

    def get_response(self, model: int) -> np.ndarray:
        k = ctypes.c_uint()
        self._ck(self._L.lfdm_fleet_get_response(self._h, int(model), None, 0, ctypes.byref(k)))
        out = np.zeros((k.value, self.NCH[model], self.count[model]))
        if out.size:
            self._ck(self._L.lfdm_fleet_get_response(self._h, int(model), _ptr(out), out.size, ctypes.byref(k)))
        return out

    def status_words(self, model: int) -> np.ndarray:
        w = np.zeros(self.count[model], dtype=np.uint32)
        if w.size:
            self._ck(self._L.lfdm_fleet_get_status_words(self._h, int(model), _ptr(w)))
        return w


# Parameters of the differentiable rollout, in the order of grad_params / theta.
ROLLOUT_PARAMS = ("m", "jz", "a", "friction_scale", "kt")
_FRICTION = ("fxmpn", "fxmp2n", "fxspn", "fxsp2n", "fympn", "fymp2n", "fyspn", "fysp2n")


class Rollout18:
    """Differentiable rollout of a d18SolverHalfImplicitGPU's vehicles (lfdm_traj18_*): `nsteps` FP64
    steps from the solver's current states with per-step controls, loss per vehicle = sum over steps
    of the squared lateral and heading error to a reference path + weight_u |u|^2, gradients by the
    hand-written adjoint with a checkpoint every `ckpt_every` steps.

    `loss(controls, ref, theta)` is a torch autograd function of the controls [nsteps, 3, N] and of
    theta [5, N], offsets of (mass, Jz, CG-to-front distance a with b held, tire friction scale
    around 1, tire vertical stiffness) applied to the solver's parameters for the rollout."""

    def __init__(self, solver: "d18SolverHalfImplicitGPU", nsteps: int, ckpt_every: int = 100,
                 weight_u: float = 1e-3):
        import torch  # noqa: F401  (the rollout works on CUDA tensors)
        self.solver = solver
        self.n = solver.n
        self.nsteps = int(nsteps)
        self.ckpt = int(ckpt_every)
        self.weight_u = float(weight_u)
        self._base = solver.get_params()
        self._fwd_token = None

    def _apply_theta(self, theta):
        t = theta.detach().cpu().numpy() if theta is not None else None
        if t is None or not t.any():
            self.solver.set_params(self._base)
            return
        p = self._base.copy()
        p[:, P["m"]] += t[0]
        p[:, P["jz"]] += t[1]
        p[:, P["a"]] += t[2]
        for f in _FRICTION:
            p[:, P[f]] *= 1.0 + t[3]
        p[:, P["kt"]] += t[4]
        self.solver.set_params(p)

    def forward_raw(self, controls, ref, loss):
        self.solver._ck(self.solver._L.lfdm_traj18_forward(
            self.solver._h, ctypes.c_void_p(controls.data_ptr()), ctypes.c_void_p(ref.data_ptr()), self.nsteps,
            self.weight_u, self.ckpt, ctypes.c_void_p(loss.data_ptr())))

    def backward_raw(self, controls, ref, grad_ctl, grad_params, grad_state0=None):
        self.solver._ck(self.solver._L.lfdm_traj18_backward(
            self.solver._h, ctypes.c_void_p(controls.data_ptr()), ctypes.c_void_p(ref.data_ptr()), self.nsteps,
            self.weight_u, self.ckpt, ctypes.c_void_p(grad_ctl.data_ptr()), ctypes.c_void_p(grad_params.data_ptr()),
            ctypes.c_void_p(grad_state0.data_ptr()) if grad_state0 is not None else None))

    def branch_signature(self, controls, out):
        """lfdm_traj18_branch_signature: per-vehicle hash (int64 CUDA tensor `out` [N]) of the branches
        the rollout with `controls` takes (at the solver's current parameters)."""
        self.solver._ck(self.solver._L.lfdm_traj18_branch_signature(
            self.solver._h, ctypes.c_void_p(controls.data_ptr()), self.nsteps, ctypes.c_void_p(out.data_ptr())))

    def last_ms(self) -> tuple[float, float]:
        f, b = ctypes.c_double(), ctypes.c_double()
        self.solver._ck(self.solver._L.lfdm_traj18_last_ms(self.solver._h, ctypes.byref(f), ctypes.byref(b)))
        return f.value, b.value

    def loss(self, controls, ref, theta=None):
        import torch
        if theta is None:
            theta = torch.zeros(5, self.n, dtype=torch.float64, device=controls.device)
        return _rollout_fn()(controls, theta, ref, self)


_ROLLOUT_FN = None


def _rollout_fn():
    """The torch.autograd.Function of Rollout18.loss (built on first use: torch is imported lazily)."""
    global _ROLLOUT_FN
    if _ROLLOUT_FN is not None:
        return _ROLLOUT_FN.apply
    import torch

    class _Fn(torch.autograd.Function):
        @staticmethod
        def forward(ctx, controls, theta, ref, ro):
            controls = controls.detach().contiguous()
            ref = ref.detach().contiguous()
            if controls.dtype != torch.float64 or controls.shape != (ro.nsteps, 3, ro.n):
                raise ValueError(f"controls must be float64 [{ro.nsteps}, 3, {ro.n}]")
            if ref.dtype != torch.float64 or ref.shape != (ro.nsteps, 3, ro.n):
                raise ValueError(f"ref must be float64 [{ro.nsteps}, 3, {ro.n}]")
            loss = torch.empty(ro.n, dtype=torch.float64, device=controls.device)
            ro._apply_theta(theta)
            ro.forward_raw(controls, ref, loss)
            ro._fwd_token = object()
            ctx.token = ro._fwd_token
            ctx.ro = ro
            ctx.save_for_backward(controls, theta, ref)
            return loss

        @staticmethod
        def backward(ctx, gl):
            controls, theta, ref = ctx.saved_tensors
            ro = ctx.ro
            ro._apply_theta(theta)
            if ro._fwd_token is not ctx.token:  # another rollout ran since: rebuild the checkpoints
                tmp = torch.empty(ro.n, dtype=torch.float64, device=controls.device)
                ro.forward_raw(controls, ref, tmp)
                ro._fwd_token = ctx.token
            gctl = torch.empty_like(controls)
            gp = torch.empty(5, ro.n, dtype=torch.float64, device=controls.device)
            ro.backward_raw(controls, ref, gctl, gp)
            # friction scale: the adjoint returns d loss / d scale at the current fields, i.e. per unit
            # of (1 + theta3)
            gp[3] = gp[3] / (1.0 + theta[3])
            gl = gl.contiguous()
            return gctl * gl[None, None, :], gp * gl[None, :], None, None

    _ROLLOUT_FN = _Fn
    return _ROLLOUT_FN.apply


NOALLOC_MAX_VEHICLES = _abi.C["LFDM_NOALLOC_MAX_VEHICLES"]
NOALLOC_SCRATCH_BYTES = _abi.C["LFDM_NOALLOC_SCRATCH_BYTES"]


def step18_noalloc(cls: Class18, params: int, states: int, steering: int, throttle: int, braking: int, n: int,
                   t0: float, dt: float, nsteps: int, stream: int = 0, tire_type: int = TireType.TMeasy) -> None:
    """lfdm_step18_noalloc: one FP64 18-DOF window over device-resident vehicles (device pointers,
    e.g. torch CUDA tensors' data_ptr(): params [n][P_COUNT], states [n][S_COUNT] in/out, controls
    [n] each), enqueued on `stream` without allocating device memory; n <= NOALLOC_MAX_VEHICLES. For
    callers that cannot allocate on their call path. The call waits for `stream` at the end to read
    one status word and raises LfdmError (LFDM_ERR_NUMERIC) when a state became non-finite. Calls
    share one static scratch array per device (NOALLOC_SCRATCH_BYTES), so calls that overlap on
    the GPU race."""
    err = ctypes.create_string_buffer(512)
    rc = lib().lfdm_step18_noalloc(ctypes.byref(cls), int(tire_type), ctypes.c_void_p(params), ctypes.c_void_p(states),
                                   ctypes.c_void_p(steering), ctypes.c_void_p(throttle), ctypes.c_void_p(braking),
                                   int(n), float(t0), float(dt), int(nsteps), ctypes.c_void_p(stream) if stream else None,
                                   err, 512)
    if rc:
        raise LfdmError(rc, err.value.decode())


def register_host(a: np.ndarray) -> None:
    """Page-lock a numpy array (for overlapped copies)."""
    rc = lib().lfdm_register_host(ctypes.c_void_p(a.ctypes.data), a.nbytes)
    if rc:
        raise LfdmError(rc, "cudaHostRegister failed")


def unregister_host(a: np.ndarray) -> None:
    lib().lfdm_unregister_host(ctypes.c_void_p(a.ctypes.data))
