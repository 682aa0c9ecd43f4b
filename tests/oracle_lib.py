"""ctypes access to the oracle (oracle/_build/liboracle.so) — test infrastructure only.

The oracle is the CPU restatement of the reference stepper (oracle/lfdm_oracle.c); tests compare
the CUDA path against it and bench.py's CPU-baseline leg times it. It is built with `make -C oracle oracle`.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
LIB = os.path.join(ORACLE_DIR, "_build", "liboracle.so")
REFRUN18 = os.path.join(ORACLE_DIR, "_ref", "refrun18")


def build() -> str:
    subprocess.run(["make", "-s", "-C", ORACLE_DIR, "oracle"], check=True)
    return LIB


LIB_FMA = os.path.join(ORACLE_DIR, "_build", "liboracle_fma.so")
LIB_O3 = os.path.join(ORACLE_DIR, "_build", "liboracle_o3.so")
_libs = {}


def lib(fma: bool = False, timing: bool = False):
    """The oracle; fma=True loads the same restatement compiled with FMA contraction, timing=True the
    build with the reference's Release flags (-O3) that the CPU baseline times."""
    path = LIB_O3 if timing else (LIB_FMA if fma else LIB)
    if path not in _libs:
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        L.oracle18_run.argtypes = [ctypes.c_void_p]
        L.oracle18_run.restype = ctypes.c_int
        L.oracle11_run.argtypes = [ctypes.c_void_p]
        L.oracle11_run.restype = ctypes.c_int
        L.oracle24_run.argtypes = [ctypes.c_void_p]
        L.oracle24_run.restype = ctypes.c_int
        L.oracle24_init_state.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.oracle_map_y.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double]
        L.oracle_map_y.restype = ctypes.c_double
        L.oracle_driver_input.argtypes = [ctypes.c_double, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.oracle_tire_init.argtypes = [ctypes.c_void_p]
        L.oracle18_rhs.argtypes = [ctypes.c_void_p] * 6
        L.oracle18_rhs.restype = ctypes.c_int
        L.oracle_rhs.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 6
        L.oracle_rhs.restype = ctypes.c_int
        L.oracle_jacobian_fd.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 4 + [ctypes.c_int] + \
            [ctypes.c_void_p] * 2
        L.oracle_jacobian_fd.restype = ctypes.c_int
        L.oracle_jacobian_fd_batch.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 4 + \
            [ctypes.c_int] * 3 + [ctypes.c_void_p] * 2
        L.oracle_jacobian_fd_batch.restype = ctypes.c_int
        _libs[path] = L
    return _libs[path]


class _Args(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int), ("tire_type", ctypes.c_int),
        ("classes", ctypes.c_void_p), ("class_of", ctypes.c_void_p),
        ("params", ctypes.c_void_p), ("states", ctypes.c_void_p),
        ("drv_rows", ctypes.c_void_p), ("drv_off", ctypes.c_void_p), ("drv_len", ctypes.c_void_p),
        ("ctl", ctypes.c_void_p),
        ("dt", ctypes.c_double), ("t0", ctypes.c_double), ("tend", ctypes.c_double), ("ksim", ctypes.c_double),
        ("schedule", ctypes.c_int),
        ("dtout", ctypes.c_double), ("resp", ctypes.c_void_p),
        ("resp_samples", ctypes.c_int64), ("samples_per_window", ctypes.c_int64),
        ("nthreads", ctypes.c_int),
    ]


def _ptr(a):
    return a.ctypes.data if a is not None else None


def run18(classes, class_of, params, states, tables=None, ctl=None, *, tire_type=0, dt=1e-3, t0=0.0,
          tend=10.0, ksim=2.0, schedule=1, dtout=0.0, nthreads=1, fma=False, model=18, timing=False):
    """Advance `states` ([n][75] for 18-DOF, [n][42] for 11-DOF; copied) with the oracle. `tables` is
    a list of per-vehicle [rows][4] arrays or one [n][rows][4] array. schedule 0 = CPU solver,
    1 = GPU Solve, 2 = one SolveStep window. Returns (states, resp or None)."""
    nch = {18: 13, 11: 9, 24: 15}[model]
    n = params.shape[0]
    cls_arr = (type(classes[0]) * len(classes))(*classes)
    class_of = np.ascontiguousarray(class_of, dtype=np.int32)
    params = np.ascontiguousarray(params, dtype=np.float64)
    st = np.array(states, dtype=np.float64, order="C", copy=True)
    rows = off = ln = None
    if tables is not None:
        if isinstance(tables, np.ndarray) and tables.ndim == 3:
            rows = np.ascontiguousarray(tables.reshape(-1, 4), dtype=np.float64)
            ln = np.full(n, tables.shape[1], dtype=np.int32)
        else:
            rows = np.ascontiguousarray(np.concatenate([np.asarray(t, np.float64).reshape(-1, 4) for t in tables]))
            ln = np.array([len(t) for t in tables], dtype=np.int32)
        off = np.zeros(n, dtype=np.int64)
        off[1:] = np.cumsum(ln[:-1].astype(np.int64))
    ctl_arr = np.ascontiguousarray(ctl, dtype=np.float64) if ctl is not None else None
    resp = None
    spw = 0
    nsamp = 0
    if dtout > 0:
        spw = int(np.ceil(ksim / dtout))
        windows = 1 if schedule == 2 else int(np.ceil((tend - t0) / ksim - 1e-12))
        # count the windows exactly as the solver loop does
        if schedule == 1:
            windows, ct = 0, t0
            while ct < tend:
                windows += 1
                ct = ct + ksim
        nsamp = windows * spw
        resp = np.full((nsamp, nch, n), np.nan, dtype=np.float64)
    a = _Args(n=n, tire_type=tire_type, classes=ctypes.addressof(cls_arr), class_of=_ptr(class_of),
              params=_ptr(params), states=_ptr(st), drv_rows=_ptr(rows), drv_off=_ptr(off), drv_len=_ptr(ln),
              ctl=_ptr(ctl_arr), dt=dt, t0=t0, tend=tend, ksim=ksim, schedule=schedule, dtout=dtout,
              resp=_ptr(resp), resp_samples=nsamp, samples_per_window=spw, nthreads=nthreads)
    L = lib(fma, timing)
    fn = {18: L.oracle18_run, 11: L.oracle11_run, 24: L.oracle24_run}[model]
    rc = fn(ctypes.byref(a))
    if rc != 0:
        raise RuntimeError(f"oracle18_run failed rc={rc}")
    return st, resp


def init_state24(params, state) -> np.ndarray:
    """initializeTireSus applied to a copy of one flat 24-DOF state (what Initialize does)."""
    p = np.ascontiguousarray(params, dtype=np.float64)
    st = np.array(state, dtype=np.float64, copy=True)
    lib().oracle24_init_state(p.ctypes.data, st.ctypes.data)
    return st


def map_y(points, x) -> float:
    m = np.ascontiguousarray(np.asarray(points, dtype=np.float64).reshape(-1, 2))
    return lib().oracle_map_y(m.ctypes.data, m.shape[0], float(x))


def driver_input(t, rows) -> np.ndarray:
    r = np.ascontiguousarray(np.asarray(rows, dtype=np.float64).reshape(-1, 4))
    out = np.zeros(4)
    lib().oracle_driver_input(float(t), r.ctypes.data, r.shape[0], out.ctypes.data)
    return out


def pack_y18(state, tc: bool) -> np.ndarray:
    """packY (18dof/dof18_halfImplicit.cpp:879-921) of a flat 18-DOF state (include/lfdm.h order)."""
    s = np.asarray(state, dtype=np.float64)
    T0, TS = 15, 15
    y = []
    for k in range(4):
        y += [s[T0 + k * TS + 0], s[T0 + k * TS + 1]]
    y += [s[T0 + k * TS + 4] for k in range(4)]
    if tc:
        y.append(s[12])
    y += [s[0], s[1], s[2], s[3], s[4], s[5], s[6], s[7]]
    return np.array(y)


def rhs18(cls, params, y, ctl, full_state=None) -> np.ndarray:
    """The reference's PerturbRhsFun (oracle18_rhs): the 18-DOF right-hand side at packed states y."""
    y = np.ascontiguousarray(y, dtype=np.float64)
    p = np.ascontiguousarray(params, dtype=np.float64)
    c = np.ascontiguousarray(ctl, dtype=np.float64)
    out = np.zeros(len(y))
    fs = None if full_state is None else np.ascontiguousarray(full_state, dtype=np.float64)
    n = lib().oracle18_rhs(ctypes.byref(cls), _ptr(p), None if fs is None else _ptr(fs), _ptr(y), _ptr(c), _ptr(out))
    assert n == len(y)
    return out


def rhs(model, tire_type, cls, params, y, ctl, full_state=None) -> np.ndarray:
    """PerturbRhsFun of the 11-, 18- or 24-DOF model (oracle_rhs) at packed states y."""
    y = np.ascontiguousarray(y, dtype=np.float64)
    p = np.ascontiguousarray(params, dtype=np.float64)
    c = np.ascontiguousarray(ctl, dtype=np.float64)
    fs = None if full_state is None else np.ascontiguousarray(full_state, dtype=np.float64)
    out = np.zeros(len(y))
    n = lib().oracle_rhs(model, tire_type, ctypes.byref(cls), _ptr(p), None if fs is None else _ptr(fs), _ptr(y),
                         _ptr(c), _ptr(out))
    assert n == len(y), (n, len(y))
    return out


def jacobian_fd(model, tire_type, cls, params, state, ctl, full_point=False):
    """IntegrateStepWithJacobian's central differences (oracle_jacobian_fd) at a flat state:
    (state Jacobian [ny][ny], control Jacobian [ny][2])."""
    p = np.ascontiguousarray(params, dtype=np.float64)
    s = np.ascontiguousarray(state, dtype=np.float64)
    c = np.ascontiguousarray(ctl, dtype=np.float64)
    js, jc = np.zeros(40 * 40), np.zeros(40 * 2)
    ny = lib().oracle_jacobian_fd(model, tire_type, ctypes.byref(cls), _ptr(p), _ptr(s), _ptr(c), int(full_point),
                                  _ptr(js), _ptr(jc))
    assert ny > 0
    return js[:ny * ny].reshape(ny, ny), jc[:2 * ny].reshape(ny, 2)


def jacobian_fd_batch(model, tire_type, cls, params, states, ctl, full_point=False, nthreads=1):
    """oracle_jacobian_fd over n vehicles of one class on nthreads host threads; ctl [3][n]. Returns
    (state Jacobians [n][ny][ny], control Jacobians [n][ny][2])."""
    p = np.ascontiguousarray(params, dtype=np.float64)
    s = np.ascontiguousarray(states, dtype=np.float64)
    n = s.shape[0]
    c = np.ascontiguousarray(np.asarray(ctl, dtype=np.float64).T)
    js, jc = np.zeros((n, 36 * 36)), np.zeros((n, 36 * 2))
    rc = lib().oracle_jacobian_fd_batch(model, tire_type, ctypes.byref(cls), _ptr(p), _ptr(s), _ptr(c), n,
                                        int(full_point), int(nthreads), _ptr(js), _ptr(jc))
    assert rc == 0
    ny = {11: 12, 18: 20, 24: 35}[model] - (0 if tire_type == 0 else {11: 4, 18: 8, 24: 8}[model]) + int(bool(cls.tcbool))
    return js[:, : ny * ny].reshape(n, ny, ny), jc[:, : 2 * ny].reshape(n, ny, 2)

