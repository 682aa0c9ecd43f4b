import importlib
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TESTS = os.path.dirname(os.path.abspath(__file__))
for p in (ROOT, TESTS):
    if p not in sys.path:
        sys.path.insert(0, p)

PKG = "low-fidelity-dynamic-models_gb300"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs the library's kernels)")


def load_pkg():
    return importlib.import_module(PKG)


def pkg_mod(name):
    return importlib.import_module(f"{PKG}.{name}")


@pytest.fixture(scope="session")
def lfdm():
    return load_pkg()


@pytest.fixture(scope="session")
def golden18():
    with open(os.path.join(TESTS, "golden", "golden18.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def golden11_cases():
    with open(os.path.join(TESTS, "golden", "golden11.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def golden24_cases():
    with open(os.path.join(TESTS, "golden", "golden24.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def built_lib():
    """Build liblfdm.so if needed (nvcc cross-compiles without a GPU)."""
    pkg_mod("build").build()
    return load_pkg()


# Parity floors s_k of the per-state check |a - b| <= rtol * max(|b|, s_k): 1 m for positions,
# 1 m/s for velocities, 1 rad for angles, 1 rad/s for body rates, 10 rad/s for wheel and crank
# speeds, 1e-3 m for tire deflections, 1 m/s^2 for accelerations.
def state_floors():
    abi = pkg_mod("_abi")
    fl = np.full(abi.S_COUNT, np.inf)  # fields not listed are not compared
    S, T = abi.S, abi.T
    for k in ("x", "y"):
        fl[S[k]] = 1.0
    for k in ("u", "v"):
        fl[S[k]] = 1.0
    for k in ("psi", "phi"):
        fl[S[k]] = 1.0
    for k in ("wz", "wx"):
        fl[S[k]] = 1.0
    for k in ("udot", "vdot"):
        fl[S[k]] = 1.0
    fl[S["crankomega"]] = 10.0
    fl[S["current_gr"]] = 1.0
    for t in range(4):
        b = abi.S_TIRE0 + t * abi.S_TIRE_STRIDE
        fl[b + T["omega"]] = 10.0
        fl[b + T["xe"]] = 1e-3
        fl[b + T["ye"]] = 1e-3
    return fl


RESP_FLOORS = np.array([1.0, 1, 1, 1, 1, 1, 1, 1, 1, 10, 10, 10, 10], dtype=np.float64)


def state_floors11():
    """Floors of the 11-DOF state vector (LFDM11_S_* layout), same scales as state_floors()."""
    abi = pkg_mod("_abi")
    fl = np.full(abi.S11_COUNT, np.inf)
    S, T = abi.S11, abi.T
    for k in ("x", "y", "u", "v", "psi", "wz", "udot", "vdot", "current_gr"):
        fl[S[k]] = 1.0
    fl[S["crankomega"]] = 10.0
    for t in range(2):
        b = abi.S11_TIRE0 + t * abi.S_TIRE_STRIDE
        fl[b + T["omega"]] = 10.0
        fl[b + T["xe"]] = 1e-3
        fl[b + T["ye"]] = 1e-3
    return fl


# time, x, y, u, v, psi, wz, front and rear wheel speed
RESP11_FLOORS = np.array([1.0, 1, 1, 1, 1, 1, 1, 10, 10], dtype=np.float64)


def case_inputs11(case):
    """(Class18, params[P], state[S11], table[rows][4]) of an 11-DOF golden case."""
    params = pkg_mod("params")
    cls, p = params.vehicle_from_json(case["vehicle"], case["tire"], case["tire_type"], model=11)
    return cls, p, np.array(case["state"], dtype=np.float64), np.array(case["driver"], dtype=np.float64)


def rel_err(a, b, floors):
    """Elementwise |a-b| / max(|b|, floor); inf floors mark fields that are not compared."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.maximum(np.abs(b), floors)
    with np.errstate(invalid="ignore", divide="ignore"):
        e = np.abs(a - b) / den
    e[..., ~np.isfinite(np.broadcast_to(floors, a.shape[-1:]))] = 0.0
    return np.where(np.isnan(e), np.inf, e)


def case_inputs(case):
    """(Class18, params[P], state[S], table[rows][4]) of a golden case."""
    params = pkg_mod("params")
    abi = pkg_mod("_abi")
    cls, p = params.vehicle_from_json(case["vehicle"], case["tire"], case["tire_type"])
    for k, v in case["vp"].items():
        p[abi.P[k.lower()]] = v
    for k, v in case["tp"].items():
        p[abi.P[k.lower()]] = v
    if case["tp"]:
        params.tire_init(p)
    return cls, p, np.array(case["state"], dtype=np.float64), np.array(case["driver"], dtype=np.float64)


def state_floors24():
    """Floors of the 24-DOF state vector (LFDM24_S_* layout): positions 1 m, speeds 1 m/s, angles
    1 rad, rates 1 rad/s, accelerations 1 m/s^2 (1 rad/s^2), wheel and crank speeds 10 rad/s, tire
    deflections and compressions and spring compressions 1e-3 m, forces 1e3 N, moments 1e3 N m, wheel
    and crank accelerations 1e3 rad/s^2 (differences of torques of order 1e3 N m over inertias of
    order 1 kg m^2)."""
    abi = pkg_mod("_abi")
    C = abi.C
    fl = np.full(C["LFDM24_S_COUNT"], 1.0)
    fl[C["LFDM24_S_CRANKOMEGA"]] = 10.0
    fl[C["LFDM24_S_DOMEGA_CRANK"]] = 1e3
    for k in range(4):
        b = C["LFDM24_S_TIRE0"] + k * C["LFDM24_T_COUNT"]
        for f in ("XE", "YE", "XT"):
            fl[b + C[f"LFDM24_T_{f}"]] = 1e-3
        fl[b + C["LFDM24_T_OMEGA"]] = 10.0
        fl[b + C["LFDM24_T_DOMEGA"]] = 1e3
        for f in ("FX", "FY", "FZ", "FXG", "FYG", "FZG", "MY", "ENGTOR"):
            fl[b + C[f"LFDM24_T_{f}"]] = 1e3
        s = C["LFDM24_S_SUS0"] + k * C["LFDM24_SUS_COUNT"]
        for f in ("XS", "XSI", "LS", "LSI"):
            fl[s + C[f"LFDM24_SUS_{f}"]] = 1e-3
        for f in ("FXS", "FYS", "FZS", "FZD", "MX", "MY", "MZ"):
            fl[s + C[f"LFDM24_SUS_{f}"]] = 1e3
    return fl


# time, x, y, u, v, phi, psi, theta, wx, wz, wy, four wheel speeds
RESP24_FLOORS = np.array([1.0] * 11 + [10.0] * 4, dtype=np.float64)


def case_inputs24(case):
    """(Class18, params[P], state[S24], table[rows][4]) of a 24-DOF golden case."""
    params = pkg_mod("params")
    abi = pkg_mod("_abi")
    cls, p = params.vehicle_from_json(case["vehicle"], case["tire"], case["tire_type"], model=24, sus=case["sus"])
    for k, v in case["vp"].items():
        p[abi.P[k.lower()]] = v
    for k, v in case["tp"].items():
        p[abi.P[k.lower()]] = v
    if case["tp"]:
        params.tire_init(p)
    return cls, p, np.array(case["state"], dtype=np.float64), np.array(case["driver"], dtype=np.float64)
