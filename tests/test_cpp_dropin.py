"""The C++ drop-in headers (include/lfdm/*.cuh): a program written like the reference's GPU tests and
demos (tests/cpp/dropin_demo.cpp) compiles against them with a plain host compiler and, on the GPU,
gives bit for bit the states the Python binding of the same library gives for the same calls; the
struct fields it prints by name are checked against the flat state vector of include/lfdm.h."""
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import pkg_mod

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "dropin_demo.cpp")


def _compile(built_lib, out, extra=()):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    libdir = os.path.dirname(pkg_mod("build").LIB)
    cmd = [gxx, "-std=c++17", "-Wall", "-Wextra", "-Werror", "-O1", "-I", os.path.join(ROOT, "include", "lfdm"),
           *extra, SRC, "-L", libdir, "-llfdm", f"-Wl,-rpath,{libdir}", "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return out


def test_dropin_headers_compile(built_lib, tmp_path):
    """All three model headers in one translation unit (TireType and DriverInput declared once),
    with the default print-and-continue error policy and with LFDM_CPP_THROW."""
    _compile(built_lib, str(tmp_path / "demo"))
    _compile(built_lib, str(tmp_path / "demo_throw"), ["-DLFDM_CPP_THROW"])


@pytest.fixture(scope="module")
def demo(built_lib, tmp_path_factory):
    return _compile(built_lib, str(tmp_path_factory.mktemp("dropin") / "demo"))


def _run(demo, *args):
    r = subprocess.run([demo, *map(str, args)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    vals = {}
    for line in r.stdout.splitlines():
        k, v = line.split()
        vals[k] = float(v)
    return vals, r.stderr


def _write(tmp, name, obj):
    p = tmp / name
    p.write_text(obj if isinstance(obj, str) else json.dumps(obj))
    return str(p)


def _driver(case):
    return "".join(" ".join(repr(float(v)) for v in r) + "\n" for r in case["driver"])


def _case(golden, name):
    return {c["name"]: c for c in golden["cases"]}[name]


@pytest.mark.gpu
def test_dropin_18dof_solve_matches_binding(built_lib, golden18, demo, tmp_path):
    """tests/18dof_gpu.cu:13-56 written against the drop-in class: 50 HMMWVs on acc3 for 10 s."""
    case = _case(golden18, "hmmwv_acc3_gpu")
    vj, tj = _write(tmp_path, "v.json", case["vehicle"]), _write(tmp_path, "t.json", case["tire"])
    dj = _write(tmp_path, "acc3.txt", _driver(case))
    got, _ = _run(demo, "solve", 18, vj, tj, "-", dj, 50, 10.0)
    sol = built_lib.d18SolverHalfImplicitGPU(50)
    sol.Construct(vj, tj, 50, dj)
    sol.SetThreadsPerBlock(32)
    sol.SetTimeStep(1e-3)
    sol.Initialize(np.zeros(built_lib.S_COUNT), 50)
    sol.SetEndTime(10.0)
    sol.Solve()
    A = pkg_mod("_abi")
    S, T0, TS, T = A.S, A.S_TIRE0, A.S_TIRE_STRIDE, A.T
    for tag, i in (("first", 0), ("last", 49)):
        s = sol.GetSimState(i)
        for f in ("x", "y", "u", "v", "psi", "wz", "phi", "wx", "current_gr"):
            assert got[f"{tag}.{f}"] == s[S[f]], (tag, f)
        assert got[f"{tag}.crankOmega"] == s[S["crankomega"]]
        assert got[f"{tag}.lf.omega"] == s[T0 + T["omega"]]
        assert got[f"{tag}.rr.omega"] == s[T0 + 3 * TS + T["omega"]]
        assert got[f"{tag}.lf.xe"] == s[T0 + T["xe"]]
        assert got[f"{tag}.rr.ye"] == s[T0 + 3 * TS + T["ye"]]
        assert got[f"{tag}.lr.fz"] == s[T0 + 2 * TS + T["fz"]]
    assert abs(got["first.x"] - 88.5335) < 1  # the reference test's own bound
    assert got["step"] == 1e-3 and got["end_time"] == 10.0 and got["tire_nr"] == 0.0
    sol.close()


@pytest.mark.gpu
def test_dropin_11dof_solve_matches_binding(built_lib, golden11_cases, demo, tmp_path):
    case = _case(golden11_cases, "hmmwv11_acc3_gpu22")
    vj, tj = _write(tmp_path, "v.json", case["vehicle"]), _write(tmp_path, "t.json", case["tire"])
    dj = _write(tmp_path, "acc3.txt", _driver(case))
    got, _ = _run(demo, "solve", 11, vj, tj, "-", dj, 40, 6.0)
    sol = built_lib.d11SolverHalfImplicitGPU(40)
    sol.Construct(vj, tj, 40, dj)
    sol.SetThreadsPerBlock(32)
    sol.SetTimeStep(1e-3)
    sol.Initialize(np.zeros(built_lib.S11_COUNT), 40)
    sol.SetEndTime(6.0)
    sol.Solve()
    s = sol.GetSimState(39)
    A = pkg_mod("_abi")
    S, T0, TS, T = A.S11, A.S11_TIRE0, A.S_TIRE_STRIDE, A.T
    for f in ("x", "y", "u", "psi", "wz", "current_gr"):
        assert got[f"last.{f}"] == s[S[f]], f
    assert got["last.f.omega"] == s[T0 + T["omega"]]
    assert got["last.r.omega"] == s[T0 + TS + T["omega"]]
    assert got["last.f.xe"] == s[T0 + T["xe"]]
    sol.close()


@pytest.mark.gpu
def test_dropin_24dof_solve_matches_binding(built_lib, golden24_cases, demo, tmp_path):
    """tests/24dof_gpu.cu's pattern: Construct with the suspension file, Initialize from default
    (zero) structs, which applies initializeTireSus, then Solve."""
    case = _case(golden24_cases, "hmmwv24_acc3_gpu22")
    vj, tj = _write(tmp_path, "v.json", case["vehicle"]), _write(tmp_path, "t.json", case["tire"])
    sj, dj = _write(tmp_path, "s.json", case["sus"]), _write(tmp_path, "acc3.txt", _driver(case))
    got, _ = _run(demo, "solve", 24, vj, tj, sj, dj, 40, 4.0)
    sol = built_lib.d24SolverHalfImplicitGPU(40)
    sol.Construct(vj, tj, sj, 40, dj)
    sol.SetThreadsPerBlock(32)
    sol.SetTimeStep(1e-3)
    sol.Initialize(np.zeros(built_lib.S24_COUNT), 40)
    s0 = sol.GetSimState(0)
    A = pkg_mod("_abi")
    S = A.S24
    T0, TN, U0, UN = 24, 23, 116, 24  # LFDM24_S_TIRE0, LFDM24_T_COUNT, LFDM24_S_SUS0, LFDM24_SUS_COUNT
    assert got["init.z"] == s0[S["z"]]
    assert got["init.lf.xt"] == s0[T0 + 6]          # LFDM24_T_XT
    assert got["init.rr.xs"] == s0[U0 + 3 * UN + 0]  # LFDM24_SUS_XS
    assert got["init.lf.ls"] == s0[U0 + 3]          # LFDM24_SUS_LS
    assert got["init.lf.xt"] != 0.0                 # initializeTireSus ran
    sol.SetEndTime(4.0)
    sol.Solve()
    s = sol.GetSimState(39)
    for f in ("x", "y", "z", "theta", "psi", "current_gr"):
        assert got[f"last.{f}"] == s[S[f]], f
    assert got["last.lf.omega"] == s[T0 + 4]
    assert got["last.rr.xt"] == s[T0 + 3 * TN + 6]
    assert got["last.lr.xs"] == s[U0 + 2 * UN + 0]
    assert got["last.rf.fzs"] == s[U0 + UN + 19]    # LFDM24_SUS_FZS
    sol.close()


@pytest.mark.gpu
def test_dropin_solve_step_scalar_and_functor(built_lib, golden18, demo, tmp_path):
    """demo_hmmwv_step_18gpu.cu and demo_hmmwv_controlsFunctor_18gpu.cu: SolveStep with scalar
    controls, then with a functor evaluated at each step start time; an Initialize beyond the
    capacity prints the library's message and the program carries on."""
    case = _case(golden18, "hmmwv_acc3_gpu")
    vj, tj = _write(tmp_path, "v.json", case["vehicle"]), _write(tmp_path, "t.json", case["tire"])
    got, err = _run(demo, "step", vj, tj, 16)
    sol = built_lib.d18SolverHalfImplicitGPU(16)
    sol.Construct(vj, tj, 16)
    sol.SetTimeStep(1e-3)
    sol.SetKernelSimTime(0.5)
    A = pkg_mod("_abi")
    s0 = np.zeros(built_lib.S_COUNT)
    s0[A.S["u"]] = 5.0
    for k in range(4):
        s0[A.S_TIRE0 + k * A.S_TIRE_STRIDE + A.T["omega"]] = 5.0 / 0.47
    sol.Initialize(s0, 16)
    t = sol.SolveStep(0.0, 0.1, 0.4, 0.0)
    t = sol.SolveStep(t, 0.0, 0.2, 0.1)
    f = lambda x: (0.0 if x < 0.7 else 0.05, 0.0 if x < 0.5 else 0.5, 0.0)  # noqa: E731
    t = sol.SolveStep(t, schedule=f)
    t = sol.SolveStep(t, schedule=f)
    s = sol.GetSimState(15)
    assert got["t"] == t == pytest.approx(2.0)
    for k in ("x", "y", "u", "v", "psi", "wz", "current_gr"):
        assert got[f"last.{k}"] == s[A.S[k]], k
    assert "lfdm: Initialize:" in err and got["after_error"] == 1.0
    sol.close()


@pytest.mark.gpu
def test_dropin_rhs_jacobians_match_binding(built_lib, golden18, demo, tmp_path):
    """GetRhsJacobians (the C++ method over lfdm_rhs_jacobian_host, per-vehicle matrices as the
    reference's GetJacobianState / GetJacobianControls) returns the binding's device Jacobians bit
    for bit, for the difference scheme and the exact Jacobian; a control vector of the wrong length
    is refused."""
    case = _case(golden18, "hmmwv_acc3_gpu")
    vj, tj = _write(tmp_path, "v.json", case["vehicle"]), _write(tmp_path, "t.json", case["tire"])
    n = 6
    got, err = _run(demo, "jac", vj, tj, n)
    sol = built_lib.d18SolverHalfImplicitGPU(n)
    sol.Construct(vj, tj, n)
    sol.SetTimeStep(1e-3)
    sol.SetKernelSimTime(0.2)
    s0 = np.zeros(built_lib.S_COUNT)
    A = pkg_mod("_abi")
    s0[A.S["u"]] = 8.0
    for k in range(4):
        s0[A.S_TIRE0 + k * A.S_TIRE_STRIDE + A.T["omega"]] = 8.0 / 0.47
    sol.Initialize(s0, n)
    sol.SolveStep(0.0, 0.1, 0.5, 0.0)
    st = 0.05 * np.arange(n)
    for tag, fn in (("fd", sol.rhs_jacobian_fd), ("exact", sol.rhs_jacobian)):
        js, ju = fn(st, np.full(n, 0.3), np.zeros(n))
        ny = js.shape[1]
        assert got[f"{tag}.ny"] == ny
        for r in range(ny):
            for c in range(ny):
                assert got[f"{tag}.s.{r}.{c}"] == js[n - 1, r, c], (tag, r, c)
            assert got[f"{tag}.u.{r}.0"] == ju[n - 1, r, 0] and got[f"{tag}.u.{r}.1"] == ju[n - 1, r, 1]
    assert got["bad_size"] == 0 and "one control value per vehicle" in err
    sol.close()

