"""SolveStep with a __device__ functor (tests/cpp/functor_demo.cu, the pattern of the reference's
18dof-gpu/demos/HMMWV/demo_hmmwv_controlsFunctor_18gpu.cu:20-110): compiled with nvcc against the
C++ drop-in headers of include/lfdm it must build unchanged, and on the GPU the states after
SolveStep windows driven by the device-side functor (and by a functor that reads a table in device
memory) equal bit for bit those of the Python binding's SolveStep with the same controls as a
per-step schedule, for the 18-, 11- and 24-DOF solvers. Compiled with --fmad=false, as the library is."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import pkg_mod

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "functor_demo.cu")
TABLE = [(0.02 * r, 0.6 if r < 6 else 0.2, 0.3 if r == 7 else 0.0) for r in range(10)]


def _nvcc():
    for c in (os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc"), shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    pytest.skip("nvcc not available")


@pytest.fixture(scope="module")
def demo(built_lib, tmp_path_factory):
    out = str(tmp_path_factory.mktemp("functor") / "functor_demo")
    libdir = os.path.dirname(pkg_mod("build").LIB)
    cmd = [_nvcc(), "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", "--fmad=false", "-O2",
           "-I", os.path.join(ROOT, "include", "lfdm"), SRC, "-L", libdir, "-llfdm", "-Xlinker", "-rpath",
           "-Xlinker", libdir, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return out


def test_functor_demo_compiles(demo):
    assert os.path.exists(demo)


def _run(demo, *args):
    r = subprocess.run([demo, *map(str, args)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and not r.stderr, r.stdout + r.stderr
    t, s = None, {}
    for line in r.stdout.splitlines():
        k, v = line.split()
        if k == "t":
            t = float(v)
        else:
            s[int(k.split(".")[1])] = float(v)
    return t, np.array([s[i] for i in range(len(s))])


def _binding_drive(sol):
    """The demo's calls through the Python binding, the functors as per-step schedules."""
    t = 0.0
    while t < 2.0 - 1e-3 / 10.0:
        t = sol.SolveStep(t, schedule=lambda x: (0.0, 0.0 if x < 1 else 0.5, 0.0))
    t0 = t
    for _ in range(10):
        t = sol.SolveStep(t, schedule=lambda x: TABLE[min(max(int((x - t0) * 10.0), 0), 9)])
    return t


def _write(tmp, name, obj):
    import json
    p = tmp / name
    p.write_text(json.dumps(obj))
    return str(p)


@pytest.mark.gpu
def test_functor18_matches_schedule_path(built_lib, golden18, demo, tmp_path):
    case = {c["name"]: c for c in golden18["cases"]}["hmmwv_acc3_gpu"]
    vj, tj = _write(tmp_path, "v.json", case["vehicle"]), _write(tmp_path, "t.json", case["tire"])
    n = 40
    t_dev, got = _run(demo, 18, vj, tj, n)
    sol = built_lib.d18SolverHalfImplicitGPU(n)
    sol.Construct(vj, tj, n)
    sol.SetTimeStep(1e-3)
    sol.SetKernelSimTime(0.1)
    S, T = built_lib.S, built_lib.T
    s0 = np.zeros(built_lib.S_COUNT)
    s0[S["u"]] = 5.0
    for k in range(4):
        s0[built_lib.S_TIRE0 + k * built_lib.S_TIRE_STRIDE + T["omega"]] = 5.0 / 0.47
    sol.Initialize(s0, n)
    t_bind = _binding_drive(sol)
    want = sol.get_states()[n - 1]
    sol.close()
    assert t_dev == t_bind
    assert np.array_equal(got, want), np.nonzero(got != want)
    assert got[S["x"]] > 5.0  # the vehicle moved


@pytest.mark.gpu
def test_functor11_matches_schedule_path(built_lib, golden11_cases, demo, tmp_path):
    case = {c["name"]: c for c in golden11_cases["cases"]}["hmmwv11_acc3_gpu22"]
    vj, tj = _write(tmp_path, "v.json", case["vehicle"]), _write(tmp_path, "t.json", case["tire"])
    n = 33
    t_dev, got = _run(demo, 11, vj, tj, n)
    sol = built_lib.d11SolverHalfImplicitGPU(n)
    sol.Construct(vj, tj, n)
    sol.SetTimeStep(1e-3)
    sol.SetKernelSimTime(0.1)
    abi = pkg_mod("_abi")
    s0 = np.zeros(abi.S11_COUNT)
    s0[abi.S11["u"]] = 5.0
    for k in range(2):
        s0[abi.S11_TIRE0 + k * abi.S_TIRE_STRIDE + abi.T["omega"]] = 5.0 / 0.47
    sol.Initialize(s0, n)
    t_bind = _binding_drive(sol)
    want = sol.get_states()[n - 1]
    sol.close()
    assert t_dev == t_bind
    assert np.array_equal(got, want), np.nonzero(got != want)


@pytest.mark.gpu
def test_functor24_matches_schedule_path(built_lib, golden24_cases, demo, tmp_path):
    case = {c["name"]: c for c in golden24_cases["cases"]}["hmmwv24_acc3_gpu22"]
    vj, tj = _write(tmp_path, "v.json", case["vehicle"]), _write(tmp_path, "t.json", case["tire"])
    sj = _write(tmp_path, "s.json", case["sus"])
    n = 20
    t_dev, got = _run(demo, 24, vj, tj, sj, n)
    sol = built_lib.d24SolverHalfImplicitGPU(n)
    sol.Construct(vj, tj, sj, n)
    sol.SetTimeStep(1e-3)
    sol.SetKernelSimTime(0.1)
    sol.Initialize(np.zeros(pkg_mod("_abi").C["LFDM24_S_COUNT"]), n)
    t_bind = _binding_drive(sol)
    want = sol.get_states()[n - 1]
    sol.close()
    assert t_dev == t_bind
    assert np.array_equal(got, want), np.nonzero(got != want)
