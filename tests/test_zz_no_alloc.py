"""lfdm_step18_noalloc on the GPU: the stepping entry point for callers that cannot allocate device
memory on their call path (its scratch is one static device array).

* two calls in a row on device-resident vehicles, bit for bit the solver API's SolveStep with the same
  per-vehicle controls, and within rounding of the oracle (or within the reference algorithm's own
  sensitivity near branch points); with TMeasy and with TMeasyNr tires;
* exactly LFDM_NOALLOC_MAX_VEHICLES vehicles, and one more rejected with the capacity error;
* no device memory allocated by a call: torch's allocator count and the driver's free-memory figure
  are unchanged across a synchronised call;
* a non-finite state is reported as LFDM_ERR_NUMERIC, as the solver reports it;
* the entry point still works after the device's primary context was reset between two calls (its
  scratch address is looked up at every call), in a child process without torch.

Named so that pytest collects it last; it also passes alone in a fresh process.
"""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle_lib as O
from conftest import ROOT, TESTS, case_inputs, pkg_mod, rel_err, state_floors

pytestmark = pytest.mark.gpu


def _fleet(n, seed):
    f = pkg_mod("fleet").fleet18(n, seed=seed, horizon=2.0)
    rng = np.random.default_rng(seed)
    ctl = np.stack([rng.uniform(-0.3, 0.3, n), rng.uniform(0.0, 1.0, n), np.where(rng.random(n) < 0.2, 0.5, 0.0)],
                   axis=1)
    return f, ctl


def _solver_two_windows(lfdm, cls, params, states, ctl, tire_type=0):
    """The same two windows of 0.02 s through the solver API; returns (states, steps0, t1, steps1)."""
    n = params.shape[0]
    sol = lfdm.d18SolverHalfImplicitGPU(n)
    sol.construct_class(cls, params, tire_type)
    sol.set_states(states)
    sol.SetKernelSimTime(0.02)
    steps0 = len(sol.window_times(0.0))
    t1 = sol.SolveStep(0.0, ctl[:, 0], ctl[:, 1], ctl[:, 2])
    steps1 = len(sol.window_times(t1))
    sol.SolveStep(t1, ctl[:, 0], ctl[:, 1], ctl[:, 2])
    want = sol.get_states()
    sol.close()
    return want, steps0, t1, steps1


def _noalloc_two_windows(lfdm, torch, cls, params, states, ctl, steps0, t1, steps1, tire_type=0):
    dev = torch.device("cuda", 0)
    n = params.shape[0]
    p = torch.from_numpy(np.ascontiguousarray(params)).to(dev)
    s = torch.from_numpy(np.ascontiguousarray(states)).to(dev)
    c = [torch.from_numpy(np.ascontiguousarray(ctl[:, k])).to(dev) for k in range(3)]
    stream = torch.cuda.current_stream(dev)
    torch.cuda.synchronize(dev)
    args = (cls, p.data_ptr(), s.data_ptr(), c[0].data_ptr(), c[1].data_ptr(), c[2].data_ptr(), n)
    lfdm.step18_noalloc(*args, 0.0, 1e-3, steps0, stream.cuda_stream, tire_type=tire_type)
    lfdm.step18_noalloc(*args, t1, 1e-3, steps1, stream.cuda_stream, tire_type=tire_type)
    torch.cuda.synchronize(dev)
    return s.cpu().numpy()


def test_two_calls_in_a_row_match_solver_and_oracle(built_lib):
    torch = pytest.importorskip("torch")
    n = 3000  # not a multiple of the block size
    f, ctl = _fleet(n, seed=11)
    cls = f["cls"][0]
    want, steps0, t1, steps1 = _solver_two_windows(built_lib, cls, f["params"], f["states"], ctl)
    got = _noalloc_two_windows(built_lib, torch, cls, f["params"], f["states"], ctl, steps0, t1, steps1)
    assert np.array_equal(got, want)

    # oracle: rounding-level agreement, or within 100x the reference algorithm's sensitivity where a
    # vehicle sits near a branch point (the largest deviation among its FMA-contracted build and
    # runs from u moved by +-1e-15 max(|u|, 1 m/s))
    def two_windows(s0, **kw):
        st = s0
        for t0 in (0.0, t1):
            st, _ = O.run18(f["cls"], f["class_of"], f["params"], st, ctl=ctl, t0=t0, ksim=0.02, schedule=2,
                            nthreads=8, **kw)
        return st

    fl = state_floors()
    ref = two_windows(f["states"])
    runs = [two_windows(f["states"], fma=True)]
    U = pkg_mod("_abi").S["u"]
    for eps in (1e-15, -1e-15):
        s2 = f["states"].copy()
        s2[:, U] += eps * np.maximum(np.abs(s2[:, U]), 1.0)  # relative, floored at 1 m/s (u0 may be 0)
        runs.append(two_windows(s2))
    env = np.max([rel_err(r, ref, fl).max(axis=1) for r in runs], axis=0)
    e = rel_err(got, ref, fl).max(axis=1)
    assert (e <= np.maximum(1e-12, 100 * env)).all(), (float(e.max()), int(e.argmax()))
    assert (e[env <= 1e-13] <= 1e-12).all()


def test_tmeasy_nr_matches_solver(built_lib):
    """The reference's Sedan with TMeasyNr tires (high-level tire parameters), 512 vehicles at
    seeded speeds and controls: bit for bit the solver API."""
    torch = pytest.importorskip("torch")
    with open(os.path.join(TESTS, "golden", "golden18.json")) as fh:
        case = {c["name"]: c for c in json.load(fh)["cases"]}["sedan_nr_acc05_gpu"]
    cls, p, s, _ = case_inputs(case)
    n = 512
    rng = np.random.default_rng(5)
    params = np.repeat(p[None], n, axis=0)
    states = pkg_mod("fleet").states_at_speed(cls, params, rng.uniform(0.5, 25.0, n))
    ctl = np.stack([rng.uniform(-0.5, 0.5, n), rng.uniform(0.0, 1.0, n), np.where(rng.random(n) < 0.3, 0.4, 0.0)],
                   axis=1)
    want, steps0, t1, steps1 = _solver_two_windows(built_lib, cls, params, states, ctl, tire_type=1)
    got = _noalloc_two_windows(built_lib, torch, cls, params, states, ctl, steps0, t1, steps1, tire_type=1)
    assert np.array_equal(got, want)
    assert not np.array_equal(got, states)


def test_full_capacity_and_no_device_allocation(built_lib):
    """Exactly LFDM_NOALLOC_MAX_VEHICLES vehicles (bit for bit the solver API), and no device memory
    allocated by a call once the library is loaded and the buffers exist."""
    torch = pytest.importorskip("torch")
    n = built_lib.NOALLOC_MAX_VEHICLES
    f, ctl = _fleet(n, seed=3)
    cls = f["cls"][0]
    want, steps0, t1, steps1 = _solver_two_windows(built_lib, cls, f["params"], f["states"], ctl)
    dev = torch.device("cuda", 0)
    p = torch.from_numpy(np.ascontiguousarray(f["params"])).to(dev)
    s = torch.from_numpy(np.ascontiguousarray(f["states"])).to(dev)
    c = [torch.from_numpy(np.ascontiguousarray(ctl[:, k])).to(dev) for k in range(3)]
    args = (cls, p.data_ptr(), s.data_ptr(), c[0].data_ptr(), c[1].data_ptr(), c[2].data_ptr(), n)
    stream = torch.cuda.current_stream(dev).cuda_stream
    # warm-up on a copy of the states: loads the library's module (and with it the static scratch
    # array) if no earlier call in this process did
    s_warm = s.clone()
    built_lib.step18_noalloc(cls, p.data_ptr(), s_warm.data_ptr(), c[0].data_ptr(), c[1].data_ptr(), c[2].data_ptr(),
                             n, 0.0, 1e-3, steps0, stream)
    torch.cuda.synchronize(dev)
    alloc0 = torch.cuda.memory_allocated(dev)
    free0, _ = torch.cuda.mem_get_info(dev)
    built_lib.step18_noalloc(*args, 0.0, 1e-3, steps0, stream)
    torch.cuda.synchronize(dev)
    free1, _ = torch.cuda.mem_get_info(dev)
    built_lib.step18_noalloc(*args, t1, 1e-3, steps1, stream)
    torch.cuda.synchronize(dev)
    free2, _ = torch.cuda.mem_get_info(dev)
    assert torch.cuda.memory_allocated(dev) == alloc0
    assert free0 == free1 == free2, (free0, free1, free2)
    assert np.array_equal(s.cpu().numpy(), want)


def test_non_finite_state_reported(built_lib):
    torch = pytest.importorskip("torch")
    n = 64
    f, ctl = _fleet(n, seed=4)
    st = f["states"].copy()
    st[17, pkg_mod("_abi").S["u"]] = np.nan
    dev = torch.device("cuda", 0)
    p = torch.from_numpy(np.ascontiguousarray(f["params"])).to(dev)
    s = torch.from_numpy(st).to(dev)
    c = [torch.from_numpy(np.ascontiguousarray(ctl[:, k])).to(dev) for k in range(3)]
    with pytest.raises(built_lib.LfdmError, match="non-finite"):
        built_lib.step18_noalloc(f["cls"][0], p.data_ptr(), s.data_ptr(), c[0].data_ptr(), c[1].data_ptr(),
                                 c[2].data_ptr(), n, 0.0, 1e-3, 10, torch.cuda.current_stream(dev).cuda_stream)
    out = s.cpu().numpy()
    assert np.isfinite(np.delete(out, 17, axis=0)[:, :15]).all()
    # the next call on finite states succeeds (the status words are cleared per call)
    s2 = torch.from_numpy(np.ascontiguousarray(f["states"])).to(dev)
    built_lib.step18_noalloc(f["cls"][0], p.data_ptr(), s2.data_ptr(), c[0].data_ptr(), c[1].data_ptr(),
                             c[2].data_ptr(), n, 0.0, 1e-3, 10, torch.cuda.current_stream(dev).cuda_stream)


_RESET_CHILD = r"""
import ctypes, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import importlib
lfdm = importlib.import_module("low-fidelity-dynamic-models_gb300")
fleet = importlib.import_module("low-fidelity-dynamic-models_gb300.fleet")
L = lfdm.lib()                                   # loads the CUDA runtime liblfdm.so links against
with open("/proc/self/maps") as fh:              # ... which is the one to reset
    rt_path = next(line.split()[-1] for line in fh if "libcudart.so" in line)
rt = ctypes.CDLL(rt_path)
rt.cudaMalloc.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t]
rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
rt.cudaFree.argtypes = [ctypes.c_void_p]
n = 300
f = fleet.fleet18(n, seed=21, horizon=1.0)
ctl = np.ascontiguousarray(np.stack([np.full(n, 0.1), np.full(n, 0.5), np.zeros(n)]))

def dev_copy(a):
    p = ctypes.c_void_p()
    assert rt.cudaMalloc(ctypes.byref(p), a.nbytes) == 0
    assert rt.cudaMemcpy(p, a.ctypes.data, a.nbytes, 1) == 0
    return p

def one_call():
    bufs = [dev_copy(np.ascontiguousarray(f["params"])), dev_copy(np.ascontiguousarray(f["states"]))]
    bufs += [dev_copy(ctl[k].copy()) for k in range(3)]
    lfdm.step18_noalloc(f["cls"][0], *[b.value for b in bufs], n, 0.0, 1e-3, 20)
    out = np.empty_like(f["states"])
    assert rt.cudaMemcpy(out.ctypes.data, bufs[1], out.nbytes, 2) == 0
    for b in bufs:
        rt.cudaFree(b)
    return out

a = one_call()
assert rt.cudaDeviceReset() == 0
b = one_call()
assert np.array_equal(a, b) and not np.array_equal(a, f["states"])
print("reset ok")
"""


def test_after_device_reset(built_lib):
    """Two calls with a reset of the device's primary context between them give the same states:
    the scratch address is looked up at every call, not cached across contexts."""
    r = subprocess.run([sys.executable, "-c", _RESET_CHILD, ROOT], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "reset ok" in r.stdout, r.stdout + r.stderr


def test_capacity_and_arguments_rejected(built_lib):
    torch = pytest.importorskip("torch")
    cls, p = pkg_mod("fleet").suv18()
    big = built_lib.NOALLOC_MAX_VEHICLES + 1
    with pytest.raises(built_lib.LfdmError, match="capacity"):
        built_lib.step18_noalloc(cls, 1, 1, 1, 1, 1, big, 0.0, 1e-3, 10)
    x = torch.zeros(8, dtype=torch.float64, device="cuda")
    with pytest.raises(built_lib.LfdmError, match="null"):
        built_lib.step18_noalloc(cls, 0, x.data_ptr(), x.data_ptr(), x.data_ptr(), x.data_ptr(), 1, 0.0, 1e-3, 10)
    with pytest.raises(built_lib.LfdmError, match="dt"):
        built_lib.step18_noalloc(cls, x.data_ptr(), x.data_ptr(), x.data_ptr(), x.data_ptr(), x.data_ptr(), 1, 0.0,
                                 -1.0, 10)
    assert built_lib.NOALLOC_SCRATCH_BYTES == 19669504
