"""The reference's OWN GPU solvers (their Integrate kernels compiled from the reference sources) on
this GPU, for the 11-, 18- and 24-DOF models: each must reproduce the reference CPU goldens, which
validates the launcher, and the CUDA path is timed against them on the same fleets. Skipped where
the reference cubins were not built (they are built where the reference checkout exists and travel
with the repository as build artefacts)."""
import numpy as np
import pytest

import refgpu_lib as R
from conftest import (case_inputs, case_inputs11, case_inputs24, pkg_mod, rel_err, state_floors, state_floors11,
                      state_floors24)

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not all(R.available(m) for m in (11, 18, 24)),
                                                  reason="reference cubins not built here")]


@pytest.fixture(scope="module")
def launcher():
    return R.build_launcher()


def _check(model, cases, inputs, floors, tol=1e-9):
    for c in cases:
        cls, p, s, tab = inputs(c)
        final, _ = R.run(cls, p[None], tab[None], s[None], model=model, dt=c["dt"], ksim=c["ksim"], tend=c["tend"])
        e = rel_err(final[0], np.array(c["expected_final"]), floors)
        assert e.max() <= tol, (c["name"], float(e.max()), int(e.argmax()))


def test_reference_gpu18_reproduces_goldens(launcher, golden18):
    """HMMWV fixtures, the audi and Sedan rear/front-wheel-drive fixtures and the calm fleet vehicles
    (TMeasy, no throttleMod): the reference's GPU kernel gives its CPU solver's states to 1e-9."""
    by = {c["name"]: c for c in golden18["cases"]}
    names = ["hmmwv_acc3_gpu", "hmmwv_dl4_gpu", "audi_dl4_gpu", "audi_rwd_ls5_gpu", "audi_fwd_ls5_gpu",
             "sedan_rwd_ls5_gpu", "calm_fleet_0", "calm_fleet_1"]
    _check(18, [by[n] for n in names], case_inputs, state_floors())


def test_reference_gpu11_reproduces_goldens(launcher, golden11_cases):
    by = {c["name"]: c for c in golden11_cases["cases"]}
    names = ["hmmwv11_acc3_gpu22", "hmmwv11_dl4_gpu", "audi11_dl4_gpu", "audi11_rwd_ls5_gpu", "audi11_fwd_ls5_gpu",
             "sedan11_rwd_ls5_gpu"]
    _check(11, [by[n] for n in names], case_inputs11, state_floors11())
    # the reference's own GPU test pins, tests/11dof_gpu.cu:76-77 (x within 1 m)
    X = pkg_mod("_abi").S11["x"]
    for name, x in (("hmmwv11_acc3_gpu22", 198.72), ("hmmwv11_dl4_gpu", 104.805)):
        cls, p, s, tab = case_inputs11(by[name])
        final, _ = R.run(cls, p[None], tab[None], s[None], model=11, ksim=2.0, tend=22.0)
        assert abs(final[0, X] - x) < 1.0, (name, final[0, X])


def test_reference_gpu24_reproduces_goldens(launcher, golden24_cases):
    """The Sedan with TMeasy tires and its suspension on the double lane change (a trajectory that
    is insensitive to rounding): 1e-9 on all 212 state fields. The HMMWV fixtures are
    rounding-chaotic (wheel chatter); there the reference's own GPU test pins hold
    (tests/24dof_gpu.cu:56, :103-104: x within 1 m)."""
    by = {c["name"]: c for c in golden24_cases["cases"]}
    _check(24, [by["sedan24_tm_dl4_gpu"]], case_inputs24, state_floors24())
    X = pkg_mod("_abi").S24["x"]
    for name, x in (("hmmwv24_acc3_gpu22", 235.685), ("hmmwv24_dl4_gpu22", 91.5211)):
        cls, p, s, tab = case_inputs24(by[name])
        final, _ = R.run(cls, p[None], tab[None], s[None], model=24, ksim=2.0, tend=22.0)
        assert abs(final[0, X] - x) < 1.0, (name, final[0, X])


def test_reference_gpu_throttle_mod_differs_from_its_cpu_solver(launcher, golden18, built_lib):
    """The reference's GPU driveTorque scales the vehicle's engine map IN PLACE on every call
    (18dof-gpu/dof18_gpu.cu:18-26), so with throttleMod its GPU solver drifts away from its CPU
    solver, which scales a copy (18dof/dof18.cpp:23-29). This library follows the CPU solver: on the
    ART fixture it matches the CPU golden to 1e-9 while the reference's GPU kernel does not."""
    c = {x["name"]: x for x in golden18["cases"]}["art_ls5_gpu"]
    cls, p, s, tab = case_inputs(c)
    exp = np.array(c["expected_final"])
    ref_gpu, _ = R.run(cls, p[None], tab[None], s[None], model=18, dt=c["dt"], ksim=c["ksim"], tend=c["tend"])
    e_ref = rel_err(ref_gpu[0], exp, state_floors()).max()
    sol = built_lib.d18SolverHalfImplicitGPU(1)
    sol.construct_class(cls, p[None])
    sol.set_driver_tables(tab[None])
    sol.set_states(s[None])
    sol.SetKernelSimTime(c["ksim"])
    sol.SetEndTime(c["tend"])
    sol.Solve()
    e_ours = rel_err(sol.get_states()[0], exp, state_floors()).max()
    sol.close()
    print(f"ART throttleMod: reference GPU vs its CPU solver {e_ref:.2e}, this library vs the CPU solver {e_ours:.2e}")
    assert e_ours <= 1e-9
    assert e_ref > 1e-6


def _ours_rate(built_lib, model, f, n, ksim, windows, output_hz):
    import torch

    sol = getattr(built_lib, f"d{model}SolverHalfImplicitGPU")(n)
    sol.construct_class(f["cls"][0], f["params"])
    sol.set_driver_tables(f["tables"])
    sol.set_states(f["states"])
    sol.SetKernelSimTime(ksim)
    sol.SetEndTime(windows * ksim)
    nch = {11: built_lib.RESP11, 18: built_lib.RESP18, 24: built_lib.RESP24}[model]
    spw = int(round(ksim * output_hz))
    buf = torch.empty(spw * nch * n, dtype=torch.float64, device="cuda")
    sol.set_response_device(buf.data_ptr(), buf.numel(), output_hz)
    sol.solve_range(-0.5 * ksim, 0.5 * ksim)
    sol.solve_range(0.5 * ksim, (windows - 0.5) * ksim)
    ms, launches = sol.last_kernel_ms()
    sol.close()
    return n * int(round(ksim / 1e-3)) * launches / (ms * 1e-3)


@pytest.mark.parametrize("model,n,ksim,windows,hz,factor", [(18, 300_000, 1.0, 3, 100.0, 2.0),
                                                           (11, 1024, 1.0, 3, 100.0, 1.0),
                                                           (24, 100_000, 1.0, 3, 100.0, 1.5)])
def test_throughput_vs_reference_gpu_kernel(launcher, built_lib, model, n, ksim, windows, hz, factor):
    """The seeded SUV fleets with outputs every 10 ms, 1 s windows; windows 2 and 3 timed for both
    (the reference at 16 and 32 threads per block, its best counts). The 18-DOF model at 300,000
    vehicles must run at least 2x as fast as the reference's GPU solver."""
    fleet = pkg_mod("fleet")
    gen = {11: fleet.fleet11, 18: fleet.fleet18, 24: fleet.fleet24}[model]
    f = gen(n, seed=20261203, horizon=windows * ksim)
    res = {}
    for tpb in (32, 16):
        _, ms = R.run(f["cls"][0], f["params"], f["tables"], f["states"], model=model, ksim=ksim,
                      tend=windows * ksim, dtout=1.0 / hz, tpb=tpb)
        res[f"reference_tpb{tpb}"] = n * 1000 * (windows - 1) / (sum(ms[1:]) * 1e-3)
    res["ours"] = _ours_rate(built_lib, model, f, n, ksim, windows, hz)
    best_ref = max(res["reference_tpb32"], res["reference_tpb16"])
    ratio = res["ours"] / best_ref
    msg = f"{model}-DOF, {n} vehicles: " + str({k: f"{v:.3e}" for k, v in res.items()}) + f", ratio {ratio:.2f}x"
    print(msg)
    assert ratio >= factor, msg
