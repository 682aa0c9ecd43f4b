"""Branches of the reference that only some vehicles take, held to 1e-9 over whole trajectories.

The golden cases below come from the reference's own CPU solvers (tests/golden/make_golden.py) on
the reference's data files:
  * ART (18dof-gpu/data/json/ART): steering map (`nonLinearSteer`, getMapY in vehToTireTransform,
    tireToVehTransform and computeTireRHS, 18dof-gpu/dof18_gpu.cu:71-109, :152-185, :382-391),
    `throttleMod` (driveTorque's scaled engine map, the CPU solver's copy semantics of
    18dof/dof18.cpp:23-29), one gear and no torque converter;
  * Sedan and audi `vehicle_RWD.json`: the 2WD torque split of computePowertrainRHS
    (18dof-gpu/dof18_gpu.cu:664-839) to the rear axle; an audi variant with `rearWheels` false
    drives the front axle; audi `vehicle.json` (4WD, its own tire file);
  * the HMMWV and Sedan vehicles with `throttleMod` and a steering map switched on (the scaled map
    with a torque converter, and with TMeasyNr tires);
  * the calm synthetic fleet (fleet.fleet18_calm): the configured SUV's parameter jitter with an
    HMMWV-class wheel inertia, whose trajectories are insensitive to rounding.
Every one of these trajectories is insensitive to rounding (the reference algorithm compiled with
fused multiply-add contraction stays within 1e-13 of its plain build along all of them), so no
sensitivity envelope is used: per state |gpu - ref| <= 1e-9 * max(|ref|, s_k), at every sample
and for the full final state.

The 24-DOF fixtures whose trajectories are rounding-chaotic (the HMMWV with a steering map and the
Sedan on the long sine, where the wheels chatter at standstill) are held to the reference's
sensitivity envelope by test_gpu_parity24.py; the others are held to 1e-9 here.
"""
import os

import numpy as np
import pytest

import oracle_lib as O
from conftest import (RESP11_FLOORS, RESP24_FLOORS, RESP_FLOORS, pkg_mod, rel_err, state_floors, state_floors11,
                      state_floors24)
from test_gpu_parity11 import _run_group as run_group11
from test_gpu_parity18 import _run_golden_group as run_group18
from test_gpu_parity24 import _run_group as run_group24

pytestmark = pytest.mark.gpu
RTOL = 1e-9
NT = os.cpu_count() or 1

BRANCH18 = ("art_ls5_gpu", "audi_dl4_gpu", "audi_rwd_ls5_gpu", "audi_fwd_ls5_gpu", "sedan_rwd_ls5_gpu",
            "sedan_rwd_nr_acc05_gpu", "hmmwv_tmod_nls_ls5_gpu", "sedan_tmod_nls_nr_dl4_gpu") + \
    tuple(f"calm_fleet_{i}" for i in range(6))
BRANCH11 = ("art11_ls5_gpu", "audi11_dl4_gpu", "audi11_rwd_ls5_gpu", "audi11_fwd_ls5_gpu", "sedan11_rwd_ls5_gpu",
            "sedan11_rwd_nr_acc05_gpu", "hmmwv11_tmod_nls_ls5_gpu", "sedan11_tmod_nls_nr_dl4_gpu")
BRANCH24 = ("sedan24_rwd_nr_acc05_gpu", "sedan24_tmod_nls_nr_dl4_gpu", "sedan24_tm_dl4_gpu")


def _groups(cases, names):
    by = {c["name"]: c for c in cases}
    g = {}
    for n in names:
        c = by[n]
        g.setdefault((c["ksim"], c["tend"], c["sample"], c["tire_type"]), []).append(c)
    return g


def _check(cases, final, resp, floors, resp_floors):
    worst = []
    for i, c in enumerate(cases):
        e = rel_err(final[i], np.array(c["expected_final"]), floors)
        assert e.max() <= RTOL, (c["name"], "final", float(e.max()), int(e.argmax()))
        exp = np.array(c["expected_samples"])
        er = rel_err(resp[: len(exp), :, i], exp[:, 1:], resp_floors)
        assert er.max() <= RTOL, (c["name"], "samples", float(er.max()), int(er.max(axis=1).argmax()))
        worst.append((c["name"], float(max(e.max(), er.max()))))
    return worst


def test_branch_fixtures18(built_lib, golden18):
    worst = []
    for (ksim, tend, sample, tt), cases in _groups(golden18["cases"], BRANCH18).items():
        final, resp = run_group18(built_lib, cases, ksim, tend, tt, 1.0 / (sample * cases[0]["dt"]))
        worst += _check(cases, final, resp, state_floors(), RESP_FLOORS)
    print("18-DOF branch fixtures, largest relative error per case:", worst)


def test_branch_fixtures11(built_lib, golden11_cases):
    worst = []
    for (ksim, tend, sample, _tt), cases in _groups(golden11_cases["cases"], BRANCH11).items():
        final, resp = run_group11(built_lib, cases, ksim, tend, 1.0 / (sample * cases[0]["dt"]))
        worst += _check(cases, final, resp, state_floors11(), RESP11_FLOORS)
    print("11-DOF branch fixtures, largest relative error per case:", worst)


def test_branch_fixtures24(built_lib, golden24_cases):
    worst = []
    for (ksim, tend, sample, _tt), cases in _groups(golden24_cases["cases"], BRANCH24).items():
        final, resp = run_group24(built_lib, cases, ksim, tend, 1.0 / (sample * cases[0]["dt"]))
        worst += _check(cases, final, resp, state_floors24(), RESP24_FLOORS)
    print("24-DOF branch fixtures, largest relative error per case:", worst)


def test_calm_fleet_whole_horizon(built_lib):
    """4,096 vehicles of the calm fleet over the 10 s horizon in 1 s windows with 10 ms outputs: every
    vehicle's full final state and every sampled response within 1e-9 of the oracle (which is pinned
    bit for bit to the reference's CPU solver, calm_fleet_* goldens included)."""
    fleet = pkg_mod("fleet")
    n, horizon, freq = 4096, 10.0, 100.0
    f = fleet.fleet18_calm(n, horizon=horizon)
    sol = built_lib.d18SolverHalfImplicitGPU(n)
    sol.construct_class(f["cls"][0], f["params"])
    sol.set_driver_tables(f["tables"])
    sol.set_states(f["states"])
    sol.SetKernelSimTime(1.0)
    sol.SetEndTime(horizon)
    nsamp = int(round(horizon * freq)) + 4
    resp = np.full((nsamp, 13, n), np.nan)
    sol.set_response_buffer(resp, freq)
    sol.Solve()
    got = sol.get_states()
    sol.close()
    ref, rresp = O.run18(f["cls"], f["class_of"], f["params"], f["states"], f["tables"], tend=horizon, ksim=1.0,
                         schedule=1, dtout=1.0 / freq, nthreads=NT)
    e = rel_err(got, ref, state_floors()).max(axis=1)
    ns = int(round(horizon * freq))
    er = rel_err(np.moveaxis(resp[:ns], 2, 1), np.moveaxis(rresp[:ns], 2, 1), RESP_FLOORS).max(axis=(0, 2))
    print(f"calm fleet: final max {e.max():.2e} median {np.median(e):.2e}; responses max {er.max():.2e}")
    assert e.max() <= RTOL, (float(e.max()), int(e.argmax()))
    assert er.max() <= RTOL, (float(er.max()), int(er.argmax()))
