"""11-DOF oracle (oracle/lfdm_oracle.c) against the reference's own 11-DOF CPU solver outputs in
tests/golden/golden11.json (bit for bit on x86-64), including the reference test pins."""
import json
import os
import platform

import numpy as np
import pytest

import oracle_lib as O
from conftest import TESTS, pkg_mod

EXACT = platform.machine() in ("x86_64", "AMD64")


@pytest.fixture(scope="module")
def golden11():
    with open(os.path.join(TESTS, "golden", "golden11.json")) as f:
        return json.load(f)


def inputs11(case):
    params = pkg_mod("params")
    cls, p = params.vehicle_from_json(case["vehicle"], case["tire"], case["tire_type"], model=11)
    return cls, p, np.array(case["state"]), np.array(case["driver"])


def run_case(case, dtout=0.0):
    cls, p, s, tab = inputs11(case)
    sched = 0 if case["ksim"] == 0 else 1
    return O.run18([cls], [0], p[None], s[None], [tab], tire_type=case["tire_type"], dt=case["dt"], tend=case["tend"],
                   ksim=case["ksim"] or 1.0, schedule=sched, dtout=dtout, model=11)


def test_golden11_final_states(golden11):
    for case in golden11["cases"]:
        st, _ = run_case(case)
        exp = np.array(case["expected_final"])
        if EXACT:
            assert np.array_equal(st[0], exp), case["name"]
        else:
            assert np.allclose(st[0], exp, rtol=1e-12, atol=1e-12), case["name"]


def test_golden11_trajectories(golden11):
    for case in golden11["cases"]:
        if case["ksim"] == 0:
            continue
        _, resp = run_case(case, dtout=case["sample"] * case["dt"])
        exp = np.array(case["expected_samples"])
        got = resp[: len(exp), :, 0]
        if EXACT:
            assert np.array_equal(got, exp[:, 1:]), case["name"]
        else:
            assert np.allclose(got, exp[:, 1:], rtol=1e-12, atol=1e-12), case["name"]


def test_reference_11dof_test_pins(golden11):
    """tests/11dof_gpu.cu:38 (70.6758) and :76-77 (198.72 / 104.805), +-1 m in the reference."""
    by = {c["name"]: c for c in golden11["cases"]}
    assert abs(by["hmmwv11_acc3_cpu"]["expected_final"][0] - 70.6758) < 1
    assert abs(by["hmmwv11_acc3_gpu22"]["expected_final"][0] - 198.72) < 1
    assert abs(by["hmmwv11_dl4_gpu"]["expected_final"][0] - 104.805) < 1
    # TMeasyNr with high-level tire parameters: tests/11dof.cpp dof11HiNr (115.1)
    assert abs(by["sedan11_nr_acc05_cpu"]["expected_final"][0] - 115.1) < 1
