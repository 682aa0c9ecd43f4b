"""The oracle (CPU restatement, oracle/lfdm_oracle.c) against the reference's own CPU solver.

tests/golden/golden18.json holds outputs of the reference's d18SolverHalfImplicit compiled from
its sources (tests/golden/make_golden.py). The oracle must reproduce them: bit for bit on x86-64
(same compiler rules, no FMA contraction), and to 1e-12 per state elsewhere (libm may differ in
the last bit on other architectures).
"""
import platform

import numpy as np
import pytest

import oracle_lib as O
from conftest import case_inputs, rel_err, state_floors, RESP_FLOORS

EXACT = platform.machine() in ("x86_64", "AMD64")


def _run_case(case, dtout=0.0):
    cls, p, s, tab = case_inputs(case)
    sched = 0 if case["ksim"] == 0 else 1
    return O.run18([cls], [0], p[None, :], s[None, :], [tab], tire_type=case["tire_type"], dt=case["dt"],
                   tend=case["tend"], ksim=case["ksim"] or 1.0, schedule=sched, dtout=dtout)


def test_golden_final_states(golden18):
    fl = state_floors()
    for case in golden18["cases"]:
        st, _ = _run_case(case)
        exp = np.array(case["expected_final"])
        if EXACT:
            assert np.array_equal(st[0], exp), case["name"]
        else:
            assert rel_err(st[0], exp, fl).max() <= 1e-12, case["name"]


def test_reference_test_goldens(golden18):
    """The reference's own test pins (tests/18dof.cpp:38, tests/18dof_gpu.cu:52, :94)."""
    by = {c["name"]: c for c in golden18["cases"]}
    assert abs(by["hmmwv_acc3_cpu"]["expected_final"][0] - 88.5335) < 1.0
    assert abs(by["hmmwv_acc3_gpu"]["expected_final"][0] - 88.5335) < 1.0
    assert abs(by["hmmwv_dl4_gpu"]["expected_final"][0] - 106.548) < 1.0
    # TMeasyNr with high-level tire parameters: tests/18dof.cpp dof18HiNr (114.973)
    assert abs(by["sedan_nr_acc05_cpu"]["expected_final"][0] - 114.973) < 1.0
    st, _ = _run_case(by["sedan_nr_acc05_cpu"])
    assert st[0, 0] == pytest.approx(114.973, abs=1e-3)
    st, _ = _run_case(by["hmmwv_acc3_cpu"])
    assert st[0, 0] == pytest.approx(88.533467841729632, abs=1e-9)


def test_golden_sampled_trajectories(golden18):
    """Sampled trajectories (GPU schedule) through the oracle's SoA response buffer."""
    for case in golden18["cases"]:
        if case["ksim"] == 0:
            continue
        dtout = case["sample"] * case["dt"]
        _, resp = _run_case(case, dtout=dtout)
        exp = np.array(case["expected_samples"])  # [k][step, t, 12 channels]
        got = resp[: len(exp), :, 0]
        assert np.isfinite(got).all()
        e = rel_err(got, exp[:, 1:], RESP_FLOORS)
        assert e.max() <= (0.0 if EXACT else 1e-12), (case["name"], e.max())


def test_cpu_and_gpu_schedules_agree(golden18):
    """The two time schedules differ only in how t is rounded; trajectories agree to ~1e-12."""
    by = {c["name"]: c for c in golden18["cases"]}
    a = by["hmmwv_acc3_cpu"]["expected_final"]
    b = by["hmmwv_acc3_gpu"]["expected_final"]
    assert rel_err(np.array(a), np.array(b), state_floors()).max() < 1e-9


def test_driver_input_edges():
    rows = np.array([[0.0, 0.0, 0.0, 0.0], [1.0, 1.0, 0.5, 0.0], [1.0, 2.0, 0.5, 0.0], [3.0, 0.0, 1.0, 1.0]])
    assert np.array_equal(O.driver_input(-1.0, rows), rows[0])
    assert np.array_equal(O.driver_input(0.0, rows), rows[0])
    assert np.array_equal(O.driver_input(3.0, rows), rows[3])
    assert np.array_equal(O.driver_input(5.0, rows), rows[3])
    # duplicate time: lower_bound picks the first row with t_k >= t, so t=1 interpolates on [0,1]
    np.testing.assert_array_equal(O.driver_input(1.0, rows), [1.0, 1.0, 0.5, 0.0])
    # past the duplicate: segment [1 (second row), 3]
    np.testing.assert_allclose(O.driver_input(2.0, rows), [2.0, 1.0, 0.75, 0.5])


def test_map_lookup_edges():
    m = [[0.0, 1.0], [1.0, 3.0], [2.0, 2.0]]
    assert O.map_y(m, -5) == 1.0
    assert O.map_y(m, 7) == 2.0
    assert O.map_y(m, 0.5) == 2.0
    assert O.map_y(m, 1.0) == 3.0
    assert O.map_y(m, 1.5) == 2.5


def test_oracle_threads_deterministic():
    fleet = __import__("conftest").pkg_mod("fleet")
    f = fleet.fleet18(64, seed=7, horizon=2.0)
    a, _ = O.run18(f["cls"], f["class_of"], f["params"], f["states"], f["tables"], tend=2.0, ksim=1.0, nthreads=1)
    b, _ = O.run18(f["cls"], f["class_of"], f["params"], f["states"], f["tables"], tend=2.0, ksim=1.0, nthreads=4)
    assert np.array_equal(a, b)
