"""The oracle's restatement of PerturbRhsFun and of IntegrateStepWithJacobian's central differences
(oracle/lfdm_oracle.c: oracle_rhs, oracle_jacobian_fd) against the Jacobians the reference's own CPU
solvers print at the final state of golden cases (tests/golden/golden{11,18,24}.json, written by
tests/golden/make_golden.py through oracle/refrun*.cpp): bit for bit on x86-64, to 1e-9 elsewhere
(libm may round differently in the last bit, which a difference quotient amplifies).

The reference's 24-DOF TMeasyNr PerturbRhsFun (24dof/dof24_halfImplicit.cpp:836-878) evaluates
default-constructed states without unpacking the perturbed vector, so its state Jacobian is
identically zero; that case is recorded to show it and is not a pin of the restatement, which
unpacks the states for both tire types."""
import json
import os
import platform

import numpy as np
import pytest

import oracle_lib as O
from conftest import TESTS, case_inputs, case_inputs11, case_inputs24

EXACT = platform.machine() in ("x86_64", "AMD64")
INPUTS = {11: case_inputs11, 18: case_inputs, 24: case_inputs24}


def _cases(model):
    with open(os.path.join(TESTS, "golden", f"golden{model}.json")) as f:
        return [c for c in json.load(f)["cases"] if "jacobian" in c]


def _check(got, exp, name):
    if EXACT:
        assert np.array_equal(got, exp), (name, np.argwhere(got != exp)[:5].tolist())
    else:
        scale = np.maximum(np.abs(exp).max(axis=1, keepdims=True), 1e-300)
        assert np.all(np.abs(got - exp) <= 1e-9 * np.maximum(np.abs(exp), 1e-6 * scale)), name


@pytest.mark.parametrize("model", [11, 18, 24])
def test_fd_jacobians_match_the_reference(model):
    cases = _cases(model)
    assert len(cases) >= 3
    checked = 0
    for case in cases:
        if model == 24 and case["tire_type"] == 1:
            continue
        cls, p, _, _ = INPUTS[model](case)
        jac = case["jacobian"]
        js, jc = O.jacobian_fd(model, case["tire_type"], cls, p, np.array(case["expected_final"]), jac["controls"])
        ny = jac["ny"]
        assert js.shape == (ny, ny)
        _check(js, np.array(jac["state"]).reshape(ny, ny), case["name"])
        _check(jc, np.array(jac["control"]).reshape(ny, 2), case["name"])
        checked += 1
    assert checked >= 3


def test_reference_24dof_nr_perturbation_ignores_the_states():
    (case,) = [c for c in _cases(24) if c["tire_type"] == 1]
    jac = case["jacobian"]
    assert jac["ny"] == 27 and not np.any(jac["state"])
    cls, p, _, _ = case_inputs24(case)
    js, _ = O.jacobian_fd(24, 1, cls, p, np.array(case["expected_final"]), jac["controls"])
    assert np.count_nonzero(js) > 50  # the restatement unpacks the perturbed states


@pytest.mark.parametrize("model,tire_type", [(11, 0), (11, 1), (18, 0), (18, 1), (24, 0), (24, 1)])
def test_fd_jacobian_is_the_difference_quotient_of_oracle_rhs(model, tire_type):
    """The Jacobian loop against difference quotients of oracle_rhs built here, at the full state
    (full_point) of a golden case; and the reference's packed sizes."""
    cases = [c for c in _cases(model) if c["tire_type"] == tire_type] or _cases(model)
    case = cases[0]
    cls, p, _, _ = INPUTS[model](case)
    s = np.array(case["expected_final"])
    ctl = case["jacobian"]["controls"]
    js, jc = O.jacobian_fd(model, tire_type, cls, p, s, ctl, full_point=True)
    ny = js.shape[0]
    tc = bool(cls.tcbool)
    sizes = {(11, 0): 12, (11, 1): 8, (18, 0): 20, (18, 1): 12, (24, 0): 35, (24, 1): 27}
    assert ny == sizes[(model, tire_type)] + tc
    # y from the Jacobian's own evaluation point: a zero perturbation of the identity
    y = _pack(model, tire_type, tc, s)
    assert len(y) == ny
    for i in (0, ny // 2, ny - 1):
        d = max(abs(y[i] * 1e-3), 1e-3 if abs(y[i] * 1e-3) < 1e-8 else 0.0)
        yp, ym = y.copy(), y.copy()
        yp[i] += d
        ym[i] -= d
        col = (O.rhs(model, tire_type, cls, p, yp, ctl, s) - O.rhs(model, tire_type, cls, p, ym, ctl, s)) / (2 * d)
        assert np.array_equal(col, js[:, i])


def _pack(model, tire_type, tc, s):
    """packY of a flat state, written out here from the reference's pack order."""
    abi = __import__("conftest").pkg_mod("_abi")
    C, S, T = abi.C, abi.S, abi.T
    nr = tire_type == 1
    y = []
    if model == 18:
        tire = lambda k, f: s[abi.S_TIRE0 + k * C["LFDM_S_TIRE_STRIDE"] + T[f]]
        if not nr:
            for k in range(4):
                y += [tire(k, "xe"), tire(k, "ye")]
        y += [tire(k, "omega") for k in range(4)]
        y += [s[S["crankomega"]]] if tc else []
        y += [s[S[f]] for f in ("x", "y", "u", "v", "psi", "wz", "phi", "wx")]
    elif model == 11:
        tire = lambda k, f: s[C["LFDM11_S_TIRE0"] + k * C["LFDM_S_TIRE_STRIDE"] + T[f]]
        if not nr:
            for k in range(2):
                y += [tire(k, "xe"), tire(k, "ye")]
        y += [tire(k, "omega") for k in range(2)]
        y += [s[C["LFDM11_S_CRANKOMEGA"]]] if tc else []
        y += [s[C[f"LFDM11_S_{f}"]] for f in ("X", "Y", "U", "V", "PSI", "WZ")]
    else:
        tire = lambda k, f: s[C["LFDM24_S_TIRE0"] + k * C["LFDM24_T_COUNT"] + C[f"LFDM24_T_{f}"]]
        sus = lambda k, f: s[C["LFDM24_S_SUS0"] + k * C["LFDM24_SUS_COUNT"] + C[f"LFDM24_SUS_{f}"]]
        for k in range(4):
            y += ([] if nr else [tire(k, "XE"), tire(k, "YE")]) + [tire(k, "XT")]
        y += [tire(k, "OMEGA") for k in range(4)]
        for k in range(4):
            y += [sus(k, "WU"), sus(k, "XS")]
        y += [s[C["LFDM24_S_CRANKOMEGA"]]] if tc else []
        y += [s[C[f"LFDM24_S_{f}"]] for f in ("X", "Y", "U", "V", "W", "WZ", "WX", "WY", "PSI", "PHI", "THETA")]
    return np.array(y)


@pytest.mark.parametrize("model", [11, 18, 24])
def test_threaded_batch_equals_the_single_vehicle_jacobians(model):
    fleet = __import__("conftest").pkg_mod("fleet")
    n = 12
    f = {11: fleet.fleet11, 18: fleet.fleet18, 24: fleet.fleet24}[model](n, seed=9, horizon=2.0)
    rng = np.random.default_rng(model)
    ctl = np.stack([rng.uniform(-0.3, 0.3, n), rng.uniform(0.0, 1.0, n), rng.uniform(0.0, 0.2, n)])
    js, jc = O.jacobian_fd_batch(model, 0, f["cls"][0], f["params"], f["states"], ctl, full_point=True, nthreads=4)
    for i in range(n):
        a, b = O.jacobian_fd(model, 0, f["cls"][0], f["params"][i], f["states"][i], ctl[:, i], full_point=True)
        assert np.array_equal(js[i], a) and np.array_equal(jc[i], b)


@pytest.mark.parametrize("model", [11, 18, 24])
def test_threaded_batch_tmeasy_nr(model):
    """The batch entry with TMeasyNr tires (golden Sedan state, spread controls) equals the single-
    vehicle restatement, at the fresh and the full evaluation point."""
    case = [c for c in _cases(model) if c["tire_type"] == 1][0]
    cls, p, _, _ = INPUTS[model](case)
    n = 8
    states = np.repeat(np.array(case["expected_final"])[None], n, axis=0)
    rng = np.random.default_rng(model + 100)
    ctl = np.stack([rng.uniform(-0.3, 0.3, n), rng.uniform(0.0, 1.0, n), rng.uniform(0.0, 0.2, n)])
    params = np.repeat(p[None], n, axis=0)
    for full in (False, True):
        js, jc = O.jacobian_fd_batch(model, 1, cls, params, states, ctl, full_point=full, nthreads=3)
        for i in range(n):
            a, b = O.jacobian_fd(model, 1, cls, p, states[i], ctl[:, i], full_point=full)
            assert np.array_equal(js[i], a) and np.array_equal(jc[i], b)

