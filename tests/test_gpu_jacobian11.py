"""Exact right-hand-side Jacobians of the 11-DOF model on the GPU (lfdm_rhs_jacobian_exact, TMeasy
and TMeasyNr tires) against central differences of the reference algorithm's own right-hand side
(the oracle's restatement of PerturbRhsFun, 11dof/dof11_halfImplicit.cpp), in the reference's packed
order ({xe, ye} front, rear; omega front, rear; crank with a torque converter; x, y, u, v, psi, wz),
at the point the reference differentiates at (fresh vehicle state) and at the full current state;
against the Jacobians the reference's CPU solver prints (its 1e-3 differences); and against the
library's own difference scheme.

Tolerances as for the 18-DOF exact Jacobian: over the entries that are not zero in both (relative to
max(|entry|, 1e-7 x the row's largest entry)), median <= 1e-6 and at least 95 % <= 1e-5 against
small-step central differences (the remainder straddle a branch of the tire curve or drivetrain);
median <= 1e-4 against differences with steps of 1e-3 of each state (their truncation error)."""
import ctypes

import numpy as np
import pytest

import oracle_lib as O
from conftest import case_inputs11, pkg_mod
from test_gpu_jacobian_fd import _batch, _cases

pytestmark = pytest.mark.gpu


def _pack11(state, tc, nr=False):
    abi = pkg_mod("_abi")
    C = abi.C
    y = []
    t = [C["LFDM11_S_TIRE0"] + k * C["LFDM_S_TIRE_STRIDE"] for k in range(2)]
    if not nr:
        for k in range(2):
            y += [state[t[k] + abi.T["xe"]], state[t[k] + abi.T["ye"]]]
    y += [state[t[k] + abi.T["omega"]] for k in range(2)]
    if tc:
        y.append(state[abi.S11["crankomega"]])
    y += [state[abi.S11[k]] for k in ("x", "y", "u", "v", "psi", "wz")]
    return np.array(y)


def _fd(cls, p, y, ctl, full_state, steps, tire_type=0):
    def f(yy, cc):
        return O.rhs(11, tire_type, cls, p, yy, cc, full_state)

    m = len(y)
    J = np.zeros((m, m))
    for c in range(m):
        h = steps[c]
        yp, ym = y.copy(), y.copy()
        yp[c] += h
        ym[c] -= h
        J[:, c] = (f(yp, ctl) - f(ym, ctl)) / (2 * h)
    Ju = np.zeros((m, 2))
    for c in range(2):
        h = 1e-7
        cp, cm = np.array(ctl, dtype=float), np.array(ctl, dtype=float)
        cp[c] += h
        cm[c] -= h
        Ju[:, c] = (f(y, cp) - f(y, cm)) / (2 * h)
    return J, Ju


def _rel(a, b):
    scale = np.maximum(np.abs(b).max(axis=1, keepdims=True), 1e-300)
    floor = 1e-7 * scale
    e = np.abs(a - b) / np.maximum(np.abs(b), floor)
    keep = (np.abs(a) > floor) | (np.abs(b) > floor)
    return e[keep]


def _fleet(lfdm, n=48, seed=11):
    fleet = pkg_mod("fleet")
    f = fleet.fleet11(n, seed=seed, horizon=3.0)
    sol = lfdm.d11SolverHalfImplicitGPU(n)
    sol.construct_class(f["cls"][0], f["params"])
    sol.set_driver_tables(f["tables"])
    sol.set_states(f["states"])
    sol.SetKernelSimTime(1.0)
    sol.SetEndTime(2.0)
    sol.Solve()  # diverse speeds, slips and gears after 2 s of the seeded drivers
    rng = np.random.default_rng(seed)
    ctl = np.stack([rng.uniform(-0.3, 0.3, n), rng.uniform(0.0, 1.0, n), rng.uniform(0.0, 0.3, n)])
    return f, sol, sol.get_states(), ctl


def _check(js, ju, cls, params, states, ctl, reference_point, tire_type=0):
    tc = bool(cls.tcbool)
    errs, errs_u = [], []
    for i in range(states.shape[0]):
        y = _pack11(states[i], tc, tire_type == 1)
        full = None if reference_point else states[i]
        steps = 1e-6 * np.maximum(np.abs(y), 1e-2)
        J, Ju = _fd(cls, params[i], y, ctl[:, i], full, steps, tire_type)
        errs.append(_rel(js[i], J))
        errs_u.append(_rel(ju[i], Ju))
    e, eu = np.concatenate(errs), np.concatenate(errs_u)
    print(f"state Jacobian ({e.size} nonzero entries): median {np.median(e):.1e}, 95% {np.quantile(e, 0.95):.1e}; "
          f"controls: median {np.median(eu):.1e}, 95% {np.quantile(eu, 0.95):.1e}")
    assert np.median(e) <= 1e-6 and (e <= 1e-5).mean() >= 0.95
    assert np.median(eu) <= 1e-6 and (eu <= 1e-5).mean() >= 0.95


@pytest.mark.parametrize("reference_point", [True, False])
def test_jacobian11_matches_central_differences_of_the_reference_rhs(built_lib, reference_point):
    f, sol, states, ctl = _fleet(built_lib)
    js, ju = sol.rhs_jacobian(ctl[0], ctl[1], ctl[2], reference_point=reference_point)
    sol.close()
    cls = f["cls"][0]
    assert js.shape[1:] == (13 if cls.tcbool else 12,) * 2 and ju.shape[2] == 2
    _check(js, ju, cls, f["params"], states, ctl, reference_point)


@pytest.mark.parametrize("reference_point", [True, False])
def test_jacobian11_tmeasy_nr(built_lib, reference_point):
    """The Sedan TMeasyNr case's final state spread over 48 vehicles (packed order without
    deflection states)."""
    cls, p, states, ctl = _batch(11, 1, 48, 7)
    params = np.repeat(p[None], len(states), axis=0)
    sol = built_lib.d11SolverHalfImplicitGPU(len(states))
    sol.construct_class(cls, params, 1)
    sol.set_states(states)
    js, ju = sol.rhs_jacobian(ctl[0], ctl[1], ctl[2], reference_point=reference_point)
    sol.close()
    assert js.shape[1:] == (9 if cls.tcbool else 8,) * 2
    _check(js, ju, cls, params, states, ctl, reference_point, tire_type=1)


def test_jacobian11_agrees_with_the_reference_cpu_solver(built_lib):
    """The Jacobians the reference's 11-DOF CPU solver prints (IntegrateStepWithJacobian, steps of
    1e-3 of each state) at golden final states, both tire types: their truncation error apart."""
    errs = []
    for case in _cases(11):
        cls, p, _, _ = case_inputs11(case)
        jac = case["jacobian"]
        ny = jac["ny"]
        sol = built_lib.d11SolverHalfImplicitGPU(1)
        sol.construct_class(cls, p[None], case["tire_type"])
        sol.set_states(np.array(case["expected_final"])[None])
        js, jc = sol.rhs_jacobian(*[[x] for x in jac["controls"]])
        sol.close()
        assert js.shape == (1, ny, ny)
        errs.append(_rel(js[0], np.array(jac["state"]).reshape(ny, ny)))
        errs.append(_rel(jc[0], np.array(jac["control"]).reshape(ny, 2)))
    e = np.concatenate(errs)
    print(f"vs the reference's printed Jacobians ({e.size} nonzero entries): median {np.median(e):.1e}, "
          f"90% {np.quantile(e, 0.9):.1e}")
    assert np.median(e) <= 1e-4


def test_jacobian11_exact_against_the_difference_scheme_and_host_form(built_lib):
    """On the driven fleet: the library's difference scheme (the reference's steps) agrees with the
    exact Jacobian to its truncation error, and the host-buffer form (lfdm_rhs_jacobian_host,
    exact = 1) returns the device results per vehicle."""
    f, sol, states, ctl = _fleet(built_lib, n=32, seed=5)
    js, ju = sol.rhs_jacobian(ctl[0], ctl[1], 0.0)
    fs, fu = sol.rhs_jacobian_fd(ctl[0], ctl[1], 0.0)
    e = np.concatenate([_rel(fs[i], js[i]) for i in range(len(js))])
    print(f"difference scheme vs exact: median {np.median(e):.1e}")
    assert np.median(e) <= 1e-4
    n, ny = js.shape[0], js.shape[1]
    hs, hu = np.zeros((n, ny, ny)), np.zeros((n, ny, 2))
    c3 = np.ascontiguousarray(np.stack([ctl[0], ctl[1], np.zeros(n)]))
    got = ctypes.c_int()
    dp = ctypes.POINTER(ctypes.c_double)
    rc = sol._L.lfdm_rhs_jacobian_host(sol._h, 1, c3.ctypes.data_as(dp), 1, hs.ctypes.data_as(dp),
                                       hu.ctypes.data_as(dp), ctypes.byref(got))
    sol.close()
    assert rc == 0 and got.value == ny
    assert np.array_equal(hs, js) and np.array_equal(hu, ju)
