"""Exact right-hand-side Jacobians of the 18-DOF model on the GPU (lfdm_rhs_jacobian18, TMeasy and
TMeasyNr tires) against
central differences of the reference algorithm's own right-hand side (the oracle's restatement of
PerturbRhsFun, 18dof/dof18_halfImplicit.cpp:679-745), in the reference's packed order, at the point
the reference differentiates at (fresh vehicle state) and at the full current state.

Tolerance, over the entries that are not zero in both (relative to max(|entry|, 1e-7 x the row's
largest entry)): median <= 1e-6 and at least 95 % <= 1e-5 against small-step central differences.
The remainder are entries whose +-h perturbation crosses a branch of the tire curve or the
drivetrain, which a finite difference straddles and the exact derivative does not. Against the reference's own scheme (steps
of 1e-3 of each state) the agreement is at its truncation error: median <= 1e-4."""
import numpy as np
import pytest

import oracle_lib as O
from conftest import pkg_mod

pytestmark = pytest.mark.gpu


def _fleet(lfdm, n=48, seed=11):
    fleet = pkg_mod("fleet")
    f = fleet.fleet18(n, seed=seed, horizon=3.0)
    sol = lfdm.d18SolverHalfImplicitGPU(n)
    sol.construct_class(f["cls"][0], f["params"])
    sol.set_driver_tables(f["tables"])
    sol.set_states(f["states"])
    sol.SetKernelSimTime(1.0)
    sol.SetEndTime(2.0)
    sol.Solve()  # diverse speeds, slips and gears after 2 s of the seeded drivers
    rng = np.random.default_rng(seed)
    ctl = np.stack([rng.uniform(-0.3, 0.3, n), rng.uniform(0.0, 1.0, n), rng.uniform(0.0, 0.3, n)])
    return f, sol, sol.get_states(), ctl


def _fd(cls, p, y, ctl, full_state, steps, tire_type=0):
    def f(yy, cc):
        return O.rhs(18, tire_type, cls, p, yy, cc, full_state)

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
    """Relative differences of the entries that are not zero in both (structural zeros excluded)."""
    scale = np.maximum(np.abs(b).max(axis=1, keepdims=True), 1e-300)
    floor = 1e-7 * scale
    e = np.abs(a - b) / np.maximum(np.abs(b), floor)
    keep = (np.abs(a) > floor) | (np.abs(b) > floor)
    return e[keep]


@pytest.mark.parametrize("reference_point", [True, False])
def test_jacobian_matches_central_differences_of_the_reference_rhs(built_lib, reference_point):
    f, sol, states, ctl = _fleet(built_lib)
    js, ju = sol.rhs_jacobian(ctl[0], ctl[1], ctl[2], reference_point=reference_point)
    sol.close()
    cls = f["cls"][0]
    tc = bool(cls.tcbool)
    assert js.shape[1:] == (21 if tc else 20,) * 2 and ju.shape[2] == 2
    errs, errs_u = [], []
    for i in range(states.shape[0]):
        y = O.pack_y18(states[i], tc)
        full = None if reference_point else states[i]
        steps = 1e-6 * np.maximum(np.abs(y), 1e-2)
        J, Ju = _fd(cls, f["params"][i], y, ctl[:, i], full, steps)
        errs.append(_rel(js[i], J))
        errs_u.append(_rel(ju[i], Ju))
    e, eu = np.concatenate(errs), np.concatenate(errs_u)
    print(f"state Jacobian ({e.size} nonzero entries): median {np.median(e):.1e}, 95% {np.quantile(e, 0.95):.1e}; "
          f"controls: median {np.median(eu):.1e}, 95% {np.quantile(eu, 0.95):.1e}")
    assert np.median(e) <= 1e-6 and (e <= 1e-5).mean() >= 0.95
    assert np.median(eu) <= 1e-6 and (eu <= 1e-5).mean() >= 0.95


def test_jacobian_agrees_with_the_reference_scheme(built_lib):
    """IntegrateStepWithJacobian's own differences: steps of 1e-3 of each state (1e-3 where the state
    is below 1e-8), 1e-3 on steering and throttle, braking 0."""
    f, sol, states, ctl = _fleet(built_lib, n=16, seed=5)
    js, ju = sol.rhs_jacobian(ctl[0], ctl[1], 0.0)
    sol.close()
    cls = f["cls"][0]
    tc = bool(cls.tcbool)
    errs = []
    for i in range(states.shape[0]):
        y = O.pack_y18(states[i], tc)
        steps = np.abs(y * 1e-3)
        steps[steps < 1e-8] = 1e-3
        J, _ = _fd(cls, f["params"][i], y, [ctl[0, i], ctl[1, i], 0.0], None, steps)
        errs.append(_rel(js[i], J))
    e = np.concatenate(errs)
    print(f"vs the reference's 1e-3 differences ({e.size} nonzero entries): median {np.median(e):.1e}")
    assert np.median(e) <= 1e-4


def _nr_states(n, seed):
    """The Sedan TMeasyNr golden case's final state, spread: velocities and wheel speeds scaled by
    U[0.6, 1.4], and a third of the vehicles at 0.3-4 m/s with lateral slip (the Coulomb force, its
    clamp to the friction circle and the blend into the slip forces)."""
    import json
    import os

    from conftest import TESTS, case_inputs
    with open(os.path.join(TESTS, "golden", "golden18.json")) as fh:
        case = [c for c in json.load(fh)["cases"] if c["tire_type"] == 1][0]
    cls, p, _, _ = case_inputs(case)
    abi = pkg_mod("_abi")
    rng = np.random.default_rng(seed)
    s0 = np.array(case["expected_final"])
    states = np.repeat(s0[None], n, axis=0)
    om = [abi.S_TIRE0 + k * abi.C["LFDM_S_TIRE_STRIDE"] + abi.T["omega"] for k in range(4)]
    fields = [abi.S[k] for k in ("u", "v", "wz", "wx")] + om
    states[:, fields] *= rng.uniform(0.6, 1.4, (n, len(fields)))
    r0 = float(p[abi.P["r0"]])
    for i in range(0, n, 3):
        u = rng.uniform(0.3, 4.0)
        states[i, abi.S["u"]] = u
        states[i, abi.S["v"]] = rng.uniform(-1.0, 1.0)
        states[i, om] = u / r0 * rng.uniform(0.7, 1.3, 4)
    ctl = np.stack([rng.uniform(-0.3, 0.3, n), rng.uniform(0.0, 1.0, n), rng.uniform(0.0, 0.3, n)])
    return cls, p, states, ctl


def _pack_nr(state, tc):
    abi = pkg_mod("_abi")
    y = [state[abi.S_TIRE0 + k * abi.C["LFDM_S_TIRE_STRIDE"] + abi.T["omega"]] for k in range(4)]
    y += [state[abi.S["crankomega"]]] if tc else []
    y += [state[abi.S[k]] for k in ("x", "y", "u", "v", "psi", "wz", "phi", "wx")]
    return np.array(y)


@pytest.mark.parametrize("reference_point", [True, False])
def test_tmeasy_nr_jacobian_matches_central_differences(built_lib, reference_point):
    """The exact Jacobian of the 18-DOF model with TMeasyNr tires (packed order without deflection
    states: omega x 4, crank, x, y, u, v, psi, wz, phi, wx) against central differences of the
    reference algorithm's TMeasyNr right-hand side, with the TMeasy test's tolerance."""
    n = 48
    cls, p, states, ctl = _nr_states(n, seed=17)
    sol = built_lib.d18SolverHalfImplicitGPU(n)
    sol.construct_class(cls, np.repeat(p[None], n, axis=0), 1)
    sol.set_states(states)
    js, ju = sol.rhs_jacobian(ctl[0], ctl[1], ctl[2], reference_point=reference_point)
    sol.close()
    tc = bool(cls.tcbool)
    assert js.shape[1:] == (13 if tc else 12,) * 2 and ju.shape[2] == 2
    errs, errs_u = [], []
    for i in range(n):
        y = _pack_nr(states[i], tc)
        full = None if reference_point else states[i]
        steps = 1e-6 * np.maximum(np.abs(y), 1e-2)
        J, Ju = _fd(cls, p, y, ctl[:, i], full, steps, tire_type=1)
        errs.append(_rel(js[i], J))
        errs_u.append(_rel(ju[i], Ju))
    e, eu = np.concatenate(errs), np.concatenate(errs_u)
    print(f"TMeasyNr state Jacobian ({e.size} nonzero entries): median {np.median(e):.1e}, "
          f"95% {np.quantile(e, 0.95):.1e}; controls: median {np.median(eu):.1e}, 95% {np.quantile(eu, 0.95):.1e}")
    assert np.median(e) <= 1e-6 and (e <= 1e-5).mean() >= 0.95
    assert np.median(eu) <= 1e-6 and (eu <= 1e-5).mean() >= 0.95


def test_tmeasy_nr_exact_against_the_reference_scheme(built_lib):
    """Exact and difference-scheme TMeasyNr Jacobians of the same vehicles agree to the scheme's
    truncation error."""
    n = 32
    cls, p, states, ctl = _nr_states(n, seed=4)
    sol = built_lib.d18SolverHalfImplicitGPU(n)
    sol.construct_class(cls, np.repeat(p[None], n, axis=0), 1)
    sol.set_states(states)
    ex, _ = sol.rhs_jacobian(ctl[0], ctl[1], 0.0)
    fd, _ = sol.rhs_jacobian_fd(ctl[0], ctl[1], 0.0)
    sol.close()
    e = np.concatenate([_rel(fd[i], ex[i]) for i in range(n)])
    print(f"TMeasyNr difference scheme vs exact ({e.size} entries): median {np.median(e):.1e}")
    assert np.median(e) <= 1e-4


def test_kinematic_rows_and_errors(built_lib):
    f, sol, states, ctl = _fleet(built_lib, n=8, seed=2)
    js, _ = sol.rhs_jacobian(ctl[0], ctl[1], ctl[2])
    o = 13 if f["cls"][0].tcbool else 12
    psi, u, v = states[:, 4], states[:, 2], states[:, 3]
    assert np.allclose(js[:, o, o + 2], np.cos(psi), rtol=1e-15, atol=1e-15)
    assert np.allclose(js[:, o + 1, o + 4], u * np.cos(psi) - v * np.sin(psi), rtol=1e-13, atol=1e-13)
    assert np.all(js[:, o + 4, o + 5] == 1.0) and np.all(js[:, o + 6, o + 7] == 1.0)
    sol.close()
    s11 = built_lib.d11SolverHalfImplicitGPU(2)
    jac = built_lib.d18SolverHalfImplicitGPU.rhs_jacobian.__get__(s11)  # the 18-DOF call on an 11-DOF solver
    with pytest.raises(built_lib.LfdmError):
        jac(0.0, 0.0)
    s11.close()


def test_host_jacobian_rejects_unsupported_configurations_before_sizing(built_lib):
    """lfdm_rhs_jacobian_host checks the configuration first: the size query of the exact Jacobian on
    a 24-DOF solver with TMeasyNr tires, or on an 18-DOF solver whose vehicle has throttleMod, fails
    like the call; on 11-DOF and 24-DOF TMeasy solvers both Jacobians are sized."""
    import ctypes

    fleet = pkg_mod("fleet")
    L = built_lib.lib()
    ny = ctypes.c_int(-1)
    f11 = fleet.fleet11(8, seed=2, horizon=1.0)
    s11 = built_lib.d11SolverHalfImplicitGPU(8)
    s11.construct_class(f11["cls"][0], f11["params"])
    s11.set_states(f11["states"])
    for exact in (1, 0):
        ny.value = -1
        assert L.lfdm_rhs_jacobian_host(s11._h, exact, None, 1, None, None, ctypes.byref(ny)) == 0 and ny.value == 13
    s11.close()
    f24 = fleet.fleet24(4, seed=2, horizon=1.0)
    for tire, want in ((0, 0), (1, built_lib._abi.C["LFDM_ERR_ARG"])):
        s24 = built_lib.d24SolverHalfImplicitGPU(4)
        s24.construct_class(f24["cls"][0], f24["params"], tire)
        s24.set_states(f24["states"])
        ny.value = -1
        assert L.lfdm_rhs_jacobian_host(s24._h, 1, None, 1, None, None, ctypes.byref(ny)) == want
        assert ny.value == (36 if want == 0 else -1)
        s24.close()
    cls, p = fleet.suv18()
    cls.throttleMod = 1
    s18 = built_lib.d18SolverHalfImplicitGPU(4)
    s18.construct_class(cls, np.repeat(p[None], 4, axis=0))
    ny.value = -1
    assert L.lfdm_rhs_jacobian_host(s18._h, 1, None, 1, None, None, ctypes.byref(ny)) == \
        built_lib._abi.C["LFDM_ERR_ARG"]
    assert ny.value == -1
    assert L.lfdm_rhs_jacobian_host(s18._h, 0, None, 1, None, None, ctypes.byref(ny)) == 0 and ny.value == 21
    s18.close()
