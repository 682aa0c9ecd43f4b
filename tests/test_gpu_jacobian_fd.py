"""Right-hand-side Jacobians by the reference's own difference scheme on the GPU
(lfdm_rhs_jacobian_fd, every model and tire type) against

* the Jacobians the reference's CPU solvers print (IntegrateStepWithJacobian at the final state of
  golden cases, tests/golden/golden{11,18,24}.json), and
* the oracle's restatement of the same scheme (oracle_jacobian_fd) on batches of diverse states,
  at the reference's evaluation point (fresh state) and at the full current state.

The kernel and the reference take the same perturbations and quotients of right-hand sides that
differ only in the last bits (libm, fused multiply-adds); a quotient (f(y+h) - f(y-h)) / 2h magnifies
those differences by |f| / h. Each entry is therefore compared against the size of its row: its
relative difference is |gpu - ref| / max(|ref|, 1e-4 x the largest |entry| of the row across the
state and control Jacobians). At least 97 % of the entries of the non-zero rows must agree to 1e-9,
99.9 % to 1e-6, and none may differ by more than 1e-4. The 24-DOF rows (suspension and chassis
accelerations: sums of forces of order 1e4 N over masses and inertias) carry the largest rounding
magnification."""
import json
import os

import numpy as np
import pytest

import oracle_lib as O
from conftest import TESTS, case_inputs, case_inputs11, case_inputs24, pkg_mod

pytestmark = pytest.mark.gpu
INPUTS = {11: case_inputs11, 18: case_inputs, 24: case_inputs24}
SOLVER = {11: "d11SolverHalfImplicitGPU", 18: "d18SolverHalfImplicitGPU", 24: "d24SolverHalfImplicitGPU"}
TOL, FLOOR = 1e-9, 1e-4


def _cases(model):
    with open(os.path.join(TESTS, "golden", f"golden{model}.json")) as f:
        return [c for c in json.load(f)["cases"] if "jacobian" in c]


def _errors(a, b, ac, bc):
    """Relative differences of a state Jacobian (a against b) and a control Jacobian (ac against bc):
    |a - b| / max(|b|, FLOOR x the largest |entry| of the row across b and bc), over rows that are not
    zero in both."""
    scale = np.maximum(np.abs(b).max(axis=-1), np.abs(bc).max(axis=-1))[:, None]

    def rel(x, y):
        den = np.maximum(np.abs(y), FLOOR * scale)
        rows = np.broadcast_to(scale > 0, y.shape)
        return (np.abs(x - y) / np.where(den > 0, den, 1.0))[rows]

    return rel(a, b), rel(ac, bc)


def _worst(a, b, ac, bc, name, k=3):
    """The k largest relative differences (matrix, row, column, value, expected) of one vehicle."""
    scale = np.maximum(np.abs(b).max(axis=-1), np.abs(bc).max(axis=-1))[:, None]
    out = []
    for tag, x, y in (("state", a, b), ("control", ac, bc)):
        e = np.abs(x - y) / np.maximum(np.maximum(np.abs(y), FLOOR * scale), 1e-300)
        for idx in np.argsort(e, axis=None)[::-1][:k]:
            r, c = np.unravel_index(idx, e.shape)
            if e[r, c] > TOL:
                out.append(f"{name} {tag}[{r},{c}] {x[r, c]!r} vs {y[r, c]!r} (rel {e[r, c]:.1e}, "
                           f"row scale {scale[r, 0]:.2e})")
    return out


def _assess(e, what, worst=()):
    print(f"{what}: {e.size} entries, median {np.median(e):.1e}, 99% {np.quantile(e, 0.99):.1e}, "
          f"max {e.max():.1e}, above {TOL:g}: {(e > TOL).mean():.2%}")
    for w in worst[:6]:
        print("   ", w)
    assert (e <= TOL).mean() >= 0.97, what
    assert (e <= 1e-6).mean() >= 0.999, what
    assert e.max() <= 1e-4, what


def _compare(pairs, what):
    """pairs: (gpu state, gpu control, expected state, expected control, name) per vehicle."""
    es, ec, w = [], [], []
    for a, ac, b, bc, name in pairs:
        e1, e2 = _errors(a, b, ac, bc)
        es.append(e1)
        ec.append(e2)
        w += _worst(a, b, ac, bc, name)
    _assess(np.concatenate(es), what + ", state Jacobians", w)
    _assess(np.concatenate(ec), what + ", control Jacobians")


def _solver(lfdm, model, cls, params, states, tire_type):
    sol = getattr(lfdm, SOLVER[model])(len(states))
    sol.construct_class(cls, params, tire_type)
    sol.set_states(states)
    return sol


@pytest.mark.parametrize("model", [11, 18, 24])
def test_fd_jacobians_match_the_reference_cpu_solver(built_lib, model):
    pairs = []
    for case in _cases(model):
        if model == 24 and case["tire_type"] == 1:
            continue  # the reference's 24-DOF TMeasyNr PerturbRhsFun ignores the states (oracle tests)
        cls, p, _, _ = INPUTS[model](case)
        jac = case["jacobian"]
        ny = jac["ny"]
        sol = _solver(built_lib, model, cls, p[None], np.array(case["expected_final"])[None], case["tire_type"])
        js, jc = sol.rhs_jacobian_fd(*[[x] for x in jac["controls"]])
        sol.close()
        assert js.shape == (1, ny, ny) and jc.shape == (1, ny, 2)
        pairs.append((js[0], jc[0], np.array(jac["state"]).reshape(ny, ny), np.array(jac["control"]).reshape(ny, 2),
                      case["name"]))
    _compare(pairs, f"{model}-DOF vs the reference")


def _batch(model, tire_type, n, seed):
    """n diverse states of a golden case with a Jacobian of this model and tire: its final state with
    the packed velocity-like fields scaled by U[0.6, 1.4] and random controls."""
    abi = pkg_mod("_abi")
    C = abi.C
    case = [c for c in _cases(model) if c["tire_type"] == tire_type][0]
    cls, p, _, _ = INPUTS[model](case)
    rng = np.random.default_rng(seed)
    s0 = np.array(case["expected_final"])
    states = np.repeat(s0[None], n, axis=0)
    if model == 18:
        fields = [abi.S[k] for k in ("u", "v", "wz", "wx")]
        fields += [abi.S_TIRE0 + k * C["LFDM_S_TIRE_STRIDE"] + abi.T["omega"] for k in range(4)]
    elif model == 11:
        fields = [C[f"LFDM11_S_{k}"] for k in ("U", "V", "WZ")]
        fields += [C["LFDM11_S_TIRE0"] + k * C["LFDM_S_TIRE_STRIDE"] + abi.T["omega"] for k in range(2)]
    else:
        fields = [C[f"LFDM24_S_{k}"] for k in ("U", "V", "W", "WZ", "WX", "WY")]
        fields += [C["LFDM24_S_TIRE0"] + k * C["LFDM24_T_COUNT"] + C["LFDM24_T_OMEGA"] for k in range(4)]
    states[:, fields] *= rng.uniform(0.6, 1.4, (n, len(fields)))
    ctl = np.stack([rng.uniform(-0.4, 0.4, n), rng.uniform(0.0, 1.0, n), rng.uniform(0.0, 0.3, n)])
    return cls, p, states, ctl


@pytest.mark.parametrize("model,tire_type", [(11, 0), (11, 1), (18, 0), (18, 1), (24, 0), (24, 1)])
@pytest.mark.parametrize("reference_point", [True, False])
def test_fd_jacobians_match_the_oracle_on_diverse_states(built_lib, model, tire_type, reference_point):
    n = 48
    cls, p, states, ctl = _batch(model, tire_type, n, seed=model * 10 + tire_type)
    sol = _solver(built_lib, model, cls, np.repeat(p[None], n, axis=0), states, tire_type)
    js, jc = sol.rhs_jacobian_fd(ctl[0], ctl[1], ctl[2], reference_point=reference_point)
    sol.close()
    pairs = []
    for i in range(n):
        Js, Jc = O.jacobian_fd(model, tire_type, cls, p, states[i], ctl[:, i], full_point=not reference_point)
        assert js.shape[1:] == Js.shape
        pairs.append((js[i], jc[i], Js, Jc, f"vehicle {i}"))
    _compare(pairs, f"{model}-DOF {'TMeasyNr' if tire_type else 'TMeasy'} {'fresh' if reference_point else 'full'} state")


@pytest.mark.parametrize("model", [11, 18, 24])
def test_fd_jacobians_on_a_driven_fleet(built_lib, model):
    """Realistic states: the seeded SUV fleet of the model after 2 s of its drivers."""
    fleet = pkg_mod("fleet")
    n = 64
    f = {11: fleet.fleet11, 18: fleet.fleet18, 24: fleet.fleet24}[model](n, seed=7, horizon=3.0)
    sol = getattr(built_lib, SOLVER[model])(n)
    params = f["params"] if f["params"].ndim == 2 else np.repeat(f["params"][None], n, axis=0)
    cls = f["cls"][0] if isinstance(f["cls"], list) else f["cls"]
    sol.construct_class(cls, params)
    sol.set_driver_tables(f["tables"])
    sol.set_states(f["states"])
    sol.SetKernelSimTime(1.0)
    sol.SetEndTime(2.0)
    sol.Solve()
    states = sol.get_states()
    rng = np.random.default_rng(model)
    ctl = np.stack([rng.uniform(-0.3, 0.3, n), rng.uniform(0.0, 1.0, n), rng.uniform(0.0, 0.3, n)])
    js, jc = sol.rhs_jacobian_fd(ctl[0], ctl[1], ctl[2])
    sol.close()
    pairs = []
    for i in range(n):
        Js, Jc = O.jacobian_fd(model, 0, cls, params[i], states[i], ctl[:, i])
        pairs.append((js[i], jc[i], Js, Jc, f"vehicle {i}"))
    _compare(pairs, f"{model}-DOF driven fleet")


def test_fd_scheme_against_the_exact_18dof_jacobian(built_lib):
    """The two GPU paths of the 18-DOF TMeasy model at the same point: the difference scheme agrees
    with the exact Jacobian to its truncation error (median relative difference <= 1e-4)."""
    fleet = pkg_mod("fleet")
    n = 32
    f = fleet.fleet18(n, seed=3, horizon=3.0)
    sol = built_lib.d18SolverHalfImplicitGPU(n)
    sol.construct_class(f["cls"][0], f["params"])
    sol.set_driver_tables(f["tables"])
    sol.set_states(f["states"])
    sol.SetKernelSimTime(1.0)
    sol.SetEndTime(2.0)
    sol.Solve()
    ex, _ = sol.rhs_jacobian(0.1, 0.5, 0.0)
    fd, _ = sol.rhs_jacobian_fd(0.1, 0.5, 0.0)
    sol.close()
    scale = np.abs(ex).max(axis=2, keepdims=True)
    keep = (np.abs(ex) > 1e-7 * scale) | (np.abs(fd) > 1e-7 * scale)
    e = (np.abs(fd - ex) / np.maximum(np.abs(ex), 1e-7 * scale))[keep]
    print(f"difference scheme vs exact: median {np.median(e):.1e}")
    assert np.median(e) <= 1e-4


def test_fd_jacobian_argument_errors(built_lib):
    sol = built_lib.d24SolverHalfImplicitGPU(2)
    with pytest.raises(built_lib.LfdmError):  # no vehicles constructed
        sol.rhs_jacobian_fd(0.0, 0.0)
    sol.close()
