"""Edge regimes of every model and tire type on the GPU against the oracle, one window of 10 steps
(SolveStep, per-vehicle controls): standstill under full brake, rolling backwards, 60 m/s, wheels
locked at speed, wheels spinning under full throttle, and wheel lift-off (roll and lateral load
transfer for the 18-/24-DOF models, pitch transfer for the 11-DOF model, a negative tire compression
for the 24-DOF model) — the zero-load branch of computeTireRHS that the fleets rarely reach.

Tolerance: per state |gpu - oracle| <= 1e-12 max(|oracle|, s_k) (the floors of the parity tests)
for all but at most 2 of the 96 vehicles of each case, and <= 1e-9 for every vehicle: in these
regimes a wheel speed can pass through zero, where the brake torque's sign (sgn(omega)) decides on
the last bit of a rounding-level value, so an occasional vehicle agrees only to the amplified
rounding of that step."""
import json
import os

import numpy as np
import pytest

import oracle_lib as O
from conftest import TESTS, case_inputs, case_inputs11, case_inputs24, pkg_mod, rel_err, state_floors, \
    state_floors24

pytestmark = pytest.mark.gpu
INPUTS = {11: case_inputs11, 18: case_inputs, 24: case_inputs24}
SOLVER = {11: "d11SolverHalfImplicitGPU", 18: "d18SolverHalfImplicitGPU", 24: "d24SolverHalfImplicitGPU"}
N = 96


def _case(model, tire_type):
    with open(os.path.join(TESTS, "golden", f"golden{model}.json")) as f:
        return [c for c in json.load(f)["cases"] if c["tire_type"] == tire_type][0]


def _fields(model):
    abi = pkg_mod("_abi")
    C = abi.C
    if model == 18:
        ntire, t0, stride = 4, abi.S_TIRE0, C["LFDM_S_TIRE_STRIDE"]
        S = {k: abi.S[k] for k in ("u", "v", "wz", "phi", "wx", "udot", "vdot")}
        fz = abi.T["fz"]
        omega = abi.T["omega"]
        xt = None
    elif model == 11:
        ntire, t0, stride = 2, C["LFDM11_S_TIRE0"], C["LFDM_S_TIRE_STRIDE"]
        S = {k: C[f"LFDM11_S_{k.upper()}"] for k in ("u", "v", "wz", "udot", "vdot")}
        fz = abi.T["fz"]
        omega = abi.T["omega"]
        xt = None
    else:
        ntire, t0, stride = 4, C["LFDM24_S_TIRE0"], C["LFDM24_T_COUNT"]
        S = {k: C[f"LFDM24_S_{k.upper()}"] for k in ("u", "v", "wz", "phi", "wx", "udot", "vdot")}
        fz = C["LFDM24_T_FZ"]
        omega = C["LFDM24_T_OMEGA"]
        xt = C["LFDM24_T_XT"]
    return ntire, t0, stride, S, fz, omega, xt


def _edge_states(model, s0, r0, seed):
    """N states from s0 in eight regimes (vehicle k in regime k % 8) and their controls [3][N]."""
    ntire, t0, stride, S, _, omega, xt = _fields(model)
    rng = np.random.default_rng(seed)
    states = np.repeat(s0[None], N, axis=0)
    ctl = np.stack([rng.uniform(-0.3, 0.3, N), rng.uniform(0.0, 0.6, N), np.zeros(N)])

    def wheels(i, w):
        for k in range(ntire):
            states[i, t0 + k * stride + omega] = w

    for i in range(N):
        reg = i % 8
        u = rng.uniform(5.0, 25.0)
        states[i, S["u"]] = u
        wheels(i, u / r0)
        if reg == 0:  # standstill, full brake
            states[i, S["u"]] = 0.0
            states[i, S["v"]] = 0.0
            states[i, S["wz"]] = 0.0
            wheels(i, 0.0)
            ctl[1, i], ctl[2, i] = 0.0, 1.0
        elif reg == 1:  # rolling backwards
            states[i, S["u"]] = -rng.uniform(0.5, 4.0)
            wheels(i, states[i, S["u"]] / r0)
        elif reg == 2:  # 60 m/s
            states[i, S["u"]] = 60.0
            wheels(i, 60.0 / r0)
            ctl[0, i] *= 0.1
        elif reg == 3:  # wheels locked at speed
            wheels(i, 0.0)
            ctl[1, i], ctl[2, i] = 0.0, 1.0
        elif reg == 4:  # wheels spinning under full throttle
            wheels(i, 3.0 * u / r0)
            ctl[1, i] = 1.0
        elif reg in (5, 6):  # lift-off: large lateral / longitudinal load transfer
            states[i, S["wz"]] = rng.uniform(0.6, 1.2) * (1 if reg == 5 else -1)
            states[i, S["vdot"]] = 15.0 * np.sign(states[i, S["wz"]])
            states[i, S["udot"]] = -45.0 if reg == 5 else 45.0
            if "phi" in S:
                states[i, S["phi"]] = 0.3 * np.sign(states[i, S["wz"]])
                states[i, S["wx"]] = 1.5 * np.sign(states[i, S["wz"]])
            ctl[0, i] = 0.8 * np.sign(states[i, S["wz"]])
        else:  # 24-DOF: two tires with negative compression; others: strong steering at speed
            if xt is not None:
                for k in (0, 3):
                    states[i, t0 + k * stride + xt] = -0.01
            ctl[0, i] = rng.choice([-1.0, 1.0])
    return states, ctl


@pytest.mark.parametrize("tire_type", [0, 1])
@pytest.mark.parametrize("model", [11, 18, 24])
def test_edge_regimes_one_window(built_lib, model, tire_type):
    case = _case(model, tire_type)
    cls, p, _, _ = INPUTS[model](case)
    s0 = np.array(case["expected_final"])
    r0 = float(p[pkg_mod("_abi").P["r0"]])
    states, ctl = _edge_states(model, s0, r0, seed=model * 2 + tire_type)
    params = np.repeat(p[None], N, axis=0)
    sol = getattr(built_lib, SOLVER[model])(N)
    sol.construct_class(cls, params, tire_type)
    sol.set_states(states)
    sol.SetKernelSimTime(0.01)
    sol.SolveStep(0.0, ctl[0], ctl[1], ctl[2])
    got = sol.get_states()
    sol.close()
    ref, _ = O.run18([cls], np.zeros(N, np.int32), params, states, ctl=ctl.T.copy(), t0=0.0, ksim=0.01, schedule=2,
                     tire_type=tire_type, model=model, nthreads=os.cpu_count() or 1)
    floors = state_floors24() if model == 24 else (state_floors() if model == 18 else None)
    if floors is None:  # 11-DOF: a floor of 1 for every field
        abi = pkg_mod("_abi")
        floors = np.full(abi.C["LFDM11_S_COUNT"], 1.0)
    e = rel_err(got, ref, floors).max(axis=1)
    ntire, t0, stride, _, fz, _, _ = _fields(model)
    one, _ = O.run18([cls], np.zeros(N, np.int32), params, states, ctl=ctl.T.copy(), t0=0.0, ksim=0.001, schedule=2,
                     tire_type=tire_type, model=model)
    lifted = sum(int((one[:, t0 + k * stride + fz] == 0.0).sum()) for k in range(ntire))
    print(f"{model}-DOF tire {tire_type}: max {e.max():.1e}, vehicles above 1e-12: {int((e > 1e-12).sum())}/{N}, "
          f"tires at zero load after the first step: {lifted}")
    assert lifted > 0  # the zero-load branch ran
    assert np.isfinite(got).all() and np.isfinite(ref).all()
    assert (e > 1e-12).sum() <= 2, (model, tire_type, float(e.max()), int(e.argmax()))
    assert e.max() <= 1e-9, (model, tire_type, float(e.max()), int(e.argmax()))
