"""24-DOF CUDA path (through the C ABI) against the reference's own 24-DOF CPU solver outputs
(tests/golden/golden24.json), the reference's GPU test pins and the oracle.

Per state |gpu - ref| <= 1e-9 * max(|ref|, s_k) with the floors of conftest.state_floors24()
(every one of the 212 fields of the reference's SimState is compared, including the ones the
kernel writes from a window's last step only). Rounding-chaotic trajectories (wheel chatter of the
light SUV wheels) are held to max(1e-9, 100 x the reference algorithm's sensitivity envelope): the
largest deviation, sample by sample, among the reference algorithm built with FMA contraction and
started from u moved by +-1e-15 max(|u|, 1 m/s). A single window from many diverse states is held to 1e-12.

The seeded 24-DOF SUV fleet is strongly chaotic: over 10 s about 330 of 512 vehicles of the
reference algorithm itself move beyond 1e-9 under a 1e-15 perturbation of u, and about 40 saturate
at relative deviations of order 1-10, where different perturbations land anywhere on the
attractor. Per vehicle the 100 x envelope bound is therefore applied below saturation (envelope
< 1e-3); saturated vehicles are checked through the fleet statistics.
"""
import json
import os
import tempfile

import numpy as np
import pytest

import oracle_lib as O
from conftest import RESP24_FLOORS, TESTS, case_inputs24, pkg_mod, rel_err, state_floors24

pytestmark = pytest.mark.gpu
RTOL = 1e-9
CHAOS_FACTOR = 100.0
NT = os.cpu_count() or 1


@pytest.fixture(scope="module")
def golden24():
    with open(os.path.join(TESTS, "golden", "golden24.json")) as f:
        return json.load(f)


def _groups(cases):
    g = {}
    for c in cases:
        if c["ksim"] > 0:
            g.setdefault((c["ksim"], c["tend"], c["sample"], c["tire_type"]), []).append(c)
    return g


def _run_group(lfdm, cases, ksim, tend, freq):
    n = len(cases)
    sol = lfdm.d24SolverHalfImplicitGPU(n)
    states = []
    for i, c in enumerate(cases):
        cls, p, s, tab = case_inputs24(c)
        sol.construct_class(cls, p[None, :], c["tire_type"])
        sol.set_driver_tables(tab[None, :, :], first=i)
        states.append(s)
    sol.set_states(np.array(states))
    sol.SetTimeStep(cases[0]["dt"])
    sol.SetKernelSimTime(ksim)
    sol.SetEndTime(tend)
    nsamp = int(round(tend * freq)) + 4
    resp = np.full((nsamp, lfdm.RESP24, n), np.nan)
    sol.set_response_buffer(resp, freq)
    sol.Solve()
    final = sol.get_states()
    sol.close()
    return final, resp


def _perturbed_runs(cls, class_of, params, states, tables, **kw):
    """The reference algorithm under the three perturbations of the sensitivity envelope."""
    U = pkg_mod("_abi").S24["u"]
    out = [O.run18(cls, class_of, params, states, tables, fma=True, model=24, **kw)]
    for eps in (1e-15, -1e-15):
        s2 = np.array(states, dtype=np.float64, copy=True)
        s2[:, U] += eps * np.maximum(np.abs(s2[:, U]), 1.0)  # relative, floored at 1 m/s (u0 may be 0)
        out.append(O.run18(cls, class_of, params, s2, tables, model=24, **kw))
    return out


def test_golden24_trajectories_within_reference_sensitivity(built_lib, golden24):
    """HMMWV (reference data files and driver tables, 22 s) and seeded SUV cases: the full final
    state and every sample within max(1e-9, 100 x the sensitivity envelope)."""
    fl = state_floors24()
    for (ksim, tend, sample, _tire), cases in _groups(golden24["cases"]).items():
        freq = 1.0 / (sample * cases[0]["dt"])
        final, resp = _run_group(built_lib, cases, ksim, tend, freq)
        for i, c in enumerate(cases):
            cls, p, s, tab = case_inputs24(c)
            runs = _perturbed_runs([cls], [0], p[None], s[None], [tab], tire_type=c["tire_type"], dt=c["dt"],
                                   tend=c["tend"], ksim=c["ksim"], schedule=1, dtout=sample * c["dt"])
            exp_f = np.array(c["expected_final"])
            exp = np.array(c["expected_samples"])
            env_f = max(rel_err(st[0], exp_f, fl).max() for st, _ in runs)
            env_r = np.max([rel_err(r[: len(exp), :, 0], exp[:, 1:], RESP24_FLOORS).max(axis=1) for _, r in runs],
                           axis=0)
            e = rel_err(final[i], exp_f, fl)
            assert e.max() <= max(RTOL, CHAOS_FACTOR * env_f), (c["name"], float(e.max()), int(e.argmax()),
                                                               float(env_f))
            e_r = rel_err(resp[: len(exp), :, i], exp[:, 1:], RESP24_FLOORS).max(axis=1)
            bound = np.maximum(RTOL, CHAOS_FACTOR * env_r)
            assert (e_r <= bound).all(), (c["name"], int(np.argmax(e_r > bound)), float(e_r.max()))


def _write(tmp, name, obj):
    p = os.path.join(tmp, name)
    with open(p, "w") as f:
        if isinstance(obj, str):
            f.write(obj)
        else:
            json.dump(obj, f)
    return p


def test_reference_24dof_gpu_tests(built_lib, golden24):
    """tests/24dof_gpu.cu:13-61 and :63-110 through the reference-style API: Construct from the
    HMMWV vehicle, tire and suspension files with a driver file, Initialize from zero states
    (initializeTireSus applied), Solve. x after 10 s of acc3 is 89.1625; with 500 vehicles on acc3
    and 500 on double_lane4 for 22 s, vehicles 499 and 999 end at 235.685 and 91.5211 (+-1 m)."""
    by = {c["name"]: c for c in golden24["cases"]}
    acc, dl = by["hmmwv24_acc3_gpu22"], by["hmmwv24_dl4_gpu22"]
    S24 = built_lib.S24_COUNT
    with tempfile.TemporaryDirectory() as tmp:
        vj, tj, sj = (_write(tmp, "v.json", acc["vehicle"]), _write(tmp, "t.json", acc["tire"]),
                      _write(tmp, "s.json", acc["sus"]))
        d_acc = _write(tmp, "acc3.txt", "".join(" ".join(repr(x) for x in r) + "\n" for r in acc["driver"]))
        d_dl = _write(tmp, "dl4.txt", "".join(" ".join(repr(x) for x in r) + "\n" for r in dl["driver"]))
        sol = built_lib.d24SolverHalfImplicitGPU(50)
        sol.Construct(vj, tj, sj, 50, d_acc)
        sol.SetThreadsPerBlock(32)
        sol.SetTimeStep(1e-3)
        sol.Initialize(np.zeros(S24), 50)
        sol.SetEndTime(10.0)
        sol.Solve()
        st = sol.GetSimState(0)
        sol.close()
        assert abs(st[built_lib.S24["x"]] - 89.1625) < 1
        # Initialize applied initializeTireSus: the state at t = 0 equals the fixture's initial state
        sol = built_lib.d24SolverHalfImplicitGPU(1000)
        sol.Construct(vj, tj, sj, 500, d_acc)
        sol.Construct(vj, tj, sj, 500, d_dl)
        sol.SetThreadsPerBlock(32)
        sol.SetTimeStep(1e-3)
        sol.Initialize(np.zeros(S24), 1000)
        assert np.allclose(sol.get_states(0, 1)[0], np.array(acc["state"]), rtol=1e-14, atol=0)
        sol.SetEndTime(22.0)
        sol.Solve()
        x1 = sol.GetSimState(499)[built_lib.S24["x"]]
        x2 = sol.GetSimState(999)[built_lib.S24["x"]]
        sol.close()
    assert abs(x1 - 235.685) < 1
    assert abs(x2 - 91.5211) < 1


def _fleet(built_lib, n, horizon, ksim, seed):
    fleet = pkg_mod("fleet")
    f = fleet.fleet24(n, seed=seed, horizon=horizon)
    sol = built_lib.d24SolverHalfImplicitGPU(n)
    sol.construct_class(f["cls"][0], f["params"])
    sol.set_driver_tables(f["tables"])
    sol.set_states(f["states"])
    sol.SetKernelSimTime(ksim)
    sol.SetEndTime(horizon)
    sol.Solve()
    got = sol.get_states()
    sol.close()
    args = (f["cls"], f["class_of"], f["params"], f["states"], f["tables"])
    kw = dict(tend=horizon, ksim=ksim, schedule=1, nthreads=NT)
    ref, _ = O.run18(*args, model=24, **kw)
    fl = state_floors24()
    env = np.max([rel_err(st, ref, fl).max(axis=1) for st, _ in _perturbed_runs(*args, **kw)], axis=0)
    return got, ref, env


@pytest.mark.parametrize("n,horizon,ksim", [(512, 10.0, 1.0), (1, 1.0, 0.3), (33, 2.0, 0.7), (129, 1.5, 1.5)])
def test_seeded_fleet24_within_reference_sensitivity(built_lib, n, horizon, ksim):
    """Vehicles the perturbations leave quiet (envelope <= 1e-13) agree within 1e-9; no more vehicles
    exceed 1e-9 than under the perturbations (+5%); each vehicle below saturation stays within 100 x
    its envelope or 1e-9."""
    got, ref, env = _fleet(built_lib, n, horizon, ksim, seed=20261203 + n)
    e = rel_err(got, ref, state_floors24()).max(axis=1)
    print(f"fleet24 n={n}: gpu>1e-9 {int((e > RTOL).sum())} (perturbed reference {int((env > RTOL).sum())}); "
          f"median gpu {np.median(e):.2e} envelope {np.median(env):.2e}")
    assert (e[env <= 1e-13] <= RTOL).all()
    assert (e > RTOL).sum() <= (env > RTOL).sum() + 0.05 * n
    below = env < 1e-3
    assert (e[below] <= np.maximum(RTOL, CHAOS_FACTOR * env[below])).all(), float(e[below].max())


def test_one_window24_parity_from_diverse_states(built_lib):
    """10 steps from states spread along the fleet's trajectories: rounding-level agreement on all
    212 fields."""
    fleet = pkg_mod("fleet")
    n = 512
    f = fleet.fleet24(n, seed=7, horizon=10.0)
    outs, ctls = [], []
    st = f["states"]
    for k in range(9):
        st, _ = O.run18(f["cls"], f["class_of"], f["params"], st, f["tables"], t0=float(k), ksim=1.0, schedule=2,
                        nthreads=NT, model=24)
        outs.append(st.copy())
        ctls.append(np.stack([O.driver_input(k + 1.0, f["tables"][i])[1:] for i in range(n)]))
    S = np.concatenate(outs)
    P = np.concatenate([f["params"]] * 9)
    ctl = np.concatenate(ctls)
    m = P.shape[0]
    sol = built_lib.d24SolverHalfImplicitGPU(m)
    sol.construct_class(f["cls"][0], P)
    sol.set_states(S)
    sol.SetKernelSimTime(0.01)
    sol.SolveStep(0.0, ctl[:, 0], ctl[:, 1], ctl[:, 2])
    got = sol.get_states()
    sol.close()
    ref, _ = O.run18(f["cls"], np.zeros(m, np.int32), P, S, ctl=ctl, t0=0.0, ksim=0.01, schedule=2, nthreads=NT,
                     model=24)
    e = rel_err(got, ref, state_floors24())
    assert e.max() <= 1e-12, (float(e.max()), int(e.max(axis=1).argmax()), int(e.max(axis=0).argmax()))


def test_model24_rejects_mixed_tire_types_and_missing_suspension(built_lib):
    sol = built_lib.d24SolverHalfImplicitGPU(4)
    with pytest.raises(built_lib.LfdmError):
        sol.set_precision(pkg_mod("_abi").PREC_MIXED)
    with pytest.raises(built_lib.LfdmError):
        sol.Initialize(np.zeros(built_lib.S24_COUNT), 1)  # Initialize needs the vehicle's parameters
    cls, p = pkg_mod("fleet").suv24()
    sol.construct_class(cls, p[None, :], built_lib.TireType.TMeasyNr)
    with pytest.raises(built_lib.LfdmError):  # one tire type per solver
        sol.construct_class(cls, p[None, :], built_lib.TireType.TMeasy)
    sol.close()
