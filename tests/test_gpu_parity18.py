"""CUDA path (through the C ABI) against the reference's CPU solver outputs and the oracle.

Tolerance (floating point): per state |gpu - ref| <= 1e-9 * max(|ref|, s_k), with the floors s_k
of conftest.state_floors() (1 m, 1 m/s, 1 rad, 1 rad/s, 10 rad/s for wheel/crank speeds, 1e-3 m
for tire deflections). The kernel reorders FP64 arithmetic (fused multiply-adds, shared
reciprocals, trigonometric identities), so agreement is to rounding level, not bit level.
"""
import os

import numpy as np
import pytest

import oracle_lib as O
from conftest import RESP_FLOORS, case_inputs, pkg_mod, rel_err, state_floors

pytestmark = pytest.mark.gpu
RTOL = 1e-9


def _group(cases):
    groups = {}
    for c in cases:
        if c["ksim"] > 0:
            groups.setdefault((c["ksim"], c["tend"], c["tire_type"]), []).append(c)
    return groups


def _solver_for(lfdm, cases, ksim, tend, tire_type, freq=None):
    n = len(cases)
    sol = lfdm.d18SolverHalfImplicitGPU(n)
    states = []
    for i, c in enumerate(cases):
        cls, p, s, tab = case_inputs(c)
        sol.construct_class(cls, p[None, :], tire_type)
        sol.set_driver_tables(tab[None, :, :], first=i)
        states.append(s)
    sol.set_states(np.array(states))
    sol.SetTimeStep(cases[0]["dt"])
    sol.SetKernelSimTime(ksim)
    sol.SetEndTime(tend)
    resp = None
    if freq:
        nsamp = int(round(tend * freq)) + 4
        resp = np.full((nsamp, 13, n), np.nan)
        sol.set_response_buffer(resp, freq)
    return sol, resp


def test_golden_cases_final_state(built_lib, golden18):
    fl = state_floors()
    for (ksim, tend, tt), cases in _group(golden18["cases"]).items():
        sol, _ = _solver_for(built_lib, cases, ksim, tend, tt)
        sol.Solve()
        got = sol.get_states()
        for i, c in enumerate(cases):
            e = rel_err(got[i], np.array(c["expected_final"]), fl)
            assert e.max() <= RTOL, (c["name"], float(e.max()), int(e.argmax()))
        sol.close()


def test_golden_cases_sampled_response(built_lib, golden18):
    for (ksim, tend, tt), cases in _group(golden18["cases"]).items():
        sample = cases[0]["sample"]
        freq = 1.0 / (sample * cases[0]["dt"])
        sol, resp = _solver_for(built_lib, cases, ksim, tend, tt, freq=freq)
        sol.Solve()
        for i, c in enumerate(cases):
            exp = np.array(c["expected_samples"])
            got = resp[: len(exp), :, i]
            e = rel_err(got, exp[:, 1:], RESP_FLOORS)
            assert e.max() <= RTOL, (c["name"], float(e.max()))
        sol.close()


def _fleet_vs_oracle(built_lib, n, horizon, ksim, seed, threads=None):
    fleet = pkg_mod("fleet")
    f = fleet.fleet18(n, seed=seed, horizon=horizon)
    sol = built_lib.d18SolverHalfImplicitGPU(n)
    sol.construct_class(f["cls"][0], f["params"])
    sol.set_driver_tables(f["tables"])
    sol.set_states(f["states"])
    sol.SetKernelSimTime(ksim)
    sol.SetEndTime(horizon)
    if threads:
        sol.SetThreadsPerBlock(threads)
    sol.Solve()
    got = sol.get_states()
    sol.close()
    ref, _ = O.run18(f["cls"], f["class_of"], f["params"], f["states"], f["tables"], tend=horizon, ksim=ksim,
                     schedule=1, nthreads=os.cpu_count() or 1)
    return got, ref


@pytest.mark.parametrize("threads", [32, 128])
def test_seeded_fleet_matches_oracle(built_lib, threads):
    got, ref = _fleet_vs_oracle(built_lib, 512, 10.0, 1.0, seed=20261203, threads=threads)
    e = rel_err(got, ref, state_floors()).max(axis=1)
    bad = np.nonzero(e > RTOL)[0]
    print(f"fleet parity: max {e.max():.3e}, p99 {np.quantile(e, 0.99):.3e}, outliers {bad.tolist()[:20]}")
    assert len(bad) == 0, (bad.tolist()[:20], e[bad][:20])


def test_odd_sizes_and_window_lengths(built_lib):
    """Vehicle counts that are not multiples of the block, and window lengths that do not divide
    the horizon (the last window runs past the end time, as in the reference)."""
    for n, horizon, ksim in ((1, 1.0, 0.3), (33, 2.0, 0.7), (129, 1.5, 1.5)):
        got, ref = _fleet_vs_oracle(built_lib, n, horizon, ksim, seed=n)
        e = rel_err(got, ref, state_floors())
        assert e.max() <= RTOL, (n, horizon, ksim, float(e.max()))
