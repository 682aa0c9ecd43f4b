"""The two mixed-precision forms against the FP64 form, which is their oracle (the FP64 stepper is
pinned to the reference's CPU solver by the parity tests):
  * LFDM_PREC_MIXED (18-DOF): FP32 right-hand side; FP64 states, X/Y/yaw accumulation and the
    low-speed slip normalisation;
  * LFDM_PREC_MIXED_TIRE (11/18/24-DOF): only the TMeasy tire core (load interpolation of the curve
    parameters, combined slip, force curve, relaxation rates) in FP32; everything else FP64.
Accuracy is judged against the rounding noise of the reference algorithm itself (its FMA-contracted
build against its plain build, both run by the oracle)."""
import os

import numpy as np
import pytest

import oracle_lib as O
from conftest import case_inputs, pkg_mod

pytestmark = pytest.mark.gpu
NT = os.cpu_count() or 1
PRECS = (1, 2)  # LFDM_PREC_MIXED, LFDM_PREC_MIXED_TIRE


def _solver(lfdm, model, n):
    return {18: lfdm.d18SolverHalfImplicitGPU, 11: lfdm.d11SolverHalfImplicitGPU,
            24: lfdm.d24SolverHalfImplicitGPU}[model](n)


def _solve(lfdm, cls, params, tables, states, horizon, prec, ksim=1.0, model=18):
    n = params.shape[0]
    s = _solver(lfdm, model, n)
    s.construct_class(cls, params)
    s.set_driver_tables(tables)
    s.set_states(states)
    s.SetKernelSimTime(ksim)
    s.SetEndTime(horizon)
    s.set_precision(prec)
    s.Solve()
    out = s.get_states()
    ms, launches = s.last_kernel_ms()
    s.close()
    return out, ms


def _xy(model):
    abi = pkg_mod("_abi")
    lay = {18: abi.S, 11: abi.S11, 24: abi.S24}[model]
    return lay["x"], lay["y"]


def _pos_err(a, b, model=18):
    ix, iy = _xy(model)
    return np.hypot(a[:, ix] - b[:, ix], a[:, iy] - b[:, iy])


def test_precision_enum_matches_header(built_lib):
    abi = pkg_mod("_abi")
    assert (abi.PREC_FP64, abi.PREC_MIXED, abi.PREC_MIXED_TIRE) == (0, 1, 2)


@pytest.mark.parametrize("prec", PRECS)
def test_mixed_on_reference_fixtures(built_lib, golden18, prec):
    """Well-conditioned trajectories: end position within 1 mm, yaw within 1e-4 rad, speed within
    1e-4 m/s of the reference's FP64 result."""
    for c in golden18["cases"]:
        if not c["name"].startswith("hmmwv") or c["ksim"] == 0:
            continue
        cls, p, s, tab = case_inputs(c)
        m, _ = _solve(built_lib, cls, p[None], tab[None], s[None], c["tend"], prec, ksim=c["ksim"])
        e = np.array(c["expected_final"])
        assert np.hypot(m[0, 0] - e[0], m[0, 1] - e[1]) <= 1e-3, c["name"]
        assert abs(m[0, 4] - e[4]) <= 1e-4, c["name"]
        assert abs(m[0, 2] - e[2]) <= 1e-4, c["name"]


def _within_floor(noise, gap, n):
    """The least fraction of n vehicles within 1 cm of FP64 a form may reach: the reference build's
    noise floor less the form's allowed gap, less two binomial standard deviations of the fraction
    at n vehicles. On a rounding-chaotic fleet each vehicle's end point flips in or out of 1 cm
    under an ulp-level change of either run (a change of FP64 rounding in one tire-curve regime
    moved the 24-DOF fraction by 0.003 at 2,048 vehicles with the FP32 code untouched), so the
    fraction carries that sampling noise."""
    p = min(max(noise - gap, 0.0), 1.0)
    return noise - gap - 2.0 * np.sqrt(p * (1.0 - p) / n)


def _noise_within(model, f, horizon, tol=0.01):
    args = (f["cls"], f["class_of"], f["params"], f["states"], f["tables"])
    ref, _ = O.run18(*args, tend=horizon, ksim=1.0, nthreads=NT, model=model)
    fma, _ = O.run18(*args, tend=horizon, ksim=1.0, nthreads=NT, fma=True, model=model)
    return float(np.mean(_pos_err(fma, ref, model) <= tol))


@pytest.mark.parametrize("prec", PRECS)
def test_mixed_error_distribution_on_seeded_fleet(built_lib, prec):
    """The rounding-chaotic SUV fleet (10 s): median end-position error within 1 cm, and the
    fraction of vehicles within 1 cm no more than 0.15 (MIXED) or 0.08 (MIXED_TIRE) below that of
    the reference's own FMA-contracted FP64 build (its rounding-noise floor), to the fraction's
    sampling noise at 2,048 vehicles."""
    fleet = pkg_mod("fleet")
    n, H = 2048, 10.0
    f = fleet.fleet18(n, seed=5, horizon=H)
    fp64, _ = _solve(built_lib, f["cls"][0], f["params"], f["tables"], f["states"], H, 0)
    mixed, _ = _solve(built_lib, f["cls"][0], f["params"], f["tables"], f["states"], H, prec)
    e_mix = _pos_err(mixed, fp64)
    noise = _noise_within(18, f, H)
    print(f"prec {prec} vs fp64: p50 {np.median(e_mix):.2e} m, within 1 cm {np.mean(e_mix <= 0.01):.3f}; "
          f"reference FMA-build noise within 1 cm {noise:.3f}")
    assert np.median(e_mix) <= 0.01
    assert np.mean(e_mix <= 0.01) >= _within_floor(noise, 0.15 if prec == 1 else 0.08, n)


def test_mixed_on_calm_fleet(built_lib):
    """On the calm fleet (trajectories insensitive to FP64-level rounding) both forms end within 1 cm
    of FP64 on at least 99 % of the vehicles over 10 s, with a median below 1 mm. FP32-level rounding
    can still move a discrete event (a gear shift, the converter's flow direction) by a step on a
    few vehicles; their count is printed."""
    fleet = pkg_mod("fleet")
    n, H = 2048, 10.0
    f = fleet.fleet18_calm(n, horizon=H)
    fp64, _ = _solve(built_lib, f["cls"][0], f["params"], f["tables"], f["states"], H, 0)
    res = {}
    for prec in PRECS:
        m, _ = _solve(built_lib, f["cls"][0], f["params"], f["tables"], f["states"], H, prec)
        e = _pos_err(m, fp64)
        res[prec] = e
        print(f"calm fleet prec {prec}: max {e.max():.2e} m (vehicle {int(e.argmax())}), p50 {np.median(e):.2e} m, "
              f"p99 {np.quantile(e, 0.99):.2e} m, beyond 1 cm {int((e > 0.01).sum())} of {n}")
    for prec, e in res.items():
        assert np.mean(e <= 0.01) >= 0.99, (prec, float(np.mean(e <= 0.01)))
        assert np.median(e) <= 1e-3, (prec, float(np.median(e)))


@pytest.mark.parametrize("prec,factor", [(1, 1.8), (2, 1.5)])
def test_mixed_is_faster(built_lib, prec, factor):
    fleet = pkg_mod("fleet")
    n = 65536
    f = fleet.fleet18(n, seed=9, horizon=1.0)
    _, ms64 = _solve(built_lib, f["cls"][0], f["params"], f["tables"], f["states"], 1.0, 0)
    _, ms32 = _solve(built_lib, f["cls"][0], f["params"], f["tables"], f["states"], 1.0, prec)
    print(f"fp64 {ms64:.1f} ms, prec {prec} {ms32:.1f} ms, speed-up {ms64 / ms32:.2f}x")
    assert ms64 / ms32 >= factor


@pytest.mark.parametrize("model", [11, 24])
def test_mixed_tire_11_and_24dof(built_lib, model):
    """The FP32 tire core in the single-track and 24-DOF steppers: on the seeded SUV fleets (10 s)
    median end-position error within 1 cm of FP64 and the fraction within 1 cm no more than 0.08
    below the reference's FMA-build noise floor (to its sampling noise); at 65,536 vehicles at least
    1.3 times as fast."""
    fleet = pkg_mod("fleet")
    gen = {11: fleet.fleet11, 24: fleet.fleet24}[model]
    n, H = 2048, 10.0
    f = gen(n, seed=5, horizon=H)
    fp64, _ = _solve(built_lib, f["cls"][0], f["params"], f["tables"], f["states"], H, 0, model=model)
    mt, _ = _solve(built_lib, f["cls"][0], f["params"], f["tables"], f["states"], H, 2, model=model)
    e = _pos_err(mt, fp64, model)
    noise = _noise_within(model, f, H)
    print(f"{model}-DOF tire core FP32 vs fp64: p50 {np.median(e):.2e} m, within 1 cm {np.mean(e <= 0.01):.3f}; "
          f"reference FMA-build noise within 1 cm {noise:.3f}")
    assert np.median(e) <= 0.01
    assert np.mean(e <= 0.01) >= _within_floor(noise, 0.08, n)
    g = gen(65536, seed=9, horizon=1.0)
    _, ms64 = _solve(built_lib, g["cls"][0], g["params"], g["tables"], g["states"], 1.0, 0, model=model)
    _, ms32 = _solve(built_lib, g["cls"][0], g["params"], g["tables"], g["states"], 1.0, 2, model=model)
    print(f"{model}-DOF at 65,536: fp64 {ms64:.1f} ms, tire core FP32 {ms32:.1f} ms, {ms64 / ms32:.2f}x")
    assert ms64 / ms32 >= 1.3


def test_fp32_probe_rate(built_lib):
    """The FP32 FMA probe runs at least 16 times the FP64 one (GB300: 128 against 2 lane FMA per
    clock and SM) and reports a plausible SM clock."""
    r64, g64 = built_lib.measure_fp64_peak_clock(0)
    r32, g32 = built_lib.measure_fp32_peak_clock(0)
    print(f"FP64 {r64:.3e} DFMA/s at {g64:.3f} GHz; FP32 {r32:.3e} FFMA/s at {g32:.3f} GHz")
    assert r32 >= 16 * r64
    assert 0.5 < g32 < 3.0


@pytest.mark.parametrize("model", [18, 11, 24])
def test_mixed_rejects_tmeasy_nr(built_lib, model):
    """The FP32 right-hand-side form is built for the 18-DOF model with TMeasy tires only."""
    lfdm = built_lib
    if model != 18:
        s = _solver(lfdm, model, 2)
        with pytest.raises(lfdm.LfdmError):
            s.set_precision(1)
        s.close()
        return
    fleet = pkg_mod("fleet")
    cls, p = fleet.suv18()
    s = _solver(lfdm, model, 2)
    s.construct_class(cls, np.repeat(p[None], 2, 0), tire_type=1)
    s.set_states(np.zeros((2, lfdm.S_COUNT)))
    s.set_driver_tables(np.array([[0.0, 0, 0, 0], [1.0, 0, 0, 0]]))
    s.SetEndTime(0.1)
    s.SetKernelSimTime(0.1)
    s.set_precision(1)
    with pytest.raises(lfdm.LfdmError):
        s.Solve()
    s.close()


@pytest.mark.parametrize("model,case", [(18, "sedan_rwd_nr_acc05_gpu"), (11, "sedan11_rwd_nr_acc05_gpu"),
                                        (24, "sedan24_rwd_nr_acc05_gpu"), (18, "sedan_tmod_nls_nr_dl4_gpu")])
def test_mixed_tire_with_tmeasy_nr(built_lib, golden18, golden11_cases, golden24_cases, model, case):
    """The FP32 tire core with TMeasyNr tires (Coulomb force, slips, curve, blend in FP32) on the
    Sedan TMeasyNr fixtures (trajectories insensitive to rounding): the end position within 1 cm of
    the reference's FP64 result."""
    from conftest import case_inputs11, case_inputs24
    golden = {18: golden18, 11: golden11_cases, 24: golden24_cases}[model]
    inputs = {18: case_inputs, 11: case_inputs11, 24: case_inputs24}[model]
    c = {x["name"]: x for x in golden["cases"]}[case]
    cls, p, st, tab = inputs(c)
    sol = _solver(built_lib, model, 1)
    sol.construct_class(cls, p[None], 1)
    sol.set_driver_tables(tab[None])
    sol.set_states(st[None])
    sol.SetKernelSimTime(c["ksim"])
    sol.SetEndTime(c["tend"])
    sol.set_precision(2)
    sol.Solve()
    got = sol.get_states()
    sol.close()
    e = _pos_err(got, np.array(c["expected_final"])[None], model)[0]
    print(f"{case}: FP32 Nr tire core end-position error {e:.2e} m")
    assert e <= 0.01
