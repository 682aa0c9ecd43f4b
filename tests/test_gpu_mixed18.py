"""Mixed-precision form (FP32 right-hand side; FP64 states, X/Y/yaw accumulation and the low-speed
slip normalisation) against the FP64 form, which is its oracle."""
import os

import numpy as np
import pytest

import oracle_lib as O
from conftest import case_inputs, pkg_mod

pytestmark = pytest.mark.gpu


def _solve(lfdm, cls, params, tables, states, horizon, prec, ksim=1.0):
    n = params.shape[0]
    s = lfdm.d18SolverHalfImplicitGPU(n)
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


def _pos_err(a, b):
    return np.hypot(a[:, 0] - b[:, 0], a[:, 1] - b[:, 1])


def test_mixed_on_reference_fixtures(built_lib, golden18):
    """Well-conditioned trajectories: end position within 1 mm, yaw within 1e-4 rad, speed within
    1e-4 m/s of the reference's FP64 result."""
    for c in golden18["cases"]:
        if not c["name"].startswith("hmmwv") or c["ksim"] == 0:
            continue
        cls, p, s, tab = case_inputs(c)
        m, _ = _solve(built_lib, cls, p[None], tab[None], s[None], c["tend"], 1, ksim=c["ksim"])
        e = np.array(c["expected_final"])
        assert np.hypot(m[0, 0] - e[0], m[0, 1] - e[1]) <= 1e-3, c["name"]
        assert abs(m[0, 4] - e[4]) <= 1e-4, c["name"]
        assert abs(m[0, 2] - e[2]) <= 1e-4, c["name"]


def test_mixed_error_distribution_on_seeded_fleet(built_lib):
    """The rounding-chaotic SUV fleet (10 s): median end-position error within 1 cm, and the
    fraction of vehicles within 1 cm no more than 0.15 below that of the reference's own
    FMA-contracted FP64 build (its rounding-noise floor)."""
    fleet = pkg_mod("fleet")
    n, H = 2048, 10.0
    f = fleet.fleet18(n, seed=5, horizon=H)
    fp64, _ = _solve(built_lib, f["cls"][0], f["params"], f["tables"], f["states"], H, 0)
    mixed, _ = _solve(built_lib, f["cls"][0], f["params"], f["tables"], f["states"], H, 1)
    args = (f["cls"], f["class_of"], f["params"], f["states"], f["tables"])
    ref, _ = O.run18(*args, tend=H, ksim=1.0, nthreads=os.cpu_count() or 1)
    fma, _ = O.run18(*args, tend=H, ksim=1.0, nthreads=os.cpu_count() or 1, fma=True)
    e_mix = _pos_err(mixed, fp64)
    e_noise = _pos_err(fma, ref)
    print(f"mixed vs fp64: p50 {np.median(e_mix):.2e} m, within 1 cm {np.mean(e_mix <= 0.01):.3f}; "
          f"reference FMA-build noise within 1 cm {np.mean(e_noise <= 0.01):.3f}")
    assert np.median(e_mix) <= 0.01
    assert np.mean(e_mix <= 0.01) >= np.mean(e_noise <= 0.01) - 0.15


def test_mixed_is_faster(built_lib):
    fleet = pkg_mod("fleet")
    n = 65536
    f = fleet.fleet18(n, seed=9, horizon=1.0)
    _, ms64 = _solve(built_lib, f["cls"][0], f["params"], f["tables"], f["states"], 1.0, 0)
    _, ms32 = _solve(built_lib, f["cls"][0], f["params"], f["tables"], f["states"], 1.0, 1)
    print(f"fp64 {ms64:.1f} ms, mixed {ms32:.1f} ms, speed-up {ms64 / ms32:.2f}x")
    assert ms64 / ms32 >= 1.8


def test_mixed_rejects_tmeasy_nr(built_lib):
    lfdm = built_lib
    cls, p = pkg_mod("fleet").suv18()
    s = lfdm.d18SolverHalfImplicitGPU(2)
    s.construct_class(cls, np.repeat(p[None], 2, 0), tire_type=1)
    s.set_states(np.zeros((2, lfdm.S_COUNT)))
    s.set_driver_tables(np.array([[0.0, 0, 0, 0], [1.0, 0, 0, 0]]))
    s.SetEndTime(0.1)
    s.SetKernelSimTime(0.1)
    s.set_precision(1)
    with pytest.raises(lfdm.LfdmError):
        s.Solve()
