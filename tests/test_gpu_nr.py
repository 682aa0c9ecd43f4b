"""TMeasyNr tires on the GPU through the reference-style API for the 11-, 18- and 24-DOF models:
Construct from the reference's Sedan files (high-level tire parameters guessed from load index 97)
with TireType.TMeasyNr, Initialize from zero states, Solve over acc05. Checked against the reference
tests' own pins (tests/11dof.cpp dof11HiNr 115.1, tests/18dof.cpp dof18HiNr 114.973, tests/24dof.cpp
dof24HiNr 114.938, +-1 m there) and against the golden GPU-schedule trajectory of the reference CPU
solver (tests/golden, cases sedan*_nr_acc05_gpu)."""
import json

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _files(tmp_path, case):
    paths = []
    for name in ("vehicle", "tire", "sus"):
        if name in case:
            p = tmp_path / f"{name}.json"
            p.write_text(json.dumps(case[name]))
            paths.append(str(p))
    d = tmp_path / "acc05.txt"
    d.write_text("".join(" ".join(repr(float(v)) for v in r) + "\n" for r in case["driver"]))
    return paths, str(d)


@pytest.mark.parametrize("model,case_name,pin", [
    (18, "sedan_nr_acc05_gpu", 114.973),
    (11, "sedan11_nr_acc05_gpu", 115.1),
    (24, "sedan24_nr_acc05_gpu", 114.938),
])
def test_reference_nr_case_through_construct(built_lib, golden18, golden11_cases, golden24_cases, tmp_path, model,
                                             case_name, pin):
    golden = {18: golden18, 11: golden11_cases, 24: golden24_cases}[model]
    case = {c["name"]: c for c in golden["cases"]}[case_name]
    paths, drv = _files(tmp_path, case)
    cls_ = {11: built_lib.d11SolverHalfImplicitGPU, 18: built_lib.d18SolverHalfImplicitGPU,
            24: built_lib.d24SolverHalfImplicitGPU}[model]
    n = 40
    sol = cls_(n)
    sol.Construct(*paths, n, drv, built_lib.TireType.TMeasyNr)
    assert sol.GetTireType() == built_lib.TireType.TMeasyNr
    sol.SetTimeStep(1e-3)
    sol.SetKernelSimTime(case["ksim"])
    sol.Initialize(np.zeros(sol.STATE_COUNT), n)
    sol.SetEndTime(case["tend"])
    sol.Solve()
    st = sol.get_states()
    sol.close()
    assert np.isfinite(st).all()
    assert np.array_equal(st[0], st[-1])  # identical vehicles stay identical
    assert abs(st[0, 0] - pin) < 1.0
    # the reference CPU solver on the same schedule: this is a smooth straight-line run (no chaotic
    # wheel chatter), so the FP64 kernel agrees to rounding level on the chassis states
    exp = np.array(case["expected_final"])
    e = np.abs(st[0, :6] - exp[:6]) / np.maximum(np.abs(exp[:6]), 1.0)
    assert e.max() <= 1e-9, e
