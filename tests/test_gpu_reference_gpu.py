"""The reference's OWN GPU solver (its Integrate kernel compiled from its sources) on this GPU:
it must reproduce the reference CPU goldens (which validates the launcher), and the CUDA path is
timed against it on the same fleet. Skipped where the reference cubin was not built."""
import numpy as np
import pytest

import refgpu_lib as R
from conftest import case_inputs, pkg_mod, rel_err, state_floors

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not R.available(), reason="reference cubin not built here")]


@pytest.fixture(scope="module")
def launcher():
    return R.build_launcher()


def test_reference_gpu_kernel_reproduces_goldens(launcher, golden18):
    by = {c["name"]: c for c in golden18["cases"]}
    for name in ("hmmwv_acc3_gpu", "hmmwv_dl4_gpu"):
        c = by[name]
        cls, p, s, tab = case_inputs(c)
        final, _ = R.run(cls, p[None], tab[None], s[None], dt=c["dt"], ksim=c["ksim"], tend=c["tend"])
        e = rel_err(final[0], np.array(c["expected_final"]), state_floors())
        assert e.max() <= 1e-9, (name, float(e.max()))


def test_throughput_vs_reference_gpu_kernel(launcher, built_lib):
    """300,000 SUV vehicles, 1 s windows, outputs every 10 ms: window 2 and 3 timed for both."""
    fleet = pkg_mod("fleet")
    n, ksim, windows = 300_000, 1.0, 3
    f = fleet.fleet18(n, seed=20261203, horizon=windows * ksim)
    res = {}
    for tpb in (32, 16):
        _, ms = R.run(f["cls"][0], f["params"], f["tables"], f["states"], ksim=ksim, tend=windows * ksim,
                      dtout=0.01, tpb=tpb)
        res[f"reference_tpb{tpb}"] = n * 1000 * (windows - 1) / (sum(ms[1:]) * 1e-3)
    sol = built_lib.d18SolverHalfImplicitGPU(n)
    sol.construct_class(f["cls"][0], f["params"])
    sol.set_driver_tables(f["tables"])
    sol.set_states(f["states"])
    sol.SetKernelSimTime(ksim)
    sol.SetEndTime(windows * ksim)
    import torch

    buf = torch.empty(100 * 13 * n, dtype=torch.float64, device="cuda")
    sol.set_response_device(buf.data_ptr(), buf.numel(), 100.0)
    sol.solve_range(-0.5, 0.5)
    sol.solve_range(0.5, windows - 0.5)
    ms, launches = sol.last_kernel_ms()
    res["ours"] = n * 1000 * launches / (ms * 1e-3)
    best_ref = max(res["reference_tpb32"], res["reference_tpb16"])
    print("vehicle-steps/s:", {k: f"{v:.3e}" for k, v in res.items()}, f"speed-up {res['ours'] / best_ref:.2f}x")
    assert res["ours"] >= 1.5 * best_ref
