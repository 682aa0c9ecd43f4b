"""bench.py's reference arm on the CPU, as rank 0 of a one-process run prints it: one JSON line with
the headline's metric and unit, `impl: reference`, a `cpu_baseline` describing the run (the oracle
port on the host cores, kind "port") and an `e2e` object carrying the line's own value with no host
copies; the trajectories continue from window to window."""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


class _Args:
    cpu_sample, warmup, steps, ksim, gpus, vehicles = 16, 1, 2, 0.05, 1, 16


def test_reference_arm_prints_the_contract_line(capsys, monkeypatch):
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    sys.path.insert(0, ROOT)
    import bench
    bench.run_reference(_Args, bench.Dist(0))
    lines = [ln for ln in capsys.readouterr().out.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == "vehicle-steps/s"
    assert d["higher_is_better"] is True and d["steps"] == 2 and d["warmup"] == 1 and d["n_gpus"] == 1
    assert np.isfinite(d["value"]) and d["value"] > 0
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == d["value"] and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["vehicles"] == 16 and d["config"]["kernel_sim_time"] == 0.05


def test_cpu_trajectory_continues_across_windows():
    """Two calls of one 0.05 s window each continue one trajectory: bit for bit the oracle's run of
    the same two windows in one call (a window length of 0.1 s would round the step times
    differently)."""
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import bench
    import oracle_lib as O
    fleet = bench.importlib.import_module(bench.PKG + ".fleet")
    f = fleet.fleet18(8, seed=bench.SEED, horizon=0.1)
    cpu = bench.CpuTrajectory(f, 8, 0.05, 1)
    cpu.window()
    cpu.window()
    want, _ = O.run18(f["cls"], f["class_of"], f["params"], np.array(f["states"], copy=True), f["tables"],
                      t0=0.0, tend=0.1, ksim=0.05, schedule=1, nthreads=1, model=18, timing=True)
    assert np.array_equal(cpu.states, want)
    assert not np.array_equal(cpu.states, f["states"])
