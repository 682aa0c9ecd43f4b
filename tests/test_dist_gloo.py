"""The multi-process path of bench.py on the CPU with gloo, world size 2: the timing reductions (max
over ranks of the device time, sum of the vehicle-steps), the barrier, the per-rank fleets (weak
scaling: each rank a replica with its own seed; vehicles are independent, so there is no data
exchange), and the reference arm, which rank 0 alone runs while the others return at once."""
import multiprocessing as mp
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, q) -> None:
    os.environ.update(WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    try:
        import bench
        d = bench.Dist(0)
        out = {"rank": d.rank, "world": d.world, "max": d.max(10.0 * (rank + 1)), "sum": d.sum(float(rank + 1))}
        d.barrier()
        fleet = bench.importlib.import_module(bench.PKG + ".fleet")
        f = fleet.fleet18(8, seed=bench.SEED + d.rank, horizon=1.0)
        out["u0"] = f["states"][:, 0:8].sum()

        class A:  # the reference arm's arguments; rank 1 must return before doing any work
            cpu_sample, warmup, steps, ksim = 4, 0, 0, 1.0
        out["ref_skipped"] = bench.run_reference(A, d) is None if d.rank != 0 else None
        d.barrier()
        d.pg.destroy_process_group()
        q.put(out)
    except Exception as e:  # reported to the parent
        q.put({"rank": rank, "error": repr(e)})


def test_two_ranks_with_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=180) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res = sorted(res, key=lambda r: r["rank"])
    for r in res:
        assert "error" not in r, r
        assert r["world"] == 2
        assert r["max"] == 20.0 and r["sum"] == 3.0
    assert res[1]["ref_skipped"] is True
    assert not np.isclose(res[0]["u0"], res[1]["u0"])  # each rank its own seeded replica fleet
