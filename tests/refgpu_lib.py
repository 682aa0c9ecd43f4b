"""Runs the reference's own GPU kernels (oracle/_ref/ref{11,18,24}.cubin, built from the reference
sources by `make -C oracle refgpu` where the checkout exists) through oracle/refgpu_launch — test
infrastructure only (tests and the bench's reference-GPU comparison)."""
from __future__ import annotations

import json
import os
import subprocess
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE = os.path.join(ROOT, "oracle")
LAUNCHER = os.path.join(ORACLE, "_build", "refgpu_launch")


def cubin(model: int = 18) -> str:
    return os.path.join(ORACLE, "_ref", f"ref{model}.cubin")


def available(model: int = 18) -> bool:
    return os.path.exists(cubin(model))


def build_launcher() -> str:
    subprocess.run(["make", "-s", "-C", ORACLE, "launcher"], check=True)
    return LAUNCHER


def run(cls, params, tables, states, *, model=18, dt=1e-3, ksim=2.0, tend=10.0, dtout=0.0, tpb=32):
    """The reference GPU solver's Solve over n vehicles of one class (TMeasy tires); returns (final
    states [n][state count of the model] in this library's flat layout, per-window kernel ms)."""
    n = params.shape[0]
    tables = np.ascontiguousarray(tables, dtype=np.float64)
    assert tables.ndim == 3 and tables.shape[0] == n
    with tempfile.TemporaryDirectory() as tmp:
        inp, out = os.path.join(tmp, "in.bin"), os.path.join(tmp, "out.bin")
        with open(inp, "wb") as f:
            f.write(np.array([model, n, tables.shape[1], tpb], dtype=np.int32).tobytes())
            f.write(np.array([dt, ksim, tend, dtout], dtype=np.float64).tobytes())
            f.write(bytes(cls))
            f.write(np.ascontiguousarray(params, dtype=np.float64).tobytes())
            f.write(tables.tobytes())
            f.write(np.ascontiguousarray(states, dtype=np.float64).tobytes())
        r = subprocess.run([LAUNCHER, cubin(model), inp, out], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference GPU launcher failed ({r.returncode}): {r.stderr}")
        final = np.fromfile(out, dtype=np.float64).reshape(n, -1)
        info = json.loads(r.stdout.strip().splitlines()[-1])
    return final, info["window_ms"]
