"""Runs the reference's own GPU kernel (oracle/_ref/ref18.cubin, built from the reference sources
by `make -C oracle refgpu` where the checkout exists) through oracle/refgpu18_launch — test
infrastructure only."""
from __future__ import annotations

import ctypes
import json
import os
import subprocess
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE = os.path.join(ROOT, "oracle")
CUBIN = os.path.join(ORACLE, "_ref", "ref18.cubin")
LAUNCHER = os.path.join(ORACLE, "_build", "refgpu18_launch")


def available() -> bool:
    return os.path.exists(CUBIN)


def build_launcher() -> str:
    subprocess.run(["make", "-s", "-C", ORACLE, "launcher"], check=True)
    return LAUNCHER


def run(cls, params, tables, states, *, dt=1e-3, ksim=2.0, tend=10.0, dtout=0.0, tpb=32):
    """Reference GPU Solve over n vehicles of one class; returns (final states [n][75], window ms)."""
    n = params.shape[0]
    tables = np.ascontiguousarray(tables, dtype=np.float64)
    assert tables.ndim == 3 and tables.shape[0] == n
    with tempfile.TemporaryDirectory() as tmp:
        inp, out = os.path.join(tmp, "in.bin"), os.path.join(tmp, "out.bin")
        with open(inp, "wb") as f:
            f.write(np.array([n, tables.shape[1], tpb, 0], dtype=np.int32).tobytes())
            f.write(np.array([dt, ksim, tend, dtout], dtype=np.float64).tobytes())
            f.write(bytes(cls))
            f.write(np.ascontiguousarray(params, dtype=np.float64).tobytes())
            f.write(tables.tobytes())
            f.write(np.ascontiguousarray(states, dtype=np.float64).tobytes())
        r = subprocess.run([LAUNCHER, CUBIN, inp, out], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference GPU launcher failed ({r.returncode}): {r.stderr}")
        final = np.fromfile(out, dtype=np.float64).reshape(n, -1)
        info = json.loads(r.stdout.strip().splitlines()[-1])
    return final, info["window_ms"]
