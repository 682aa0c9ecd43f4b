"""Build liblfdm.so (the C-ABI library) in-tree: nvcc for the sm_103a kernels, g++ for the host side.

    python -m <package>.build      or     from <package> import build; build.build()

Translation units are compiled in parallel; the library is rebuilt only when a source is newer.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "liblfdm.so")
ROOT_INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


def _sources():
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    cpp = sorted(glob.glob(os.path.join(CSRC, "*.cpp")))
    hdr = sorted(glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) +
                 glob.glob(os.path.join(ROOT_INCLUDE, "*.h")) +
                 glob.glob(os.path.join(ROOT_INCLUDE, "lfdm", "device", "*.cuh")))
    return cu, cpp, hdr


def _stale(lib: str, deps) -> bool:
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False, extra_nvcc: list[str] | None = None) -> str:
    cu, cpp, hdr = _sources()
    if not force and not _stale(LIB, cu + cpp + hdr + [__file__]):
        return LIB
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(OUT, exist_ok=True)
    jobs = []
    objs = []
    for src in cu:
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        # --fmad=false: only the fma() calls written in the source fuse. Implicit contraction of a
        # multiply and an add depends on the surrounding code (a product with a second use is not
        # fused), so the same device function could round differently in the window kernels and in
        # the fleet kernel; with it off, every kernel that runs a step computes it bit for bit alike.
        cmd = [nvcc, *ARCH, "-O3", "--fmad=false", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas",
               "-warn-spills", "-c", src, "-o", obj, *(extra_nvcc or [])]
        jobs.append((cmd, obj))
    for src in cpp:
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", f"-I{cuda}/include", "-c", src, "-o", obj]
        jobs.append((cmd, obj))
    procs = []
    for cmd, obj in jobs:
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True), cmd, obj))
    failed = []
    for p, cmd, obj in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((cmd, out))
        elif verbose and out.strip():
            print(out, file=sys.stderr)
        objs.append(obj)
    if failed:
        msg = "\n".join(" ".join(c) + "\n" + o for c, o in failed)
        raise RuntimeError("liblfdm build failed:\n" + msg)
    tmp = LIB + ".tmp"
    link = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("liblfdm link failed:\n" + " ".join(link) + "\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
