"""Build recipe for the native parts (no CMake): the sm_103a engine library
and the C++ host front end that mirrors the reference's classes.

    python -m mps_gb300.build            # engine + host
    python -m mps_gb300.build --engine   # engine only

Products land in mps_gb300/lib/ (git-ignored).  Translation units are
compiled in parallel; each is recompiled only when it or a header changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
LIB = os.path.join(HERE, "lib")
OBJ = os.path.join(LIB, "obj")
ENGINE_SO = os.path.join(LIB, "libmps_gb300.so")
HOST_EXE = os.path.join(LIB, "mps")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "--extended-lambda", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-ffp-contract=off", "-I", os.path.join(REPO, "include")]
ENGINE_SRCS = ["sort.cu", "sweeps.cu", "solver.cu", "mg.cu", "capi.cu", "adjoint.cu", "batch.cu", "noalloc.cu",
               "io.cu", "symcheck.cu", "selftest.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r


def build_engine(verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith(".cuh")]
    headers.append(os.path.join(REPO, "include", "mps_gb300.h"))
    jobs = []
    objs = []
    for src in ENGINE_SRCS:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src.replace(".cu", ".o"))
        objs.append(o)
        if _newer(o, [s] + headers):
            cmd = [nvcc()] + NVCC_FLAGS + ["-c", s, "-o", o]
            if verbose:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for r in ex.map(_run, jobs):
            if verbose:
                sys.stderr.write(r.stderr)
    if _newer(ENGINE_SO, objs):
        _run([nvcc()] + ARCH + ["-shared", "-o", ENGINE_SO] + objs + ["-lpthread"])
    return ENGINE_SO


def build_host() -> str:
    """The C++ front end (Simulation/MPS/Particle/Bucket/Settings/Exporter)."""
    if not os.path.isdir(HOST):
        return ""
    srcs = sorted(os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".cpp"))
    hdrs = [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".hpp")]
    if not srcs:
        return ""
    deps = srcs + hdrs + [ENGINE_SO, os.path.join(REPO, "include", "mps_gb300.h")]
    if _newer(HOST_EXE, deps):
        cxx = os.environ.get("CXX", "g++")
        _run([cxx, "-std=c++20", "-O2", "-pthread", "-ffp-contract=off", "-I", os.path.join(REPO, "include"),
              "-o", HOST_EXE] + srcs + ["-L", LIB, "-lmps_gb300", f"-Wl,-rpath,{LIB}",
                                         "-Wl,-rpath,$ORIGIN"])
    return HOST_EXE


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    build_engine(verbose="--verbose" in argv)
    if "--engine" not in argv:
        build_host()


if __name__ == "__main__":
    main()
