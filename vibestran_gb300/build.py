"""Build libvsgb.so (sm_103a) in-tree: vibestran_gb300/_lib/libvsgb.so.

Each CUDA translation unit is compiled by nvcc in parallel with
``-gencode arch=compute_103a,code=sm_103a -lineinfo -O3``, host C++ with g++,
and the objects are linked by nvcc into one shared library with the CUDA
runtime linked statically (no torch types anywhere in the ABI).
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
LIB = os.path.join(OUT_DIR, "libvsgb.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xptxas", "-warn-spills", "-DNDEBUG"]
CXX_FLAGS = ["-O2", "-std=c++20", "-fPIC", "-Wall", "-DNDEBUG"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    return cu, cpp


def _digest() -> str:
    h = hashlib.sha256()
    for d in (CSRC, os.path.join(ROOT, "include")):
        for f in sorted(os.listdir(d)):
            p = os.path.join(d, f)
            if os.path.isfile(p):
                h.update(f.encode())
                with open(p, "rb") as fh:
                    h.update(fh.read())
    h.update(" ".join(ARCH + NVCC_FLAGS + CXX_FLAGS).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compile (if sources changed) and return the path of libvsgb.so."""
    os.makedirs(OBJ_DIR, exist_ok=True)
    stamp = os.path.join(OUT_DIR, "build.stamp")
    dig = _digest()
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as fh:
            if fh.read().strip() == dig:
                return LIB
    cu, cpp = _sources()
    jobs = []
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    for f in cu:
        obj = os.path.join(OBJ_DIR, f + ".o")
        jobs.append(([nvcc()] + ARCH + NVCC_FLAGS + extra +
                     ["-c", os.path.join(CSRC, f), "-o", obj], obj))
    for f in cpp:
        obj = os.path.join(OBJ_DIR, f + ".o")
        jobs.append((["g++"] + CXX_FLAGS + ["-c", os.path.join(CSRC, f), "-o", obj], obj))
    logs = []
    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        futs = {ex.submit(_run, cmd): cmd for cmd, _ in jobs}
        for fut in cf.as_completed(futs):
            logs.append(fut.result())
    tmp = LIB + f".tmp{os.getpid()}"
    _run([nvcc()] + ARCH + ["-shared", "-o", tmp] + [o for _, o in jobs] +
         ["-cudart", "static", "-Xcompiler", "-fPIC", "-lpthread", "-ldl", "-lrt"])
    os.replace(tmp, LIB)
    with open(stamp, "w") as fh:
        fh.write(dig)
    if verbose or ptxas_info:
        sys.stdout.write("\n".join(logs))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
