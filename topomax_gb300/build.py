"""Build the sm_103a C-ABI library ``libtopomax_gb300.so`` in-tree.

Each ``csrc/*.cu`` translation unit is compiled in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a`` and linked into one shared
library next to this file.  No CMake, no torch extension machinery: the
library exports the plain C ABI declared in ``include/topomax_gb300.h``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libtopomax_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code is compiled without floating-point contraction: gcc fuses a*b+c into
# one FMA by default on aarch64 but not on x86-64, and the set-up values (node
# coordinates, flow profiles, load weights) must round the same on both.
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
         "-I", INCLUDE, "-I", CSRC, "--expt-relaxed-constexpr"]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build topomax_gb300")
    return path


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    """Compile (if anything changed) and return the library path."""
    deps = _deps() + [os.path.abspath(__file__)]
    if not force and not _stale(LIB, deps):
        return LIB
    os.makedirs(OBJ, exist_ok=True)
    cc = nvcc()
    srcs = _sources()
    objs = [os.path.join(OBJ, os.path.basename(s)[:-3] + ".o") for s in srcs]

    def compile_one(pair):
        src, obj = pair
        cmd = [cc, *ARCH, *FLAGS, "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        for msg in ex.map(compile_one, zip(srcs, objs)):
            if verbose and msg:
                print(msg)
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-cudart", "shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
