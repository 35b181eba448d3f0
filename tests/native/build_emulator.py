"""Build the CPU emulator of the kernel phases (test-only shared library).

``emulate.cu`` runs the load/compute/gather phase functions of the GPU
kernels sequentially on the host.  It is compiled with nvcc (host code only
is executed) into ``tests/native/_emulate.so``, which is git-ignored.
"""
from __future__ import annotations

import ctypes
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
CSRC = os.path.join(ROOT, "topomax_gb300", "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(HERE, "_emulate.so")


def build() -> str:
    srcs = [os.path.join(HERE, "emulate.cu"), os.path.join(CSRC, "topo_mg_common.cu")]
    deps = srcs + [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    if os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps):
        return LIB
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cmd = [nvcc, "-std=c++17", "-O1", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-shared", "-I", INCLUDE, "-I", CSRC,
           "--expt-relaxed-constexpr", "-gencode", "arch=compute_103a,code=sm_103a", *srcs,
           "-o", LIB + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"emulator build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(LIB + ".tmp", LIB)
    return LIB


def load() -> ctypes.CDLL:
    return ctypes.CDLL(build())
