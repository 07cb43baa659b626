"""Builds ``libcaroli_gb300.so`` in-tree for sm_103a (nvcc, no cmake)."""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SOURCES = [os.path.join(HERE, "csrc", f) for f in ("engine.cu", "plan.cpp")]
OUT = os.path.join(HERE, "_build", "libcaroli_gb300.so")
FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
         "-shared"]


def build(verbose=False):
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    cmd = ["nvcc", *FLAGS, "-o", OUT, *SOURCES]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    return OUT


if __name__ == "__main__":
    build(verbose=True)
