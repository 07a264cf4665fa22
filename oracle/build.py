"""ORACLE build recipe -- test infrastructure only.

Compiles oracle/nufft_oracle.c into oracle/_build/liboracle_nufft.so with gcc
and OpenMP.  Portable C (no intrinsics, no -march=native), so the same source
builds on x86_64 and aarch64.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "nufft_oracle.c")
OUT_DIR = os.path.join(HERE, "_build")
OUT = os.path.join(OUT_DIR, "liboracle_nufft.so")


def build(force: bool = False) -> str:
    if (not force and os.path.exists(OUT)
            and os.path.getmtime(OUT) >= os.path.getmtime(SRC)):
        return OUT
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = OUT + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-fopenmp", "-shared", "-fPIC", "-std=c99",
           "-D_GNU_SOURCE", SRC, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
