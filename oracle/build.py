"""Builds the C oracle (test infrastructure) into oracle/_build/liboracle.so
from oracle.c (the restated algorithms and FP64 solvers) and inputs.c (input
generators, the batch semantics and the residual bound)."""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")


def lib_path() -> str:
    return os.path.join(OUT, "liboracle.so")


def build(verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    srcs = [os.path.join(HERE, "oracle.c"), os.path.join(HERE, "inputs.c")]
    lib = lib_path()
    if os.path.exists(lib) and os.path.getmtime(lib) >= max(os.path.getmtime(s) for s in srcs):
        return lib
    cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=gnu11",
           *srcs, "-o", lib, "-lm"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if verbose or p.returncode:
        sys.stderr.write(p.stdout + p.stderr)
    if p.returncode:
        raise RuntimeError("oracle build failed")
    return lib


if __name__ == "__main__":
    print(build(verbose=True))
