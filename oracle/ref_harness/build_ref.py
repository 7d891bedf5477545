"""Builds the reference harness binary oracle/_ref/ref_driver (test
infrastructure).

The reference's own sources are compiled where they lie (read-only checkout)
against the stub headers in ./stubs (single-rank MPI, glog / gflags / Cilk
shims); nothing of the reference is copied.  Its six .cu files are not
compiled: the harness runs the CPU path (-gpu_start=0) and the CUDA shim
entry points are linked as no-ops (stubs/cuda_shim.cc).  Needs the reference
checkout, g++ and the CUDA runtime library; the reference's build system
(cmake, gcc-7 / Cilk Plus, MPI, glog, gflags) is not used.

The checkout's location comes from --reference PATH or the SUMINC_REFERENCE
environment variable; without either nothing is built.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("SUMINC_REFERENCE", "")
OUT = os.path.join(os.path.dirname(HERE), "_ref")
CUDA = "/usr/local/cuda"


def set_reference(path: str) -> None:
    global REF
    REF = path


def build(verbose: bool = False) -> str | None:
    if not REF or not os.path.isdir(REF):
        return None
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "ref_driver")
    stubs = os.path.join(HERE, "stubs")
    inc = ["-I" + stubs, "-I" + REF, "-I" + os.path.join(REF, "examples/analytical_apps"),
           "-I" + os.path.join(REF, "cudaCode"), "-I" + os.path.join(REF, "thirdparty"),
           "-I" + os.path.join(CUDA, "include")]
    flags = ["-std=c++14", "-O2", "-fopenmp", "-DOPENMP", "-w", "-include",
             os.path.join(stubs, "force.h")]
    srcs = [os.path.join(HERE, "driver.cc"),
            os.path.join(REF, "examples/analytical_apps/flags.cc"),
            os.path.join(stubs, "support.cc"), os.path.join(stubs, "mpi_stub.cc"),
            os.path.join(stubs, "cuda_shim.cc"),
            os.path.join(REF, "grape/io/local_io_adaptor.cc")]
    deps = srcs + [os.path.join(stubs, f) for f in os.listdir(stubs) if f.endswith(".h")]
    if os.path.exists(exe) and os.path.getmtime(exe) >= max(os.path.getmtime(s) for s in deps):
        return exe
    cmd = ["g++", *flags, *inc, *srcs, "-o", exe, "-L" + os.path.join(CUDA, "lib64"),
           "-lcudart", "-lpthread", "-Wl,-rpath," + os.path.join(CUDA, "lib64")]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if verbose or p.returncode:
        sys.stderr.write(p.stdout + p.stderr[-20000:])
    if p.returncode:
        return None
    return exe


def check_adaptor(verbose: bool = False) -> bool | None:
    """Compiles adaptor_check.cc (the C++ workers over the reference's own
    fragment and app types) with -fsyntax-only; None without the checkout."""
    if not REF or not os.path.isdir(REF):
        return None
    stubs = os.path.join(HERE, "stubs")
    repo = os.path.dirname(os.path.dirname(HERE))
    inc = ["-I" + stubs, "-I" + REF, "-I" + os.path.join(REF, "examples/analytical_apps"),
           "-I" + os.path.join(REF, "cudaCode"), "-I" + os.path.join(REF, "thirdparty"),
           "-I" + os.path.join(CUDA, "include"), "-I" + os.path.join(repo, "include")]
    # C++17 for the adaptor's `if constexpr`
    flags = ["-std=c++17", "-fsyntax-only", "-fopenmp", "-DOPENMP", "-w", "-include",
             os.path.join(stubs, "force.h")]
    p = subprocess.run(["g++", *flags, *inc, os.path.join(HERE, "adaptor_check.cc")],
                       capture_output=True, text=True)
    if verbose or p.returncode:
        sys.stderr.write(p.stdout + p.stderr[-20000:])
    return p.returncode == 0


if __name__ == "__main__":
    if "--reference" in sys.argv:
        set_reference(sys.argv[sys.argv.index("--reference") + 1])
    print(build(verbose=True))
