"""Compiles libsuminc_gb300.so in-tree for sm_103a.

Every CUDA translation unit is compiled with
``-gencode arch=compute_103a,code=sm_103a``; host C++ goes through nvcc's host
compiler with the same flags so the library links as one shared object.
Objects are rebuilt only when a source or header is newer.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIB_NAME = "libsuminc_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC,-fopenmp,-ffp-contract=off,-O3",
    "-I" + INCLUDE, "-I" + SRC,
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources() -> list[str]:
    return sorted(
        os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".cu", ".cpp"))
    )


def headers() -> list[str]:
    hs = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _compile(src: str, obj: str) -> tuple[str, int, str]:
    cmd = [nvcc(), *ARCH, *COMMON, "-c", src, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [nvcc(), *ARCH, *COMMON, "-x", "cu", "-c", src, "-o", obj]
    p = subprocess.run(cmd, capture_output=True, text=True)
    return src, p.returncode, p.stdout + p.stderr


def lib_path() -> str:
    return os.path.join(OUT, LIB_NAME)


def build(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(OUT, exist_ok=True)
    newest_hdr = max((os.path.getmtime(h) for h in headers()), default=0.0)
    todo = []
    objs = []
    for s in sources():
        o = os.path.join(OUT, os.path.basename(s) + ".o")
        objs.append(o)
        if not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), newest_hdr):
            todo.append((s, o))
    jobs = jobs or min(len(todo) or 1, os.cpu_count() or 4)
    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
            for src, rc, log in ex.map(lambda t: _compile(*t), todo):
                if verbose or rc != 0:
                    sys.stderr.write(log)
                if rc != 0:
                    raise RuntimeError(f"nvcc failed on {os.path.basename(src)}")
    lib = lib_path()
    if todo or not os.path.exists(lib):
        cmd = [nvcc(), *ARCH, "-shared", "-o", lib, *objs, "-Xcompiler", "-fopenmp",
               "-lgomp"]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            sys.stderr.write(p.stdout + p.stderr)
            raise RuntimeError("link of libsuminc_gb300.so failed")
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
