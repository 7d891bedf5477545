"""The header-only C++ workers (include/suminc_gb300_worker.hpp) compiled
against a stand-in fragment (tests/cpp/adaptor_test.cc) give the same
results as the C ABI driven from Python on the same files."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle
import suminc_gb300 as sg
from suminc_gb300 import build as sgbuild

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def oid(v):
    return 10 * np.asarray(v, np.int64) + 7


def write_updates(path, upd, weighted):
    with open(path, "w") as f:
        for r in upd:
            s, d = oid(r["src"]), oid(r["dst"])
            if int(r["op"]) == 0:
                f.write(f"a {s} {d}" + (f" {int(r['weight'])}\n" if weighted else "\n"))
            else:
                f.write(f"d {s} {d}\n")


@pytest.fixture(scope="module")
def binary(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no C++ compiler")
    lib_dir = os.path.dirname(sgbuild.lib_path())
    out = str(tmp_path_factory.mktemp("adaptor") / "adaptor_test")
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "adaptor_test.cc"), "-L", lib_dir,
                    "-lsuminc_gb300", f"-Wl,-rpath,{lib_dir}", "-o", out], check=True)
    return out


def test_cpp_workers_match_c_abi(binary, tmp_path):
    rp, col, w = sg.rmat_host(10, 16 << 10, seed=4, weight_kind=1, wlo=1, whi=100)
    n = len(rp) - 1
    src = np.repeat(np.arange(n), np.diff(rp).astype(np.int64))
    ef = tmp_path / "g.e"
    with open(ef, "w") as f:
        for u, v, x in zip(src.tolist(), col.tolist(), w.astype(np.int64).tolist()):
            f.write(f"{10 * u + 7} {10 * v + 7} {x}\n")
    hg = sg.HostGraph(rp, col, w)
    upr = hg.gen_updates(200, 200, 0, seed=5)
    hg2 = sg.HostGraph(rp, col, w)
    uss = hg2.gen_updates(150, 150, 50, seed=6)
    write_updates(tmp_path / "pr.update", upr, False)
    write_updates(tmp_path / "sssp.update", uss, True)
    opr, oss = tmp_path / "pr.out", tmp_path / "sssp.out"
    clusters = sg.greedy_clusters(rp, col, 150, 8, seed=2)
    cf = tmp_path / "g.e.c_150"
    with open(cf, "w") as f:
        for c in clusters:
            f.write(" ".join([str(len(c))] + [str(int(v)) for v in oid(c)]) + "\n")
    r = subprocess.run([binary, str(ef), str(tmp_path / "pr.update"), str(tmp_path / "sssp.update"),
                        str(opr), str(oss), str(n), str(cf)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    pr = np.loadtxt(opr)
    ss = np.loadtxt(oss)
    assert np.array_equal(pr[:, 0].astype(np.int64), oid(np.arange(n)))
    with sg.Context(0) as ctx:
        ctx.load_csr(rp, col)
        ctx.pr_peval(out=False)
        ctx.apply_updates(upr)
        x = ctx.pr_inceval()
    assert np.abs(pr[:, 1] - x).max() <= 1e-6 * max(1.0, np.abs(x).max()) + 1e-9
    nrp, ncol, nw = hg2.csr()
    assert np.array_equal(ss[:, 1], oracle.dijkstra(nrp, ncol, nw, 3))
    # SSSP over the summary built from the same cluster file
    sss = np.loadtxt(str(oss) + ".sum")
    assert np.array_equal(sss[:, 0].astype(np.int64), oid(np.arange(n)))
    assert np.array_equal(sss[:, 1], oracle.dijkstra(nrp, ncol, nw, 3))
    # message_type = pull over the summary: same file, same batch
    pp = np.loadtxt(str(opr) + ".pull")
    assert np.array_equal(pp[:, 0].astype(np.int64), oid(np.arange(n)))
    with sg.Context(0, compress=1, message_type=sg.SG_MSG_PULL, mirror_k=1 << 30) as ctx:
        ctx.load_csr(rp, col)
        ctx.summary_build(clusters)
        ctx.pr_peval(out=False)
        ctx.apply_updates(upr)
        xp = ctx.pr_inceval()
    assert np.abs(pp[:, 1] - xp).sum() <= 2e-5
    prp, pcol, _ = hg.csr()
    assert np.abs(pp[:, 1] - oracle.pr_fixed_point(prp, pcol)).sum() <= 1e-5
