"""The reference's text formats (.e / .v / update / cluster files) read into
the device graph: results equal the ones from the same graph loaded as
arrays, and the reference's own outputs on the golden fixture, with the
vertex ids renamed to sparse oids."""
import json
import os

import numpy as np
import pytest

import oracle
import suminc_gb300 as sg

pytestmark = pytest.mark.gpu
HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    d = np.load(os.path.join(HERE, f"{name}.npz"))
    return {k: d[k] for k in d.files}


def write_case(tmp_path, fx, oid, weighted):
    rp, col, w = fx["row_ptr"], fx["col"], fx["w"]
    n = len(rp) - 1
    src = np.repeat(np.arange(n), np.diff(rp).astype(np.int64))
    e = tmp_path / "g.e"
    with open(e, "w") as f:
        f.write("# edges\n")
        for u, v, x in zip(src.tolist(), col.tolist(), w.astype(np.int64).tolist()):
            f.write(f"{oid[u]} {oid[v]} {x}\n" if weighted else f"{oid[u]} {oid[v]}\n")
        if len(src):  # a repeated line keeps the first occurrence
            f.write(f"{oid[src[0]]} {oid[col[0]]} 77\n" if weighted else f"{oid[src[0]]} {oid[col[0]]}\n")
    vf = tmp_path / "g.v"
    with open(vf, "w") as f:
        for v in np.random.default_rng(0).permutation(n):
            f.write(f"{oid[v]}\n")
    return str(e), str(vf)


def write_updates(path, upd, oid, weighted):
    with open(path, "w") as f:
        for r in upd:
            if int(r["op"]) == 0:
                f.write(f"a {oid[r['src']]} {oid[r['dst']]}" +
                        (f" {int(r['weight'])}\n" if weighted else "\n"))
            else:
                f.write(f"d {oid[r['src']]} {oid[r['dst']]}\n")


def test_files_reproduce_reference_pagerank(tmp_path):
    fx = load("planted2600")
    n = len(fx["row_ptr"]) - 1
    oid = (1000 + 3 * np.arange(n)).astype(np.int64)  # sparse oids, same order
    efile, vfile = write_case(tmp_path, fx, oid, weighted=False)
    cfile = tmp_path / "g.e.c_150"
    cp, mem = fx["clusters_ptr"], fx["clusters_members"]
    with open(cfile, "w") as f:
        for i in range(len(cp) - 1):
            m = mem[cp[i]:cp[i + 1]]
            f.write(" ".join([str(len(m))] + [str(oid[v]) for v in m]) + "\n")
    ufile = tmp_path / "pr.update"
    write_updates(ufile, fx["updates_pr"], oid, weighted=False)
    with sg.Context(0, compress=1) as ctx:
        ctx.load_files(efile, vfile)
        assert np.array_equal(ctx.vertex_oids(), oid.astype(np.uint64))
        rp, col, _ = ctx.download_csr(weights=False)
        assert np.array_equal(rp, fx["row_ptr"]) and np.array_equal(col, fx["col"])
        ctx.summary_build_file(str(cfile))
        x = ctx.pr_peval()
        assert np.abs(x - fx["ref_pr_sum_peval"]).sum() <= 2e-5
        ctx.apply_update_file(str(ufile))
        x2 = ctx.pr_inceval()
        assert np.abs(x2 - fx["ref_pr_sum_inc"]).sum() <= 2e-5


def test_files_reproduce_reference_sssp(tmp_path):
    fx = load("rmat12")
    n = len(fx["row_ptr"]) - 1
    efile, vfile = write_case(tmp_path, fx, np.arange(n), weighted=True)
    ufile = tmp_path / "sssp.update"
    write_updates(ufile, fx["updates_sssp"], np.arange(n), weighted=True)
    with sg.Context(0) as ctx:
        ctx.load_files(efile, vfile, weighted=True)
        rp, col, w = ctx.download_csr()
        assert np.array_equal(w, fx["w"])
        assert np.array_equal(ctx.sssp_peval(0), fx["ref_sssp_sum_peval"])
        ctx.apply_update_file(str(ufile))
        assert np.array_equal(ctx.sssp_inceval(), fx["ref_sssp_plain_inc"])


def test_bad_files_are_rejected(tmp_path):
    e = tmp_path / "bad.e"
    e.write_text("0 1\n1 x\n")
    u = tmp_path / "bad.update"
    u.write_text("x 0 1\n")
    good = tmp_path / "good.e"
    good.write_text("0 1\n1 2\n")
    with sg.Context(0) as ctx:
        with pytest.raises(sg.SgError):
            ctx.load_files(str(e))
        with pytest.raises(sg.SgError):
            ctx.load_files(str(tmp_path / "missing.e"))
        ctx.load_files(str(good))
        with pytest.raises(sg.SgError):
            ctx.apply_update_file(str(u))
        u.write_text("a 0 9\n")  # vertex 9 is not in the graph
        with pytest.raises(sg.SgError):
            ctx.apply_update_file(str(u))
