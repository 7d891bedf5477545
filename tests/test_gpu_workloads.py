"""Parity at the workload sizes: the device path against the reference's own
workers run on the same inputs (golden fixtures written by
tests/golden/make_golden.py) and against the FP64 oracle.

  rmat16_pr    PageRank, R-MAT scale 16 (2^20 edges), greedy clusters, one
               10,000-change batch: summarized PEval and IncEval, plain IncEval
  rmat20_sssp  SSSP from 0, R-MAT scale 20 (2^24 edges, weights U[1, 100]),
               greedy clusters, one 100,000-change batch (40/40/20):
               summarized PEval and IncEval, plain IncEval, bit-exact
  rmat12_tight PageRank on rmat12 with the stop threshold at 1e-10 on both
               sides: L1 <= 1e-6 against the reference
The graphs and batches are regenerated from their seeds on the device and on
the host, and checked against the hashes the fixtures hold."""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle
import suminc_gb300 as sg

pytestmark = pytest.mark.gpu
HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL_REF = 2e-5    # each side within 1e-5 of the FP64 fixed point
TOL_FIXED = 1e-5  # stop rule sum|delta| < 1e-6: 1e-6 / (1 - d) + FP32 rounding
TOL_TIGHT = 1e-6  # both sides stopped at sum|delta| < 1e-10


def load(name):
    path = os.path.join(HERE, f"{name}.npz")
    if not os.path.exists(path):
        pytest.skip(f"fixture {name} not generated")
    d = np.load(path)
    fx = {k: d[k] for k in d.files}
    if "clusters_ptr" in fx:
        cp, mem = fx["clusters_ptr"], fx["clusters_members"]
        fx["clusters"] = [mem[cp[i]:cp[i + 1]] for i in range(len(cp) - 1)]
    if "stats" in fx:
        fx["stats_d"] = json.loads(str(fx["stats"]))
    return fx


def sha(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        if a is not None:
            h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def dist_u32(d):
    out = np.full(len(d), 0xFFFFFFFF, np.uint32)
    fin = np.isfinite(d)
    out[fin] = d[fin].astype(np.uint32)
    return out


def test_rmat16_pagerank_matches_reference():
    fx = load("rmat16_pr")
    st = fx["stats_d"]
    with sg.Context(0, compress=1) as ctx:
        ctx.generate_rmat(16, 1 << 20, seed=1)
        rp, col, _ = ctx.download_csr(weights=False)
        assert sha(rp, col) == str(fx["input_sha256"])
        upd = oracle.gen_updates(rp, col, 5000, 5000, 0, seed=2)
        assert sha(upd) == str(fx["updates_sha256"])
        ctx.summary_build(fx["clusters"])
        info = ctx.summary_info()
        pe = st["pr_peval"]
        assert info["clusters"] == pe["ids_num"][0]
        assert info["supernodes"] == pe["spn_num"][0]
        assert info["shortcut_edges"] == pe["source_e_num"][0]
        assert info["boundary_edges"] == pe["bound_e_num"][0]
        x = ctx.pr_peval()
        assert np.abs(x - fx["ref_pr_sum_peval"]).sum() <= TOL_REF
        assert np.abs(x - oracle.pr_fixed_point(rp, col)).sum() <= TOL_FIXED
        ctx.apply_updates(upd)
        x2 = ctx.pr_inceval()
        assert np.abs(x2 - fx["ref_pr_sum_inc"]).sum() <= TOL_REF
        nrp, ncol, _ = oracle.apply_updates(rp, col, None, upd)
        x_new = oracle.pr_fixed_point(nrp, ncol)
        assert np.abs(x2 - x_new).sum() <= TOL_FIXED
        inc = st["pr_inc"]
        info = ctx.summary_info()
        assert info["shortcut_edges"] == inc["source_e_num"][-1]
        assert info["boundary_edges"] == inc["bound_e_num"][-1]
    with sg.Context(0) as ctx:
        ctx.load_csr(rp, col)
        ctx.pr_peval(out=False)
        ctx.apply_updates(upd)
        x3 = ctx.pr_inceval()
        assert np.abs(x3 - fx["ref_pr_plain_inc"]).sum() <= TOL_REF
        assert np.abs(x3 - x_new).sum() <= TOL_FIXED


def test_rmat20_sssp_matches_reference():
    fx = load("rmat20_sssp")
    with sg.Context(0, compress=1) as ctx:
        ctx.generate_rmat(20, 1 << 24, seed=1, weight_kind=1, wlo=1, whi=100)
        rp, col, w = ctx.download_csr()
        assert sha(rp, col, w) == str(fx["input_sha256"])
        upd = oracle.gen_updates(rp, col, 40000, 40000, 20000, seed=2)
        assert sha(upd) == str(fx["updates_sha256"])
        ctx.summary_build(fx["clusters"])
        d0 = ctx.sssp_peval(0)
        assert np.array_equal(dist_u32(d0), fx["ref_sssp_sum_peval"])
        assert np.array_equal(d0, oracle.dijkstra(rp, col, w, 0))
        ctx.apply_updates(upd)
        d1 = ctx.sssp_inceval()
        nrp, ncol, nw = oracle.apply_updates(rp, col, w, upd)
        d_new = oracle.dijkstra(nrp, ncol, nw, 0)
        assert np.array_equal(d1, d_new)
        assert np.array_equal(dist_u32(d1), fx["ref_sssp_plain_inc"])
        # the reference's summarized IncEval is pinned separately (CPU test):
        # where it equals its plain worker, the device result equals both
        if np.array_equal(fx["ref_sssp_sum_inc"], fx["ref_sssp_plain_inc"]):
            assert np.array_equal(dist_u32(d1), fx["ref_sssp_sum_inc"])
        # a fresh summarized PEval on the repaired summary
        assert np.array_equal(ctx.sssp_peval(0), d_new)
    with sg.Context(0) as ctx:
        ctx.load_csr(rp, col, w)
        ctx.sssp_peval(0)
        ctx.apply_updates(upd)
        assert np.array_equal(dist_u32(ctx.sssp_inceval()), fx["ref_sssp_plain_inc"])


def test_tight_threshold_within_1e6_of_reference():
    """With the stop threshold at 1e-10 on both sides, the summarized PEval and
    IncEval and the plain IncEval are within L1 1e-6 of the reference's."""
    base = load("rmat12")
    fx = load("rmat12_tight")
    assert str(fx["input_sha256"]) == str(base["input_sha256"])
    rp, col, w = base["row_ptr"], base["col"], base["w"]
    with sg.Context(0, compress=1, termcheck_threshold=1e-10) as ctx:
        ctx.load_csr(rp, col)
        ctx.summary_build(base["clusters"])
        x = ctx.pr_peval()
        assert np.abs(x - fx["ref_pr_sum_peval"]).sum() <= TOL_TIGHT
        ctx.apply_updates(base["updates_pr"])
        x2 = ctx.pr_inceval()
        assert np.abs(x2 - fx["ref_pr_sum_inc"]).sum() <= TOL_TIGHT
    with sg.Context(0, termcheck_threshold=1e-10) as ctx:
        ctx.load_csr(rp, col)
        ctx.pr_peval(out=False)
        ctx.apply_updates(base["updates_pr"])
        x3 = ctx.pr_inceval()
        assert np.abs(x3 - fx["ref_pr_plain_inc"]).sum() <= TOL_TIGHT


def test_rmat22_incremental_pagerank_and_sssp_size_independent_checks():
    """R-MAT scale 22 (67 M edges), two 0.1 % batches each: PageRank IncEval
    within the FP64 residual bound of the fixed point (||x - x*||_1 <=
    residual / (1 - d) <= 1e-5) and SSSP IncEval bit-exact against Dijkstra
    on the final graph."""
    scale, E = 22, 16 << 22
    rp, col, w = oracle.rmat(scale, E, seed=5, weight_kind=1, wlo=1, whi=100)
    with sg.Context(0) as ctx:
        ctx.generate_rmat(scale, E, seed=5, weight_kind=1, wlo=1, whi=100)
        ctx.pr_peval(out=False)
        ctx.sssp_peval(0)
        cur = (rp, col, w)
        for i in range(2):
            upd = oracle.gen_updates(cur[0], cur[1], E // 2000, E // 2000, 0, seed=60 + i)
            cur = oracle.apply_updates(*cur, upd)
            ctx.apply_updates(upd)
            x = ctx.pr_inceval()
            d = ctx.sssp_inceval()
        assert oracle.pr_residual_l1(cur[0], cur[1], x) / 0.15 <= TOL_FIXED
        assert np.array_equal(d, oracle.dijkstra(*cur, 0))
