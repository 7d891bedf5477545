"""The summary repair on the device against the host restatement of the
reference's inc_run (inc_compress_mirror, judge_out_bound_node,
build_subgraph_mirror, the touched supernodes' shortcuts, get_nodetype_mirror
and sketch2csr_mirror; compressor_base.h:5634-5924, iter_compressor.h:796-896),
whose counters tests/test_gpu_summary.py pins to the reference's own logs.
After every batch the device's node types, entry / exit / single lists,
boundary and shortcut rows and correction lists equal the host's, and
PageRank over the repaired summary stays within the FP64 fixed-point bound."""
import json
import os

import numpy as np
import pytest

import oracle
import suminc_gb300 as sg

pytestmark = pytest.mark.gpu
HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL_FIXED = 1e-5


def load(name):
    d = np.load(os.path.join(HERE, f"{name}.npz"))
    fx = {k: d[k] for k in d.files}
    cp, mem = fx["clusters_ptr"], fx["clusters_members"]
    fx["clusters"] = [mem[cp[i]:cp[i + 1]] for i in range(len(cp) - 1)]
    fx["stats_d"] = json.loads(str(fx["stats"]))
    return fx


def assert_tables_equal(ctx):
    c = ctx.summary_check()
    assert c["rows"] > 0
    for k in ("type_diff", "list_diff", "ib_diff", "is_diff", "corr_diff"):
        assert c[k] == 0, c
    assert c["max_rel"] <= 1e-4, c


def fixed_point_l1(x, rp, col):
    return np.abs(x - oracle.pr_fixed_point(rp, col)).sum()


@pytest.mark.parametrize("name", ["rmat12", "planted2600"])
def test_device_repair_equals_host_after_each_batch(name):
    fx = load(name)
    cur = (fx["row_ptr"], fx["col"], fx["w"])
    with sg.Context(0, compress=1) as ctx:
        ctx.load_csr(cur[0], cur[1])
        ctx.summary_build(fx["clusters"])
        assert_tables_equal(ctx)  # the device's first build against the host's
        ctx.pr_peval(out=False)
        for b, seed in enumerate((0, 31, 32, 33)):
            upd = (fx["updates_pr"] if b == 0
                   else oracle.gen_updates(cur[0], cur[1], 100, 100, 0, seed=seed))
            cur = oracle.apply_updates(*cur, upd)
            ctx.apply_updates(upd)
            assert fixed_point_l1(ctx.pr_inceval(), cur[0], cur[1]) <= TOL_FIXED, f"batch {b}"
            assert_tables_equal(ctx)


def test_device_repair_over_several_pending_batches():
    """Three batches before one IncEval: the device repairs after each, the
    IncEval precomputes every cluster any of them updated, and the host
    restatement replays the three logged batches in order."""
    fx = load("planted2600")
    cur = (fx["row_ptr"], fx["col"], fx["w"])
    with sg.Context(0, compress=1) as ctx:
        ctx.load_csr(cur[0], cur[1])
        ctx.summary_build(fx["clusters"])
        ctx.pr_peval(out=False)
        for seed in (51, 52, 53):
            upd = oracle.gen_updates(cur[0], cur[1], 120, 120, 0, seed=seed)
            cur = oracle.apply_updates(*cur, upd)
            ctx.apply_updates(upd)
        assert fixed_point_l1(ctx.pr_inceval(), cur[0], cur[1]) <= TOL_FIXED
        assert_tables_equal(ctx)
        # and one more batch after the replay
        upd = oracle.gen_updates(cur[0], cur[1], 60, 60, 0, seed=54)
        cur = oracle.apply_updates(*cur, upd)
        ctx.apply_updates(upd)
        assert fixed_point_l1(ctx.pr_inceval(), cur[0], cur[1]) <= TOL_FIXED
        assert_tables_equal(ctx)


def _in_lists(rp, col):
    n = len(rp) - 1
    src = np.repeat(np.arange(n, dtype=np.uint32), np.diff(rp).astype(np.int64))
    return src, col


def test_device_repair_retires_and_creates_entries():
    """A batch that removes every in-edge from outside the cluster of some
    members (entries retire) and one that adds edges from unclustered
    vertices to members with no outside in-edge (new entries): tables equal
    the host's and PageRank stays within the bound."""
    fx = load("planted2600")  # 60 clusters of 40 and 200 unclustered vertices
    cur = (fx["row_ptr"], fx["col"], fx["w"])
    n = len(cur[0]) - 1
    with sg.Context(0, compress=1) as ctx:
        ctx.load_csr(cur[0], cur[1])
        ctx.summary_build(fx["clusters"])
        ctx.pr_peval(out=False)
        cl_of = np.full(n, -1, np.int64)
        for i, c in enumerate(fx["clusters"]):
            cl_of[np.asarray(c, np.int64)] = i
        # the largest clusters' members with at most 3 in-edges from outside
        src, dst = _in_lists(cur[0], cur[1])
        outside = (cl_of[dst] >= 0) & (cl_of[src] != cl_of[dst])
        cnt = np.bincount(dst[outside], minlength=n)
        big = sorted(range(len(fx["clusters"])), key=lambda i: -len(fx["clusters"][i]))[:20]
        members = np.concatenate([np.asarray(fx["clusters"][i], np.int64) for i in big])
        pick = [int(v) for v in members if 0 < cnt[v] <= 3][:40]
        assert pick, "no member with few outside in-edges"
        sel = outside & np.isin(dst, pick)
        upd = np.zeros(int(sel.sum()), dtype=oracle.UPDATE_DTYPE)
        upd["src"], upd["dst"], upd["op"] = src[sel], dst[sel], 1  # deletes
        cur = oracle.apply_updates(*cur, upd)
        ctx.apply_updates(upd)
        assert fixed_point_l1(ctx.pr_inceval(), cur[0], cur[1]) <= TOL_FIXED
        assert_tables_equal(ctx)
        # unclustered tails into members that now have no outside in-edge
        singles = np.flatnonzero(cl_of < 0)
        assert len(singles) > 0
        rng = np.random.default_rng(5)
        rows = [(int(rng.choice(singles)), v) for v in pick[:20]]
        upd = np.zeros(len(rows), dtype=oracle.UPDATE_DTYPE)
        upd["src"] = [r[0] for r in rows]
        upd["dst"] = [r[1] for r in rows]
        upd["weight"], upd["op"] = 1.0, 0  # inserts
        cur = oracle.apply_updates(*cur, upd)
        ctx.apply_updates(upd)
        assert fixed_point_l1(ctx.pr_inceval(), cur[0], cur[1]) <= TOL_FIXED
        assert_tables_equal(ctx)


def test_device_repair_over_many_batches():
    """Ten batches on one summary: new entries take slots at the pool tail,
    retired ones leave holes, and the slots are packed again when the tail
    outgrows the pool; tables equal the host's and PageRank stays within the
    bound after every batch."""
    fx = load("planted2600")
    cur = (fx["row_ptr"], fx["col"], fx["w"])
    with sg.Context(0, compress=1) as ctx:
        ctx.load_csr(cur[0], cur[1])
        ctx.summary_build(fx["clusters"])
        ctx.pr_peval(out=False)
        for seed in range(80, 90):
            upd = oracle.gen_updates(cur[0], cur[1], 150, 150, 0, seed=seed)
            cur = oracle.apply_updates(*cur, upd)
            ctx.apply_updates(upd)
            assert fixed_point_l1(ctx.pr_inceval(), cur[0], cur[1]) <= TOL_FIXED, f"seed {seed}"
            assert_tables_equal(ctx)


def test_device_repair_under_kernel_profiler():
    """With the kernel-class profiler on, the shortcut solves stay on the
    context's stream (no side stream); the repaired tables are the same."""
    fx = load("planted2600")
    cur = (fx["row_ptr"], fx["col"], fx["w"])
    with sg.Context(0, compress=1) as ctx:
        ctx.load_csr(cur[0], cur[1])
        ctx.summary_build(fx["clusters"])
        ctx.pr_peval(out=False)
        for seed, prof in ((61, 0xFF), (62, 0), (63, 0xFF)):
            ctx.set_profile(prof)
            upd = oracle.gen_updates(cur[0], cur[1], 150, 150, 0, seed=seed)
            cur = oracle.apply_updates(*cur, upd)
            ctx.apply_updates(upd)
            assert fixed_point_l1(ctx.pr_inceval(), cur[0], cur[1]) <= TOL_FIXED, f"seed {seed}"
            assert_tables_equal(ctx)
        ctx.set_profile(0)
