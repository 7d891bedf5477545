"""Summarized-graph PageRank on the device against the reference's own
SumInc worker (golden fixtures): the summary's structure counters equal the
ones the reference logged, and PEval / IncEval values agree within the
PageRank tolerance."""
import json
import os

import numpy as np
import pytest

import oracle
import suminc_gb300 as sg

pytestmark = pytest.mark.gpu
HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL_REF = 2e-5   # two results each within 1e-5 of the FP64 fixed point
TOL_FIXED = 1e-5


def load(name):
    d = np.load(os.path.join(HERE, f"{name}.npz"))
    fx = {k: d[k] for k in d.files}
    cp, mem = fx["clusters_ptr"], fx["clusters_members"]
    fx["clusters"] = [mem[cp[i]:cp[i + 1]] for i in range(len(cp) - 1)]
    fx["stats_d"] = json.loads(str(fx["stats"]))
    return fx


@pytest.mark.parametrize("name", ["rmat12", "planted2600"])
def test_summary_structure_matches_reference(name):
    fx = load(name)
    st = fx["stats_d"]["pr_peval"]
    with sg.Context(0, compress=1) as ctx:
        ctx.load_csr(fx["row_ptr"], fx["col"])
        ctx.summary_build(fx["clusters"])
        info = ctx.summary_info()
    assert info["clusters"] == st["ids_num"][0]
    assert info["supernodes"] == st["spn_num"][0]
    assert info["cluster_members"] == st["spn_com_num"][0]
    assert info["sources"] == st["source_node_num"][0]
    assert info["bound_nodes"] == st["bound_node_num"][0]
    assert info["absorbed"] == st["mirror_node_cnt"][0]
    assert info["all_rows"] == st["all_node_num"][-1]
    assert info["boundary_edges"] == st["bound_e_num"][0]
    assert info["shortcut_edges"] == st["source_e_num"][0]
    assert info["bound_index"] == st["bound_index_num"][0]
    assert info["sync_edges"] == st["sync_e_num"][0]
    ref_types = [c for t, c in sorted(st["node_types"][:7])]
    assert info["node_type_count"] == ref_types


@pytest.mark.parametrize("name", ["rmat12", "planted2600"])
def test_summarized_pagerank_matches_reference(name):
    fx = load(name)
    with sg.Context(0, compress=1) as ctx:
        ctx.load_csr(fx["row_ptr"], fx["col"])
        ctx.summary_build(fx["clusters"])
        x = ctx.pr_peval()
        assert np.abs(x - fx["ref_pr_sum_peval"]).sum() <= TOL_REF
        xf = oracle.pr_fixed_point(fx["row_ptr"], fx["col"])
        assert np.abs(x - xf).sum() <= TOL_FIXED
        ctx.apply_updates(fx["updates_pr"])
        x2 = ctx.pr_inceval()
        assert np.abs(x2 - fx["ref_pr_sum_inc"]).sum() <= TOL_REF
        nrp, ncol, _ = oracle.apply_updates_reference(fx["row_ptr"], fx["col"], fx["w"],
                                                      fx["updates_pr"])
        assert np.abs(x2 - oracle.pr_fixed_point(nrp, ncol)).sum() <= TOL_FIXED
        inc = fx["stats_d"]["pr_inc"]
        info = ctx.summary_info()
        assert info["shortcut_edges"] == inc["source_e_num"][-1]
        assert info["boundary_edges"] == inc["bound_e_num"][-1]
        assert info["node_type_count"] == [c for t, c in sorted(inc["node_types"][7:14])]


@pytest.mark.parametrize("name", ["rmat12", "planted2600"])
def test_plain_pagerank_and_sssp_match_reference(name):
    fx = load(name)
    with sg.Context(0) as ctx:
        ctx.load_csr(fx["row_ptr"], fx["col"])
        ctx.pr_peval(out=False)
        ctx.apply_updates(fx["updates_pr"])
        x = ctx.pr_inceval()
        assert np.abs(x - fx["ref_pr_plain_inc"]).sum() <= TOL_REF
    with sg.Context(0) as ctx:
        ctx.load_csr(fx["row_ptr"], fx["col"], fx["w"])
        d = ctx.sssp_peval(0)
        assert np.array_equal(d, fx["ref_sssp_sum_peval"])
        ctx.apply_updates(fx["updates_sssp"])
        d2 = ctx.sssp_inceval()
        # exact distances: the reference's Ingress traversal worker (its
        # summarized worker deviates on planted2600, see test_cpu_golden)
        assert np.array_equal(d2, fx["ref_sssp_plain_inc"])


@pytest.mark.parametrize("name,source", [("rmat12", 0), ("planted2600", 0), ("planted2600", 5),
                                         ("planted2600", 2500)])
def test_summarized_sssp_is_exact(name, source):
    """SSSP over the summary (shortcut distances, summarized delta-stepping,
    inner correction) equals Dijkstra; also for a source inside a cluster."""
    fx = load(name)
    rp, col, w = fx["row_ptr"], fx["col"], fx["w"]
    with sg.Context(0, compress=1) as ctx:
        ctx.load_csr(rp, col, w)
        ctx.summary_build(fx["clusters"])
        d = ctx.sssp_peval(source)
        assert np.array_equal(d, oracle.dijkstra(rp, col, w, source))
        if source == 0:
            assert np.array_equal(d, fx["ref_sssp_sum_peval"])
        # IncEval after the batch, then a fresh summarized PEval on the
        # repaired summary
        ctx.apply_updates(fx["updates_sssp"])
        nrp, ncol, nw = oracle.apply_updates_reference(rp, col, w, fx["updates_sssp"])
        d_new = oracle.dijkstra(nrp, ncol, nw, source)
        assert np.array_equal(ctx.sssp_inceval(), d_new)
        assert np.array_equal(ctx.sssp_peval(source), d_new)
        parents = ctx.sssp_parents()
        reach = np.isfinite(d_new) & (np.arange(len(d_new)) != source)
        assert np.all(parents[reach] < len(d_new))


@pytest.mark.parametrize("name", ["rmat12", "planted2600"])
def test_summary_save_and_load_reference_file(name, tmp_path):
    """sg_summary_save writes the reference's serialized cluster state;
    loading the reference's own file rebuilds the same summary and values."""
    fx = load(name)
    saved = tmp_path / "ours.bin"
    with sg.Context(0, compress=1) as ctx:
        ctx.load_csr(fx["row_ptr"], fx["col"])
        ctx.summary_build(fx["clusters"])
        info0 = ctx.summary_info()
        ctx.summary_save(str(saved))
    assert saved.read_bytes() == fx["ref_serialized_summary"].tobytes()
    ref_file = tmp_path / "ref.bin"
    ref_file.write_bytes(fx["ref_serialized_summary"].tobytes())
    with sg.Context(0, compress=1) as ctx:
        ctx.load_csr(fx["row_ptr"], fx["col"])
        ctx.summary_load(str(ref_file))
        assert ctx.summary_info() == info0
        x = ctx.pr_peval()
        assert np.abs(x - fx["ref_pr_sum_peval"]).sum() <= TOL_REF
        bad = tmp_path / "bad.bin"
        bad.write_bytes(fx["ref_serialized_summary"].tobytes()[:-4])
        with pytest.raises(sg.SgError):
            ctx.summary_load(str(bad))


def _mixed_communities(seed=3):
    """Planted communities of four kinds: 40 members with ~8 inner out-edges
    each, 56 members (more than half a warp's solve holds), 200 members (more
    than a warp-staged cluster holds), and 120 members with ~24 inner
    out-edges each (more local edges than staging holds); three exits per
    community link to four other communities."""
    rng = np.random.default_rng(seed)
    spec = [(40, 8)] * 60 + [(56, 8)] * 4 + [(200, 8)] * 6 + [(120, 24)] * 4
    rng.shuffle(spec)
    starts = np.cumsum([0] + [s for s, _ in spec])
    n = int(starts[-1])
    src, dst = [], []
    for c, (size, deg) in enumerate(spec):
        b = starts[c]
        s = np.repeat(np.arange(b, b + size), deg)
        src.append(s)
        dst.append(b + rng.integers(0, size, size=s.size))
        x = np.repeat(np.arange(b + size - 3, b + size), 4)
        oc = rng.integers(0, len(spec), size=x.size)
        src.append(x)
        dst.append(starts[oc] + rng.integers(0, 3, size=x.size))
    src, dst = np.concatenate(src), np.concatenate(dst)
    keep = src != dst
    key = np.unique(src[keep] * n + dst[keep])
    src, dst = key // n, key % n
    rp = np.concatenate([[0], np.cumsum(np.bincount(src, minlength=n))]).astype(np.uint64)
    col = dst.astype(np.uint32)
    comms = [np.arange(starts[c], starts[c + 1], dtype=np.uint32) for c in range(len(spec))]
    return rp, col, comms


def test_summarized_pagerank_staged_and_global_clusters():
    """The cluster precompute stages small clusters in shared memory and
    iterates the others (too many members or too many local edges) on global
    memory: PEval and two IncEvals over a summary holding all three kinds
    stay within the FP64 bound and agree with the plain path."""
    rp, col, comms = _mixed_communities()
    hg = sg.HostGraph(rp, col)
    with sg.Context(0, compress=1) as ctx, sg.Context(0) as plain:
        ctx.load_csr(rp, col)
        ctx.summary_build(comms)
        plain.load_csr(rp, col)
        x = ctx.pr_peval()
        assert np.abs(x - oracle.pr_fixed_point(rp, col)).sum() <= TOL_FIXED
        assert np.abs(x - plain.pr_peval()).sum() <= TOL_REF
        for seed in (11, 12):
            batch = hg.gen_updates(150, 150, 0, seed=seed)
            nrp, ncol, _ = hg.csr()
            ctx.apply_updates(batch)
            plain.apply_updates(batch)
            x2 = ctx.pr_inceval()
            assert np.abs(x2 - oracle.pr_fixed_point(nrp, ncol)).sum() <= TOL_FIXED
            assert np.abs(x2 - plain.pr_inceval()).sum() <= TOL_REF
            # the device repair over every solver variant (cluster sizes up
            # to 48, 64, 160 nodes and beyond) equals the host restatement
            chk = ctx.summary_check()
            for k in ("type_diff", "list_diff", "ib_diff", "is_diff", "corr_diff"):
                assert chk[k] == 0, chk


@pytest.mark.parametrize("name,source", [("planted2600", 0), ("planted2600", 5), ("rmat12", 0)])
def test_summarized_sssp_inceval_over_several_batches(name, source):
    """IncEval over the summary (reset, rounds over boundary edges and
    repaired shortcuts, inner correction) after each of several batches:
    the fixture's batch, random changes, a deleted intra-cluster edge on a
    shortest path, and an inserted intra-cluster edge that shortens an
    entry -> exit shortcut; bit-exact against Dijkstra each time."""
    fx = load(name)
    rp, col, w = fx["row_ptr"], fx["col"], fx["w"]
    cl = fx["clusters"]
    cur = (rp, col, w)
    with sg.Context(0, compress=1) as ctx:
        ctx.load_csr(rp, col, w)
        ctx.summary_build(cl)
        ctx.sssp_peval(source)
        for b in range(4):
            if b == 0:
                upd = fx["updates_sssp"]
            elif b == 1:
                upd = oracle.gen_updates(cur[0], cur[1], 60, 60, 30, seed=40 + b)
            else:
                d_now = oracle.dijkstra(*cur, source)
                par = ctx.sssp_parents()
                c = max(cl, key=len)
                inside = set(int(v) for v in c)
                if b == 2:
                    # remove a shortest-path tree edge inside the cluster
                    cand = [int(v) for v in c if int(par[v]) in inside and np.isfinite(d_now[v])]
                    v = cand[len(cand) // 2] if cand else int(c[1])
                    u = int(par[v]) if cand else int(c[0])
                    upd = np.array([(u, v, 0, 1)], dtype=oracle.UPDATE_DTYPE)
                else:
                    # a short cut from the nearest member to the farthest one
                    order = sorted((int(v) for v in c), key=lambda v: d_now[v])
                    upd = np.array([(order[0], order[-1], 1, 0)], dtype=oracle.UPDATE_DTYPE)
            cur = oracle.apply_updates(*cur, upd)
            ctx.apply_updates(upd)
            d1 = ctx.sssp_inceval()
            assert np.array_equal(d1, oracle.dijkstra(*cur, source)), f"batch {b}"
        parents = ctx.sssp_parents()
        reach = np.isfinite(d1) & (np.arange(len(d1)) != source)
        assert np.all(parents[reach] < len(d1))


def test_summary_without_supernodes_runs_the_plain_path():
    """Clusters the benefit filter rejects (groups of the highest-degree
    vertices: few inner edges, many entries and exits) leave a summary with
    no supernode; PageRank and SSSP over it equal the plain path, before and
    after a batch, and the batch needs no repair."""
    fx = load("rmat12")
    rp, col, w = fx["row_ptr"], fx["col"], fx["w"]
    deg = np.diff(rp).astype(np.int64) + np.bincount(col, minlength=len(rp) - 1)
    top = np.argsort(-deg, kind="stable")[:64].astype(np.uint32)
    groups = [np.sort(top[i:i + 8]) for i in range(0, 64, 8)]
    upd = fx["updates_sssp"]
    with sg.Context(0, compress=1) as ctx, sg.Context(0) as plain:
        ctx.load_csr(rp, col, w)
        ctx.summary_build(groups)
        info = ctx.summary_info()
        assert info["supernodes"] == 0 and info["clusters"] == 0
        plain.load_csr(rp, col, w)
        x = ctx.pr_peval()
        assert np.abs(x - plain.pr_peval()).sum() <= TOL_REF
        assert np.array_equal(ctx.sssp_peval(0), plain.sssp_peval(0))
        ctx.apply_updates(upd)
        plain.apply_updates(upd)
        nrp, ncol, nw = oracle.apply_updates(rp, col, w, upd)
        x2 = ctx.pr_inceval()
        assert np.abs(x2 - oracle.pr_fixed_point(nrp, ncol)).sum() <= TOL_FIXED
        d2 = ctx.sssp_inceval()
        assert np.array_equal(d2, oracle.dijkstra(nrp, ncol, nw, 0))
        assert np.array_equal(d2, plain.sssp_inceval())


def test_summarized_sssp_inceval_after_two_pending_batches():
    """Two batches applied before one IncEval over the summary (the reset and
    re-seed cover both, the shortcut repair covers the supernodes both
    touched): bit-exact against Dijkstra."""
    fx = load("planted2600")
    rp, col, w = fx["row_ptr"], fx["col"], fx["w"]
    cur = (rp, col, w)
    with sg.Context(0, compress=1) as ctx:
        ctx.load_csr(rp, col, w)
        ctx.summary_build(fx["clusters"])
        ctx.sssp_peval(5)
        for seed in (71, 72):
            upd = oracle.gen_updates(cur[0], cur[1], 80, 80, 40, seed=seed)
            cur = oracle.apply_updates(*cur, upd)
            ctx.apply_updates(upd)
        assert np.array_equal(ctx.sssp_inceval(), oracle.dijkstra(*cur, 5))
