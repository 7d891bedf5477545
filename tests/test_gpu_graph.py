"""Device graph: generator twin, upload/download and the in-place applier,
checked against the host generator and the reference update semantics."""
import numpy as np
import pytest

import oracle
import suminc_gb300 as sg

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("scale,edges,wk", [(10, 8000, 0), (12, 60000, 1), (14, 200000, 2)])
def test_device_rmat_equals_host_twin(ctx, scale, edges, wk):
    ctx.generate_rmat(scale, edges, seed=11, weight_kind=wk, wlo=1.0 if wk == 1 else 0.1,
                      whi=100.0 if wk == 1 else 1.0)
    rp, col, w = ctx.download_csr(weights=wk != 0)
    hrp, hcol, hw = sg.rmat_host(scale, edges, seed=11, weight_kind=wk,
                                 wlo=1.0 if wk == 1 else 0.1, whi=100.0 if wk == 1 else 1.0)
    assert np.array_equal(rp, hrp)
    assert np.array_equal(col, hcol)
    if wk:
        assert np.array_equal(w, hw)


def test_load_download_roundtrip(ctx):
    rp, col, w = sg.rmat_host(11, 20000, seed=5, weight_kind=1)
    ctx.load_csr(rp, col, w)
    assert ctx.n == 2048 and ctx.m == 20000
    r2, c2, w2 = ctx.download_csr()
    assert np.array_equal(rp, r2) and np.array_equal(col, c2) and np.array_equal(w, w2)


def test_empty_rows_and_isolated_vertices(ctx):
    rp = np.array([0, 0, 2, 2, 3, 3], np.uint64)
    col = np.array([0, 3, 1], np.uint32)
    w = np.array([1, 2, 3], np.float32)
    ctx.load_csr(rp, col, w)
    r2, c2, w2 = ctx.download_csr()
    assert r2.tolist() == rp.tolist() and c2.tolist() == col.tolist()


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_applier_matches_reference_semantics(ctx, seed):
    rp, col, w = sg.rmat_host(11, 20000, seed=seed, weight_kind=1)
    ctx.load_csr(rp, col, w)
    hg = sg.HostGraph(rp, col, w)
    cur = (rp, col, w)
    for b in range(3):
        upd = hg.gen_updates(400, 400, 100, seed=100 * seed + b)
        ctx.apply_updates(upd)
        cur = oracle.apply_updates_reference(*cur, upd)
        r2, c2, w2 = ctx.download_csr()
        assert np.array_equal(r2, cur[0]) and np.array_equal(c2, cur[1])
        assert np.array_equal(w2, cur[2])
        assert ctx.m == int(cur[0][-1])


def test_applier_edge_cases(ctx):
    # duplicate adds keep the first weight, delete of an absent edge is
    # ignored, delete+add is a weight change, add of an existing pair replaces
    rp = np.array([0, 2, 3, 3], np.uint64)
    col = np.array([1, 2, 2], np.uint32)
    w = np.array([5, 6, 7], np.float32)
    ctx.load_csr(rp, col, w)
    U = sg.UPDATE_DTYPE
    upd = np.array([(0, 2, 9.0, 0), (0, 2, 3.0, 0),      # add existing twice: first wins
                    (2, 0, 0.0, 1),                      # delete absent: ignored
                    (1, 2, 0.0, 1), (1, 2, 8.0, 0),      # weight change
                    (2, 1, 4.0, 0), (2, 1, 1.0, 0),      # new edge, first add wins
                    (0, 1, 0.0, 1)], U)                  # delete present
    ctx.apply_updates(upd)
    ref = oracle.apply_updates_reference(rp, col, w, upd)
    r2, c2, w2 = ctx.download_csr()
    assert r2.tolist() == ref[0].tolist() and c2.tolist() == ref[1].tolist()
    assert w2.tolist() == ref[2].tolist() == [9.0, 8.0, 4.0]


def test_applier_overflow_relocates_segments(ctx):
    # a vertex that gains far more edges than its slack moves to the pool
    n = 64
    rp = np.ones(n + 1, np.uint64)
    rp[0] = 0  # vertex 0 -> 1 is the only edge
    col = np.array([1], np.uint32)
    w = np.array([1], np.float32)
    ctx.load_csr(rp, col, w)
    upd = np.array([(0, v, float(v), 0) for v in range(2, n)], sg.UPDATE_DTYPE)
    ctx.apply_updates(upd)
    ref = oracle.apply_updates_reference(rp, col, w, upd)
    r2, c2, w2 = ctx.download_csr()
    assert np.array_equal(r2, ref[0]) and np.array_equal(c2, ref[1]) and np.array_equal(w2, ref[2])


def test_invalid_update_is_rejected(ctx):
    rp, col, w = sg.rmat_host(8, 1000, seed=1, weight_kind=1)
    ctx.load_csr(rp, col, w)
    bad = np.array([(0, 1 << 20, 1.0, 0)], sg.UPDATE_DTYPE)
    with pytest.raises(sg.SgError) as e:
        ctx.apply_updates(bad)
    assert e.value.status == sg.SG_ERR_INVALID
    r2, c2, _ = ctx.download_csr()
    assert np.array_equal(c2, col)


def test_pool_repacks_under_many_inserts():
    """No slack and insert-heavy batches: segments keep moving to the pool
    tail until a batch no longer fits and the direction is repacked; the
    graph and the incremental SSSP stay exact throughout."""
    with sg.Context(0, slack=0.0) as ctx:
        ctx.generate_rmat(10, 4000, seed=3, weight_kind=1)
        rp, col, w = ctx.download_csr()
        hg = sg.HostGraph(rp, col, w)
        ctx.sssp_peval(0, out=False)
        for i in range(12):
            ctx.apply_updates(hg.gen_updates(3000, 200, 100, seed=10 + i))
            nrp, ncol, nw = hg.csr()
            drp, dcol, dw = ctx.download_csr()
            assert np.array_equal(drp, nrp) and np.array_equal(dcol, ncol)
            assert np.array_equal(dw, nw)
            assert np.array_equal(ctx.sssp_inceval(), oracle.dijkstra(nrp, ncol, nw, 0))
        assert ctx.stats()["repacks"] > 0  # the repack path ran


def test_graph_emptied_and_refilled_by_batches():
    """Every edge deleted (m = 0, no pull work), then edges back: PageRank
    and SSSP IncEval stay exact, and an empty batch changes nothing."""
    rp = np.array([0, 2, 3, 3, 4], np.uint64)
    col = np.array([1, 2, 2, 0], np.uint32)
    w = np.array([1, 5, 1, 2], np.float32)
    with sg.Context(0) as ctx:
        ctx.load_csr(rp, col, w)
        ctx.pr_peval(out=False)
        ctx.apply_updates(np.zeros(0, sg.UPDATE_DTYPE))
        hg = sg.HostGraph(rp, col, w)
        dels = np.zeros(4, sg.UPDATE_DTYPE)
        for i, (u, v) in enumerate([(0, 1), (0, 2), (1, 2), (3, 0)]):
            dels[i] = (u, v, 0.0, 1)
        ctx.apply_updates(dels)
        assert ctx.m == 0
        x = ctx.pr_inceval()
        assert np.abs(x - oracle.pr_fixed_point(np.zeros(5, np.uint64), np.zeros(0, np.uint32))).sum() <= 1e-5
        adds = np.zeros(3, sg.UPDATE_DTYPE)
        for i, (u, v, ww) in enumerate([(2, 3, 4.0), (3, 1, 1.0), (0, 3, 9.0)]):
            adds[i] = (u, v, ww, 0)
        ctx.apply_updates(adds)
        nrp = np.array([0, 1, 1, 2, 3], np.uint64)
        ncol = np.array([3, 3, 1], np.uint32)
        nw = np.array([9, 4, 1], np.float32)
        x = ctx.pr_inceval()
        assert np.abs(x - oracle.pr_fixed_point(nrp, ncol)).sum() <= 1e-5
    with sg.Context(0) as ctx:
        ctx.load_csr(rp, col, w)
        ctx.sssp_peval(0, out=False)
        ctx.apply_updates(dels)
        d = ctx.sssp_inceval()
        assert d[0] == 0 and np.all(np.isinf(d[1:]))
        ctx.apply_updates(adds)
        assert np.array_equal(ctx.sssp_inceval(), oracle.dijkstra(nrp, ncol, nw, 0))


def test_single_vertex_graph():
    with sg.Context(0) as ctx:
        ctx.load_csr(np.array([0, 0], np.uint64), np.zeros(0, np.uint32), np.zeros(0, np.float32))
        x = ctx.pr_peval()
        assert abs(float(x[0]) - 0.15) < 1e-6
        assert ctx.sssp_peval(0)[0] == 0.0
