"""SSSP PEval / IncEval on the device: distances bit-exact against FP64
Dijkstra (integer weights make every path sum exact in FP64)."""
import numpy as np
import pytest

import oracle
import suminc_gb300 as sg

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("scale,ef,src", [(10, 8, 0), (14, 16, 0), (16, 16, 123)])
def test_peval_bit_exact(ctx, scale, ef, src):
    n = 1 << scale
    ctx.generate_rmat(scale, n * ef, seed=scale + 1, weight_kind=1, wlo=1, whi=100)
    d = ctx.sssp_peval(src)
    rp, col, w = ctx.download_csr()
    ref = oracle.dijkstra(rp, col, w, src)
    assert np.array_equal(d, ref)


def test_parents_form_a_shortest_path_tree(ctx):
    ctx.generate_rmat(12, 16 << 12, seed=3, weight_kind=1)
    d = ctx.sssp_peval(0)
    par = ctx.sssp_parents()
    rp, col, w = ctx.download_csr()
    wmap = {}
    for u in range(len(rp) - 1):
        for e in range(int(rp[u]), int(rp[u + 1])):
            wmap[(u, int(col[e]))] = float(w[e])
    for v in range(len(d)):
        if v == 0 or not np.isfinite(d[v]):
            assert par[v] == 0xFFFFFFFF
        else:
            u = int(par[v])
            assert d[u] + wmap[(u, v)] == d[v]


@pytest.mark.parametrize("seed", [1, 2])
def test_inceval_bit_exact_after_batches(ctx, seed):
    scale = 14
    ctx.generate_rmat(scale, 16 << scale, seed=seed, weight_kind=1)
    rp, col, w = ctx.download_csr()
    hg = sg.HostGraph(rp, col, w)
    ctx.sssp_peval(0, out=False)
    for b in range(4):
        upd = hg.gen_updates(800, 800, 400, seed=seed * 10 + b)
        ctx.apply_updates(upd)
        d = ctx.sssp_inceval()
        nrp, ncol, nw = hg.csr()
        ref = oracle.dijkstra(nrp, ncol, nw, 0)
        assert np.array_equal(d, ref), b


def test_two_batches_before_one_inceval(ctx):
    ctx.generate_rmat(12, 16 << 12, seed=9, weight_kind=1)
    rp, col, w = ctx.download_csr()
    hg = sg.HostGraph(rp, col, w)
    ctx.sssp_peval(0, out=False)
    ctx.apply_updates(hg.gen_updates(300, 300, 100, seed=1))
    ctx.apply_updates(hg.gen_updates(300, 300, 100, seed=2))
    d = ctx.sssp_inceval()
    nrp, ncol, nw = hg.csr()
    assert np.array_equal(d, oracle.dijkstra(nrp, ncol, nw, 0))


def test_delete_whole_tree_edge_chain(ctx):
    # path 0->1->2->3 (w=1) plus a detour 0->3 (w=10): deleting 1->2 must
    # reset 2 and 3 and route 3 through the detour
    rp = np.array([0, 2, 3, 4, 4], np.uint64)
    col = np.array([1, 3, 2, 3], np.uint32)
    w = np.array([1, 10, 1, 1], np.float32)
    ctx.load_csr(rp, col, w)
    d = ctx.sssp_peval(0)
    assert d.tolist() == [0.0, 1.0, 2.0, 3.0]
    ctx.apply_updates(np.array([(1, 2, 0.0, 1)], sg.UPDATE_DTYPE))
    d = ctx.sssp_inceval()
    assert d[0] == 0 and d[1] == 1 and np.isinf(d[2]) and d[3] == 10.0
    assert ctx.stats()["reset_vertices"] == 2


def test_unweighted_graph_is_rejected(ctx):
    rp, col, _ = sg.rmat_host(8, 1000, seed=1)
    ctx.load_csr(rp, col)
    with pytest.raises(sg.SgError) as e:
        ctx.sssp_peval(0)
    assert e.value.status == sg.SG_ERR_INVALID


def _min_tight_parents(rp, col, w, d, source):
    n = len(rp) - 1
    src = np.repeat(np.arange(n), np.diff(rp).astype(np.int64))
    tight = np.isfinite(d[src]) & (d[src] + w.astype(np.float64) == d[col])
    par = np.full(n, 0xFFFFFFFF, np.uint64)
    np.minimum.at(par, col[tight], src[tight].astype(np.uint64))
    par[source] = 0xFFFFFFFF
    par[~np.isfinite(d)] = 0xFFFFFFFF
    return par.astype(np.uint32)


def test_parents_stay_min_tight_across_inceval(ctx):
    """IncEval refreshes parents only where they can change (changed
    distances, their out-neighbours, heads of changed edges); the result must
    equal the smallest tight in-neighbour everywhere."""
    ctx.generate_rmat(13, 16 << 13, seed=31, weight_kind=1)
    rp, col, w = ctx.download_csr()
    hg = sg.HostGraph(rp, col, w)
    ctx.sssp_peval(0, out=False)
    for i in range(4):
        ctx.apply_updates(hg.gen_updates(400, 400, 150, seed=40 + i))
        d = ctx.sssp_inceval()
        nrp, ncol, nw = hg.csr()
        assert np.array_equal(d, oracle.dijkstra(nrp, ncol, nw, 0))
        assert np.array_equal(ctx.sssp_parents(), _min_tight_parents(nrp, ncol, nw, d, 0))


def test_grid_barrier_wait_runs_out_and_context_survives(ctx):
    """Failure detection without a GPU fault: the persistent kernels' grid
    barrier with one CTA kept away gives up after its bounded spin and the
    call reports SG_ERR_TIMEOUT; with every CTA present it passes; the
    context keeps working afterwards (SSSP and PageRank on a small graph)."""
    assert ctx.barrier_probe(False) == sg.SG_OK
    assert ctx.barrier_probe(True) == sg.SG_ERR_TIMEOUT
    assert ctx.barrier_probe(False) == sg.SG_OK
    scale = 10
    ctx.generate_rmat(scale, 8 << scale, seed=3, weight_kind=1)
    rp, col, w = ctx.download_csr(weights=True)
    assert np.array_equal(ctx.sssp_peval(0), oracle.dijkstra(rp, col, w, 0))
    x = ctx.pr_peval()
    assert np.abs(x - oracle.pr_fixed_point(rp, col)).sum() <= 1e-5


def _hub_graph(n=40000, deg=6, hubs=(0, 7, 11), hub_deg=12000, seed=5):
    """A sparse random graph plus a few hubs with long out- and in-rows
    (longer than one warp takes: rows are split over the grid above 4,096
    entries); integer weights in [1, 100]."""
    rng = np.random.default_rng(seed)
    src = [np.repeat(np.arange(n), deg)]
    dst = [rng.integers(0, n, n * deg)]
    for h in hubs:
        src += [np.full(hub_deg, h), rng.integers(0, n, hub_deg)]
        dst += [rng.integers(0, n, hub_deg), np.full(hub_deg, h)]
    src, dst = np.concatenate(src), np.concatenate(dst)
    keep = src != dst
    key = np.unique(src[keep].astype(np.int64) * n + dst[keep])
    s, d = key // n, key % n
    rp = np.concatenate([[0], np.cumsum(np.bincount(s, minlength=n))]).astype(np.uint64)
    w = (1 + (s * 2654435761 + d * 40503) % 100).astype(np.float32)
    return rp, d.astype(np.uint32), w


def _drop_edges(rp, col, w, pairs):
    n = len(rp) - 1
    src = np.repeat(np.arange(n), np.diff(rp).astype(np.int64))
    key = src.astype(np.int64) * n + col
    keep = ~np.isin(key, [u * n + v for u, v in pairs])
    rp2 = np.concatenate([[0], np.cumsum(np.bincount(src[keep], minlength=n))]).astype(np.uint64)
    return rp2, col[keep], w[keep]


@pytest.mark.parametrize("batches_per_inceval", [1, 2])
def test_inceval_with_long_rows(ctx, batches_per_inceval):
    """Hubs whose rows are split over the grid (reset BFS, re-seed pulls,
    parent pulls, the persistent kernel's deferred rows): the first batch
    deletes the hubs' tree edges so their subtrees reset and their long
    in-rows are pulled; IncEval after one batch (new edges relaxed directly)
    and after two (heads pulled) stays bit-exact with min-tight parents."""
    rp, col, w = _hub_graph()
    ctx.load_csr(rp, col, w)
    d = ctx.sssp_peval(0)
    assert np.array_equal(d, oracle.dijkstra(rp, col, w, 0))
    par = ctx.sssp_parents()
    assert np.array_equal(par, _min_tight_parents(rp, col, w, d, 0))
    cut = [(int(par[h]), h) for h in (7, 11)]
    forced = np.array([(u, v, 0.0, 1) for u, v in cut], sg.UPDATE_DTYPE)
    rp, col, w = _drop_edges(rp, col, w, cut)
    hg = sg.HostGraph(rp, col, w)
    for b in range(3):
        for k in range(batches_per_inceval):
            upd = hg.gen_updates(1500, 1500, 500, seed=100 + 10 * b + k)
            if b == 0 and k == 0:
                upd = np.concatenate([forced, upd])
            ctx.apply_updates(upd)
        d = ctx.sssp_inceval()
        nrp, ncol, nw = hg.csr()
        assert np.array_equal(d, oracle.dijkstra(nrp, ncol, nw, 0)), b
        assert np.array_equal(ctx.sssp_parents(), _min_tight_parents(nrp, ncol, nw, d, 0))
        if b == 0:
            assert ctx.stats()["reset_vertices"] > 1000
