"""Batched personalized PageRank + multi-source SSSP (one persistent kernel)
against the single-query GPU path, the FP64 PPR fixed point and Dijkstra."""
import numpy as np
import pytest

import oracle
import suminc_gb300 as sg

pytestmark = pytest.mark.gpu
TOL_FIXED = 1e-5   # tau / (1 - d) + FP32 rounding, per query
TOL_SINGLE = 2e-5  # batched vs single query: both within TOL_FIXED of x*


def seeds_for(rng, n, q):
    out = []
    for _ in range(q):
        k = int(np.floor(np.exp(rng.uniform(0, np.log(64)))))
        out.append(np.sort(rng.choice(n, size=max(1, k), replace=False)).astype(np.uint32))
    return out


def ppr_star(rp, col, n, seeds):
    t = np.zeros(n, np.float64)
    t[seeds] = 1.0 / len(seeds)
    return oracle.pr_fixed_point(rp, col, tele=t)


@pytest.fixture(scope="module")
def graph():
    ctx = sg.Context(0)
    ctx.generate_rmat(12, 16 << 12, seed=21, weight_kind=1)
    rp, col, w = ctx.download_csr()
    yield ctx, rp, col, w
    ctx.close()


@pytest.mark.parametrize("nq", [1, 3, 37, 130])
def test_batched_ppr_matches_single_and_fixed_point(graph, nq):
    ctx, rp, col, w = graph
    n = len(rp) - 1
    rng = np.random.default_rng(nq)
    seeds = seeds_for(rng, n, nq)
    P, _ = ctx.batch_run(seeds, [])
    info = ctx.batch_info()
    assert info["ppr_not_converged"] == 0
    rounds, resid = ctx.batch_query_stats(nq)
    assert np.all(resid < 1e-6)
    for q in range(0, nq, max(1, nq // 6)):
        single = ctx.ppr(seeds[q])
        assert np.abs(P[q] - single).sum() <= TOL_SINGLE
        assert np.abs(P[q] - ppr_star(rp, col, n, seeds[q])).sum() <= TOL_FIXED


@pytest.mark.parametrize("ns", [1, 8, 64])
def test_batched_sssp_bit_exact(graph, ns):
    ctx, rp, col, w = graph
    n = len(rp) - 1
    rng = np.random.default_rng(100 + ns)
    src = rng.choice(n, size=ns, replace=False).astype(np.uint32)
    _, D = ctx.batch_run([], src)
    for s in range(ns):
        assert np.array_equal(D[s], oracle.dijkstra(rp, col, w, int(src[s])))


def test_mixed_batch_replays_graph_and_repeats(graph):
    ctx, rp, col, w = graph
    n = len(rp) - 1
    rng = np.random.default_rng(5)
    seeds = seeds_for(rng, n, 20)
    src = np.array([0, 5, 5, 77, n - 1], np.uint32)  # a repeated source
    P1, D1 = ctx.batch_run(seeds, src)
    P2, D2 = ctx.batch_run(seeds, src)
    info = ctx.batch_info()
    assert info["graph_launch"] in (0, 1)
    assert np.array_equal(D1, D2)
    assert np.abs(P1 - P2).max() < 1e-6  # FP32 atomics may reorder sums
    for s in range(len(src)):
        assert np.array_equal(D1[s], oracle.dijkstra(rp, col, w, int(src[s])))
    for q in (0, 7, 19):
        assert np.abs(P1[q] - ppr_star(rp, col, n, seeds[q])).sum() <= TOL_FIXED


def test_batch_follows_graph_updates():
    with sg.Context(0) as ctx:
        ctx.generate_rmat(11, 16 << 11, seed=3, weight_kind=1)
        rp, col, w = ctx.download_csr()
        hg = sg.HostGraph(rp, col, w)
        seeds = [np.array([1, 2, 3], np.uint32), np.array([100], np.uint32)]
        src = np.array([0, 9], np.uint32)
        ctx.batch_run(seeds, src)
        ctx.apply_updates(hg.gen_updates(500, 500, 200, seed=4))
        nrp, ncol, nw = hg.csr()
        P, D = ctx.batch_run(seeds, src)
        n = len(nrp) - 1
        for q in range(2):
            assert np.abs(P[q] - ppr_star(nrp, ncol, n, seeds[q])).sum() <= TOL_FIXED
        for s in range(2):
            assert np.array_equal(D[s], oracle.dijkstra(nrp, ncol, nw, int(src[s])))


def test_dangling_seed_and_isolated_source():
    # 0 -> 1 -> 2, 3 isolated, 4 -> 0; seed 2 has no out-edges, source 3 none
    rp = np.array([0, 1, 2, 2, 2, 3], np.uint64)
    col = np.array([1, 2, 0], np.uint32)
    w = np.array([2, 3, 1], np.float32)
    with sg.Context(0) as ctx:
        ctx.load_csr(rp, col, w)
        P, D = ctx.batch_run([np.array([2], np.uint32), np.array([4, 0], np.uint32)],
                             np.array([3, 4], np.uint32))
        assert np.array_equal(D[0], oracle.dijkstra(rp, col, w, 3))
        assert np.array_equal(D[1], oracle.dijkstra(rp, col, w, 4))
        assert np.isinf(D[0][0]) and D[0][3] == 0.0
        for q, sd in enumerate(([2], [4, 0])):
            assert np.abs(P[q] - ppr_star(rp, col, 5, np.array(sd))).sum() <= TOL_FIXED


def test_batch_rejects_bad_specs(graph):
    ctx, rp, col, w = graph
    n = len(rp) - 1
    with pytest.raises(sg.SgError):
        ctx.batch_run([np.array([n], np.uint32)], [])
    with pytest.raises(sg.SgError):
        ctx.batch_run([np.array([0], np.uint32)] * 257, [])
    with pytest.raises(sg.SgError):
        ctx.batch_run([], np.arange(65, dtype=np.uint32))
    with pytest.raises(sg.SgError):
        ctx.batch_run([np.zeros(0, np.uint32)], [])
    with sg.Context(0) as c2:
        c2.generate_rmat(8, 1000, seed=1)
        with pytest.raises(sg.SgError):
            c2.batch_run([], np.array([0], np.uint32))
