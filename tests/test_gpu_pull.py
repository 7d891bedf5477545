"""PageRank with message_type = pull (SumSyncIterWorkerPull) on the device:
PEval over the summarized graph against the reference's own pull worker
(golden fixtures, no mirrors) and the FP64 fixed point; IncEval against the
fixed point of the updated graph (the reference's pull worker faults in its
incremental stage, so it has no recorded IncEval); the plain pull rounds
(compress = 0); a summary with mirrors is refused."""
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
    p = np.load(os.path.join(HERE, "pull_pr.npz"))
    assert str(p[f"{name}_input_sha256"]) == str(fx["input_sha256"])
    fx["ref_pull"] = p[f"{name}_ref_pr_pull_peval"]
    fx["mirror_k"] = int(json.loads(str(p["params"]))["flags_pr_pull"]["mirror_k"])
    return fx


@pytest.mark.parametrize("name", ["rmat12", "planted2600"])
def test_pull_summarized_peval_matches_reference_and_inceval_converges(name):
    fx = load(name)
    with sg.Context(0, compress=1, message_type=sg.SG_MSG_PULL, mirror_k=fx["mirror_k"]) as ctx:
        ctx.load_csr(fx["row_ptr"], fx["col"])
        ctx.summary_build(fx["clusters"])
        assert ctx.summary_info()["in_mirrors"] + ctx.summary_info()["out_mirrors"] == 0
        x = ctx.pr_peval()
        st = ctx.stats()
        assert st["converged"] == 1 and st["rounds"] > 1
        assert np.abs(x - fx["ref_pull"]).sum() <= TOL_REF
        assert np.abs(x - oracle.pr_fixed_point(fx["row_ptr"], fx["col"])).sum() <= TOL_FIXED
        ctx.apply_updates(fx["updates_pr"])
        rp, col, _ = oracle.apply_updates_reference(fx["row_ptr"], fx["col"], None,
                                                    fx["updates_pr"])
        hg = sg.HostGraph(rp, col)
        for b in range(3):
            if b:
                ctx.apply_updates(hg.gen_updates(60, 60, 0, seed=70 + b))
                rp, col, _ = hg.csr()
            x = ctx.pr_inceval()
            assert ctx.stats()["converged"] == 1
            assert np.abs(x - oracle.pr_fixed_point(rp, col)).sum() <= TOL_FIXED, b


def test_pull_counts_mass_in_flight_at_entries():
    """64 planted communities, where the reference's pull worker stops its
    summarized stage with mass in flight at the entries (1.5e-3 from the
    fixed point): the device worker counts the entries' arrivals in its stop
    test and agrees with the CPU restatement that does the same; PEval and
    two IncEvals stay within the FP64 bound."""
    from oracle import pull
    z = np.load(os.path.join(HERE, "pull_pr.npz"))
    rp, col = z["community64_row_ptr"], z["community64_col"]
    cp, mem = z["community64_clusters_ptr"], z["community64_clusters_members"]
    clusters = [mem[cp[i]:cp[i + 1]] for i in range(len(cp) - 1)]
    x_oracle, _ = pull.pr_pull_summarized(rp, col, clusters, count_entry_arrivals=True)
    hg = sg.HostGraph(rp, col)
    with sg.Context(0, compress=1, message_type=sg.SG_MSG_PULL, mirror_k=1 << 30) as ctx:
        ctx.load_csr(rp, col)
        ctx.summary_build(clusters)
        x = ctx.pr_peval()
        assert np.abs(x - x_oracle).sum() <= TOL_REF
        assert np.abs(x - oracle.pr_fixed_point(rp, col)).sum() <= TOL_FIXED
        for seed in (1, 2):
            ctx.apply_updates(hg.gen_updates(200, 200, 0, seed=seed))
            nrp, ncol, _ = hg.csr()
            x = ctx.pr_inceval()
            assert np.abs(x - oracle.pr_fixed_point(nrp, ncol)).sum() <= TOL_FIXED


def test_pull_plain_rounds():
    """compress = 0: every vertex gathers along all its in-edges each round;
    PEval and two IncEvals within the FP64 bound, and equal to the push
    worker within the PageRank tolerance."""
    scale = 14
    rp, col, _ = sg.rmat_host(scale, 16 << scale, seed=5)
    hg = sg.HostGraph(rp, col)
    with sg.Context(0, message_type=sg.SG_MSG_PULL) as ctx, sg.Context(0) as push:
        ctx.load_csr(rp, col)
        push.load_csr(rp, col)
        x = ctx.pr_peval()
        assert np.abs(x - oracle.pr_fixed_point(rp, col)).sum() <= TOL_FIXED
        assert np.abs(x - push.pr_peval()).sum() <= TOL_REF
        for seed in (1, 2):
            batch = hg.gen_updates(2000, 2000, 0, seed=seed)
            nrp, ncol, _ = hg.csr()
            ctx.apply_updates(batch)
            push.apply_updates(batch)
            x = ctx.pr_inceval()
            assert np.abs(x - oracle.pr_fixed_point(nrp, ncol)).sum() <= TOL_FIXED
            assert np.abs(x - push.pr_inceval()).sum() <= TOL_REF


def _linked_communities(k=20, size=30, deg=6, links=8, seed=4):
    """k communities of `size` members with `deg` inner out-edges each; the
    last member of community c also has `links` edges into community c+1,
    which makes it a mirror candidate of that cluster (mirror_k = 4) while it
    is a member of its own."""
    rng = np.random.default_rng(seed)
    src, dst = [], []
    for c in range(k):
        b = c * size
        s = np.repeat(np.arange(b, b + size), deg)
        src.append(s)
        dst.append(b + rng.integers(0, size, s.size))
        nb = ((c + 1) % k) * size
        src.append(np.full(links, b + size - 1))
        dst.append(nb + rng.choice(size, links, replace=False))
    src, dst = np.concatenate(src), np.concatenate(dst)
    n = k * size
    keep = src != dst
    key = np.unique(src[keep] * n + dst[keep])
    s, d = key // n, key % n
    rp = np.concatenate([[0], np.cumsum(np.bincount(s, minlength=n))]).astype(np.uint64)
    comms = [np.arange(c * size, (c + 1) * size, dtype=np.uint32) for c in range(k)]
    return rp, d.astype(np.uint32), comms


def test_pull_refuses_summary_with_mirrors():
    """The pull worker indexes per-vertex arrays by shortcut targets, which
    with mirrors include mirror ids past the vertex range: refused."""
    rp, col, comms = _linked_communities()
    with sg.Context(0, compress=1, message_type=sg.SG_MSG_PULL, mirror_k=4) as ctx:
        ctx.load_csr(rp, col)
        ctx.summary_build(comms)
        assert ctx.summary_info()["all_rows"] > len(rp) - 1
        with pytest.raises(sg.SgError) as e:
            ctx.pr_peval()
        assert e.value.status == sg.SG_ERR_INVALID


def test_pull_empty_batch_and_no_kept_clusters():
    """An empty batch moves the pull worker's values by no more than the
    pending residual (another summarized stage and plain stage run from the
    state PEval left, Σ|δ| < τ, so the change is within τ/(1-d)); a
    summary that keeps no cluster (every vertex an out node) runs the
    summarized stage over all in-edges and still converges."""
    fx = load("planted2600")
    rp, col = fx["row_ptr"], fx["col"]
    x_star = oracle.pr_fixed_point(rp, col)
    with sg.Context(0, compress=1, message_type=sg.SG_MSG_PULL, mirror_k=fx["mirror_k"]) as ctx:
        ctx.load_csr(rp, col)
        ctx.summary_build(fx["clusters"])
        x0 = ctx.pr_peval()
        ctx.apply_updates(np.zeros(0, sg.UPDATE_DTYPE))
        x1 = ctx.pr_inceval()
        assert np.abs(x1 - x0).sum() <= 1e-6 / (1 - 0.85)
        assert np.abs(x1 - x_star).sum() <= TOL_FIXED
    with sg.Context(0, compress=1, message_type=sg.SG_MSG_PULL, mirror_k=fx["mirror_k"]) as ctx:
        ctx.load_csr(rp, col)
        ctx.summary_build([])
        assert ctx.summary_info()["supernodes"] == 0
        x = ctx.pr_peval()
        assert np.abs(x - x_star).sum() <= TOL_FIXED
