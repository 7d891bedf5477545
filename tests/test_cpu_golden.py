"""The golden fixtures (outputs of the reference's own CPU workers, made by
tests/golden/make_golden.py) pin the oracle: the FP64 solvers and the C
restatement agree with the reference on the same inputs."""
import json
import os

import numpy as np
import pytest

import oracle
import suminc_gb300 as sg

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["rmat12", "planted2600"]


def load(name):
    d = np.load(os.path.join(HERE, f"{name}.npz"))
    return {k: d[k] for k in d.files}


def after(fx, key):
    return oracle.apply_updates_reference(fx["row_ptr"], fx["col"], fx["w"], fx[key])


@pytest.mark.parametrize("name", CASES)
def test_fixture_inputs_regenerate(name):
    fx = load(name)
    if name == "rmat12":
        rp, col, w = sg.rmat_host(12, 16 << 12, seed=1, weight_kind=1, wlo=1, whi=100)
        assert np.array_equal(rp, fx["row_ptr"]) and np.array_equal(col, fx["col"])
        assert np.array_equal(w, fx["w"])


@pytest.mark.parametrize("name", CASES)
def test_reference_pagerank_against_fp64(name):
    fx = load(name)
    x_star = oracle.pr_fixed_point(fx["row_ptr"], fx["col"])
    # reference stops at sum|delta| < 1e-6: distance <= 1e-6 / (1 - d) + rounding
    assert np.abs(fx["ref_pr_sum_peval"] - x_star).sum() < 1e-5
    nrp, ncol, _ = after(fx, "updates_pr")
    x_new = oracle.pr_fixed_point(nrp, ncol)
    assert np.abs(fx["ref_pr_sum_inc"] - x_new).sum() < 1e-5
    assert np.abs(fx["ref_pr_plain_inc"] - x_new).sum() < 1e-5


@pytest.mark.parametrize("name", CASES)
def test_oracle_restatement_matches_reference(name):
    fx = load(name)
    rp, col = fx["row_ptr"], fx["col"]
    x, delta, _ = oracle.ingress_pr(rp, col, tau=1e-6)
    assert np.abs(x - fx["ref_pr_sum_peval"]).sum() < 1.5e-5
    nrp, ncol, _ = after(fx, "updates_pr")
    d2 = oracle.pr_amend((rp, col), (nrp, ncol), x, delta)
    x2, _, _ = oracle.ingress_pr(nrp, ncol, x=x, delta=d2, tau=1e-6)
    assert np.abs(x2 - fx["ref_pr_plain_inc"]).sum() < 1.5e-5


@pytest.mark.parametrize("name", CASES)
def test_reference_sssp_equals_dijkstra(name):
    fx = load(name)
    d0 = oracle.dijkstra(fx["row_ptr"], fx["col"], fx["w"], 0)
    assert np.array_equal(fx["ref_sssp_sum_peval"], d0)
    nrp, ncol, nw = after(fx, "updates_sssp")
    d1 = oracle.dijkstra(nrp, ncol, nw, 0)
    assert np.array_equal(fx["ref_sssp_plain_inc"], d1)
    bad = np.nonzero(fx["ref_sssp_sum_inc"] != d1)[0]
    if name == "planted2600":
        # The reference's summarized traversal worker leaves 61 distances too
        # long after the batch deletes the intra-community edge 370->380 of
        # community 9 (vertices 360..399; the excess flows on to vertices
        # reached through it): a known deviation of its IncEval, pinned here
        # so that a change of the fixture shows up.
        assert len(bad) == 61 and bad.min() == 361
        assert np.all(fx["ref_sssp_sum_inc"][bad] > d1[bad])
    else:
        assert len(bad) == 0


def test_greedy_clusters_regenerate():
    fx = load("rmat12")
    cl = sg.greedy_clusters(fx["row_ptr"], fx["col"], 150, 8, seed=1)
    cp, mem = fx["clusters_ptr"], fx["clusters_members"]
    ref = [mem[cp[i]:cp[i + 1]] for i in range(len(cp) - 1)]
    assert len(cl) == len(ref) and all(np.array_equal(a, b) for a, b in zip(cl, ref))


@pytest.mark.parametrize("name", CASES)
def test_summary_cluster_state_is_byte_identical_to_reference(name):
    """The supernode candidates and mirrors chosen from the clustering, in
    the reference's serialize_cluster layout, equal the bytes the reference
    wrote for the same graph and cluster file."""
    fx = load(name)
    cp, mem = fx["clusters_ptr"], fx["clusters_members"]
    clusters = [mem[cp[i]:cp[i + 1]] for i in range(len(cp) - 1)]
    ours = sg.summary_serialize_host(fx["row_ptr"], fx["col"], clusters, 8, 4, 1.0)
    assert ours == fx["ref_serialized_summary"].tobytes()


@pytest.mark.parametrize("name", CASES)
def test_sssp_restatement_matches_reference(name):
    """The oracle's restatement of the reference's plain SSSP traversal and of
    its incremental stage (deltaCompute over the batch's deleted edges, one
    round from every finite vertex, then the traversal) reproduces the
    distances the reference's IngressSyncTraversalWorker produced."""
    fx = load(name)
    rp, col, w = fx["row_ptr"], fx["col"], fx["w"]
    d0, par, st0 = oracle.sssp_peval(rp, col, w, 0)
    assert np.array_equal(d0, fx["ref_sssp_sum_peval"])
    assert par[0] == 0xFFFFFFFF and st0["edges"] > 0
    nrp, ncol, nw = after(fx, "updates_sssp")
    upd = fx["updates_sssp"]
    dele = upd[upd["op"] == 1]
    d1, par1, st1 = oracle.sssp_inceval((rp, col), (nrp, ncol, nw), (dele["src"], dele["dst"]),
                                        d0, par)
    assert np.array_equal(d1, fx["ref_sssp_plain_inc"])
    # every reached vertex but the source has a tight parent edge
    reach = np.isfinite(d1) & (np.arange(len(d1)) != 0)
    p = par1[reach]
    assert np.all(p < len(d1))


@pytest.mark.parametrize("name", CASES)
def test_reference_pull_worker_against_fp64(name):
    """The message_type=pull worker's PEval (pull_pr.npz, run on the same
    inputs without mirrors) lies within the PageRank bound of the FP64 fixed
    point."""
    fx = load(name)
    p = np.load(os.path.join(HERE, "pull_pr.npz"))
    assert str(p[f"{name}_input_sha256"]) == str(fx["input_sha256"])
    assert json.loads(str(p[f"{name}_stats"]))["mirror_node_cnt"] == [0]
    x = p[f"{name}_ref_pr_pull_peval"]
    assert np.abs(x - oracle.pr_fixed_point(fx["row_ptr"], fx["col"])).sum() <= 1e-5


def _pull_case(name):
    z = np.load(os.path.join(HERE, "pull_pr.npz"))
    if name == "community64":
        rp, col = z["community64_row_ptr"], z["community64_col"]
        cp, mem = z["community64_clusters_ptr"], z["community64_clusters_members"]
    else:
        fx = load(name)
        rp, col = fx["row_ptr"], fx["col"]
        cp, mem = fx["clusters_ptr"], fx["clusters_members"]
    clusters = [mem[cp[i]:cp[i + 1]] for i in range(len(cp) - 1)]
    return rp, col, clusters, z[f"{name}_ref_pr_pull_peval"]


@pytest.mark.parametrize("name", ["planted2600", "community64"])
def test_pull_restatement_matches_reference(name):
    """oracle.pull restates the pull worker (its own stop test) and lands
    within 2e-6 of the reference's output on both cases."""
    from oracle import pull
    rp, col, clusters, ref = _pull_case(name)
    x, _ = pull.pr_pull_summarized(rp, col, clusters)
    assert np.abs(x - ref).sum() <= 2e-6


def test_reference_pull_worker_loses_mass_in_flight():
    """On 64 planted communities the reference's pull worker ends its
    summarized stage after two rounds (its stop test sees values only, and
    the mass that just reached the entries changes none) and the correction
    drops that mass: 1.5e-3 in L1 from the fixed point.  Counting the
    entries' arrivals in the stop test brings it within the PageRank bound."""
    from oracle import pull
    rp, col, clusters, ref = _pull_case("community64")
    x_star = oracle.pr_fixed_point(rp, col)
    assert np.abs(ref - x_star).sum() > 1e-3
    x, _ = pull.pr_pull_summarized(rp, col, clusters, count_entry_arrivals=True)
    assert np.abs(x - x_star).sum() <= 1e-5


# ------------------------------------------------------ workload-size cases

def _sha(*arrays):
    import hashlib
    h = hashlib.sha256()
    for a in arrays:
        if a is not None:
            h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def test_rmat16_inputs_regenerate_and_reference_against_oracle():
    """rmat16_pr: the graph and batch regenerate from their seeds (oracle
    generators, no library code); the reference's results are within the
    PageRank bounds of the FP64 fixed point and of the oracle's restatement;
    its summary kept a handful of the greedy clusters."""
    fx = load("rmat16_pr")
    rp, col, _ = oracle.rmat(16, 1 << 20, seed=1)
    assert _sha(rp, col) == str(fx["input_sha256"])
    upd = oracle.gen_updates(rp, col, 5000, 5000, 0, seed=2)
    assert _sha(upd) == str(fx["updates_sha256"])
    x_star = oracle.pr_fixed_point(rp, col)
    assert np.abs(fx["ref_pr_sum_peval"] - x_star).sum() < 1e-5
    nrp, ncol, _ = oracle.apply_updates(rp, col, None, upd)
    x_new = oracle.pr_fixed_point(nrp, ncol)
    assert np.abs(fx["ref_pr_sum_inc"] - x_new).sum() < 1e-5
    assert np.abs(fx["ref_pr_plain_inc"] - x_new).sum() < 1e-5
    x, delta, _ = oracle.ingress_pr(rp, col, tau=1e-6)
    d2 = oracle.pr_amend((rp, col), (nrp, ncol), x, delta)
    x2, _, _ = oracle.ingress_pr(nrp, ncol, x=x, delta=d2, tau=1e-6)
    assert np.abs(x2 - fx["ref_pr_plain_inc"]).sum() < 2e-5
    st = json.loads(str(fx["stats"]))["pr_peval"]
    assert st["spn_num"][0] > 0 and st["all_node_num"][0] == 1 << 16


def test_tight_threshold_reference_against_fixed_point_and_oracle():
    """rmat12_tight: at termcheck_threshold 1e-10 the reference is within 5e-7
    of the FP64 fixed point (its FP32 values round at about 3e-11 each over
    4,096 vertices) and the oracle's restatement within 1e-6 of it."""
    base, fx = load("rmat12"), load("rmat12_tight")
    assert str(fx["input_sha256"]) == str(base["input_sha256"])
    rp, col = base["row_ptr"], base["col"]
    x_star = oracle.pr_fixed_point(rp, col)
    assert np.abs(fx["ref_pr_sum_peval"] - x_star).sum() < 5e-7
    nrp, ncol, _ = after(base, "updates_pr")
    x_new = oracle.pr_fixed_point(nrp, ncol)
    assert np.abs(fx["ref_pr_sum_inc"] - x_new).sum() < 5e-7
    assert np.abs(fx["ref_pr_plain_inc"] - x_new).sum() < 5e-7
    x, delta, _ = oracle.ingress_pr(rp, col, tau=1e-10)
    d2 = oracle.pr_amend((rp, col), (nrp, ncol), x, delta)
    x2, _, _ = oracle.ingress_pr(nrp, ncol, x=x, delta=d2, tau=1e-10)
    assert np.abs(x2 - fx["ref_pr_plain_inc"]).sum() < 1e-6


def _u32_dist(d):
    out = np.full(len(d), 0xFFFFFFFF, np.uint32)
    fin = np.isfinite(d)
    out[fin] = d[fin].astype(np.uint32)
    return out


def test_rmat20_inputs_regenerate_and_reference_equals_dijkstra():
    """rmat20_sssp: the weighted graph and the 100,000-change batch
    regenerate from their seeds; the reference's summarized PEval and both of
    its incremental workers equal FP64 Dijkstra bit for bit."""
    fx = load("rmat20_sssp")
    rp, col, w = oracle.rmat(20, 1 << 24, seed=1, weight_kind=1, wlo=1, whi=100)
    assert _sha(rp, col, w) == str(fx["input_sha256"])
    upd = oracle.gen_updates(rp, col, 40000, 40000, 20000, seed=2)
    assert _sha(upd) == str(fx["updates_sha256"])
    assert np.array_equal(_u32_dist(oracle.dijkstra(rp, col, w, 0)), fx["ref_sssp_sum_peval"])
    nrp, ncol, nw = oracle.apply_updates(rp, col, w, upd)
    d1 = _u32_dist(oracle.dijkstra(nrp, ncol, nw, 0))
    assert np.array_equal(d1, fx["ref_sssp_plain_inc"])
    assert np.array_equal(d1, fx["ref_sssp_sum_inc"])
    st = json.loads(str(fx["stats"]))["sssp_peval"]
    assert st["spn_num"][0] > 0
