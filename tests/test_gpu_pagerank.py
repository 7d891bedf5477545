"""PageRank PEval / IncEval on the device against the oracle.

Tolerances: the reference stops at an L1 residual below tau = 1e-6, so its
distance to the fixed point is at most tau / (1 - d) = 6.7e-6 in L1; the
bound used against the FP64 fixed point (iterated to 1e-12) is 1e-5.
"""
import numpy as np
import pytest

import oracle
import suminc_gb300 as sg

pytestmark = pytest.mark.gpu
TOL_FIXED = 1e-5


@pytest.mark.parametrize("scale,ef", [(10, 8), (13, 16), (16, 16)])
def test_peval_matches_fixed_point(ctx, scale, ef):
    n = 1 << scale
    ctx.generate_rmat(scale, n * ef, seed=scale)
    x = ctx.pr_peval()
    st = ctx.stats()
    assert st["converged"] == 1 and st["residual"] < 1e-6
    rp, col, _ = ctx.download_csr(weights=False)
    xf = oracle.pr_fixed_point(rp, col)
    assert np.abs(x - xf).sum() <= TOL_FIXED
    # and close to the reference-style CPU restatement at the same threshold
    xo, _, _ = oracle.ingress_pr(rp, col)
    assert np.abs(x - xo).sum() <= 2 * TOL_FIXED


def test_inceval_after_batches_matches_fixed_point(ctx):
    scale = 14
    n = 1 << scale
    ctx.generate_rmat(scale, 16 * n, seed=5)
    rp, col, _ = ctx.download_csr(weights=False)
    hg = sg.HostGraph(rp, col)
    ctx.pr_peval(out=False)
    for b in range(4):
        upd = hg.gen_updates(500, 500, seed=40 + b)
        ctx.apply_updates(upd)
        x = ctx.pr_inceval()
        st = ctx.stats()
        assert st["converged"] == 1
        nrp, ncol, _ = hg.csr()
        xf = oracle.pr_fixed_point(nrp, ncol)
        assert np.abs(x - xf).sum() <= TOL_FIXED, b


def test_inceval_matches_oracle_amend_sequence(ctx):
    rp, col, _ = sg.rmat_host(12, 50000, seed=8)
    ctx.load_csr(rp, col)
    x0 = ctx.pr_peval()
    d0 = ctx.pr_deltas()
    hg = sg.HostGraph(rp, col)
    upd = hg.gen_updates(1000, 1000, seed=2)
    nrp, ncol, _ = hg.csr()
    ctx.apply_updates(upd)
    # amended deltas equal the reference's full AmendValue(-1)/(+1) (up to
    # float rounding of terms that cancel)
    d_gpu = ctx.pr_deltas()
    d_ref = oracle.pr_amend((rp, col), (nrp, ncol), x0, d0)
    assert np.abs(d_gpu - d_ref).sum() < 1e-6
    x = ctx.pr_inceval()
    xo, _, _ = oracle.ingress_pr(nrp, ncol, x=x0, delta=d_ref)
    assert np.abs(x - xo).sum() < 2 * TOL_FIXED


def test_dangling_and_isolated_vertices(ctx):
    # 0 -> 1 -> 2, 3 isolated, 2 dangling
    rp = np.array([0, 1, 2, 2, 2], np.uint64)
    col = np.array([1, 2], np.uint32)
    ctx.load_csr(rp, col)
    x = ctx.pr_peval()
    xf = oracle.pr_fixed_point(rp, col)
    assert np.abs(x - xf).sum() < 1e-6


def test_inceval_before_peval_is_a_state_error(ctx):
    rp, col, _ = sg.rmat_host(8, 1000, seed=1)
    ctx.load_csr(rp, col)
    with pytest.raises(sg.SgError) as e:
        ctx.pr_inceval()
    assert e.value.status == sg.SG_ERR_STATE


def test_pull_hub_cache_matches_uncached_pull():
    """The pull that keeps the push values of the highest out-degree
    vertices in shared memory (reading an encoded copy of the in-CSR
    columns) against the pull without that cache, over PEval and IncEvals
    after batches (each batch makes the encoded copy stale)."""
    scale = 16
    n = 1 << scale
    with sg.Context(0) as a, sg.Context(0, pull_hubs=-1) as b:
        a.generate_rmat(scale, 16 * n, seed=7)
        rp, col, _ = a.download_csr(weights=False)
        b.load_csr(rp, col)
        xa, xb = a.pr_peval(), b.pr_peval()
        assert np.abs(xa - xb).sum() <= 5e-6
        assert np.abs(xa - oracle.pr_fixed_point(rp, col)).sum() <= TOL_FIXED
        hg = sg.HostGraph(rp, col)
        for k in range(3):
            upd = hg.gen_updates(2000, 2000, seed=90 + k)
            a.apply_updates(upd)
            b.apply_updates(upd)
            xa, xb = a.pr_inceval(), b.pr_inceval()
            assert np.abs(xa - xb).sum() <= 5e-6, k
            nrp, ncol, _ = hg.csr()
            assert np.abs(xa - oracle.pr_fixed_point(nrp, ncol)).sum() <= TOL_FIXED, k
