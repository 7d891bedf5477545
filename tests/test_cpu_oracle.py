"""The oracle restatement agrees with its own FP64 solvers and with the
reference semantics it restates."""
import numpy as np
import pytest

import oracle
import suminc_gb300 as sg


def test_ingress_pr_converges_to_fixed_point():
    rp, col, _ = sg.rmat_host(12, 60000, seed=2)
    x, delta, st = oracle.ingress_pr(rp, col, tau=1e-6)
    assert st["converged"] == 1 and st["residual"] < 1e-6
    xf = oracle.pr_fixed_point(rp, col)
    # distance to the fixed point is bounded by residual / (1 - d)
    assert np.abs(x - xf).sum() <= 1e-5


def test_amend_then_inceval_equals_fresh_batch():
    rp, col, w = sg.rmat_host(11, 30000, seed=7, weight_kind=1)
    hg = sg.HostGraph(rp, col, w)
    upd = hg.gen_updates(300, 300, seed=3)
    nrp, ncol, _ = hg.csr()
    x, delta, _ = oracle.ingress_pr(rp, col, tau=1e-9)
    delta = oracle.pr_amend((rp, col), (nrp, ncol), x, delta)
    x2, _, st = oracle.ingress_pr(nrp, ncol, tau=1e-9, x=x, delta=delta)
    xf = oracle.pr_fixed_point(nrp, ncol)
    assert st["converged"] == 1
    assert np.abs(x2 - xf).sum() < 5e-6


def test_dijkstra_small_known_graph():
    # 0->1 (4), 0->2 (1), 2->1 (2), 1->3 (5); 4 unreachable
    rp = np.array([0, 2, 3, 4, 4, 4], np.uint64)
    col = np.array([1, 2, 3, 1], np.uint32)
    w = np.array([4, 1, 5, 2], np.float32)
    d = oracle.dijkstra(rp, col, w, 0)
    assert d.tolist()[:4] == [0.0, 3.0, 1.0, 8.0] and np.isinf(d[4])


def test_adjoint_solve_matches_dense_linear_algebra():
    rng = np.random.default_rng(0)
    n = 40
    rows = [sorted(rng.choice(n, size=rng.integers(1, 6), replace=False)) for _ in range(n)]
    rp = np.zeros(n + 1, np.uint64)
    for i, r in enumerate(rows):
        rp[i + 1] = rp[i] + len(r)
    col = np.concatenate(rows).astype(np.uint32)
    w = rng.uniform(0.1, 1.0, len(col)).astype(np.float32)
    for i in range(n):  # column-normalise (out-weights of each source sum to 1)
        s = w[rp[i]:rp[i + 1]].astype(np.float64).sum()
        w[rp[i]:rp[i + 1]] = (w[rp[i]:rp[i + 1]] / s).astype(np.float32)
    P = np.zeros((n, n))
    for u in range(n):
        for e in range(int(rp[u]), int(rp[u + 1])):
            P[u, col[e]] = w[e]
    g = rng.normal(size=n)
    lam = oracle.pr_adjoint_solve(rp, col, w, g)
    lam_ref = np.linalg.solve(np.eye(n) - 0.85 * P, g)
    assert np.abs(lam - lam_ref).max() < 1e-10
    x = oracle.pr_fixed_point(rp, col, w)
    x_ref = np.linalg.solve(np.eye(n) - 0.85 * P.T, np.full(n, 0.15 / n))
    assert np.abs(x - x_ref).max() < 1e-12


def test_oracle_adjoint_matches_central_differences():
    """FP64 transposed solve + dL/dw_uv = d*lambda_v*x_u against central
    differences of the FP64 fixed point (pins the adjoint the GPU is
    checked against)."""
    import suminc_gb300 as sg
    rp, col, w = sg.rmat_host(8, 2000, seed=3, weight_kind=2, wlo=0.1, whi=1.0)
    n = len(rp) - 1
    w = w.astype(np.float64)
    src = np.repeat(np.arange(n), np.diff(rp).astype(np.int64))
    s = np.bincount(src, weights=w, minlength=n)
    w = w / s[src]
    tele = np.full(n, 1.0 / n)
    rng = np.random.default_rng(1)
    tgt = rng.choice(n, size=60, replace=False)
    y = rng.uniform(0, 2.0 / n, size=60)

    def loss(ww, tt):
        x = oracle.pr_fixed_point(rp, col, ww, tele=tt, tol=1e-15)
        return 0.5 * np.sum((x[tgt] - y) ** 2), x

    L0, x = loss(w, tele)
    g = np.zeros(n)
    g[tgt] = x[tgt] - y
    lam = oracle.pr_adjoint_solve(rp, col, w, g, tol=1e-16)
    dw = 0.85 * lam[col] * x[src]
    h = 1e-5
    for e in rng.choice(len(col), size=12, replace=False):
        wp = w.copy(); wp[e] += h
        wm = w.copy(); wm[e] -= h
        fd = (loss(wp, tele)[0] - loss(wm, tele)[0]) / (2 * h)
        assert abs(dw[e] - fd) <= 1e-6 * abs(fd) + 1e-9 * np.abs(dw).max()
    v = int(tgt[0])
    tp = tele.copy(); tp[v] += h
    tm = tele.copy(); tm[v] -= h
    fd = (loss(w, tp)[0] - loss(w, tm)[0]) / (2 * h)
    assert abs(0.15 * lam[v] - fd) <= 1e-6 * abs(fd) + 1e-12


@pytest.mark.parametrize("scale,kind", [(12, 0), (12, 1), (12, 2), (16, 0), (16, 1)])
def test_oracle_rmat_equals_library_host_generator(scale, kind):
    """The oracle's R-MAT restatement (no library code) gives the same graph
    and weights as the library's host twin of its device generator."""
    lo, hi = (0.1, 1.0) if kind == 2 else (1.0, 100.0)
    a = sg.rmat_host(scale, 16 << scale, seed=5, weight_kind=kind, wlo=lo, whi=hi)
    b = oracle.rmat(scale, 16 << scale, seed=5, weight_kind=kind, wlo=lo, whi=hi)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    if kind:
        assert np.array_equal(a[2], b[2])


def test_oracle_updates_equal_library_batches_and_reference_semantics():
    """Batches drawn by the oracle equal the library's HostGraph batches on the
    same graph and seed; the oracle's apply equals the pure-Python restatement
    of the reference's update semantics and the library's mirror."""
    rp, col, w = sg.rmat_host(12, 16 << 12, seed=1, weight_kind=1)
    hg = sg.HostGraph(rp, col, w)
    cur = (rp, col, w)
    for i in range(3):
        u_lib = hg.gen_updates(300, 200, 100, seed=10 + i)
        u_or = oracle.gen_updates(cur[0], cur[1], 300, 200, 100, seed=10 + i)
        assert np.array_equal(u_lib, u_or)
        nxt = oracle.apply_updates(*cur, u_or)
        ref = oracle.apply_updates_reference(*cur, u_or)
        assert all(np.array_equal(a, b) for a, b in zip(nxt, ref))
        assert all(np.array_equal(a, b) for a, b in zip(nxt, hg.csr()))
        cur = nxt


def test_apply_updates_edge_cases():
    # 0->1, 0->2, 1->2; batch: delete absent 2->0, add existing 0->1 (new
    # weight), two adds of 1->0 (the first wins), delete + add of 1->2
    rp = np.array([0, 2, 3, 3], np.uint64)
    col = np.array([1, 2, 2], np.uint32)
    w = np.array([5, 6, 7], np.float32)
    upd = np.array([(2, 0, 0, 1), (0, 1, 9, 0), (1, 0, 3, 0), (1, 0, 4, 0), (1, 2, 0, 1),
                    (1, 2, 8, 0)], dtype=oracle.UPDATE_DTYPE)
    nrp, ncol, nw = oracle.apply_updates(rp, col, w, upd)
    assert nrp.tolist() == [0, 2, 4, 4]
    assert ncol.tolist() == [1, 2, 0, 2] and nw.tolist() == [9, 6, 3, 8]
    ref = oracle.apply_updates_reference(rp, col, w, upd)
    assert all(np.array_equal(a, b) for a, b in zip((nrp, ncol, nw), ref))
    e = oracle.apply_updates(rp, col, w, np.zeros(0, oracle.UPDATE_DTYPE))
    assert all(np.array_equal(a, b) for a, b in zip(e, (rp, col, w)))


def test_residual_bound_holds():
    """||x - x*||_1 <= residual / (1 - d) for the delta iteration's result."""
    rp, col, _ = sg.rmat_host(12, 16 << 12, seed=4)
    xf = oracle.pr_fixed_point(rp, col)
    for tau in (1e-4, 1e-6):
        x, _, _ = oracle.ingress_pr(rp, col, tau=tau)
        bound = oracle.pr_residual_l1(rp, col, x) / 0.15
        assert np.abs(x - xf).sum() <= bound * (1 + 1e-9) + 1e-12
    assert oracle.pr_residual_l1(rp, col, xf.astype(np.float32)) < 1e-7
