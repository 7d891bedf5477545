"""The PageRank adjoint kernel against central finite differences (FP64)
and an FP64 transposed solve, through the C ABI and the torch.autograd
binding."""
import numpy as np
import pytest

import oracle
import suminc_gb300 as sg

pytestmark = pytest.mark.gpu
D = 0.85


def weighted_graph(scale, seed):
    """R-MAT with float weights U[0.1, 1.0], column-normalised."""
    with sg.Context(0) as ctx:
        ctx.generate_rmat(scale, 16 << scale, seed=seed, weight_kind=2, wlo=0.1, whi=1.0)
        ctx.normalize_weights()
        return ctx.download_csr()


def loss_parts(n, seed, n_targets):
    rng = np.random.default_rng(seed)
    tgt = rng.choice(n, size=n_targets, replace=False)
    y = rng.uniform(0.0, 2.0 / n, size=n_targets)
    return tgt, y


def loss64(x, tgt, y):
    return 0.5 * float(np.sum((x[tgt] - y) ** 2))


def grad_x(x, n, tgt, y):
    g = np.zeros(n, np.float64)
    g[tgt] = x[tgt] - y
    return g


@pytest.fixture(scope="module")
def case():
    rp, col, w = weighted_graph(12, 5)
    n = len(rp) - 1
    tele = np.full(n, 1.0 / n)
    tgt, y = loss_parts(n, 6, 1000)
    return rp, col, w, n, tele, tgt, y


def test_columns_are_normalised(case):
    rp, col, w, n, *_ = case
    src = np.repeat(np.arange(n), np.diff(rp).astype(np.int64))
    s = np.bincount(src, weights=w.astype(np.float64), minlength=n)[np.diff(rp) > 0]
    assert np.allclose(s, 1.0, atol=1e-5)


def test_forward_matches_fp64(case):
    rp, col, w, n, tele, *_ = case
    with sg.Context(0) as ctx:
        ctx.load_csr(rp, col, w)
        x = ctx.pr_weighted(tele.astype(np.float32))
    xs = oracle.pr_fixed_point(rp, col, w, tele=tele)
    assert np.abs(x - xs).sum() <= 1e-5


def test_adjoint_matches_fp64_transposed_solve(case):
    rp, col, w, n, tele, tgt, y = case
    xs = oracle.pr_fixed_point(rp, col, w, tele=tele)
    with sg.Context(0) as ctx:
        ctx.load_csr(rp, col, w)
        x = ctx.pr_weighted(tele.astype(np.float32))
        g = grad_x(x.astype(np.float64), n, tgt, y)
        dw, dt = ctx.pr_adjoint(g.astype(np.float32))
        _, lam = ctx.adjoint_values()
    lam64 = oracle.pr_adjoint_solve(rp, col, w, g)
    rel = np.abs(lam - lam64).sum() / np.abs(lam64).sum()
    assert rel <= 1e-5
    src = np.repeat(np.arange(n), np.diff(rp).astype(np.int64))
    dw64 = D * lam64[col] * xs[src]
    assert np.abs(dw - dw64).sum() / np.abs(dw64).sum() <= 1e-4
    assert np.abs(dt - (1 - D) * lam64).sum() / np.abs(lam64).sum() <= 1e-5


def test_gradients_match_central_differences(case):
    rp, col, w, n, tele, tgt, y = case
    with sg.Context(0) as ctx:
        ctx.load_csr(rp, col, w)
        x = ctx.pr_weighted(tele.astype(np.float32))
        dw, dt = ctx.pr_adjoint(grad_x(x.astype(np.float64), n, tgt, y).astype(np.float32))
    rng = np.random.default_rng(9)
    edges = rng.choice(len(col), size=64, replace=False)
    h = 1e-4
    w64 = w.astype(np.float64)
    fd = []
    for e in edges:
        wp = w64.copy(); wp[e] += h
        wm = w64.copy(); wm[e] -= h
        lp = loss64(oracle.pr_fixed_point(rp, col, wp, tele=tele, tol=1e-15), tgt, y)
        lm = loss64(oracle.pr_fixed_point(rp, col, wm, tele=tele, tol=1e-15), tgt, y)
        fd.append((lp - lm) / (2 * h))
    fd = np.array(fd)
    scale = np.abs(fd).max()
    assert np.all(np.abs(dw[edges] - fd) <= 2e-3 * np.abs(fd) + 1e-3 * scale)
    # teleport entries
    vs = rng.choice(n, size=8, replace=False)
    for v in vs:
        tp = tele.copy(); tp[v] += h
        tm = tele.copy(); tm[v] -= h
        lp = loss64(oracle.pr_fixed_point(rp, col, w64, tele=tp, tol=1e-15), tgt, y)
        lm = loss64(oracle.pr_fixed_point(rp, col, w64, tele=tm, tol=1e-15), tgt, y)
        f = (lp - lm) / (2 * h)
        assert abs(dt[v] - f) <= 2e-3 * abs(f) + 1e-3 * np.abs(dt).max()


def test_torch_autograd_binding(case):
    torch = pytest.importorskip("torch")
    from suminc_gb300.autograd import pagerank
    rp, col, w, n, tele, tgt, y = case
    with sg.Context(0) as ctx:
        wt = torch.tensor(w, dtype=torch.float32, requires_grad=True)
        tt = torch.tensor(tele, dtype=torch.float32, requires_grad=True)
        x = pagerank(wt, tt, ctx, rp, col)
        loss = 0.5 * ((x[torch.from_numpy(tgt)] - torch.from_numpy(y).float()) ** 2).sum()
        loss.backward()
        dw, dt = ctx.pr_adjoint(grad_x(x.detach().numpy().astype(np.float64), n, tgt, y)
                                .astype(np.float32))
    assert np.allclose(wt.grad.numpy(), dw, rtol=1e-4, atol=1e-12)
    assert np.allclose(tt.grad.numpy(), dt, rtol=1e-4, atol=1e-12)


def test_adjoint_needs_current_forward():
    rp, col, w = weighted_graph(8, 2)
    with sg.Context(0) as ctx:
        ctx.load_csr(rp, col, w)
        with pytest.raises(sg.SgError):
            ctx.pr_adjoint(np.ones(len(rp) - 1, np.float32))
        ctx.pr_weighted()
        hg = sg.HostGraph(rp, col, w)
        ctx.apply_updates(hg.gen_updates(10, 10, 0, seed=1, integer_weights=False, wlo=0.1, whi=1.0))
        with pytest.raises(sg.SgError):
            ctx.pr_adjoint(np.ones(len(rp) - 1, np.float32))
    with sg.Context(0) as ctx:
        ctx.generate_rmat(8, 1000, seed=1)
        with pytest.raises(sg.SgError):
            ctx.pr_weighted()
