"""The allocation-free PageRank entry point (sg_pr_peval_noalloc).

It serves callers that cannot allocate device memory (memory owned by
another framework's pool, loops that must not synchronise on cudaMalloc): they hand in the graph and the outputs in
device memory, and the kernels use a fixed scratch array inside the library.
Checked through the C ABI against sg_pr_peval on the same graph, on two calls
in a row (the scratch array is shared and must be re-initialised by every
call).  This file sorts last so that a failure here cannot hide any other
test in a run that stops at the first failure.
"""
import ctypes as C

import numpy as np
import pytest

import suminc_gb300 as sg

pytestmark = pytest.mark.gpu
TOL = 2e-5  # both results are within 1e-5 (L1) of the FP64 fixed point


def _noalloc(lib, rp_d, col_d, n, m, x_d, d_d):
    rounds = C.c_int32()
    res = C.c_double()
    st = lib.sg_pr_peval_noalloc(n, m, C.c_void_p(rp_d.data_ptr()), C.c_void_p(col_d.data_ptr()),
                                 0.85, 1e-6, 1000, None, C.c_void_p(x_d.data_ptr()),
                                 C.c_void_p(d_d.data_ptr()), C.byref(rounds), C.byref(res))
    return st, rounds.value, res.value


def test_noalloc_matches_peval_twice():
    torch = pytest.importorskip("torch")
    lib = sg.load_library()
    rp, col, _ = sg.rmat_host(14, 16 << 14, seed=21)
    n, m = len(rp) - 1, int(rp[-1])
    with sg.Context(0) as ctx:
        ctx.load_csr(rp, col)
        ref = ctx.pr_peval()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    rp_d = torch.from_numpy(rp.view(np.int64)).to(dev)
    col_d = torch.from_numpy(col.view(np.int32)).to(dev)
    for call in range(2):
        x_d = torch.full((n,), float("nan"), dtype=torch.float32, device=dev)
        d_d = torch.full((n,), float("nan"), dtype=torch.float32, device=dev)
        torch.cuda.synchronize()
        st, rounds, res = _noalloc(lib, rp_d, col_d, n, m, x_d, d_d)
        assert st == sg.SG_OK, (call, st)
        assert res < 1e-6 and rounds > 0
        x = x_d.cpu().numpy()
        assert np.isfinite(x).all()
        assert np.abs(x - ref).sum() <= TOL, call


def test_noalloc_rejects_oversize_graph():
    lib = sg.load_library()
    n = sg.PR_NOALLOC_MAX_VERTICES + 1
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    st = lib.sg_pr_peval_noalloc(n, 0, dummy, dummy, 0.85, 1e-6, 10, None, dummy, dummy, None,
                                 None)
    assert st == sg.SG_ERR_TOO_LARGE
