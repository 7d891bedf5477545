"""CPU oracle -- test infrastructure only.

Imported by ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg
of ``bench.py``, and only as the checker.  The product path
(``suminc_gb300``) never imports it.  ``liboracle.so`` is built from
``oracle.c`` by ``oracle/build.py``.

Parity pins: the PageRank and SSSP restatements are checked against golden
vectors produced by the reference's own CPU worker (tests/golden/, see
make_golden.py there) and against the FP64 solvers in this module.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build
from .updates import apply_updates_reference  # noqa: F401

_lib = None


class OrStats(C.Structure):
    _fields_ = [("rounds", C.c_int32), ("converged", C.c_int32), ("residual", C.c_double),
                ("edges", C.c_uint64), ("visits", C.c_uint64)]


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        P = C.c_void_p
        L.or_ingress_pr.argtypes = [C.c_uint32, P, P, C.c_double, C.c_double, C.c_int, C.c_int,
                                    C.c_int, P, P, C.POINTER(OrStats)]
        L.or_ingress_pr.restype = C.c_int
        L.or_pr_amend.argtypes = [C.c_uint32, P, P, P, P, C.c_double, P, P]
        L.or_pr_amend.restype = None
        L.or_pr_fixed_point.argtypes = [C.c_uint32, P, P, P, C.c_double, P, C.c_double, C.c_int, P]
        L.or_pr_fixed_point.restype = C.c_int
        L.or_pr_adjoint_solve.argtypes = [C.c_uint32, P, P, P, C.c_double, P, C.c_double, C.c_int, P]
        L.or_pr_adjoint_solve.restype = C.c_int
        L.or_dijkstra.argtypes = [C.c_uint32, P, P, P, C.c_uint32, P]
        L.or_dijkstra.restype = C.c_int
        L.or_sssp_peval.argtypes = [C.c_uint32, P, P, P, C.c_uint32, C.c_int, P, P,
                                    C.POINTER(OrStats)]
        L.or_sssp_peval.restype = C.c_int
        L.or_sssp_inceval.argtypes = [C.c_uint32, P, P, P, P, P, C.c_uint64, P, P, C.c_int, P, P,
                                      C.POINTER(OrStats)]
        L.or_sssp_inceval.restype = C.c_int
        L.or_rmat.argtypes = [C.c_int, C.c_uint64, C.c_double, C.c_double, C.c_double,
                              C.c_uint64, C.c_int, C.c_double, C.c_double, P, P, P]
        L.or_rmat.restype = C.c_int
        L.or_gen_updates.argtypes = [C.c_uint32, P, P, C.c_uint64, C.c_uint64, C.c_uint64,
                                     C.c_uint64, C.c_int, C.c_double, C.c_double, P]
        L.or_gen_updates.restype = C.c_int
        L.or_apply_updates.argtypes = [C.c_uint32, P, P, P, P, C.c_uint64, P, P, P]
        L.or_apply_updates.restype = C.c_int
        L.or_pr_residual_l1.argtypes = [C.c_uint32, P, P, C.c_double, P, C.POINTER(C.c_double)]
        L.or_pr_residual_l1.restype = C.c_int
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _csr(rp, col, w=None):
    rp = np.ascontiguousarray(rp, np.uint64)
    col = np.ascontiguousarray(col, np.uint32)
    w = None if w is None else np.ascontiguousarray(w, np.float32)
    return rp, col, w


def ingress_pr(rp, col, damping=0.85, tau=1e-6, x=None, delta=None, max_rounds=100000,
               threads=0):
    """Delta PageRank rounds (PEval when x is None, else continue from x/delta)."""
    rp, col, _ = _csr(rp, col)
    n = len(rp) - 1
    init = x is None
    x = np.zeros(n, np.float32) if init else np.array(x, np.float32, copy=True)
    delta = np.zeros(n, np.float32) if init else np.array(delta, np.float32, copy=True)
    st = OrStats()
    lib().or_ingress_pr(n, _p(rp), _p(col), damping, tau, 1 if init else 0, max_rounds, threads,
                        _p(x), _p(delta), C.byref(st))
    return x, delta, {k: getattr(st, k) for k, _ in OrStats._fields_}


def pr_amend(old, new, x, delta, damping=0.85):
    rpo, colo, _ = _csr(*old[:2])
    rpn, coln, _ = _csr(*new[:2])
    x = np.ascontiguousarray(x, np.float32)
    delta = np.array(delta, np.float32, copy=True)
    lib().or_pr_amend(len(rpo) - 1, _p(rpo), _p(colo), _p(rpn), _p(coln), damping, _p(x),
                      _p(delta))
    return delta


def pr_fixed_point(rp, col, w=None, damping=0.85, tele=None, tol=1e-12, max_iter=100000):
    """FP64 Jacobi solve of x = (1-d) t + d M x; unweighted: M[v][u] =
    1/outdeg(u); weighted: M[v][u] = w_uv (taken in FP64)."""
    rp, col, _ = _csr(rp, col)
    w = None if w is None else np.ascontiguousarray(w, np.float64)
    n = len(rp) - 1
    x = np.zeros(n, np.float64)
    t = None if tele is None else np.ascontiguousarray(tele, np.float64)
    lib().or_pr_fixed_point(n, _p(rp), _p(col), _p(w), damping, _p(t), tol, max_iter, _p(x))
    return x


def pr_adjoint_solve(rp, col, w, g, damping=0.85, tol=1e-13, max_iter=100000):
    """FP64 solve of lambda = g + d M^T lambda (M[v][u] = w_uv)."""
    rp, col, _ = _csr(rp, col)
    w = np.ascontiguousarray(w, np.float64)
    n = len(rp) - 1
    lam = np.zeros(n, np.float64)
    g = np.ascontiguousarray(g, np.float64)
    lib().or_pr_adjoint_solve(n, _p(rp), _p(col), _p(w), damping, _p(g), tol, max_iter, _p(lam))
    return lam


def dijkstra(rp, col, w, source=0):
    rp, col, w = _csr(rp, col, w)
    n = len(rp) - 1
    d = np.empty(n, np.float64)
    lib().or_dijkstra(n, _p(rp), _p(col), _p(w), source, _p(d))
    return d


def sssp_peval(rp, col, w, source=0, threads=0):
    """The reference's SSSP traversal from `source` (integer weights):
    returns (distances f64 with inf, parents u32, stats)."""
    rp, col, w = _csr(rp, col, w)
    n = len(rp) - 1
    d = np.empty(n, np.float64)
    par = np.empty(n, np.uint32)
    st = OrStats()
    if lib().or_sssp_peval(n, _p(rp), _p(col), _p(w), source, threads, _p(d), _p(par),
                           C.byref(st)):
        raise ValueError("or_sssp_peval: bad source or non-integer weights")
    return d, par, {k: getattr(st, k) for k, _ in OrStats._fields_}


def sssp_inceval(old, new, deleted, dist, parent, threads=0):
    """The reference's incremental SSSP stage (deltaCompute, then one round
    from every vertex with a finite delta, then the traversal) after a batch:
    `old` = (row_ptr, col) before it, `new` = (row_ptr, col, w) after it,
    `deleted` = (src, dst) arrays of the removed edges (a re-weighted edge is
    a removal plus an insert, as in the reference's update files).  Returns
    (distances, parents, stats); stats["residual"] holds the reset count."""
    rpo, colo, _ = _csr(*old[:2])
    rp, col, w = _csr(*new[:3])
    n = len(rp) - 1
    ds = np.ascontiguousarray(deleted[0], np.uint32)
    dd = np.ascontiguousarray(deleted[1], np.uint32)
    d = np.array(dist, np.float64, copy=True)
    par = np.array(parent, np.uint32, copy=True)
    st = OrStats()
    if lib().or_sssp_inceval(n, _p(rpo), _p(colo), _p(rp), _p(col), _p(w), len(ds), _p(ds),
                             _p(dd), threads, _p(d), _p(par), C.byref(st)):
        raise ValueError("or_sssp_inceval: non-integer weights")
    return d, par, {k: getattr(st, k) for k, _ in OrStats._fields_}



# update records: u32 src, u32 dst, f32 weight, u32 op (0 add, 1 delete)
UPDATE_DTYPE = np.dtype([("src", "<u4"), ("dst", "<u4"), ("weight", "<f4"), ("op", "<u4")])


def rmat(scale, edges, a=0.57, b=0.19, c=0.19, seed=1, weight_kind=0, wlo=1.0, whi=100.0):
    """Seeded R-MAT graph (first `edges` distinct non-loop pairs of the draw
    stream, rows sorted): (row_ptr u64, col u32, w f32 or None)."""
    n = 1 << scale
    rp = np.empty(n + 1, np.uint64)
    col = np.empty(edges, np.uint32)
    w = np.empty(edges, np.float32) if weight_kind else None
    if lib().or_rmat(scale, edges, a, b, c, seed, weight_kind, wlo, whi, _p(rp), _p(col), _p(w)):
        raise ValueError("or_rmat failed")
    return rp, col, w


def gen_updates(rp, col, n_ins, n_del, n_rew=0, seed=1, integer_weights=True, wlo=1.0,
                whi=100.0):
    """One update batch valid for the graph (rows sorted): deletes, re-weights
    (delete + add), inserts, as UPDATE_DTYPE records."""
    rp, col, _ = _csr(rp, col)
    out = np.zeros(n_ins + n_del + 2 * n_rew, UPDATE_DTYPE)
    if lib().or_gen_updates(len(rp) - 1, _p(rp), _p(col), n_ins, n_del, n_rew, seed,
                            1 if integer_weights else 0, wlo, whi, _p(out)):
        raise ValueError("or_gen_updates: sizes do not fit the graph")
    return out


def apply_updates(rp, col, w, upd):
    """The graph after a batch, with the reference's update semantics:
    (row_ptr, col, w or None)."""
    rp, col, w = _csr(rp, col, w)
    upd = np.ascontiguousarray(upd, UPDATE_DTYPE)
    n = len(rp) - 1
    rpn = np.empty(n + 1, np.uint64)
    L = lib()
    if L.or_apply_updates(n, _p(rp), _p(col), _p(w), _p(upd), len(upd), _p(rpn), None, None):
        raise MemoryError("or_apply_updates")
    coln = np.empty(int(rpn[-1]), np.uint32)
    wn = np.empty(int(rpn[-1]), np.float32) if w is not None else None
    if L.or_apply_updates(n, _p(rp), _p(col), _p(w), _p(upd), len(upd), _p(rpn), _p(coln),
                          _p(wn)):
        raise MemoryError("or_apply_updates")
    return rpn, coln, wn


def pr_residual_l1(rp, col, x, damping=0.85):
    """|| (1-d)/N + d P^T x - x ||_1 in FP64; ||x - x*||_1 <= this / (1 - d)."""
    rp, col, _ = _csr(rp, col)
    x = np.ascontiguousarray(x, np.float32)
    r = C.c_double()
    if lib().or_pr_residual_l1(len(rp) - 1, _p(rp), _p(col), damping, _p(x), C.byref(r)):
        raise MemoryError("or_pr_residual_l1")
    return r.value
