"""Python binding of libsuminc_gb300 (ctypes over the C ABI in
``include/suminc_gb300.h``).

The binding only marshals arrays; every computation runs in the CUDA library.
Importing works without a GPU (host utilities such as the R-MAT twin and the
update-batch mirror need none); a missing or unbuilt library raises
``ImportError`` -- there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

__all__ = [
    "SgError", "Options", "Stats", "Context", "HostGraph", "UPDATE_DTYPE",
    "rmat_host", "lib_path", "load_library", "K_NAMES",
]

_HERE = os.path.dirname(os.path.abspath(__file__))


def lib_path() -> str:
    return os.path.join(_HERE, "_build", "libsuminc_gb300.so")


class SgError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"sg status {status}: {msg}")
        self.status = status


SG_OK = 0
SG_ERR_INVALID = 1
SG_ERR_CUDA = 2
SG_ERR_OOM = 3
SG_ERR_STATE = 4
SG_ERR_NOT_CONVERGED = 5
SG_ERR_TIMEOUT = 6
SG_ERR_UNSUPPORTED = 7
SG_ERR_TOO_LARGE = 8

SG_MSG_PUSH = 0
SG_MSG_PULL = 1
PR_NOALLOC_MAX_VERTICES = 1 << 22

SG_UPD_ADD = 0
SG_UPD_DEL = 1

UPDATE_DTYPE = np.dtype([("src", "<u4"), ("dst", "<u4"), ("weight", "<f4"), ("op", "<u4")])

K_NAMES = ["pr_pull", "sum_local", "pr_vertex", "apply", "sssp", "summary", "batch", "adjoint"]


class Options(C.Structure):
    _fields_ = [
        ("damping", C.c_double),
        ("termcheck_threshold", C.c_double),
        ("max_rounds", C.c_int32),
        ("compress", C.c_int32),
        ("max_node_num", C.c_int32),
        ("min_node_num", C.c_int32),
        ("mirror_k", C.c_int32),
        ("profile", C.c_int32),
        ("compress_threshold", C.c_double),
        ("sssp_delta", C.c_double),
        ("slack", C.c_double),
        ("adjoint_rel_tol", C.c_double),
        ("pull_hubs", C.c_int32),
        ("message_type", C.c_int32),
        ("reserved", C.c_int32 * 6),
    ]


class SummaryInfo(C.Structure):
    _fields_ = [(k, C.c_uint64) for k in (
        "clusters", "supernodes", "cluster_members", "sources", "bound_nodes", "bound_index",
        "inner_index", "inner_value_index", "all_rows", "absorbed", "in_mirrors", "out_mirrors",
        "sync_edges", "boundary_edges", "shortcut_edges")] + [("node_type_count", C.c_uint64 * 7)]

    def as_dict(self) -> dict:
        d = {k: int(getattr(self, k)) for k, _ in self._fields_ if k != "node_type_count"}
        d["node_type_count"] = [int(x) for x in self.node_type_count]
        return d


class SummaryCheck(C.Structure):
    _fields_ = [(k, C.c_uint64) for k in (
        "rows", "type_diff", "list_diff", "ib_diff", "is_diff", "corr_diff")] + [
        ("max_rel", C.c_double)]

    def as_dict(self) -> dict:
        return {k: (float(getattr(self, k)) if k == "max_rel" else int(getattr(self, k)))
                for k, _ in self._fields_}


class BatchSpec(C.Structure):
    _fields_ = [
        ("ppr_queries", C.c_uint32),
        ("ppr_seed_ptr", C.c_void_p),
        ("ppr_seeds", C.c_void_p),
        ("sssp_sources", C.c_uint32),
        ("sources", C.c_void_p),
    ]


class BatchInfo(C.Structure):
    _fields_ = [
        ("ppr_queries", C.c_uint32),
        ("sssp_sources", C.c_uint32),
        ("chunk_quads", C.c_uint32),
        ("blocks_per_sm", C.c_uint32),
        ("sssp_bucket", C.c_double),
        ("graph_launch", C.c_int32),
        ("tune_ms", C.c_double),
        ("iterations", C.c_uint32),
        ("ppr_pulls", C.c_uint32),
        ("sssp_steps", C.c_uint32),
        ("sssp_scans", C.c_uint32),
        ("ppr_not_converged", C.c_uint32),
        ("ppr_edge_visits", C.c_uint64),
        ("sssp_relaxations", C.c_uint64),
        ("sssp_improvements", C.c_uint64),
        ("elapsed_ms", C.c_double),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class AdjointInfo(C.Structure):
    _fields_ = [
        ("forward_rounds", C.c_int32),
        ("adjoint_rounds", C.c_int32),
        ("forward_ms", C.c_double),
        ("adjoint_ms", C.c_double),
        ("forward_residual", C.c_double),
        ("adjoint_residual", C.c_double),
        ("forward_edges", C.c_uint64),
        ("adjoint_edges", C.c_uint64),
        ("gradient_edges", C.c_uint64),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class Stats(C.Structure):
    _fields_ = [
        ("rounds", C.c_int32),
        ("converged", C.c_int32),
        ("residual", C.c_double),
        ("edges_relaxed", C.c_uint64),
        ("vertex_visits", C.c_uint64),
        ("shortcut_edges", C.c_uint64),
        ("improvements", C.c_uint64),
        ("elapsed_ms", C.c_double),
        ("kernel_ms", C.c_double * 8),
        ("kernel_launches", C.c_uint64 * 8),
        ("live_edges", C.c_uint64),
        ("reset_vertices", C.c_uint64),
        ("launches_total", C.c_uint64),
        ("edges_pull", C.c_uint64),
        ("edges_push", C.c_uint64),
        ("repacks", C.c_uint64),
    ]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_ if k not in ("kernel_ms", "kernel_launches")}
        d["kernel_ms"] = {K_NAMES[i]: self.kernel_ms[i] for i in range(8)}
        d["kernel_launches"] = {K_NAMES[i]: int(self.kernel_launches[i]) for i in range(8)}
        return d


_P = C.c_void_p
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")

_SIGS = {
    "sg_options_default": ([C.POINTER(Options)], C.c_int),
    "sg_ctx_create": ([C.c_int, C.POINTER(Options), C.POINTER(_P)], C.c_int),
    "sg_ctx_destroy": ([_P], C.c_int),
    "sg_last_error": ([_P], C.c_char_p),
    "sg_ctx_set_stream": ([_P, _P], C.c_int),
    "sg_get_stats": ([_P, C.POINTER(Stats)], C.c_int),
    "sg_graph_load_csr": ([_P, C.c_uint32, _P, _P, _P], C.c_int),
    "sg_graph_generate_rmat": ([_P, C.c_int, C.c_uint64, C.c_double, C.c_double, C.c_double,
                                C.c_uint64, C.c_int, C.c_double, C.c_double], C.c_int),
    "sg_graph_num_vertices": ([_P, C.POINTER(C.c_uint32)], C.c_int),
    "sg_graph_num_edges": ([_P, C.POINTER(C.c_uint64)], C.c_int),
    "sg_graph_download_csr": ([_P, _P, _P, _P], C.c_int),
    "sg_apply_updates": ([_P, C.c_uint64, _P], C.c_int),
    "sg_apply_updates_device": ([_P, C.c_uint64, _P], C.c_int),
    "sg_reset_stats": ([_P], C.c_int),
    "sg_ctx_record_event": ([_P, C.c_int], C.c_int),
    "sg_ctx_elapsed_ms": ([_P, C.c_int, C.c_int, C.POINTER(C.c_double)], C.c_int),
    "sg_ctx_synchronize": ([_P], C.c_int),
    "sg_ctx_set_profile": ([_P, C.c_int32], C.c_int),
    "sg_pr_peval": ([_P, _P], C.c_int),
    "sg_pr_inceval": ([_P, _P], C.c_int),
    "sg_pr_values": ([_P, _P], C.c_int),
    "sg_pr_deltas": ([_P, _P], C.c_int),
    "sg_pr_values_device": ([_P, C.POINTER(_P)], C.c_int),
    "sg_sssp_peval": ([_P, C.c_uint32, _P], C.c_int),
    "sg_sssp_inceval": ([_P, _P], C.c_int),
    "sg_sssp_distances": ([_P, _P], C.c_int),
    "sg_sssp_parents": ([_P, _P], C.c_int),
    "sg_debug_barrier_probe": ([_P, C.c_int32], C.c_int),
    "sg_util_rmat_host": ([C.c_int, C.c_uint64, C.c_double, C.c_double, C.c_double, C.c_uint64,
                           C.c_int, C.c_double, C.c_double, _P, _P, _P], C.c_int),
    "sg_hostgraph_create": ([C.c_uint32, _P, _P, _P, C.POINTER(_P)], C.c_int),
    "sg_hostgraph_destroy": ([_P], C.c_int),
    "sg_hostgraph_gen_updates": ([_P, C.c_uint64, C.c_uint64, C.c_uint64, C.c_uint64, C.c_int,
                                  C.c_double, C.c_double, _P], C.c_int),
    "sg_hostgraph_num_edges": ([_P, C.POINTER(C.c_uint64)], C.c_int),
    "sg_hostgraph_csr": ([_P, _P, _P, _P], C.c_int),
    "sg_pr_peval_noalloc": ([C.c_uint32, C.c_uint64, _P, _P, C.c_double, C.c_double, C.c_int32,
                             _P, _P, _P, C.POINTER(C.c_int32), C.POINTER(C.c_double)], C.c_int),
    "sg_summary_build": ([_P, C.c_uint32, _P, _P], C.c_int),
    "sg_ppr": ([_P, C.c_uint32, _P, _P], C.c_int),
    "sg_graph_load_files": ([_P, C.c_char_p, C.c_char_p, C.c_int], C.c_int),
    "sg_graph_vertex_oids": ([_P, _P], C.c_int),
    "sg_graph_set_vertex_oids": ([_P, _P], C.c_int),
    "sg_apply_update_file": ([_P, C.c_char_p], C.c_int),
    "sg_summary_build_file": ([_P, C.c_char_p], C.c_int),
    "sg_summary_save": ([_P, C.c_char_p], C.c_int),
    "sg_summary_load": ([_P, C.c_char_p], C.c_int),
    "sg_pr_weighted": ([_P, _P, _P], C.c_int),
    "sg_graph_normalize_weights": ([_P], C.c_int),
    "sg_pr_adjoint": ([_P, _P, _P, _P], C.c_int),
    "sg_pr_adjoint_device": ([_P, _P, _P, _P], C.c_int),
    "sg_adjoint_info_get": ([_P, C.POINTER(AdjointInfo)], C.c_int),
    "sg_adjoint_values": ([_P, _P, _P], C.c_int),
    "sg_batch_run": ([_P, C.POINTER(BatchSpec), _P, _P], C.c_int),
    "sg_batch_tune_run": ([_P, C.POINTER(BatchSpec), _P, _P], C.c_int),
    "sg_batch_info_get": ([_P, C.POINTER(BatchInfo)], C.c_int),
    "sg_batch_query_stats": ([_P, _P, _P], C.c_int),
    "sg_batch_outputs_device": ([_P, C.POINTER(_P), C.POINTER(_P)], C.c_int),
    "sg_summary_info_get": ([_P, C.POINTER(SummaryInfo)], C.c_int),
    "sg_summary_check_tables": ([_P, C.POINTER(SummaryCheck)], C.c_int),
    "sg_util_summary_serialize": ([C.c_uint32, _P, _P, C.c_uint32, _P, _P, C.c_int, C.c_int,
                                   C.c_double, _P, C.POINTER(C.c_uint64)], C.c_int),
    "sg_util_greedy_clusters": ([C.c_uint32, _P, _P, C.c_int, C.c_int, C.c_uint64, _P, _P,
                                 C.POINTER(C.c_uint32)], C.c_int),
}

_lib = None


def load_library():
    """Loads the in-tree library once; raises ImportError when it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        raise ImportError(
            f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(path)
    for name, (args, res) in _SIGS.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _check(st: int, ctx=None, what: str = ""):
    if st == SG_OK:
        return
    msg = what
    if ctx is not None and ctx._h:
        msg = f"{what}: {load_library().sg_last_error(ctx._h).decode(errors='replace')}"
    raise SgError(st, msg)


def default_options(**kw) -> Options:
    o = Options()
    _check(load_library().sg_options_default(C.byref(o)), None, "sg_options_default")
    for k, v in kw.items():
        if not hasattr(o, k):
            raise TypeError(f"unknown option {k}")
        setattr(o, k, v)
    return o


class Context:
    """One device context (graph + application states) on one GPU."""

    def __init__(self, device: int = 0, **options):
        self._lib = load_library()
        self._h = None
        self.options = default_options(**options)
        h = _P()
        st = self._lib.sg_ctx_create(device, C.byref(self.options), C.byref(h))
        if st != SG_OK:
            raise SgError(st, "sg_ctx_create failed (no CUDA device?)")
        self._h = h

    def close(self):
        if self._h:
            self._lib.sg_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- graph ------------------------------------------------------------
    def load_csr(self, row_ptr, col, w=None):
        row_ptr = np.ascontiguousarray(row_ptr, dtype=np.uint64)
        col = np.ascontiguousarray(col, dtype=np.uint32)
        w = None if w is None else np.ascontiguousarray(w, dtype=np.float32)
        n = len(row_ptr) - 1
        _check(self._lib.sg_graph_load_csr(self._h, n, _ptr(row_ptr), _ptr(col), _ptr(w)), self,
               "sg_graph_load_csr")

    def generate_rmat(self, scale, edges, a=0.57, b=0.19, c=0.19, seed=1, weight_kind=0,
                      wlo=1.0, whi=100.0):
        _check(self._lib.sg_graph_generate_rmat(self._h, scale, edges, a, b, c, seed, weight_kind,
                                                wlo, whi), self, "sg_graph_generate_rmat")

    @property
    def n(self) -> int:
        v = C.c_uint32()
        _check(self._lib.sg_graph_num_vertices(self._h, C.byref(v)), self)
        return v.value

    @property
    def m(self) -> int:
        v = C.c_uint64()
        _check(self._lib.sg_graph_num_edges(self._h, C.byref(v)), self)
        return v.value

    def download_csr(self, weights=True):
        n, m = self.n, self.m
        rp = np.empty(n + 1, np.uint64)
        col = np.empty(m, np.uint32)
        w = np.empty(m, np.float32) if weights else None
        _check(self._lib.sg_graph_download_csr(self._h, _ptr(rp), _ptr(col), _ptr(w)), self,
               "sg_graph_download_csr")
        return rp, col, w

    def apply_updates(self, upd: np.ndarray):
        upd = np.ascontiguousarray(upd, dtype=UPDATE_DTYPE)
        _check(self._lib.sg_apply_updates(self._h, len(upd), _ptr(upd)), self, "sg_apply_updates")

    def apply_updates_ptr(self, count: int, ptr: int, on_device: bool):
        """Batch given as a raw pointer (pinned host or device memory)."""
        fn = self._lib.sg_apply_updates_device if on_device else self._lib.sg_apply_updates
        _check(fn(self._h, count, C.c_void_p(ptr)), self, "apply_updates_ptr")

    def pr_inceval_into(self, out_ptr: int | None):
        _check(self._lib.sg_pr_inceval(self._h, None if out_ptr is None else C.c_void_p(out_ptr)),
               self, "sg_pr_inceval")

    def record_event(self, slot: int):
        _check(self._lib.sg_ctx_record_event(self._h, slot), self, "sg_ctx_record_event")

    def elapsed_ms(self, a: int, b: int) -> float:
        v = C.c_double()
        _check(self._lib.sg_ctx_elapsed_ms(self._h, a, b, C.byref(v)), self, "sg_ctx_elapsed_ms")
        return v.value

    def set_profile(self, mask: int):
        _check(self._lib.sg_ctx_set_profile(self._h, mask), self, "sg_ctx_set_profile")

    def synchronize(self):
        _check(self._lib.sg_ctx_synchronize(self._h), self, "sg_ctx_synchronize")

    def reset_stats(self):
        _check(self._lib.sg_reset_stats(self._h), self, "sg_reset_stats")

    # -- PageRank ---------------------------------------------------------
    def pr_peval(self, out=True):
        x = np.empty(self.n, np.float32) if out else None
        _check(self._lib.sg_pr_peval(self._h, _ptr(x)), self, "sg_pr_peval")
        return x

    def pr_inceval(self, out=True):
        x = np.empty(self.n, np.float32) if out else None
        _check(self._lib.sg_pr_inceval(self._h, _ptr(x)), self, "sg_pr_inceval")
        return x

    def pr_values(self):
        x = np.empty(self.n, np.float32)
        _check(self._lib.sg_pr_values(self._h, _ptr(x)), self, "sg_pr_values")
        return x

    def pr_deltas(self):
        x = np.empty(self.n, np.float32)
        _check(self._lib.sg_pr_deltas(self._h, _ptr(x)), self, "sg_pr_deltas")
        return x

    # -- summarized graph -------------------------------------------------
    def summary_build(self, clusters):
        """clusters: list of member arrays (the cluster file's records)."""
        cp = np.zeros(len(clusters) + 1, np.uint32)
        for i, c in enumerate(clusters):
            cp[i + 1] = cp[i] + len(c)
        mem = (np.concatenate([np.asarray(c, np.uint32) for c in clusters])
               if clusters else np.zeros(1, np.uint32))
        _check(self._lib.sg_summary_build(self._h, len(clusters), _ptr(cp), _ptr(mem)), self,
               "sg_summary_build")

    def summary_info(self) -> dict:
        info = SummaryInfo()
        _check(self._lib.sg_summary_info_get(self._h, C.byref(info)), self, "sg_summary_info_get")
        return info.as_dict()

    def summary_check(self) -> dict:
        """Device-repaired summary tables against the host restatement."""
        out = SummaryCheck()
        _check(self._lib.sg_summary_check_tables(self._h, C.byref(out)), self,
               "sg_summary_check_tables")
        return out.as_dict()

    # -- the reference's text files ---------------------------------------
    def load_files(self, efile, vfile=None, weighted=False):
        _check(self._lib.sg_graph_load_files(self._h, efile.encode(),
                                             vfile.encode() if vfile else None, int(weighted)),
               self, "sg_graph_load_files")

    def vertex_oids(self):
        o = np.empty(self.n, np.uint64)
        _check(self._lib.sg_graph_vertex_oids(self._h, _ptr(o)), self, "sg_graph_vertex_oids")
        return o

    def set_vertex_oids(self, oids):
        o = np.ascontiguousarray(oids, np.uint64)
        _check(self._lib.sg_graph_set_vertex_oids(self._h, _ptr(o)), self, "sg_graph_set_vertex_oids")

    def apply_update_file(self, path):
        _check(self._lib.sg_apply_update_file(self._h, path.encode()), self, "sg_apply_update_file")

    def summary_save(self, path):
        _check(self._lib.sg_summary_save(self._h, path.encode()), self, "sg_summary_save")

    def summary_load(self, path):
        _check(self._lib.sg_summary_load(self._h, path.encode()), self, "sg_summary_load")

    def summary_build_file(self, path):
        _check(self._lib.sg_summary_build_file(self._h, path.encode()), self,
               "sg_summary_build_file")

    # -- personalized PageRank and batches -------------------------------
    def ppr(self, seeds, out=True):
        seeds = np.ascontiguousarray(seeds, np.uint32)
        x = np.empty(self.n, np.float32) if out else None
        _check(self._lib.sg_ppr(self._h, len(seeds), _ptr(seeds), _ptr(x)), self, "sg_ppr")
        return x

    def batch_run(self, ppr_seeds=(), sources=(), out=True, retune=False):
        """ppr_seeds: list of seed arrays (one PPR query each); sources: SSSP
        sources.  Returns (ppr float32[Q, n], sssp float64[S, n]) or Nones."""
        q = len(ppr_seeds)
        sp = np.zeros(q + 1, np.uint32)
        for i, sd in enumerate(ppr_seeds):
            sp[i + 1] = sp[i] + len(sd)
        seeds = (np.concatenate([np.asarray(x, np.uint32) for x in ppr_seeds])
                 if q else np.zeros(1, np.uint32))
        src = np.ascontiguousarray(sources, np.uint32) if len(sources) else np.zeros(1, np.uint32)
        spec = BatchSpec(q, sp.ctypes.data, seeds.ctypes.data, len(sources), src.ctypes.data)
        po = np.empty((q, self.n), np.float32) if (out and q) else None
        so = np.empty((len(sources), self.n), np.float64) if (out and len(sources)) else None
        fn = self._lib.sg_batch_tune_run if retune else self._lib.sg_batch_run
        _check(fn(self._h, C.byref(spec), _ptr(po), _ptr(so)), self, "sg_batch_run")
        return po, so

    def batch_info(self) -> dict:
        info = BatchInfo()
        _check(self._lib.sg_batch_info_get(self._h, C.byref(info)), self, "sg_batch_info_get")
        return info.as_dict()

    def batch_query_stats(self, nq):
        r = np.empty(nq, np.int32)
        res = np.empty(nq, np.float64)
        _check(self._lib.sg_batch_query_stats(self._h, _ptr(r), _ptr(res)), self,
               "sg_batch_query_stats")
        return r, res

    # -- weighted PageRank and its adjoint ---------------------------------
    def normalize_weights(self):
        _check(self._lib.sg_graph_normalize_weights(self._h), self, "sg_graph_normalize_weights")

    def pr_weighted(self, tele=None, out=True):
        t = None if tele is None else np.ascontiguousarray(tele, np.float32)
        x = np.empty(self.n, np.float32) if out else None
        _check(self._lib.sg_pr_weighted(self._h, _ptr(t), _ptr(x)), self, "sg_pr_weighted")
        return x

    def pr_adjoint(self, dl_dx, out=True):
        """Returns (dL/dw in download_csr edge order, dL/dtele)."""
        g = np.ascontiguousarray(dl_dx, np.float32)
        dw = np.empty(self.m, np.float32) if out else None
        dt = np.empty(self.n, np.float32) if out else None
        _check(self._lib.sg_pr_adjoint(self._h, _ptr(g), _ptr(dw), _ptr(dt)), self, "sg_pr_adjoint")
        return dw, dt

    def adjoint_info(self) -> dict:
        info = AdjointInfo()
        _check(self._lib.sg_adjoint_info_get(self._h, C.byref(info)), self, "sg_adjoint_info_get")
        return info.as_dict()

    def adjoint_values(self):
        x = np.empty(self.n, np.float32)
        lam = np.empty(self.n, np.float32)
        _check(self._lib.sg_adjoint_values(self._h, _ptr(x), _ptr(lam)), self, "sg_adjoint_values")
        return x, lam

    # -- SSSP -------------------------------------------------------------
    def sssp_peval(self, source=0, out=True):
        d = np.empty(self.n, np.float64) if out else None
        _check(self._lib.sg_sssp_peval(self._h, source, _ptr(d)), self, "sg_sssp_peval")
        return d

    def sssp_inceval(self, out=True):
        d = np.empty(self.n, np.float64) if out else None
        _check(self._lib.sg_sssp_inceval(self._h, _ptr(d)), self, "sg_sssp_inceval")
        return d

    def sssp_distances(self):
        d = np.empty(self.n, np.float64)
        _check(self._lib.sg_sssp_distances(self._h, _ptr(d)), self, "sg_sssp_distances")
        return d

    def barrier_probe(self, skip_one_block: bool) -> int:
        """Runs the persistent kernels' bounded grid barrier with one CTA kept
        away (or none); returns the status code, SG_ERR_TIMEOUT when the wait
        ran out."""
        return int(self._lib.sg_debug_barrier_probe(self._h, 1 if skip_one_block else 0))

    def sssp_parents(self):
        p = np.empty(self.n, np.uint32)
        _check(self._lib.sg_sssp_parents(self._h, _ptr(p)), self, "sg_sssp_parents")
        return p

    def stats(self) -> dict:
        s = Stats()
        _check(self._lib.sg_get_stats(self._h, C.byref(s)), self)
        return s.as_dict()


def rmat_host(scale, edges, a=0.57, b=0.19, c=0.19, seed=1, weight_kind=0, wlo=1.0, whi=100.0):
    """Host twin of Context.generate_rmat: returns (row_ptr, col, w or None)."""
    lib = load_library()
    n = 1 << scale
    rp = np.empty(n + 1, np.uint64)
    col = np.empty(edges, np.uint32)
    w = np.empty(edges, np.float32) if weight_kind else None
    _check(lib.sg_util_rmat_host(scale, edges, a, b, c, seed, weight_kind, wlo, whi, _ptr(rp),
                                 _ptr(col), _ptr(w)), None, "sg_util_rmat_host")
    return rp, col, w


def summary_serialize_host(row_ptr, col, clusters, min_node_num=8, mirror_k=4,
                           compress_threshold=1.0) -> bytes:
    """The summary's cluster state in the reference's serialized layout,
    computed on the host (no GPU)."""
    lib = load_library()
    rp = np.ascontiguousarray(row_ptr, np.uint64)
    col = np.ascontiguousarray(col, np.uint32)
    cp = np.zeros(len(clusters) + 1, np.uint32)
    for i, c in enumerate(clusters):
        cp[i + 1] = cp[i] + len(c)
    mem = (np.concatenate([np.asarray(c, np.uint32) for c in clusters])
           if len(clusters) else np.zeros(1, np.uint32))
    size = C.c_uint64(0)
    args = (len(rp) - 1, _ptr(rp), _ptr(col), len(clusters), _ptr(cp), _ptr(mem), min_node_num,
            mirror_k, compress_threshold)
    _check(lib.sg_util_summary_serialize(*args, None, C.byref(size)), None,
           "sg_util_summary_serialize")
    buf = np.zeros(size.value, np.uint8)
    _check(lib.sg_util_summary_serialize(*args, _ptr(buf), C.byref(size)), None,
           "sg_util_summary_serialize")
    return buf.tobytes()


def greedy_clusters(row_ptr, col, max_node_num=150, min_node_num=8, seed=1):
    """In-repo greedy clustering; returns a list of sorted member arrays."""
    lib = load_library()
    row_ptr = np.ascontiguousarray(row_ptr, np.uint64)
    col = np.ascontiguousarray(col, np.uint32)
    n = len(row_ptr) - 1
    cp = np.zeros(n + 1, np.uint32)
    mem = np.zeros(max(n, 1), np.uint32)
    k = C.c_uint32()
    _check(lib.sg_util_greedy_clusters(n, _ptr(row_ptr), _ptr(col), max_node_num, min_node_num,
                                       seed, _ptr(cp), _ptr(mem), C.byref(k)), None,
           "sg_util_greedy_clusters")
    return [mem[cp[i]:cp[i + 1]].copy() for i in range(k.value)]


class HostGraph:
    """Host adjacency mirror that draws valid update batches."""

    def __init__(self, row_ptr, col, w=None):
        self._lib = load_library()
        self._h = None
        row_ptr = np.ascontiguousarray(row_ptr, dtype=np.uint64)
        col = np.ascontiguousarray(col, dtype=np.uint32)
        self.weighted = w is not None
        w = None if w is None else np.ascontiguousarray(w, dtype=np.float32)
        h = _P()
        _check(self._lib.sg_hostgraph_create(len(row_ptr) - 1, _ptr(row_ptr), _ptr(col), _ptr(w),
                                             C.byref(h)), None, "sg_hostgraph_create")
        self._h = h
        self.n = len(row_ptr) - 1

    def __del__(self):
        if self._h:
            self._lib.sg_hostgraph_destroy(self._h)
            self._h = None

    @property
    def m(self) -> int:
        v = C.c_uint64()
        _check(self._lib.sg_hostgraph_num_edges(self._h, C.byref(v)))
        return v.value

    def gen_updates(self, n_ins, n_del, n_rew=0, seed=1, integer_weights=True, wlo=1.0,
                    whi=100.0) -> np.ndarray:
        out = np.zeros(n_ins + n_del + 2 * n_rew, UPDATE_DTYPE)
        _check(self._lib.sg_hostgraph_gen_updates(self._h, n_ins, n_del, n_rew, seed,
                                                  1 if integer_weights else 0, wlo, whi,
                                                  _ptr(out)), None, "sg_hostgraph_gen_updates")
        return out

    def csr(self):
        m = self.m
        rp = np.empty(self.n + 1, np.uint64)
        col = np.empty(m, np.uint32)
        w = np.empty(m, np.float32) if self.weighted else None
        _check(self._lib.sg_hostgraph_csr(self._h, _ptr(rp), _ptr(col), _ptr(w)))
        return rp, col, w
