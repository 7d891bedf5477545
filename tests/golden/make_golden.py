#!/usr/bin/env python
"""Generates the golden fixtures in this directory by running the
reference's own CPU workers (built by oracle/ref_harness/build_ref.py from
the reference checkout) on seeded inputs.

Run where a reference checkout exists, naming it:
    python tests/golden/make_golden.py --reference PATH
(or with SUMINC_REFERENCE=PATH in the environment).
Each case writes <case>.npz with:
  params        json: generator parameters and reference flags
  input_sha256  hash of the (row_ptr, col, weights) the case was run on
  clusters_*    the cluster file both sides consume (in-repo greedy builder)
  updates       the update batch (sg_update records)
  ref_*         per-vertex results of the reference (float64):
                  pr_sum_peval / pr_sum_inc   SumSyncIterWorker (compress=1)
                  pr_plain_inc                IngressSyncIterWorker (compress=0)
                  sssp_sum_peval / sssp_sum_inc  SumSyncTraversalWorker
                  sssp_plain_inc              IngressSyncTraversalWorker (compress=0)
  stats         json: counters the reference logged while building its
                summary (node types, supernodes, mirrors, sketch edges)
  ref_serialized_summary  the bytes of the reference's serialize_cluster file
                (written with serialization_cmp_prefix)

    python tests/golden/make_golden.py --pull
runs the message_type=pull worker (SumSyncIterWorkerPull) on the inputs of
the cases above, with mirror_k large enough that no mirror is made, and
writes pull_pr.npz: params (flags), <case>_input_sha256 and
<case>_ref_pr_pull_peval; plus community64 (64 planted communities of 40,
bench.py's community generator, seed 1) with its inputs
community64_row_ptr / _col / _clusters_ptr / _clusters_members, on which the
reference's pull worker ends its summarized stage after two rounds and
stays 1.5e-3 in L1 from the fixed point.  Its IncEval is not recorded: with an update file
the reference's pull worker stops with a segmentation fault inside
inc_run (after inc_compute_index_mirror_spid) on both cases.
"""
from __future__ import annotations

import hashlib
import json
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import suminc_gb300 as sg  # noqa: E402

REF_FLAGS_PR = dict(application="pagerank", cilk="true", compress="1", compress_type="2", portion="1",
                    termcheck_threshold="1e-6", message_type="push", gpu_start="0",
                    max_node_num="150", min_node_num="8", mirror_k="4",
                    compress_threshold="1", app_concurrency="4", directed="true")
REF_FLAGS_SSSP = dict(REF_FLAGS_PR, application="sssp", cilk="false", sssp_source="0")


def input_hash(rp, col, w):
    h = hashlib.sha256()
    for a in (rp, col) + ((w,) if w is not None else ()):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def planted_graph(n_clusters=60, size=40, p_in=0.2, n_free=200, seed=7):
    """Directed graph with planted communities (seeded).  Each community has
    three entry and three exit vertices; free vertices carry random edges and
    some of them send / receive more than mirror_k edges to / from one
    community, which makes them in- and out-mirror candidates."""
    rng = np.random.default_rng(seed)
    n = n_clusters * size + n_free
    edges = set()
    for c in range(n_clusters):
        base = c * size
        m = rng.random((size, size)) < p_in
        np.fill_diagonal(m, False)
        for a, b in zip(*np.nonzero(m)):
            edges.add((base + int(a), base + int(b)))
        for x in range(size - 3, size):  # exits -> entries of other communities
            for _ in range(4):
                oc = int(rng.integers(n_clusters))
                if oc != c:
                    edges.add((base + x, oc * size + int(rng.integers(3))))
    free0 = n_clusters * size
    for f in range(free0, n):
        for _ in range(3):
            v = int(rng.integers(n))
            if v != f:
                edges.add((f, v))
        if (f - free0) % 10 == 0:  # mirror candidates
            c = int(rng.integers(n_clusters))
            for mbr in rng.choice(size, 6, replace=False):
                edges.add((f, c * size + int(mbr)))
            for mbr in rng.choice(size, 6, replace=False):
                edges.add((c * size + int(mbr), f))
    edges = sorted(edges)
    rp = np.zeros(n + 1, np.uint64)
    for u, _ in edges:
        rp[u + 1] += 1
    rp = np.cumsum(rp).astype(np.uint64)
    col = np.array([v for _, v in edges], np.uint32)
    w = np.array([1 + (u * 2654435761 + v * 40503) % 100 for u, v in edges], np.float32)
    return rp, col, w


def write_graph(d, rp, col, w):
    n = len(rp) - 1
    src = np.repeat(np.arange(n), np.diff(rp).astype(np.int64))
    with open(os.path.join(d, "g.e"), "w") as f:
        for u, v in zip(src.tolist(), col.tolist()):
            f.write(f"{u} {v}\n")
    with open(os.path.join(d, "g_w.e"), "w") as f:
        for u, v, x in zip(src.tolist(), col.tolist(), w.astype(np.int64).tolist()):
            f.write(f"{u} {v} {x}\n")
    with open(os.path.join(d, "g.v"), "w") as f:
        for v in range(n):
            f.write(f"{v}\n")


def write_updates(path, upd, weighted):
    with open(path, "w") as f:
        for r in upd:
            if int(r["op"]) == 0:
                f.write(f"a {r['src']} {r['dst']}" + (f" {int(r['weight'])}\n" if weighted else "\n"))
            else:
                f.write(f"d {r['src']} {r['dst']}\n")


def parse_stats(log):
    st = {}
    for key, pat in [("spn_num", r"#global_spn_num: (\d+)"), ("ids_num", r"#global_ids_num: (\d+)"),
                     ("spn_com_num", r"#global_spn_com_num: (\d+)"),
                     ("bound_node_num", r"#global_bound_node_num: (\d+)"),
                     ("source_node_num", r"#global_source_node_num: (\d+)"),
                     ("bound_index_num", r"#global_bound_index_num: (\d+)"),
                     ("all_node_num", r" all_node_num=(\d+)"),
                     ("mirror_node_cnt", r"mirror_node_cnt=(\d+)"),
                     ("sync_e_num", r" sync_e_num=(\d+)"), ("bound_e_num", r" bound_e_num=(\d+)"),
                     ("source_e_num", r" source_e_num=(\d+)")]:
        m = re.findall(pat, log)
        if m:
            st[key] = [int(x) for x in m]
    types = re.findall(r"  type(\d)=(\d+) rate", log)
    if types:
        st["node_types"] = [[int(a), int(b)] for a, b in types]
    for key, pat in [("batch_time", r"#?Batch time: ([0-9.e-]+)"),
                     ("inc_time", r"#?Inc time: ([0-9.e-]+)")]:
        m = re.findall(pat, log)
        if m:
            st[key] = [float(x) for x in m]
    return st


def run_ref(exe, d, app, flags, update=None, threads=4):
    out = os.path.join(d, f"{app}.bin")
    args = [exe, app, out] + [f"{k}={v}" for k, v in flags.items()]
    efile = "g_w.e" if app.startswith("sssp") else "g.e"
    args += [f"efile={os.path.join(d, efile)}", f"vfile={os.path.join(d, 'g.v')}"]
    if update:
        args.append(f"efile_update={update}")
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="", OMP_NUM_THREADS=str(threads))
    p = subprocess.run(args, capture_output=True, text=True, env=env, timeout=3600)
    if p.returncode != 0:
        sys.stderr.write(p.stderr[-4000:])
        raise RuntimeError(f"reference run failed: {app}")
    return np.fromfile(out, dtype=np.float64), p.stderr


def make_case(name, rp, col, w, exe, seed, clusters=None):
    n = len(rp) - 1
    if clusters is None:
        clusters = sg.greedy_clusters(rp, col, 150, 8, seed=seed)
    hg = sg.HostGraph(rp, col, w)
    m = int(rp[-1])
    n_upd = max(100, m // 100)
    upd_pr = hg.gen_updates(n_upd // 2, n_upd // 2, 0, seed=seed + 1)
    hg2 = sg.HostGraph(rp, col, w)
    upd_ss = hg2.gen_updates(int(n_upd * 0.4), int(n_upd * 0.4), int(n_upd * 0.2), seed=seed + 2)
    res = {}
    stats = {}
    with tempfile.TemporaryDirectory() as d:
        write_graph(d, rp, col, w)
        with open(os.path.join(d, "g.e.c_150"), "w") as f:
            for c in clusters:
                f.write(" ".join([str(len(c))] + [str(int(v)) for v in c]) + "\n")
        upd_pr_path = os.path.join(d, "pr.update")
        write_updates(upd_pr_path, upd_pr, False)
        upd_ss_path = os.path.join(d, "sssp.update")
        write_updates(upd_ss_path, upd_ss, True)
        ser_dir = os.path.join(d, "ser")
        os.makedirs(ser_dir)
        res["pr_sum_peval"], log = run_ref(exe, d, "pagerank",
                                           dict(REF_FLAGS_PR, serialization_cmp_prefix=ser_dir))
        stats["pr_peval"] = parse_stats(log)
        ser_files = sorted(os.listdir(ser_dir))
        if len(ser_files) != 1:
            raise RuntimeError(f"expected one serialized summary, found {ser_files}")
        with open(os.path.join(ser_dir, ser_files[0]), "rb") as f:
            ref_serialized = np.frombuffer(f.read(), dtype=np.uint8)
        res["pr_sum_inc"], log = run_ref(exe, d, "pagerank", REF_FLAGS_PR, upd_pr_path)
        stats["pr_inc"] = parse_stats(log)
        res["pr_plain_inc"], log = run_ref(exe, d, "pagerank_plain", dict(REF_FLAGS_PR, compress="0"),
                                           upd_pr_path)
        stats["pr_plain"] = parse_stats(log)
        res["sssp_sum_peval"], log = run_ref(exe, d, "sssp", REF_FLAGS_SSSP)
        stats["sssp_peval"] = parse_stats(log)
        res["sssp_sum_inc"], log = run_ref(exe, d, "sssp", REF_FLAGS_SSSP, upd_ss_path)
        stats["sssp_inc"] = parse_stats(log)
        res["sssp_plain_inc"], log = run_ref(exe, d, "sssp_plain", dict(REF_FLAGS_SSSP, compress="0"),
                                             upd_ss_path)
    cp = np.zeros(len(clusters) + 1, np.uint32)
    for i, c in enumerate(clusters):
        cp[i + 1] = cp[i] + len(c)
    mem = np.concatenate(clusters).astype(np.uint32) if clusters else np.zeros(0, np.uint32)
    params = {"name": name, "n": n, "m": m, "cluster_seed": seed, "flags_pr": REF_FLAGS_PR,
              "flags_sssp": REF_FLAGS_SSSP, "n_updates": n_upd}
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), params=json.dumps(params),
                        input_sha256=input_hash(rp, col, w), row_ptr=rp, col=col, w=w,
                        clusters_ptr=cp, clusters_members=mem, updates_pr=upd_pr,
                        updates_sssp=upd_ss, stats=json.dumps(stats),
                        ref_serialized_summary=ref_serialized,
                        **{f"ref_{k}": v for k, v in res.items()})
    print(name, {k: (len(v), float(np.nansum(np.where(np.isfinite(v), v, 0)))) for k, v in res.items()},
          "clusters", len(clusters))


PULL_MIRROR_K = "1000000000"


def make_pull(exe):
    flags = dict(REF_FLAGS_PR, message_type="pull", mirror_k=PULL_MIRROR_K)
    out = {"params": json.dumps({"flags_pr_pull": flags})}
    for name in ("rmat12", "planted2600"):
        z = np.load(os.path.join(HERE, f"{name}.npz"))
        rp, col, w = z["row_ptr"], z["col"], z["w"]
        cp, mem = z["clusters_ptr"], z["clusters_members"]
        with tempfile.TemporaryDirectory() as d:
            write_graph(d, rp, col, w)
            with open(os.path.join(d, "g.e.c_150"), "w") as f:
                for i in range(len(cp) - 1):
                    c = mem[cp[i]:cp[i + 1]]
                    f.write(" ".join([str(len(c))] + [str(int(v)) for v in c]) + "\n")
            res, log = run_ref(exe, d, "pagerank_pull", flags)
        out[f"{name}_input_sha256"] = str(z["input_sha256"])
        out[f"{name}_ref_pr_pull_peval"] = res
        out[f"{name}_stats"] = json.dumps(parse_stats(log))
        print(name, "pull", len(res), float(res.sum()))
    import bench
    rp, col, w, comms = bench.community_graph(64, 40, 1)
    cp = np.zeros(len(comms) + 1, np.uint32)
    for i, c in enumerate(comms):
        cp[i + 1] = cp[i] + len(c)
    mem = np.concatenate(comms).astype(np.uint32)
    with tempfile.TemporaryDirectory() as d:
        write_graph(d, rp, col, w)
        with open(os.path.join(d, "g.e.c_150"), "w") as f:
            for c in comms:
                f.write(" ".join([str(len(c))] + [str(int(v)) for v in c]) + "\n")
        res, log = run_ref(exe, d, "pagerank_pull", flags)
    out.update(community64_row_ptr=rp, community64_col=col, community64_clusters_ptr=cp,
               community64_clusters_members=mem, community64_ref_pr_pull_peval=res,
               community64_stats=json.dumps(parse_stats(log)))
    print("community64", "pull", len(res), float(res.sum()))
    np.savez_compressed(os.path.join(HERE, "pull_pr.npz"), **out)


# ----------------------------------------------------- workload-size cases
#
#   rmat16_pr.npz    PageRank on R-MAT scale 16 (65,536 vertices, 2^20 edges,
#                    seed 1), greedy clusters (max 150, min 8, seed 1), one
#                    10,000-change batch (50 % inserts / 50 % deletes, seed 2):
#                    the reference's SumInc PEval and IncEval (compress=1) and
#                    its plain Ingress IncEval (compress=0), values as float32
#                    (the reference's value type, so exact).
#   rmat20_sssp.npz  SSSP from vertex 0 on R-MAT scale 20 (1,048,576
#                    vertices, 2^24 edges, integer weights U[1, 100], seed 1),
#                    greedy clusters, one 100,000-change batch (40 % inserts,
#                    40 % deletes, 20 % re-weights, seed 2): summarized PEval
#                    and IncEval and the plain IncEval, distances as uint32
#                    (0xFFFFFFFF = unreachable).
# The inputs are not stored: tests regenerate the graph and the batch from the
# seeds (oracle.rmat / oracle.gen_updates, or the library's generators, which
# draw the same) and check them against the stored hashes.  The clusters are
# stored (the greedy builder takes minutes at scale 20).

def write_graph_fast(d, rp, col, w):
    n = len(rp) - 1
    src = np.repeat(np.arange(n, dtype=np.int64), np.diff(rp).astype(np.int64))
    np.savetxt(os.path.join(d, "g.e"), np.stack([src, col.astype(np.int64)], 1), fmt="%d %d")
    if w is not None:
        np.savetxt(os.path.join(d, "g_w.e"),
                   np.stack([src, col.astype(np.int64), w.astype(np.int64)], 1), fmt="%d %d %d")
    np.savetxt(os.path.join(d, "g.v"), np.arange(n, dtype=np.int64), fmt="%d")


def write_clusters(path, clusters):
    with open(path, "w") as f:
        for c in clusters:
            f.write(" ".join([str(len(c))] + [str(int(v)) for v in c]) + "\n")


def pack_clusters(clusters):
    cp = np.zeros(len(clusters) + 1, np.uint32)
    for i, c in enumerate(clusters):
        cp[i + 1] = cp[i] + len(c)
    mem = np.concatenate(clusters).astype(np.uint32) if clusters else np.zeros(0, np.uint32)
    return cp, mem


def update_hash(upd):
    return hashlib.sha256(np.ascontiguousarray(upd).tobytes()).hexdigest()


def make_rmat16_pr(exe, threads):
    import oracle
    rp, col, _ = oracle.rmat(16, 1 << 20, seed=1)
    clusters = sg.greedy_clusters(rp, col, 150, 8, seed=1)
    upd = oracle.gen_updates(rp, col, 5000, 5000, 0, seed=2)
    flags = dict(REF_FLAGS_PR, app_concurrency=str(threads))
    res, stats = {}, {}
    with tempfile.TemporaryDirectory() as d:
        write_graph_fast(d, rp, col, None)
        write_clusters(os.path.join(d, "g.e.c_150"), clusters)
        up = os.path.join(d, "pr.update")
        write_updates(up, upd, False)
        res["pr_sum_peval"], log = run_ref(exe, d, "pagerank", flags, threads=threads)
        stats["pr_peval"] = parse_stats(log)
        res["pr_sum_inc"], log = run_ref(exe, d, "pagerank", flags, up, threads=threads)
        stats["pr_inc"] = parse_stats(log)
        res["pr_plain_inc"], log = run_ref(exe, d, "pagerank_plain", dict(flags, compress="0"), up,
                                           threads=threads)
        stats["pr_plain"] = parse_stats(log)
    cp, mem = pack_clusters(clusters)
    params = {"graph": "oracle.rmat(16, 1 << 20, seed=1)", "clusters": "greedy(150, 8, seed=1)",
              "updates": "oracle.gen_updates(rp, col, 5000, 5000, 0, seed=2)", "flags_pr": flags}
    np.savez_compressed(os.path.join(HERE, "rmat16_pr.npz"), params=json.dumps(params),
                        input_sha256=input_hash(rp, col, None), updates_sha256=update_hash(upd),
                        clusters_ptr=cp, clusters_members=mem, stats=json.dumps(stats),
                        **{f"ref_{k}": v.astype(np.float32) for k, v in res.items()})
    print("rmat16_pr", {k: float(v.sum()) for k, v in res.items()}, "clusters", len(clusters))


def as_u32_dist(d):
    out = np.full(len(d), 0xFFFFFFFF, np.uint32)
    fin = np.isfinite(d) & (d < 2147483647)
    assert np.all(d[fin] == np.round(d[fin]))
    out[fin] = d[fin].astype(np.uint32)
    return out


def make_rmat20_sssp(exe, threads, clusters_path=None):
    import oracle
    rp, col, w = oracle.rmat(20, 1 << 24, seed=1, weight_kind=1, wlo=1, whi=100)
    if clusters_path:
        z = np.load(clusters_path)
        cp, mem = z["clusters_ptr"], z["clusters_members"]
        clusters = [mem[cp[i]:cp[i + 1]] for i in range(len(cp) - 1)]
    else:
        clusters = sg.greedy_clusters(rp, col, 150, 8, seed=1)
    upd = oracle.gen_updates(rp, col, 40000, 40000, 20000, seed=2)
    flags = dict(REF_FLAGS_SSSP, app_concurrency=str(threads))
    res, stats = {}, {}
    with tempfile.TemporaryDirectory() as d:
        write_graph_fast(d, rp, col, w)
        write_clusters(os.path.join(d, "g.e.c_150"), clusters)
        up = os.path.join(d, "sssp.update")
        write_updates(up, upd, True)
        res["sssp_sum_peval"], log = run_ref(exe, d, "sssp", flags, threads=threads)
        stats["sssp_peval"] = parse_stats(log)
        res["sssp_sum_inc"], log = run_ref(exe, d, "sssp", flags, up, threads=threads)
        stats["sssp_inc"] = parse_stats(log)
        res["sssp_plain_inc"], log = run_ref(exe, d, "sssp_plain", dict(flags, compress="0"), up,
                                             threads=threads)
        stats["sssp_plain"] = parse_stats(log)
    cp, mem = pack_clusters(clusters)
    params = {"graph": "oracle.rmat(20, 1 << 24, seed=1, weight_kind=1, wlo=1, whi=100)",
              "clusters": "greedy(150, 8, seed=1)",
              "updates": "oracle.gen_updates(rp, col, 40000, 40000, 20000, seed=2)",
              "source": 0, "flags_sssp": flags}
    np.savez_compressed(os.path.join(HERE, "rmat20_sssp.npz"), params=json.dumps(params),
                        input_sha256=input_hash(rp, col, w), updates_sha256=update_hash(upd),
                        clusters_ptr=cp, clusters_members=mem, stats=json.dumps(stats),
                        **{f"ref_{k}": as_u32_dist(v) for k, v in res.items()})
    print("rmat20_sssp", {k: int(np.isfinite(v).sum()) for k, v in res.items()},
          "clusters", len(clusters))


def make_rmat12_tight(exe):
    """rmat12 with termcheck_threshold 1e-10: the reference's summarized PEval
    and IncEval and its plain IncEval, to show L1 <= 1e-6 against the
    reference where the stop rule allows it."""
    z = np.load(os.path.join(HERE, "rmat12.npz"))
    rp, col, w = z["row_ptr"], z["col"], z["w"]
    cp, mem = z["clusters_ptr"], z["clusters_members"]
    clusters = [mem[cp[i]:cp[i + 1]] for i in range(len(cp) - 1)]
    flags = dict(REF_FLAGS_PR, termcheck_threshold="1e-10")
    res = {}
    with tempfile.TemporaryDirectory() as d:
        write_graph(d, rp, col, w)
        write_clusters(os.path.join(d, "g.e.c_150"), clusters)
        up = os.path.join(d, "pr.update")
        write_updates(up, z["updates_pr"], False)
        res["pr_sum_peval"], _ = run_ref(exe, d, "pagerank", flags)
        res["pr_sum_inc"], _ = run_ref(exe, d, "pagerank", flags, up)
        res["pr_plain_inc"], _ = run_ref(exe, d, "pagerank_plain", dict(flags, compress="0"), up)
    np.savez_compressed(os.path.join(HERE, "rmat12_tight.npz"), params=json.dumps({"flags_pr": flags}),
                        input_sha256=str(z["input_sha256"]),
                        **{f"ref_{k}": v.astype(np.float32) for k, v in res.items()})
    print("rmat12_tight", {k: float(v.sum()) for k, v in res.items()})


def main():
    sys.path.insert(0, os.path.join(ROOT, "oracle", "ref_harness"))
    import build_ref
    if "--reference" in sys.argv:
        build_ref.set_reference(sys.argv[sys.argv.index("--reference") + 1])
    exe = build_ref.build()
    if exe is None:
        raise SystemExit("reference checkout or harness build unavailable")
    if "--pull" in sys.argv[1:]:
        make_pull(exe)
        return
    threads = os.cpu_count() or 4
    if "--rmat16" in sys.argv[1:]:
        make_rmat16_pr(exe, threads)
        return
    if "--rmat20" in sys.argv[1:]:
        cl = sys.argv[sys.argv.index("--rmat20") + 1] if len(sys.argv) > sys.argv.index("--rmat20") + 1 else None
        make_rmat20_sssp(exe, threads, cl if cl and cl.endswith(".npz") else None)
        return
    if "--tight" in sys.argv[1:]:
        make_rmat12_tight(exe)
        return
    rp, col, w = sg.rmat_host(12, 16 << 12, seed=1, weight_kind=1, wlo=1, whi=100)
    make_case("rmat12", rp, col, w, exe, seed=1)
    rp, col, w = planted_graph()
    # the planted communities are the cluster file (the role of the external
    # community-detection output the reference reads)
    planted = [np.arange(c * 40, (c + 1) * 40, dtype=np.uint32) for c in range(60)]
    make_case("planted2600", rp, col, w, exe, seed=3, clusters=planted)


if __name__ == "__main__":
    main()
