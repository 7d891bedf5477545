#!/usr/bin/env python
"""Headline benchmark: incremental PageRank re-evaluation on one GB300.

Workload (the reference's "plain incremental PageRank at scale" case):
R-MAT scale 24 (16,777,216 vertices, 268,435,456 distinct directed edges,
a/b/c/d = 0.57/0.19/0.19/0.05, self loops and duplicates removed, seeded),
damping 0.85, FP32 values, L1 residual < 1e-6 (FP64 reduction).  After the
batch evaluation (PEval, untimed), every step applies one update batch of
0.1 % of the edges (50 % inserts of absent uniform pairs, 50 % deletes of
uniformly chosen edges) and runs IncEval to convergence.

Metric: GTEPS = edge relaxations performed during IncEval / IncEval time.
  value  batches already resident in HBM (sg_apply_updates_device +
         sg_pr_inceval without output copy), CUDA events on the library stream
  e2e    the C-ABI call a user makes: batch in pinned host memory
         (sg_apply_updates), result copied back to pinned host memory
         (sg_pr_inceval with an output buffer), both inside the timed region
The graph (>1 GB per direction) is larger than the 126 MB L2, so no flush is
needed between steps.

The line also carries `summarized`: the same graph and first batches with
compress = 1 (summary from the greedy builder's clusters of the low-degree
subgraph, shortcut weights on the GPU, the batch apply that repairs the
summary timed with each IncEval) and the summary's counters.

--impl reference times the CPU restatement of the reference worker
(oracle/, no library code: the same graph and batches, complete IncEvals
from a converged PEval, OpenMP over every host core) within a time budget.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L2_BYTES = 126 * 1024 * 1024
BYTES_PER_RELAXED_EDGE = 12   # 4 B neighbour + 4 B delta read + 4 B delta write
BYTES_PER_VERTEX_VISIT = 24   # 8 B row offset + 4 B delta read/reset + 8 B value RMW
# DRAM bytes (read + write) per k_pr_pull_warp launch on the default
# workload (R-MAT scale 24), from one single-pass ncu capture of
# dram__bytes_read.sum + dram__bytes_write.sum
PULL_DRAM_BYTES_RMAT24 = 2.06e9


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--scale", type=int, default=24)
    p.add_argument("--edge-factor", type=int, default=16)
    p.add_argument("--batch-frac", type=float, default=0.001)
    p.add_argument("--seed", type=int, default=1)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-community", action="store_true",
                   help="skip the summarized planted-community sub-record")
    p.add_argument("--community-batches", type=int, default=5)
    p.add_argument("--summary-batches", type=int, default=2,
                   help="headline workload: batches of the summarized sub-record (0: none)")
    p.add_argument("--ref-budget-s", type=float, default=150.0,
                   help="--impl reference: stop timing complete IncEvals once this many "
                        "seconds are spent (at least two steps)")
    p.add_argument("--no-clocks", action="store_true")
    p.add_argument("--pull-hubs", type=int, default=0,
                   help="hub cache of the PageRank pull: 0 automatic, -1 none, k at most k (16384 cap)")
    p.add_argument("--workload", default="inceval",
                   choices=["inceval", "batched", "adjoint", "sssp", "summarized"],
                   help="inceval: the headline IncEval line; batched: 256 PPR + 64 SSSP "
                        "queries in one persistent launch vs looping the single-query path; "
                        "adjoint: weighted PageRank forward vs forward + adjoint; sssp: "
                        "incremental SSSP at R-MAT scale 20; summarized: PageRank and SSSP "
                        "over the summarized graph of a community graph vs the plain graph")
    p.add_argument("--batch-scale", type=int, default=22)
    p.add_argument("--ppr-queries", type=int, default=256)
    p.add_argument("--sssp-sources", type=int, default=64)
    return p.parse_args()


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Barrier and max-over-ranks for replicas (gloo on CPU tensors)."""

    def __init__(self):
        self.ws, self.rank, self.local = dist_info()
        self.pg = None
        if self.ws > 1:
            import torch.distributed as td
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.ws > 1:
            self.td.barrier()

    def max(self, v: float) -> float:
        if self.ws == 1:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v: float) -> float:
        if self.ws == 1:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.SUM)
        return float(t.item())


class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int, enabled: bool):
        self.proc = None
        self.path = None
        if not enabled:
            return
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict | None:
        if self.proc is None:
            return None
        time.sleep(0.3)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append(parts)
            except ValueError:
                pass
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def make_batches(hg, count, size, seed0):
    half = size // 2
    return [hg.gen_updates(half, size - half, 0, seed=seed0 + i, integer_weights=True)
            for i in range(count)]


def cpu_inceval(cur, upd, x, delta, tau=1e-6):
    """One complete IncEval of the reference's worker on the host cores: the
    batch applied to the graph (the fragment rebuild of reloadGraph),
    AmendValue(-1) over the old graph and AmendValue(+1) over the new one,
    then delta rounds until sum|delta| < tau.  Returns (new graph, x, delta,
    relaxations, seconds, rounds)."""
    import oracle
    t0 = time.perf_counter()
    new = oracle.apply_updates(cur[0], cur[1], None, upd)[:2]
    d2 = oracle.pr_amend(cur, new, x, delta)
    x2, d3, st = oracle.ingress_pr(new[0], new[1], tau=tau, x=x, delta=d2)
    dt = time.perf_counter() - t0
    relax = int(cur[0][-1]) + int(new[0][-1]) + int(st["edges"])
    return new, x2, d3, relax, dt, int(st["rounds"])


def run_reference(args, D: Dist):
    """The reference's worker restated on the CPU (oracle/), all host cores,
    on the headline workload: the same graph and the same batches as the GPU
    arm's device-resident steps.  Each step is one complete IncEval from a
    converged state.  The library under test is not loaded."""
    if D.rank != 0:
        return
    import oracle
    n = 1 << args.scale
    E = n * args.edge_factor
    bsz = int(round(E * args.batch_frac))
    half = bsz // 2
    t0 = time.perf_counter()
    rp, col, _ = oracle.rmat(args.scale, E, seed=args.seed)
    gen_s = time.perf_counter() - t0
    # PEval to convergence (untimed)
    t0 = time.perf_counter()
    x, delta, pst = oracle.ingress_pr(rp, col, tau=1e-6)
    peval_s = time.perf_counter() - t0
    W, K = args.warmup, args.steps
    # the GPU arm draws batch i (seed 100 + i) from the graph after batches
    # < i; warm-up batches are applied here with one IncEval over all of them
    # (untimed), so the timed steps start from the same graph, converged
    cur = (rp, col)
    if W > 0:
        g0 = cur
        for i in range(W):
            upd = oracle.gen_updates(cur[0], cur[1], half, bsz - half, 0, seed=100 + i)
            cur = oracle.apply_updates(cur[0], cur[1], None, upd)[:2]
        delta = oracle.pr_amend(g0, cur, x, delta)
        x, delta, _ = oracle.ingress_pr(cur[0], cur[1], tau=1e-6, x=x, delta=delta)
    relax_t, time_t, steps_ms, rounds = 0, 0.0, [], []
    for i in range(W, W + K):
        upd = oracle.gen_updates(cur[0], cur[1], half, bsz - half, 0, seed=100 + i)
        cur, x, delta, relax, dt, r = cpu_inceval(cur, upd, x, delta)
        relax_t += relax
        time_t += dt
        steps_ms.append(round(dt * 1e3, 1))
        rounds.append(r)
        # bounded sample: stop once the budget is spent (at least two steps)
        if len(steps_ms) >= 2 and time_t > args.ref_budget_s:
            break
    k = len(steps_ms)
    gteps = relax_t / time_t / 1e9
    res = oracle.pr_residual_l1(cur[0], cur[1], x)
    cores = os.cpu_count() or 1
    sample = (f"complete IncEvals (batch apply + AmendValue(-1/+1) + delta rounds to "
              f"sum|delta| < 1e-6) of batches {W}..{W + k - 1}, the GPU arm's device-resident "
              f"steps, from a converged PEval; {k} of the {K} steps within a "
              f"{args.ref_budget_s:.0f} s budget")
    line = {
        "metric": "GTEPS for PR incremental re-eval (IncEval)",
        "value": round(gteps, 4), "unit": "GTEPS", "n_gpus": args.gpus,
        "steps": K, "warmup": W, "steps_timed": k,
        "ms_per_step": round(time_t / k * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic R-MAT (seeded), random update batches", "impl": "reference",
        "config": workload_config(args, n, E, bsz),
        "cpu_baseline": {"value": round(gteps, 4), "unit": "GTEPS", "cores": cores,
                         "kind": "port", "sample": sample},
        "e2e": {"value": round(gteps, 4), "unit": "GTEPS", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "step_ms": steps_ms, "rounds_per_step": rounds,
        "graph_gteps": round(E * k / time_t / 1e9, 4),
        "setup_s": {"rmat": round(gen_s, 1), "peval": round(peval_s, 1),
                    "peval_rounds": int(pst["rounds"])},
        "accuracy": {"residual_l1": res, "l1_bound_vs_fixed_point": res / 0.15,
                     "method": "||x - x*||_1 <= ||(1-d)/N + d P^T x - x||_1 / (1 - d), FP64"},
    }
    print(json.dumps(line), flush=True)


def workload_config(args, n, E, bsz):
    return {"workload": f"incremental PageRank, R-MAT scale {args.scale}",
            "vertices": n, "edges": E, "edge_factor": args.edge_factor,
            "rmat_abcd": [0.57, 0.19, 0.19, 0.05], "damping": 0.85,
            "termcheck_threshold": 1e-6, "batch_changes": bsz,
            "batch_mix": "50% insert / 50% delete", "seed": args.seed,
            "l2": "inputs larger than L2 (graph > 1 GB per direction), no flush",
            "parallelism": f"replicas x{args.gpus}" if args.gpus > 1 else "single GPU"}


def run_ours(args, D: Dist):
    import torch
    import suminc_gb300 as sg

    dev = D.local
    n = 1 << args.scale
    E = n * args.edge_factor
    bsz = int(round(E * args.batch_frac))
    ctx = sg.Context(dev, pull_hubs=args.pull_hubs)
    ctx.generate_rmat(args.scale, E, seed=args.seed)
    ctx.pr_peval(out=False)
    peval_stats = ctx.stats()
    rp0, col0, _ = ctx.download_csr(weights=False)
    hg = sg.HostGraph(rp0, col0)
    clusters, cl_s = (low_degree_clusters(rp0, col0, n) if args.summary_batches > 0 and D.rank == 0
                      else (None, 0.0))
    del rp0, col0
    K, W = args.steps, args.warmup
    batches = make_batches(hg, W + 2 * K, bsz, 100)
    # device-resident copies for `value`, pinned host copies for `e2e`
    dev_b = [torch.from_numpy(b.view(np.uint8)).to(f"cuda:{dev}") for b in batches[: W + K]]
    pin_b = [torch.from_numpy(b.view(np.uint8)).pin_memory() for b in batches[W + K: W + 2 * K]]
    out_pin = torch.empty(n, dtype=torch.float32).pin_memory()
    torch.cuda.synchronize(dev)

    clocks = Clocks(dev, not args.no_clocks)
    # warm-up
    for i in range(W):
        ctx.apply_updates_ptr(bsz, dev_b[i].data_ptr(), True)
        ctx.pr_inceval_into(None)
    # timed: device-resident batches, with CUDA events around every kernel
    # of the PageRank classes on the library stream (the per-launch
    # duration of the dominant kernel for the roofline)
    ctx.set_profile(0xFF)
    ctx.reset_stats()
    D.barrier()
    ctx.synchronize()
    ctx.record_event(0)
    relax = 0
    pe_pull = 0
    rounds = []
    visits = []
    step_ms, inc_ms = [], []
    for i in range(W, W + K):
        # events 4/5 bracket the step on the library stream; IncEval has
        # synchronised when it returns, so reading them adds no wait
        ctx.record_event(4)
        ctx.apply_updates_ptr(bsz, dev_b[i].data_ptr(), True)
        ctx.pr_inceval_into(None)
        ctx.record_event(5)
        st = ctx.stats()
        relax += st["edges_relaxed"]
        pe_pull += st["edges_pull"]
        rounds.append(st["rounds"])
        visits.append(int(st["vertex_visits"]))
        inc_ms.append(st["elapsed_ms"])
        step_ms.append(ctx.elapsed_ms(4, 5))
    repacks_value = ctx.stats()["repacks"]
    ctx.record_event(1)
    ctx.synchronize()
    D.barrier()
    t_ms = ctx.elapsed_ms(0, 1)
    st = ctx.stats()
    launches = st["launches_total"]
    kms, kl = st["kernel_ms"], st["kernel_launches"]
    ctx.set_profile(0)
    t_ms_max = D.max(t_ms)
    relax_all = D.sum(relax)
    value = relax_all / (t_ms_max * 1e-3) / 1e9

    # timed: end to end through the C ABI with pinned host buffers
    D.barrier()
    ctx.synchronize()
    ctx.record_event(2)
    relax_e = 0
    step_e_ms = []
    rep0 = ctx.stats()["repacks"]
    for i in range(K):
        ctx.record_event(4)
        ctx.apply_updates_ptr(bsz, pin_b[i].data_ptr(), False)
        ctx.pr_inceval_into(out_pin.data_ptr())
        ctx.record_event(5)
        relax_e += ctx.stats()["edges_relaxed"]
        step_e_ms.append(ctx.elapsed_ms(4, 5))
    repacks_e2e = ctx.stats()["repacks"] - rep0
    ctx.record_event(3)
    ctx.synchronize()
    D.barrier()
    te_ms = D.max(ctx.elapsed_ms(2, 3))
    e2e = D.sum(relax_e) / (te_ms * 1e-3) / 1e9
    clk = clocks.stop()

    total_k = sum(kms.values()) or 1.0
    kernels = {k: {"launches": kl[k], "ms": round(kms[k], 4), "share": round(kms[k] / total_k, 4)}
               for k in kms if kl[k]}
    dom = max(kernels, key=lambda k: kernels[k]["ms"])
    avg_ms = kms[dom] / kl[dom]
    if dom == "pr_pull":
        bytes_per_launch = BYTES_PER_RELAXED_EDGE * pe_pull / kl[dom]
    else:
        bytes_per_launch = BYTES_PER_VERTEX_VISIT * n
    peak, peak_kind = measured_peaks()
    achieved = bytes_per_launch / (avg_ms * 1e-3) / 1e9
    traffic = (PULL_DRAM_BYTES_RMAT24 if (dom == "pr_pull" and args.scale == 24
                                          and args.edge_factor == 16) else None)
    roofline = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1),
                "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                "traffic": traffic,
                "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum, one "
                                   "capture of this workload" if traffic else None),
                "avg_launch_ms": round(avg_ms, 4),
                "algorithmic_bytes_per_launch": int(bytes_per_launch),
                "kernels": kernels}

    # accuracy of the final state (after every timed batch):
    # the FP64 residual of x on the final graph bounds ||x - x*||_1
    import oracle
    x = ctx.pr_values()
    delta = ctx.pr_deltas()
    fin = hg.csr()[:2]
    res = oracle.pr_residual_l1(fin[0], fin[1], x)
    accuracy = {"residual_l1": res, "l1_bound_vs_fixed_point": res / 0.15,
                "tolerance": 1e-5, "within_tolerance": bool(res / 0.15 <= 1e-5),
                "method": "||x - x*||_1 <= ||(1-d)/N + d P^T x - x||_1 / (1 - d), FP64 "
                          "residual on the host over the final graph"}
    cpu = None
    if not args.no_cpu_baseline and D.rank == 0:
        # one complete IncEval of the reference's worker restated on the host
        # cores, from the GPU's converged state, on the next batch
        upd = oracle.gen_updates(fin[0], fin[1], bsz // 2, bsz - bsz // 2, 0, seed=99999)
        _, _, _, relax_c, dt, rc = cpu_inceval(fin, upd, x, delta)
        cpu = {"value": round(relax_c / dt / 1e9, 4), "unit": "GTEPS",
               "cores": os.cpu_count() or 1, "kind": "port",
               "sample": (f"one complete IncEval on the host (batch apply + AmendValue(-1/+1) "
                          f"over the scale-{args.scale} graph + {rc} delta rounds to "
                          f"sum|delta| < 1e-6) after a {bsz}-change batch, from the GPU's "
                          f"converged state ({dt:.1f} s)"),
               "ms_per_step": round(dt * 1e3, 1)}
    ctx.close()
    summarized = None
    if clusters is not None:
        summarized = summarized_subrecord(args, D, batches, clusters, cl_s)
    community = None
    if not args.no_community and D.rank == 0:
        community = community_subrecord(args, D)

    result = {
        "metric": "GTEPS for PR incremental re-eval (IncEval)",
        "value": round(value, 4), "unit": "GTEPS", "n_gpus": D.ws,
        "steps": K, "warmup": W, "ms_per_step": round(t_ms_max / K, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic R-MAT (seeded), random update batches",
        "config": workload_config(args, n, E, bsz),
        "e2e": {"value": round(e2e, 4), "unit": "GTEPS",
                "h2d_bytes_per_step": int(bsz * 16), "d2h_bytes_per_step": int(n * 4),
                "ms_per_step": round(te_ms / K, 4)},
        "gpu_launches": int(launches),
        "rounds_per_step": rounds,
        "activations_per_step": visits,
        "relaxations_per_step": int(relax / K),
        "step_ms": {"value": [round(v, 3) for v in step_ms],
                    "e2e": [round(v, 3) for v in step_e_ms],
                    "inceval_only": [round(v, 3) for v in inc_ms],
                    "value_median": round(statistics.median(step_ms), 3),
                    "value_max": round(max(step_ms), 3),
                    "e2e_median": round(statistics.median(step_e_ms), 3),
                    "batches": {"value": [W, W + K - 1], "e2e": [W + K, W + 2 * K - 1]},
                    "repacks": {"value": int(repacks_value), "e2e": int(repacks_e2e)}},
        "accuracy": accuracy,
        "graph_gteps": round(E * K / (t_ms_max * 1e-3) / 1e9, 4),
        "peval": {"rounds": peval_stats["rounds"], "ms": round(peval_stats["elapsed_ms"], 3)},
        "roofline": roofline,
    }
    if cpu:
        result["cpu_baseline"] = cpu
    if clk:
        result["clocks"] = clk
    if summarized:
        result["summarized"] = summarized
    if community:
        result["summarized_community"] = community
    return result, hg, batches, None


LOW_DEGREE_CAP = 32  # in + out degree of the vertices the clusters are drawn from


def low_degree_clusters(rp, col, n):
    """Clusters for the summary at R-MAT scale 24: the repository's greedy
    builder (max 150, min 8 members, seed 1) run on the subgraph induced by
    the vertices of in + out degree <= 32.  On the whole graph the builder's
    steps scan the rows of every hub it tries, which takes hours at this
    scale; without the hubs it takes seconds.  Hubs cannot be inner members
    of a profitable supernode anyway (their outside edges make them entries
    and exits).  Returns (clusters, seconds)."""
    import suminc_gb300 as sg
    t0 = time.perf_counter()
    outd = np.diff(rp).astype(np.int64)
    ind = np.bincount(col, minlength=n)
    low = (outd + ind) <= LOW_DEGREE_CAP
    src = np.repeat(np.arange(n, dtype=np.uint32), outd)
    keep = low[src] & low[col]
    srck, colk = src[keep], col[keep]
    del src, keep
    rps = np.zeros(n + 1, np.uint64)
    np.add.at(rps, srck.astype(np.int64) + 1, 1)
    rps = np.cumsum(rps).astype(np.uint64)
    cl = sg.greedy_clusters(rps, colk.astype(np.uint32), 150, 8, seed=1)
    return cl, time.perf_counter() - t0


def summarized_subrecord(args, D, batches, clusters, cl_s):
    """The same workload over the summarized graph (compress = 1): summary
    built from the clusters, shortcut weights on the GPU, then IncEval after
    the first batches of the headline sequence, each timed with the batch
    apply (which repairs the summary) on the host clock and the IncEval on
    the device."""
    import oracle
    import suminc_gb300 as sg
    n = 1 << args.scale
    E = n * args.edge_factor
    ctx = sg.Context(D.local, compress=1)
    ctx.generate_rmat(args.scale, E, seed=args.seed)
    t0 = time.perf_counter()
    ctx.set_profile(0xFF)
    ctx.reset_stats()
    ctx.summary_build(clusters)
    build_s = time.perf_counter() - t0
    sc_ms = ctx.stats()["kernel_ms"].get("summary", 0.0)
    info = ctx.summary_info()
    ctx.set_profile(0)
    ctx.pr_peval(out=False)
    pe = ctx.stats()
    steps = []
    for b in batches[: args.summary_batches]:
        ctx.synchronize()
        t1 = time.perf_counter()
        ctx.apply_updates(b)
        t2 = time.perf_counter()
        ctx.pr_inceval_into(None)
        t3 = time.perf_counter()
        st = ctx.stats()
        steps.append({"apply_and_repair_ms": round((t2 - t1) * 1e3, 1),
                      "inceval_ms": round(st["elapsed_ms"], 3),
                      "inceval_wall_ms": round((t3 - t2) * 1e3, 1),
                      "rounds": st["rounds"], "edges_relaxed": int(st["edges_relaxed"]),
                      "shortcut_edges": int(st["shortcut_edges"])})
    x = ctx.pr_values()
    rp, col, _ = ctx.download_csr(weights=False)
    ctx.close()
    res = oracle.pr_residual_l1(rp, col, x)
    members = int(sum(len(c) for c in clusters))
    return {
        "clusters": {"source": f"greedy builder (max 150, min 8, seed 1) on the subgraph "
                               f"induced by vertices of in + out degree <= {LOW_DEGREE_CAP}",
                     "count": len(clusters), "members": members, "seconds": round(cl_s, 1)},
        "summary": {k: info[k] for k in ("clusters", "supernodes", "cluster_members",
                                         "shortcut_edges", "boundary_edges", "all_rows")},
        "summary_build_s": round(build_s, 1),
        "shortcut_kernels_ms": round(sc_ms, 2),
        "peval_ms": round(pe["elapsed_ms"], 2), "peval_rounds": pe["rounds"],
        "steps": steps,
        "accuracy": {"l1_bound_vs_fixed_point": res / 0.15, "within_tolerance": bool(res / 0.15 <= 1e-5)},
    }


def community_subrecord(args, D):
    """The summarized path on a graph whose clusters are profitable
    supernodes: planted communities (batch scale 22: 131,072 communities of
    40, 5.24 M vertices, 39 M edges) with the communities as the cluster
    file.  PageRank IncEval after 0.1 % batches, each step the batch's apply
    (which repairs the summary on the device) on the host clock plus the
    IncEval on the device, against the plain path on the same batches
    (medians over the batches after the first); then the device-repaired
    tables against the host restatement."""
    import oracle
    import suminc_gb300 as sg
    n_comm = 1 << max(args.batch_scale - 5, 4)
    rp, col, _, comms = community_graph(n_comm, 40, args.seed)
    E = len(col)
    rec = {"graph": {"communities": n_comm, "size": 40, "vertices": len(rp) - 1, "edges": E,
                     "clusters": "the planted communities"}}
    # 0.1 % batches (the scale-24 headline's size), then 0.01 %: the repair
    # scales with the clusters a batch touches, the plain IncEval does not
    for frac, key in ((1e-3, "batch_0.1pct"), (1e-4, "batch_0.01pct")):
        rec[key] = community_batches(args, D, rp, col, comms, max(1000, int(E * frac)))
    return rec


def community_batches(args, D, rp, col, comms, bsz):
    import oracle
    import suminc_gb300 as sg
    hg = sg.HostGraph(rp, col)
    batches = [hg.gen_updates(bsz // 2, bsz - bsz // 2, 0, seed=700 + i)
               for i in range(args.community_batches)]
    nrp, ncol, _ = hg.csr()
    out = {}
    for mode in (1, 0):
        ctx = sg.Context(D.local, compress=mode)
        ctx.load_csr(rp, col)
        rec = {}
        if mode:
            t0 = time.perf_counter()
            ctx.summary_build(comms)
            rec["summary_build_s"] = round(time.perf_counter() - t0, 2)
            info = ctx.summary_info()
            rec["summary"] = {k: info[k] for k in ("clusters", "supernodes", "shortcut_edges",
                                                   "boundary_edges", "all_rows")}
        ctx.pr_peval(out=False)
        rec["peval_ms"] = round(ctx.stats()["elapsed_ms"], 3)
        apply_ms, inc_ms = [], []
        for b in batches:
            ctx.synchronize()
            t1 = time.perf_counter()
            ctx.apply_updates(b)
            ctx.synchronize()
            apply_ms.append(round((time.perf_counter() - t1) * 1e3, 3))
            ctx.pr_inceval_into(None)
            inc_ms.append(round(ctx.stats()["elapsed_ms"], 3))
        x = ctx.pr_values()
        if mode:
            rec["repair_vs_host_restatement"] = ctx.summary_check()
        ctx.close()
        rec["apply_ms"] = apply_ms
        rec["inceval_ms"] = inc_ms
        rec["step_ms"] = [round(a + i, 3) for a, i in zip(apply_ms, inc_ms)]
        rec["l1_bound_vs_fixed_point"] = float(oracle.pr_residual_l1(nrp, ncol, x) / 0.15)
        out["summarized" if mode else "plain"] = rec
    # the first batch of each mode warms up (first-use allocations of the
    # applier and the repair): the medians are over the batches after it
    first = 1 if len(batches) > 1 else 0
    s_step = statistics.median(out["summarized"]["step_ms"][first:])
    p_step = statistics.median(out["plain"]["step_ms"][first:])
    return {
        "batch_changes": bsz,
        "summarized": out["summarized"], "plain": out["plain"],
        "step_ms_median": {"summarized": round(s_step, 3), "plain": round(p_step, 3),
                           "summarized_over_plain": round(s_step / p_step, 3),
                           "over_steps": f"{first + 1}-{len(batches)}"},
    }


def batch_queries(n, nq, ns, seed):
    """256 PPR queries teleporting to 1..64 seeds (count log-uniform), 64
    uniform SSSP sources."""
    rng = np.random.default_rng(seed)
    seeds = []
    for _ in range(nq):
        k = max(1, int(np.floor(np.exp(rng.uniform(0.0, np.log(64.0))))))
        seeds.append(np.sort(rng.choice(n, size=k, replace=False)).astype(np.uint32))
    sources = rng.choice(n, size=ns, replace=False).astype(np.uint32)
    return seeds, sources


def run_batched(args, D: Dist):
    """Batched queries vs looping the single-query GPU path on the same GPU."""
    import torch
    import suminc_gb300 as sg

    dev = D.local
    n = 1 << args.batch_scale
    E = n * args.edge_factor
    ctx = sg.Context(dev)
    ctx.generate_rmat(args.batch_scale, E, seed=args.seed, weight_kind=1, wlo=1, whi=100)
    seeds, sources = batch_queries(n, args.ppr_queries, args.sssp_sources, args.seed + 7)
    K, W = args.steps, args.warmup
    # the first run tunes the schedule and captures the launch sequence
    t0 = time.perf_counter()
    ctx.batch_run(seeds, sources, out=False)
    first_s = time.perf_counter() - t0
    info0 = ctx.batch_info()
    for _ in range(max(0, W - 1)):
        ctx.batch_run(seeds, sources, out=False)
    clocks = Clocks(dev, not args.no_clocks)
    D.barrier()
    ctx.synchronize()
    ctx.record_event(0)
    work = 0
    for _ in range(K):
        ctx.batch_run(seeds, sources, out=False)
        bi = ctx.batch_info()
        work += bi["ppr_edge_visits"] + bi["sssp_relaxations"]
    ctx.record_event(1)
    ctx.synchronize()
    D.barrier()
    t_ms = D.max(ctx.elapsed_ms(0, 1))
    value = D.sum(work) / (t_ms * 1e-3) / 1e9
    info = ctx.batch_info()
    # end to end: query arrays from the host, results copied back to host
    ppr_host = torch.empty((len(seeds), n), dtype=torch.float32).pin_memory()
    sssp_host = torch.empty((len(sources), n), dtype=torch.float64).pin_memory()
    spec_ptr = np.zeros(len(seeds) + 1, np.uint32)
    for i, sd in enumerate(seeds):
        spec_ptr[i + 1] = spec_ptr[i] + len(sd)
    all_seeds = np.concatenate(seeds)
    spec = sg.BatchSpec(len(seeds), spec_ptr.ctypes.data, all_seeds.ctypes.data, len(sources),
                        sources.ctypes.data)
    import ctypes as C
    ctx.synchronize()
    ctx.record_event(2)
    for _ in range(K):
        sg._check(ctx._lib.sg_batch_run(ctx._h, C.byref(spec), C.c_void_p(ppr_host.data_ptr()),
                                        C.c_void_p(sssp_host.data_ptr())), ctx, "sg_batch_run")
    ctx.record_event(3)
    ctx.synchronize()
    te_ms = D.max(ctx.elapsed_ms(2, 3))
    clk = clocks.stop()
    P = ppr_host.numpy()
    S = sssp_host.numpy()

    # the loop baseline: one sg_ppr / sg_sssp_peval per query, same GPU
    ctx.synchronize()
    ctx.record_event(4)
    loop_ppr = [ctx.ppr(sd) for sd in seeds]
    ctx.record_event(5)
    loop_sssp = [ctx.sssp_peval(int(s)) for s in sources]
    ctx.record_event(6)
    ctx.synchronize()
    loop_ppr_ms = ctx.elapsed_ms(4, 5)
    loop_sssp_ms = ctx.elapsed_ms(5, 6)
    l1 = [float(np.abs(P[q] - loop_ppr[q]).sum()) for q in range(len(seeds))]
    sssp_equal = all(np.array_equal(S[s], loop_sssp[s]) for s in range(len(sources)))
    ctx.close()

    # algorithmic bytes of the launch: per pull 4 B of neighbour id per edge
    # (read once for the whole batch) + 4 B of push value per edge and query
    # pulled + 20 B per vertex and query (delta and value read/write, next
    # push value); SSSP 16 B per (edge, source) relaxed + 8 B per improvement
    pulls = info["ppr_pulls"]
    qe = info["ppr_edge_visits"]
    ppr_bytes = 4 * E * pulls + 4 * qe + 20 * n * (qe / max(E, 1))
    sssp_bytes = 16 * info["sssp_relaxations"] + 8 * info["sssp_improvements"]
    peak, peak_kind = measured_peaks()
    achieved = (ppr_bytes + sssp_bytes) / (info["elapsed_ms"] * 1e-3) / 1e9
    result = {
        "metric": "GTEPS for batched PPR + SSSP queries (one persistent launch)",
        "value": round(value, 4), "unit": "GTEPS", "n_gpus": D.ws, "steps": K, "warmup": W,
        "ms_per_step": round(t_ms / K, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (PPR), f64 (SSSP)",
        "data": "synthetic R-MAT (seeded), seeded query sets",
        "config": {"workload": f"batched queries, R-MAT scale {args.batch_scale}",
                   "vertices": n, "edges": E, "weights": "uniform integers [1, 100]",
                   "ppr_queries": len(seeds), "ppr_seeds_per_query": "floor(exp(U[0, ln 64]))",
                   "sssp_sources": len(sources), "termcheck_threshold": 1e-6,
                   "l2": "state (>4 GB) larger than L2, no flush",
                   "parallelism": "single GPU"},
        "speedup_vs_loop": round((loop_ppr_ms + loop_sssp_ms) / (te_ms / K), 3),
        "speedup_vs_loop_device_resident": round((loop_ppr_ms + loop_sssp_ms) / (t_ms / K), 3),
        "loop": {"ppr_ms": round(loop_ppr_ms, 2), "sssp_ms": round(loop_sssp_ms, 2),
                 "path": "sg_ppr / sg_sssp_peval once per query, same GPU, results to host; "
                         "speedup_vs_loop compares it with the end-to-end batch"},
        "accuracy": {"ppr_l1_vs_loop_max": max(l1), "sssp_bit_equal_to_loop": sssp_equal},
        "schedule": {"chunk_quads": info["chunk_quads"], "blocks_per_sm": info["blocks_per_sm"],
                     "sssp_bucket": info["sssp_bucket"], "graph_launch": info["graph_launch"],
                     "tune_ms": round(info0["tune_ms"], 1), "first_call_s": round(first_s, 2)},
        "iterations": {"ppr_pulls": pulls, "sssp_steps": info["sssp_steps"],
                       "sssp_scans": info["sssp_scans"], "total": info["iterations"]},
        "e2e": {"value": round(D.sum(work) / (te_ms * 1e-3) / 1e9, 4), "unit": "GTEPS",
                "h2d_bytes_per_step": int(4 * (len(spec_ptr) + len(all_seeds) + len(sources))),
                "d2h_bytes_per_step": int(P.nbytes + S.nbytes),
                "ms_per_step": round(te_ms / K, 3)},
        "gpu_launches": int(6 * K),
        "roofline": {"bound": "hbm", "kernel": "k_batch", "achieved": round(achieved, 1),
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                     "traffic": None,
                     "algorithmic_bytes_per_launch": int(ppr_bytes + sssp_bytes),
                     "launch_ms": round(info["elapsed_ms"], 3)},
    }
    if clk:
        result["clocks"] = clk
    return result


def run_adjoint(args, D: Dist):
    """Weighted PageRank forward alone vs forward + adjoint (gradients wrt
    every edge weight and the teleport vector), R-MAT scale 22 with
    column-normalised float weights, loss over 10,000 targets."""
    import torch
    import oracle
    import suminc_gb300 as sg

    dev = D.local
    n = 1 << args.batch_scale
    E = n * args.edge_factor
    ctx = sg.Context(dev)
    ctx.generate_rmat(args.batch_scale, E, seed=args.seed, weight_kind=2, wlo=0.1, whi=1.0)
    ctx.normalize_weights()
    rng = np.random.default_rng(args.seed + 11)
    tgt = rng.choice(n, size=10000, replace=False)
    y = rng.uniform(0.0, 2.0 / n, size=10000).astype(np.float32)
    tele = np.full(n, 1.0 / n, np.float32)
    x_pin = torch.empty(n, dtype=torch.float32).pin_memory()
    g_pin = torch.empty(n, dtype=torch.float32).pin_memory()
    dw_pin = torch.empty(E, dtype=torch.float32).pin_memory()
    dt_pin = torch.empty(n, dtype=torch.float32).pin_memory()
    import ctypes as C
    lib, h = ctx._lib, ctx._h

    def fwd():
        sg._check(lib.sg_pr_weighted(h, tele.ctypes.data_as(C.c_void_p),
                                     C.c_void_p(x_pin.data_ptr())), ctx, "sg_pr_weighted")

    def bwd():
        x = x_pin.numpy()
        g = g_pin.numpy()
        g[:] = 0.0
        g[tgt] = x[tgt] - y
        sg._check(lib.sg_pr_adjoint(h, C.c_void_p(g_pin.data_ptr()), C.c_void_p(dw_pin.data_ptr()),
                                    C.c_void_p(dt_pin.data_ptr())), ctx, "sg_pr_adjoint")

    K, W = args.steps, args.warmup
    for _ in range(W):
        fwd()
        bwd()
    clocks = Clocks(dev, not args.no_clocks)
    ctx.synchronize()
    ctx.record_event(0)
    f_edges = 0
    f_dev_ms = 0.0
    for _ in range(K):
        fwd()
        ai = ctx.adjoint_info()
        f_edges += ai["forward_edges"]
        f_dev_ms += ai["forward_ms"]
    ctx.record_event(1)
    ctx.synchronize()
    t_f = ctx.elapsed_ms(0, 1)
    ctx.record_event(2)
    fb_edges = 0
    a_dev_ms = 0.0
    for _ in range(K):
        fwd()
        bwd()
        ai = ctx.adjoint_info()
        fb_edges += ai["forward_edges"] + ai["adjoint_edges"] + ai["gradient_edges"]
        a_dev_ms += ai["adjoint_ms"]
    ctx.record_event(3)
    ctx.synchronize()
    t_fb = ctx.elapsed_ms(2, 3)
    clk = clocks.stop()
    info = ctx.adjoint_info()
    # the plain-loop alternative: central differences over teleport entries,
    # two forward solves per parameter on the same GPU (FP32), against the
    # adjoint's dL/dtele from the last backward
    dt_adj = dt_pin.numpy().copy()
    fd_params = [int(v) for v in tgt[:8]]
    fd_h = 1.0 / n  # x is linear in tele and L quadratic: no truncation error
    x_base = None
    ctx.synchronize()
    ctx.record_event(4)
    fd_vals = []
    for v in fd_params:
        l2 = []
        for sign in (1.0, -1.0):
            tp = tele.copy()
            tp[v] += sign * fd_h
            xs = ctx.pr_weighted(tp)
            l2.append(0.5 * float(np.sum((xs[tgt].astype(np.float64) - y) ** 2)))
        fd_vals.append((l2[0] - l2[1]) / (2 * fd_h))
    ctx.record_event(5)
    ctx.synchronize()
    fd_ms = ctx.elapsed_ms(4, 5)
    fd_rel = [abs(fd_vals[i] - float(dt_adj[v])) / max(abs(float(dt_adj[v])), 1e-30)
              for i, v in enumerate(fd_params)]
    # per-kernel device time of the adjoint's weighted pull (profiled run)
    ctx.set_profile(0xFF)
    ctx.reset_stats()
    fwd()
    bwd()
    st = ctx.stats()
    ctx.set_profile(0)
    kms, kl = st["kernel_ms"], st["kernel_launches"]
    ctx.close()

    # accuracy on a scale-12 induced subgraph: the first 4096 vertices, weights
    # re-normalised; GPU adjoint vs the FP64 transposed solve and central
    # differences on 64 random edges
    sub = 4096
    with sg.Context(dev) as c2:
        c2.generate_rmat(args.batch_scale, E, seed=args.seed, weight_kind=2, wlo=0.1, whi=1.0)
        rp, col, w = c2.download_csr()
    keep_rows = rp[: sub + 1]
    cols = col[: int(keep_rows[-1])]
    ws = w[: int(keep_rows[-1])].astype(np.float64)
    srcs = np.repeat(np.arange(sub), np.diff(keep_rows).astype(np.int64))
    mask = cols < sub
    srcs, cols, ws = srcs[mask], cols[mask], ws[mask]
    srp = np.zeros(sub + 1, np.uint64)
    np.add.at(srp, srcs + 1, 1)
    srp = np.cumsum(srp).astype(np.uint64)
    ssum = np.bincount(srcs, weights=ws, minlength=sub)
    ws = ws / ssum[srcs]
    stele = np.full(sub, 1.0 / sub)
    srng = np.random.default_rng(3)
    stgt = srng.choice(sub, size=1000, replace=False)
    sy = srng.uniform(0.0, 2.0 / sub, size=1000)
    with sg.Context(dev) as c3:
        c3.load_csr(srp, cols.astype(np.uint32), ws.astype(np.float32))
        xs = c3.pr_weighted(stele.astype(np.float32))
        gs = np.zeros(sub)
        gs[stgt] = xs[stgt] - sy
        dws, dts = c3.pr_adjoint(gs.astype(np.float32))
        _, lam32 = c3.adjoint_values()
    w32 = ws.astype(np.float32).astype(np.float64)
    lam64 = oracle.pr_adjoint_solve(srp, cols, w32, gs)
    x64 = oracle.pr_fixed_point(srp, cols, w32, tele=stele)
    dw64 = 0.85 * lam64[cols] * x64[srcs]
    rel_lam = float(np.abs(lam32 - lam64).sum() / np.abs(lam64).sum())
    rel_dw = float(np.abs(dws - dw64).sum() / np.abs(dw64).sum())
    hstep = 1e-4
    fd_err = []
    for e in srng.choice(len(cols), size=64, replace=False):
        wp = w32.copy(); wp[e] += hstep
        wm = w32.copy(); wm[e] -= hstep
        lp = 0.5 * np.sum((oracle.pr_fixed_point(srp, cols, wp, tele=stele, tol=1e-15)[stgt] - sy) ** 2)
        lm = 0.5 * np.sum((oracle.pr_fixed_point(srp, cols, wm, tele=stele, tol=1e-15)[stgt] - sy) ** 2)
        fd = (lp - lm) / (2 * hstep)
        fd_err.append(abs(float(dws[e]) - fd) / max(abs(fd), 1e-30))

    peak, peak_kind = measured_peaks()
    # adjoint class = weighted pulls along out-edges (4 B neighbour + 4 B
    # weight + 4 B push value per edge) + the gradient pass (4 B neighbour +
    # 4 B lambda + 4 B dL/dw per edge; x_u once per row)
    adj_pull_ms = kms.get("adjoint", 0.0)
    adj_launches = kl.get("adjoint", 0)
    adj_bytes = 12 * info["adjoint_edges"] + 12 * info["gradient_edges"]
    achieved = adj_bytes / (adj_pull_ms * 1e-3) / 1e9 if adj_pull_ms else None
    result = {
        "metric": "PageRank adjoint: forward + backward vs forward alone",
        "value": round(fb_edges / (t_fb * 1e-3) / 1e9, 4), "unit": "GTEPS",
        "n_gpus": D.ws, "steps": K, "warmup": W, "ms_per_step": round(t_fb / K, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic R-MAT (seeded), float weights U[0.1, 1.0] column-normalised",
        "config": {"workload": f"PageRank adjoint, R-MAT scale {args.batch_scale}",
                   "vertices": n, "edges": E, "damping": 0.85, "loss_targets": 10000,
                   "targets": "uniform, t_v ~ U[0, 2/N]", "termcheck_threshold": 1e-6,
                   "adjoint_rel_tol": 1e-7, "parallelism": "single GPU",
                   "l2": "graph larger than L2, no flush"},
        "forward_ms": round(t_f / K, 3), "forward_backward_ms": round(t_fb / K, 3),
        "backward_over_forward": round((t_fb - t_f) / t_f, 3),
        "vs_plain_loop": {
            "path": "central differences over teleport entries, 2 x sg_pr_weighted per "
                    "parameter on the same GPU (FP32), step 1/N",
            "params_timed": len(fd_params), "loop_ms": round(fd_ms, 2),
            "loop_ms_per_param": round(fd_ms / len(fd_params), 3),
            "adjoint_params": int(n + E),
            "speedup_for_all_params": round((fd_ms / len(fd_params)) * (n + E) / (t_fb / K), 1),
            "speedup_for_64_params": round((fd_ms / len(fd_params)) * 64 / (t_fb / K), 2),
            "fd_rel_err_vs_adjoint_max": max(fd_rel)},
        "device_ms": {"forward": round(f_dev_ms / K, 3), "adjoint_and_gradients": round(a_dev_ms / K, 3)},
        "rounds": {"forward": info["forward_rounds"], "adjoint": info["adjoint_rounds"]},
        "accuracy_scale12_subgraph": {"lambda_rel_l1_vs_fp64": rel_lam, "dw_rel_l1_vs_fp64": rel_dw,
                                      "fd_64_edges_max_rel_err": max(fd_err),
                                      "fd_64_edges_median_rel_err": float(np.median(fd_err))},
        "e2e": {"value": round(fb_edges / (t_fb * 1e-3) / 1e9, 4), "unit": "GTEPS",
                "h2d_bytes_per_step": int(8 * n), "d2h_bytes_per_step": int(4 * n + 4 * E + 4 * n),
                "ms_per_step": round(t_fb / K, 3)},
        "gpu_launches": int(st["launches_total"]),
        "roofline": {"bound": "hbm", "kernel": "k_pr_pull<weighted> (adjoint)",
                     "achieved": round(achieved, 1) if achieved else None, "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4) if achieved else None,
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)", "traffic": None,
                     "avg_launch_ms": round(adj_pull_ms / adj_launches, 4) if adj_launches else None,
                     "algorithmic_bytes": int(adj_bytes), "launches": int(adj_launches)},
    }
    if clk:
        result["clocks"] = clk
    return result


def run_sssp(args, D: Dist):
    """Incremental SSSP: R-MAT scale 20, integer weights U[1, 100], source 0,
    batches of 100,000 changes (40 % inserts, 40 % deletes, 20 % re-weights),
    IncEval per batch; distances bit-exact (checked against Dijkstra on the
    host for the last batch)."""
    import torch
    import oracle
    import suminc_gb300 as sg

    dev = D.local
    scale = 20
    n = 1 << scale
    E = n * args.edge_factor
    ctx = sg.Context(dev)
    ctx.generate_rmat(scale, E, seed=args.seed, weight_kind=1, wlo=1, whi=100)
    t0 = time.perf_counter()
    ctx.sssp_peval(0, out=False)
    pe = ctx.stats()
    rp, col, w = ctx.download_csr()
    hg = sg.HostGraph(rp, col, w)
    K, W = args.steps, args.warmup
    batches = [hg.gen_updates(40000, 40000, 10000, seed=500 + i) for i in range(W + 2 * K)]
    dev_b = [torch.from_numpy(b.view(np.uint8)).to(f"cuda:{dev}") for b in batches[: W + K]]
    pin_b = [torch.from_numpy(b.view(np.uint8)).pin_memory() for b in batches[W + K:]]
    out_pin = torch.empty(n, dtype=torch.float64).pin_memory()
    import ctypes as C
    for i in range(W):
        ctx.apply_updates_ptr(len(batches[i]), dev_b[i].data_ptr(), True)
        sg._check(ctx._lib.sg_sssp_inceval(ctx._h, None), ctx, "sg_sssp_inceval")
    clocks = Clocks(dev, not args.no_clocks)
    ctx.synchronize()
    ctx.record_event(0)
    relax = 0
    resets = []
    for i in range(W, W + K):
        ctx.apply_updates_ptr(len(batches[i]), dev_b[i].data_ptr(), True)
        sg._check(ctx._lib.sg_sssp_inceval(ctx._h, None), ctx, "sg_sssp_inceval")
        st = ctx.stats()
        relax += st["edges_relaxed"]
        resets.append(int(st["reset_vertices"]))
    ctx.record_event(1)
    ctx.synchronize()
    t_ms = D.max(ctx.elapsed_ms(0, 1))
    ctx.record_event(2)
    relax_e = 0
    for i in range(K):
        b = batches[W + K + i]
        ctx.apply_updates_ptr(len(b), pin_b[i].data_ptr(), False)
        sg._check(ctx._lib.sg_sssp_inceval(ctx._h, C.c_void_p(out_pin.data_ptr())), ctx,
                  "sg_sssp_inceval")
        relax_e += ctx.stats()["edges_relaxed"]
    ctx.record_event(3)
    ctx.synchronize()
    te_ms = D.max(ctx.elapsed_ms(2, 3))
    clk = clocks.stop()
    # where a step's time goes: applier vs IncEval, and inside IncEval the
    # delta-stepping kernel vs the reset / re-seed / parent passes
    ctx.set_profile(0xFF)
    ctx.reset_stats()
    prof = {"apply_ms": 0.0, "inceval_ms": 0.0, "sssp_kernel_ms": 0.0}
    extra = [hg.gen_updates(40000, 40000, 10000, seed=900 + i) for i in range(2)]
    for b in extra:
        ctx.synchronize()
        ctx.record_event(4)
        ctx.apply_updates(b)
        ctx.record_event(5)
        sg._check(ctx._lib.sg_sssp_inceval(ctx._h, None), ctx, "sg_sssp_inceval")
        ctx.record_event(6)
        ctx.synchronize()
        prof["apply_ms"] += ctx.elapsed_ms(4, 5) / len(extra)
        prof["inceval_ms"] += ctx.elapsed_ms(5, 6) / len(extra)
    st = ctx.stats()
    prof["sssp_kernel_ms"] = st["kernel_ms"]["sssp"] / len(extra)
    ctx.set_profile(0)
    # CPU baseline: the reference's incremental stage restated in the oracle
    # (deltaCompute over the deleted and re-weighted edges, a round from every
    # finite vertex, the traversal) on all host threads, for one more batch,
    # from the GPU's converged distances and parents
    d_prev, p_prev = ctx.sssp_distances(), ctx.sssp_parents()
    orp, ocol, _ = hg.csr()
    cb = hg.gen_updates(40000, 40000, 10000, seed=950)
    nrp, ncol, nw = hg.csr()
    old_keys = np.repeat(np.arange(n, dtype=np.int64), np.diff(orp).astype(np.int64)) * n + ocol
    ckeys = cb["src"].astype(np.int64) * n + cb["dst"].astype(np.int64)
    if not np.all(old_keys[1:] > old_keys[:-1]):
        old_keys = np.sort(old_keys)
    pos = np.minimum(np.searchsorted(old_keys, ckeys), len(old_keys) - 1)
    gone = (cb["op"] == 1) | ((cb["op"] == 0) & (old_keys[pos] == ckeys))
    t1 = time.perf_counter()
    d_cpu, _, cst = oracle.sssp_inceval((orp, ocol), (nrp, ncol, nw),
                                        (cb["src"][gone], cb["dst"][gone]), d_prev, p_prev)
    cpu_s = time.perf_counter() - t1
    ctx.apply_updates(cb)
    sg._check(ctx._lib.sg_sssp_inceval(ctx._h, None), ctx, "sg_sssp_inceval")
    d_last = ctx.sssp_distances()
    ref = oracle.dijkstra(nrp, ncol, nw, 0)
    exact = bool(np.array_equal(d_last, ref))
    cpu_exact = bool(np.array_equal(d_cpu, ref))
    ctx.close()
    result = {
        "metric": "GTEPS for SSSP incremental re-eval (IncEval)",
        "value": round(D.sum(relax) / (t_ms * 1e-3) / 1e9, 4), "unit": "GTEPS",
        "n_gpus": D.ws, "steps": K, "warmup": W, "ms_per_step": round(t_ms / K, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic R-MAT (seeded), random update batches",
        "config": {"workload": "incremental SSSP, R-MAT scale 20", "vertices": n, "edges": E,
                   "weights": "uniform integers [1, 100]", "source": 0,
                   "batch_changes": 100000, "batch_mix": "40% insert / 40% delete / 20% re-weight",
                   "summary": "plain graph (no cluster file at this scale)",
                   "l2": "graph larger than L2, no flush", "parallelism": "single GPU"},
        "graph_gteps": round(E * K / (t_ms * 1e-3) / 1e9, 4),
        "reset_vertices_per_step": resets,
        "step_breakdown_ms": {k: round(v, 3) for k, v in prof.items()},
        "peval_ms": round(pe["elapsed_ms"], 3),
        "exact_vs_dijkstra": exact,
        "e2e": {"value": round(D.sum(relax_e) / (te_ms * 1e-3) / 1e9, 4), "unit": "GTEPS",
                "h2d_bytes_per_step": 16 * 100000, "d2h_bytes_per_step": 8 * n,
                "ms_per_step": round(te_ms / K, 3)},
        # the reference's IncEval relaxes every edge in its first round, the
        # GPU path only the affected region: compare time (ms per IncEval)
        # or graph-GTEPS (graph edges / IncEval time), not relaxation counts
        "cpu_baseline": {"value": round(cst["edges"] / cpu_s / 1e9, 4), "unit": "GTEPS",
                         "ms_per_step": round(cpu_s * 1e3, 3),
                         "graph_gteps": round(len(ncol) / cpu_s / 1e9, 4),
                         "cores": os.cpu_count(), "kind": "port",
                         "sample": f"one IncEval of the reference's plain incremental SSSP "
                                   f"(oracle restatement of deltaCompute + traversal) after a "
                                   f"100,000-change batch: {cst['edges']} relaxations, "
                                   f"{int(cst['residual'])} reset vertices, {cpu_s:.3f} s; "
                                   f"distances equal Dijkstra: {cpu_exact}"},
    }
    if clk:
        result["clocks"] = clk
    return result


def community_graph(n_comm, size, seed):
    """Directed graph with planted communities (vectorised, seeded): inside
    each community every member links to ~8 random members; the last 3
    members of each community link to the first 3 members of 4 random other
    communities.  Integer weights U[1, 100].  Returns CSR and the
    communities (the cluster file)."""
    rng = np.random.default_rng(seed)
    n = n_comm * size
    deg_in = 8
    src_i = np.repeat(np.arange(n, dtype=np.int64), deg_in)
    dst_i = (src_i // size) * size + rng.integers(0, size, size=src_i.size)
    exits = (np.arange(n_comm, dtype=np.int64)[:, None] * size + np.arange(size - 3, size)).ravel()
    src_x = np.repeat(exits, 4)
    oc = rng.integers(0, n_comm, size=src_x.size)
    dst_x = oc * size + rng.integers(0, 3, size=src_x.size)
    src = np.concatenate([src_i, src_x])
    dst = np.concatenate([dst_i, dst_x])
    keep = src != dst
    key = np.unique(src[keep] * n + dst[keep])
    src, dst = key // n, key % n
    rp = np.zeros(n + 1, np.uint64)
    np.add.at(rp, src + 1, 1)
    rp = np.cumsum(rp).astype(np.uint64)
    col = dst.astype(np.uint32)
    w = (1 + (src * 2654435761 + dst * 40503) % 100).astype(np.float32)
    comms = [np.arange(c * size, (c + 1) * size, dtype=np.uint32) for c in range(n_comm)]
    return rp, col, w, comms


def run_summarized(args, D: Dist):
    """The summarized graph at scale: PageRank PEval/IncEval and SSSP PEval with
    compress=1 (supernodes, shortcuts computed on the GPU) against compress=0
    on the same community graph and batches."""
    import oracle
    import suminc_gb300 as sg

    dev = D.local
    n_comm = 1 << max(args.batch_scale - 5, 4)  # communities of 32..40 members
    rp, col, w, comms = community_graph(n_comm, 40, args.seed)
    n, E = len(rp) - 1, len(col)
    hg = sg.HostGraph(rp, col, w)
    bsz = max(1000, E // 1000)
    batches = [hg.gen_updates(bsz // 2, bsz - bsz // 2, 0, seed=700 + i) for i in range(args.steps)]
    prof_batch = hg.gen_updates(bsz // 2, bsz - bsz // 2, 0, seed=799)
    out = {}
    for mode in (1, 0):
        # PageRank on its own context: with compress = 1 the apply repairs the
        # summary's PageRank tables on the device
        ctx = sg.Context(dev, compress=mode)
        ctx.load_csr(rp, col, w)
        t0 = time.perf_counter()
        if mode:
            ctx.summary_build(comms)
            info = ctx.summary_info()
        build_s = time.perf_counter() - t0
        ctx.pr_peval(out=False)
        pe = ctx.stats()
        inc_ms, rounds, apply_ms = [], [], []
        for b in batches:
            t1 = time.perf_counter()
            ctx.apply_updates(b)  # with compress=1 this includes the summary repair
            apply_ms.append((time.perf_counter() - t1) * 1e3)
            ctx.pr_inceval_into(None)
            st = ctx.stats()
            inc_ms.append(st["elapsed_ms"])
            rounds.append(st["rounds"])
        # one more batch (the same one in both modes) with CUDA events around
        # every kernel class
        ctx.set_profile(0xFF)
        ctx.apply_updates(prof_batch)
        ctx.reset_stats()
        ctx.pr_inceval_into(None)
        stp = ctx.stats()
        ctx.set_profile(0)
        kms = {k: round(v, 3) for k, v in stp["kernel_ms"].items() if v}
        x = ctx.pr_values()
        check = ctx.summary_check() if mode else None
        ctx.close()
        # SSSP from 0 on a second context, re-evaluated after the same batches
        # (with compress=1 over the summary: reset, rounds over the summarized
        # CSR and repaired shortcuts, inner correction; its apply also brings
        # the host restatement of the summary up to date)
        ctx = sg.Context(dev, compress=mode)
        ctx.load_csr(rp, col, w)
        if mode:
            ctx.summary_build(comms)
        d0 = ctx.sssp_peval(0)
        sp_first = ctx.stats()
        d0 = ctx.sssp_peval(0)  # shortcut distances and sketch now built
        sp = ctx.stats()
        sssp_inc_ms, sssp_apply_ms = [], []
        for b in batches:
            t1 = time.perf_counter()
            ctx.apply_updates(b)
            sssp_apply_ms.append((time.perf_counter() - t1) * 1e3)
            d1 = ctx.sssp_inceval()
            sssp_inc_ms.append(ctx.stats()["elapsed_ms"])
        ctx.close()
        out[mode] = {"peval_ms": round(pe["elapsed_ms"], 3), "peval_rounds": pe["rounds"],
                     "inceval_kernel_ms": kms, "inceval_profiled_ms": round(stp["elapsed_ms"], 3),
                     "sssp_peval_ms": round(sp["elapsed_ms"], 3),
                     "sssp_peval_first_ms": round(sp_first["elapsed_ms"], 3),
                     "inceval_ms": [round(v, 3) for v in inc_ms], "inceval_rounds": rounds,
                     "apply_ms": [round(v, 3) for v in apply_ms],
                     "sssp_apply_ms": [round(v, 3) for v in sssp_apply_ms],
                     "sssp_inceval_ms": [round(v, 3) for v in sssp_inc_ms],
                     "build_s": round(build_s, 2), "x": x, "d0": d0, "d1": d1}
        if mode:
            out[mode]["summary"] = {k: info[k] for k in ("clusters", "supernodes", "shortcut_edges",
                                                         "boundary_edges", "all_rows")}
            out[mode]["repair_vs_host_restatement"] = check
    # the pull worker (message_type=pull) over a summary without mirrors
    ctx = sg.Context(dev, compress=1, message_type=sg.SG_MSG_PULL, mirror_k=1 << 30)
    ctx.load_csr(rp, col, w)
    ctx.summary_build(comms)
    ctx.pr_peval(out=False)
    pe = ctx.stats()
    inc_ms, rounds = [], []
    for b in batches + [prof_batch]:
        ctx.apply_updates(b)
        ctx.pr_inceval_into(None)
        st = ctx.stats()
        inc_ms.append(st["elapsed_ms"])
        rounds.append(st["rounds"])
    out["pull"] = {"peval_ms": round(pe["elapsed_ms"], 3), "peval_rounds": pe["rounds"],
                   "inceval_ms": [round(v, 3) for v in inc_ms[:-1]],
                   "inceval_rounds": rounds[:-1], "x": ctx.pr_values()}
    ctx.close()
    nrp, ncol, nw = hg.csr()
    xs = oracle.pr_fixed_point(nrp, ncol)
    out["pull"]["l1_vs_fp64"] = float(np.abs(out["pull"].pop("x") - xs).sum())
    d_ref = oracle.dijkstra(rp, col, w, 0)
    # both contexts applied the same batches (the profiled one last); hg holds
    # the graph after them
    l1 = {m: float(np.abs(out[m]["x"] - xs).sum()) for m in (0, 1)}
    exact = {m: bool(np.array_equal(out[m]["d0"], d_ref)) for m in (0, 1)}
    # the graph after the regular batches (before the profiled one): SSSP
    # IncEval's last result against Dijkstra there
    g1 = (rp, col, w)
    for b in batches:
        g1 = oracle.apply_updates(*g1, b)
    d1_ref = oracle.dijkstra(*g1, 0)
    exact_inc = {m: bool(np.array_equal(out[m]["d1"], d1_ref)) for m in (0, 1)}
    for m in (0, 1):
        del out[m]["x"], out[m]["d0"], out[m]["d1"]
    s_inc = float(np.mean(out[1]["inceval_ms"]))
    p_inc = float(np.mean(out[0]["inceval_ms"]))
    # a batch's whole cost: the apply (with compress = 1 it repairs the
    # summary's PageRank tables on the device) plus the IncEval
    s_step = float(np.mean(np.add(out[1]["apply_ms"], out[1]["inceval_ms"])))
    p_step = float(np.mean(np.add(out[0]["apply_ms"], out[0]["inceval_ms"])))
    return {
        "metric": "PageRank batch (apply + summary repair + IncEval) over the summarized graph (ms per batch)",
        "value": round(s_step, 3), "unit": "ms", "n_gpus": D.ws, "steps": args.steps, "warmup": 0,
        "ms_per_step": round(s_step, 3), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic community graph (seeded)",
        "config": {"workload": f"summarized PageRank / SSSP, {n_comm} communities of 40",
                   "vertices": n, "edges": E, "batch_changes": bsz,
                   "clusters": "the planted communities (cluster file)",
                   "parallelism": "single GPU"},
        "summarized": out[1], "plain": out[0], "summarized_pull": out["pull"],
        "summarized_over_plain_inceval": round(s_inc / p_inc, 3),
        "step_ms": {"summarized": round(s_step, 3), "plain": round(p_step, 3),
                    "summarized_over_plain": round(s_step / p_step, 3)},
        "pr_l1_vs_fp64": l1, "sssp_exact_vs_dijkstra": exact,
        "sssp_inceval_exact_vs_dijkstra": exact_inc,
        "sssp_inceval_ms": {"summarized": round(float(np.mean(out[1]["sssp_inceval_ms"])), 3),
                            "plain": round(float(np.mean(out[0]["sssp_inceval_ms"])), 3)},
    }


def main():
    args = parse()
    D = Dist()
    if args.impl == "reference":
        run_reference(args, D)
        return
    if args.workload in ("batched", "adjoint", "sssp", "summarized"):
        result = {"batched": run_batched, "adjoint": run_adjoint, "sssp": run_sssp,
                  "summarized": run_summarized}[args.workload](args, D)
        if D.rank == 0:
            print(json.dumps(result), flush=True)
        return
    result, hg, batches, _ = run_ours(args, D)
    if D.rank == 0:
        print(json.dumps(result), flush=True)


if __name__ == "__main__":
    main()
