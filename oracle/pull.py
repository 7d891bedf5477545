"""CPU restatement of the message_type=pull PageRank worker over a summary
-- test infrastructure only (imported by tests/, never by the product path).

Follows SumSyncIterWorkerPull::Query (grape/worker/sum_sync_iter_worker_pull.h):
vertex classes (:286-320), the per-vertex in-indexes (:321-509), the init of
the values (:510-535), the summarized rounds (:757-980; pull functions
pagerank_ingress.h:210-310), termCheck (:1430-1462), the correction
(:1045-1131) and the plain rounds (:600-630); the shortcut weights come
from the cluster-local iteration of build_iter_index_mirror
(iter_compressor.h:318-491: unit delta at the entry, divisor d / out-degree,
at most 100 sweeps, stop at sum|delta| <= termcheck_threshold * |C| / N;
values of exits become bound_delta, of the other members inner_value, the
remaining deltas inner_delta).

Scope: summaries in which every cluster is kept and no mirror is made
(mirror_k above every candidate's edge count), the form the pull worker
accepts.  Entries are the members with an in-edge from outside the cluster,
exits the members with an out-edge leaving it.

``count_entry_arrivals=False`` is the reference's stop test (values only);
``True`` also counts the mass that reached the entries in the round, which
keeps the summarized stage running while mass is in flight.
"""
from __future__ import annotations

import numpy as np


def pr_pull_summarized(rp, col, clusters, damping=0.85, tau=1e-6, count_entry_arrivals=False):
    rp = np.asarray(rp, np.int64)
    col = np.asarray(col, np.int64)
    n = len(rp) - 1
    d = damping
    outdeg = np.diff(rp)
    src = np.repeat(np.arange(n), outdeg)
    cl = np.full(n, -1, np.int64)
    for i, c in enumerate(clusters):
        cl[np.asarray(c, np.int64)] = i
    ext = cl[src] != cl[col]
    out_bound = np.zeros(n, bool)
    out_bound[src[ext & (cl[src] >= 0)]] = True
    entry = np.zeros(n, bool)
    entry[col[ext & (cl[col] >= 0)]] = True
    t = np.full(n, 4)
    t[cl < 0] = 0
    t[entry] = 2
    t[out_bound] = 1
    t[entry & out_bound] = 3
    pub = lambda dl: np.where(outdeg > 0, dl * d / np.maximum(outdeg, 1), 0.0)  # noqa: E731

    # shortcut weights: (members, val, del) per entry
    sc = {}
    for c in clusters:
        mem = np.asarray(c, np.int64)
        L = len(mem)
        loc = {int(v): i for i, v in enumerate(mem)}
        m = np.zeros((L, L))
        for i, u in enumerate(mem):
            for e in range(rp[u], rp[u + 1]):
                j = loc.get(int(col[e]))
                if j is not None:
                    m[j, i] += d / outdeg[u]
        for i, s in enumerate(mem):
            if not entry[s]:
                continue
            delta = np.zeros(L)
            delta[i] = 1.0
            value = np.zeros(L)
            step = 1
            while True:
                value += delta
                diff = np.abs(delta).sum()
                delta = m @ delta
                if diff <= tau / n * L or step > 100:
                    break
                step += 1
            sc[int(s)] = (mem, value, delta)

    def exits_gather(li):
        b = np.zeros(n)
        for s, (mem, val, _) in sc.items():
            b[mem] += li[s] * val * out_bound[mem]
        return b

    x = np.zeros(n)
    dl = np.full(n, (1 - d) / n)
    lastx = x.copy()
    bsave = np.zeros(n)
    li = np.zeros(n)
    spd = np.zeros(n)
    m0 = t == 0
    x[m0] += dl[m0]
    m14 = (t == 1) | (t == 4)
    bsave[m14] = dl[m14]
    dl[m14] = 0
    m23 = (t == 2) | (t == 3)
    li[m23] = dl[m23]
    spd[m23] = dl[m23]
    dl[m23] = 0
    ld = pub(dl)
    m13 = (t == 1) | (t == 3)
    step = 0
    rounds = 0
    while True:
        step += 1
        rounds += 1
        a = np.zeros(n)
        mf = ext | (t[col] == 0)
        np.add.at(a, col[mf], ld[src[mf]])
        b = exits_gather(li)
        nd = np.zeros(n)
        nl = np.zeros(n)
        x[m0] += a[m0]
        dl[m0] = a[m0]
        nd[m0] = a[m0]
        spd[m23] += a[m23]
        nl[m23] = a[m23]
        x[m13] += b[m13]
        dl[m13] = b[m13]
        nd[m13] = b[m13]
        ld, li = pub(nd), nl
        res = np.abs(lastx - x).sum()
        lastx = x.copy()
        if count_entry_arrivals:
            res += np.abs(a[m23]).sum()
        if res < tau or step > 200:
            break
    # correction
    dl[m14] = bsave[m14]
    x[m14] += bsave[m14]
    for s, (mem, val, rem) in sc.items():
        tt = t[mem]
        x[mem] += np.where((tt == 2) | (tt == 4), spd[s] * val * ~out_bound[mem], 0.0)
        x[mem] += np.where(tt >= 1, spd[s] * rem, 0.0)
        dl[mem] += np.where(tt >= 1, spd[s] * rem, 0.0)
    # plain rounds; `continue` skips ++step once
    while True:
        rounds += 1
        a = np.zeros(n)
        np.add.at(a, col, pub(dl)[src])
        dl = a
        x += a
        res = np.abs(lastx - x).sum()
        lastx = x.copy()
        if res < tau or step > 200:
            break
        step += 1
    return x, {"rounds": rounds}
