"""Restatement of the reference's update-file semantics (test infrastructure).

IncFragmentBuilder::Init / Build (grape/fragment/inc_fragment_builder.h:29-133):
  * ``a u v w`` records go into a map keyed by (u, v); emplace keeps the
    FIRST add of a pair (:57);
  * ``d u v`` records go into a set (:65);
  * the new graph = every old edge whose pair is neither deleted nor re-added
    (:100-125) plus every added pair with its first weight (:85-95).
Consequently an add of an existing pair replaces it (weight change), and a
delete of an absent pair is ignored.
"""
from __future__ import annotations

import numpy as np


def apply_updates_reference(rp, col, w, upd):
    """Returns the post-batch CSR (rows sorted by destination)."""
    n = len(rp) - 1
    added = {}
    deleted = set()
    for r in upd:
        key = (int(r["src"]), int(r["dst"]))
        if int(r["op"]) == 0:
            added.setdefault(key, float(r["weight"]))
        else:
            deleted.add(key)
    rows = [[] for _ in range(n)]
    for u in range(n):
        for e in range(int(rp[u]), int(rp[u + 1])):
            v = int(col[e])
            if (u, v) in deleted or (u, v) in added:
                continue
            rows[u].append((v, float(w[e]) if w is not None else 1.0))
    for (u, v), wt in added.items():
        rows[u].append((v, wt))
    nrp = np.zeros(n + 1, np.uint64)
    ncol = []
    nw = []
    for u in range(n):
        rows[u].sort()
        nrp[u + 1] = nrp[u] + len(rows[u])
        ncol.extend(v for v, _ in rows[u])
        nw.extend(x for _, x in rows[u])
    return nrp, np.asarray(ncol, np.uint32), np.asarray(nw, np.float32)
