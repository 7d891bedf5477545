"""torch.autograd binding of the weighted PageRank and its adjoint kernel.

Used to check the hand-written adjoint (sg_pr_adjoint) against central
finite differences and an FP64 transposed solve: `pagerank(w, tele)` runs
sg_pr_weighted on a fixed edge list with edge weights `w` (float32[m], in the
order of the CSR it was given) and teleport vector `tele` (float32[n]);
backward hands dL/dx to sg_pr_adjoint and returns dL/dw and dL/dtele.  Each
forward reloads the graph with the new weights, so this binding is for
checks, not for speed.
"""
from __future__ import annotations

import numpy as np
import torch

from . import Context


class _PageRank(torch.autograd.Function):
    @staticmethod
    def forward(fctx, w, tele, graph: Context, row_ptr, col):
        graph.load_csr(row_ptr, col, w.detach().cpu().numpy().astype(np.float32))
        x = graph.pr_weighted(tele.detach().cpu().numpy().astype(np.float32))
        fctx.graph = graph
        return torch.from_numpy(x)

    @staticmethod
    def backward(fctx, grad_x):
        dw, dt = fctx.graph.pr_adjoint(grad_x.detach().cpu().numpy().astype(np.float32))
        return torch.from_numpy(dw), torch.from_numpy(dt), None, None, None


def pagerank(w: torch.Tensor, tele: torch.Tensor, graph: Context, row_ptr: np.ndarray,
             col: np.ndarray) -> torch.Tensor:
    """Weighted PageRank x(w, tele) with gradients through the adjoint kernel.
    row_ptr / col: the edge list (rows sorted by neighbour), fixed."""
    return _PageRank.apply(w, tele, graph, row_ptr, col)
