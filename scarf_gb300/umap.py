"""f3: the UMAP layout scarf computes on the fused kNN graph (scarf/umap.py),
with the graph union and the layout epochs on the GPU.

``fit_transform`` keeps the reference's signature (scarf/umap.py:126-163):
``find_ab_params`` and ``make_epochs_per_sample`` are restated from umap-learn
(umap/umap_.py) on the host, the fuzzy union is ``sg_fuzzy_union`` and the
epochs are ``sg_umap_layout`` (see its header comment: all edges of an epoch
run concurrently, as umap-learn's parallel mode, so the layout follows the
same stochastic process rather than the sequential run's exact trajectory).
densMAP is not part of this build.
"""
from __future__ import annotations

import numpy as np
import torch

from . import kernels as K

__all__ = ["find_ab_params", "make_epochs_per_sample", "fuzzy_simplicial_set", "simplicial_set_embedding",
           "fit_transform"]


def find_ab_params(spread: float, min_dist: float):
    """umap-learn find_ab_params: least-squares fit of 1 / (1 + a x^(2b)) to
    the offset exponential of ``spread`` and ``min_dist`` on 300 points of
    [0, 3 spread]."""
    from scipy.optimize import curve_fit

    def curve(x, a, b):
        return 1.0 / (1.0 + a * x ** (2 * b))

    xv = np.linspace(0, spread * 3, 300)
    yv = np.zeros(xv.shape)
    yv[xv < min_dist] = 1.0
    yv[xv >= min_dist] = np.exp(-(xv[xv >= min_dist] - min_dist) / spread)
    params, _ = curve_fit(curve, xv, yv)
    return float(params[0]), float(params[1])


def make_epochs_per_sample(weights: np.ndarray, n_epochs: int) -> np.ndarray:
    """umap-learn make_epochs_per_sample: an edge of weight w is sampled every
    n_epochs / (n_epochs * w / max w) epochs; -1 for weight 0."""
    result = -1.0 * np.ones(weights.shape[0], dtype=np.float64)
    n_samples = n_epochs * (weights / weights.max())
    result[n_samples > 0] = float(n_epochs) / np.float64(n_samples[n_samples > 0])
    return result


def fuzzy_simplicial_set(g, set_op_mix_ratio: float):
    """scarf/umap.py:117-123 on the GPU (sg_fuzzy_union): returns the union as
    device tensors ``(rows int32, cols int32, weights float64)``, zeros removed."""
    coo = g.tocoo()
    n = g.shape[0]
    edges = torch.from_numpy(np.stack([coo.row, coo.col], 1).astype(np.int64)).cuda()
    w = torch.from_numpy(coo.data.astype(np.float64)).cuda()
    indptr, ind, dat = K.fuzzy_union(edges, w, n, 1, mix=float(set_op_mix_ratio))
    nnz = int(indptr[-1].item())
    counts = indptr[1:] - indptr[:-1]
    rows = torch.repeat_interleave(torch.arange(n, device=edges.device, dtype=torch.int32), counts)
    return rows, ind[:nnz], dat[:nnz]


def simplicial_set_embedding(g, embedding, n_epochs, a, b, random_seed, gamma, initial_alpha,
                             negative_sample_rate, densmap_kwds, parallel, nthreads, verbose):
    """scarf/umap.py:41-115 with the epochs on the GPU; ``g`` is the output of
    ``fuzzy_simplicial_set``."""
    if densmap_kwds:
        raise NotImplementedError("densMAP is not part of the GPU path")
    rows, cols, w = g
    eps = make_epochs_per_sample(w.cpu().numpy(), n_epochs)
    y = torch.from_numpy(np.ascontiguousarray(embedding, dtype=np.float32)).cuda()
    K.umap_layout(rows, cols, torch.from_numpy(eps.astype(np.float64)).cuda(), y, n_epochs, a, b, gamma,
                  initial_alpha, negative_sample_rate, seed=int(random_seed))
    return y.cpu().numpy()


def fit_transform(graph, ini_embed, spread, min_dist, n_epochs, random_seed, repulsion_strength, initial_alpha,
                  negative_sample_rate, densmap_kwds, parallel, nthreads, verbose):
    """scarf/umap.py:126-163: returns ``(embedding, a, b)``."""
    a, b = find_ab_params(spread=spread, min_dist=min_dist)
    embedding = simplicial_set_embedding(fuzzy_simplicial_set(graph, 1.0), ini_embed, n_epochs, a, b, random_seed,
                                         repulsion_strength, initial_alpha, negative_sample_rate, densmap_kwds,
                                         parallel, nthreads, verbose)
    return embedding, a, b
