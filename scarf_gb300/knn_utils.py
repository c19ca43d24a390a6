"""kNN graph construction with scarf's own signatures (scarf/knn_utils.py).

``self_query_knn`` and ``smoothen_dists`` write the same datasets with the
same dtypes as the reference (``indices`` (n, k) u8, ``distances`` (n, k) f8;
``edges`` (n*k, 2) u8, ``weights`` (n*k,) f8). ``make_knn_graph`` is the
composite of the two that this build adds (the reference has no function of
that name).
"""
from __future__ import annotations

import numpy as np
import torch

from . import kernels as K
from .store import create_zarr_dataset

__all__ = ["self_query_knn", "smoothen_dists", "make_knn_graph"]


def self_query_knn(ann_obj, store, chunk_size: int, nthreads: int) -> float:
    """scarf/knn_utils.py:23-76: every cell's k nearest other cells and the
    percentage of cells whose first hit was themselves. One exact device
    query over all cells replaces the per-block HNSW queries; the self rule is
    fix_knn_query's (scarf/ann.py:31-52), applied on the device."""
    n, k = ann_obj.nCells, ann_obj.k
    idx = ann_obj.annIdx
    s = idx.scores
    ind, dist, nm = K.knn(s, s, ann_obj.dims, k, self_offset=0, margin=idx._margin(), precision=idx.precision)
    z_knn = create_zarr_dataset(store, "indices", (chunk_size,), "u8", (n, k))
    z_dist = create_zarr_dataset(store, "distances", (chunk_size,), "f8", (n, k))
    z_knn[:, :] = ind.cpu().numpy().astype(np.uint64)
    z_dist[:, :] = dist.cpu().numpy().astype(np.float64)
    ann_obj._last_knn = (ind, dist)
    return 100.0 * (n - int(nm.item())) / n


def _device_knn(z_idx, z_dist):
    if isinstance(z_idx, torch.Tensor):
        return z_idx.to(torch.int64).contiguous(), z_dist.to(torch.float32).contiguous()
    i = torch.from_numpy(np.ascontiguousarray(np.asarray(z_idx[:]), dtype=np.int64)).cuda()
    d = torch.from_numpy(np.ascontiguousarray(np.asarray(z_dist[:]), dtype=np.float32)).cuda()
    return i, d


def smoothen_dists(store, z_idx, z_dist, lc: float, bw: float, chunk_size: int):
    """scarf/knn_utils.py:89-159 on the GPU (umap-learn's smooth_knn_dist and
    compute_membership_strengths per chunk of ``chunk_size`` rows, then the
    zero weights replaced by the chunk-derived global minimum)."""
    ki, kd = _device_knn(z_idx, z_dist)
    n, k = ki.shape
    edges, w = K.smooth(ki, kd, lc, bw, chunk_size)
    zge = create_zarr_dataset(store, "edges", (chunk_size * k,), ("u8", "u8"), (n * k, 2))
    zgw = create_zarr_dataset(store, "weights", (chunk_size * k,), "f8", (n * k,))
    zge[:, :] = edges.cpu().numpy().astype(np.uint64)
    zgw[:] = w.cpu().numpy()
    return None


def make_knn_graph(ann_obj, knn_store, graph_store, chunk_size: int, lc: float = 1.0, bw: float = 1.5) -> float:
    """``self_query_knn`` then ``smoothen_dists`` without a host round trip of
    the neighbour lists; returns the recall percentage."""
    recall = self_query_knn(ann_obj, knn_store, chunk_size, 1)
    ind, dist = ann_obj._last_knn
    smoothen_dists(graph_store, ind, dist, lc, bw, chunk_size)
    return recall


def calc_snn(indices: np.ndarray) -> np.ndarray:
    """scarf/knn_utils.py:195-211 on the GPU: for every edge (i, j) the number of
    neighbours row i shares with its j-th neighbour, over k - 1."""
    t = torch.as_tensor(np.ascontiguousarray(indices), dtype=torch.int64).cuda()
    return K.calc_snn(t).cpu().numpy()


def merge_graphs(csr_mats):
    """scarf/knn_utils.py:236-274 on the GPU: merge kNN graphs of the same shape
    and size so that every row keeps k edges, chosen by weight + shared
    neighbours. Returns a ``scipy.sparse.coo_matrix``."""
    from scipy.sparse import coo_matrix
    if len(set(x.shape for x in csr_mats)) != 1:
        raise ValueError("ERROR: All graphs do not have the same shape.")
    if len(set(x.size for x in csr_mats)) != 1:
        raise ValueError("ERROR: All graphs do not have the same number of edges")
    n = csr_mats[0].shape[0]
    nk = int(csr_mats[0].indptr[1] - csr_mats[0].indptr[0])
    idx, w, snn = [], [], []
    for mat in csr_mats:
        i = torch.as_tensor(mat.indices.reshape(n, nk).astype(np.int64)).cuda()
        idx.append(i)
        w.append(torch.as_tensor(mat.data.reshape(n, nk).astype(np.float64)).cuda())
        snn.append(K.calc_snn(i))
    oi, ow = K.merge_graphs(idx, w, snn)
    row = np.repeat(np.arange(n), nk)
    return coo_matrix((ow.cpu().numpy().ravel(), (row, oi.cpu().numpy().ravel())), shape=csr_mats[0].shape)
