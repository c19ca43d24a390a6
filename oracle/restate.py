"""numpy/scipy restatement of scarf's graph-construction path (the oracle).

Test infrastructure only: see the package docstring. Reference citations are
``file:line`` relative to the scarf project root (``scarf/...``).

Third-party arithmetic that the reference calls and that is not vendored with
it is restated from its published algorithm:

* umap-learn ``smooth_knn_dist`` / ``compute_membership_strengths``
  (unpinned in ``requirements.txt:23``; the 0.5 line is restated, float32
  locals as in its numba kernels);
* scikit-learn 1.6.1 ``IncrementalPCA.partial_fit`` and ``svd_flip``
  (``requirements.txt:16``);
* hnswlib 0.8.0 (``requirements.txt:3``) is *not* restated: the oracle is an
  exact FP64 kNN, which is what the GPU path is measured against;
* umap-learn (unpinned) ``find_ab_params``, ``make_epochs_per_sample`` and
  the single-threaded ``optimize_layout_euclidean`` (move_other=True, densMAP
  off) that scarf's UMAP step calls, with the negative samples drawn from a
  caller-given generator (``umap_layout_sequential``);
* scikit-learn 1.6.1 ``MiniBatchKMeans.partial_fit`` / ``predict``
  (``sklearn/cluster/_kmeans.py``: ``_mini_batch_step``, ``_random_reassign``,
  ``_kmeans_plusplus``; ``_k_means_minibatch.pyx``: ``_minibatch_update_dense``)
  with its random draws taken from the counter hash of the GPU kernel instead
  of numpy's generator (``kmeans_minibatch``).
"""

from __future__ import annotations

import math
from typing import Optional, Tuple

import numpy as np
import scipy.sparse as sp

__all__ = [
    "normed_csr",
    "clean_array",
    "zstats",
    "IncrementalPCARestated",
    "fit_pca_reference_order",
    "pca_exact",
    "svd_flip_v",
    "reducer",
    "exact_knn",
    "fix_knn_query",
    "self_query_knn",
    "smooth_knn_dist",
    "compute_membership_strengths",
    "smoothen_dists",
    "kmeans_hash",
    "kmeans_minibatch",
    "calc_snn",
    "weight_sort_indices",
    "merge_graphs",
    "umap_find_ab_params",
    "umap_make_epochs_per_sample",
    "umap_layout_sequential",
    "umap_negative_vertex",
    "store_to_sparse",
    "symmetrize",
    "fuzzy_simplicial_set",
    "align_target",
    "map_queries",
    "recall_at_k",
    "subspace_angles",
    "make_graph",
]

SMOOTH_K_TOLERANCE = 1e-5
MIN_K_DIST_SCALE = 1e-3


# --------------------------------------------------------------------------
# a1: library-size normalisation (scarf/assay.py:780-828, :41-64)
# --------------------------------------------------------------------------
def normed_csr(indptr, indices, data, n_genes: int, feat_idx, sf: float = 1000,
               log_transform: bool = True, renormalize_subset: bool = True,
               n_counts: Optional[np.ndarray] = None) -> Tuple[np.ndarray, np.ndarray]:
    """Dense normalised matrix over the selected features, FP64.

    ``counts = rawData[:, feat_idx][cell_idx, :]`` (assay.py:814) with
    ``feat_idx`` ascending (metadata.py:236-250 returns a boolean-mask index);
    the library size is the integer row sum over the subset with 0 -> 1
    (assay.py:818-823) or the stored full-row ``nCounts`` (assay.py:825);
    values are ``sf * c / s`` (assay.py:41-51), ``log1p`` of it when
    ``log_transform`` (assay.py:54-64). Returns ``(x, scalar)``.
    """
    n = len(indptr) - 1
    m = sp.csr_matrix((np.asarray(data), np.asarray(indices), np.asarray(indptr)),
                      shape=(n, n_genes))
    sub = m[:, np.asarray(feat_idx)].tocsr()
    if renormalize_subset:
        s = np.asarray(sub.sum(axis=1, dtype=np.int64)).ravel()
        s[s == 0] = 1
        scalar = s.astype(np.float64)
    else:
        scalar = np.asarray(n_counts, dtype=np.float64)
    dense = sub.toarray().astype(np.float64)
    x = (sf * dense) / scalar.reshape(-1, 1)
    if log_transform:
        x = np.log1p(x)
    return x, scalar


# --------------------------------------------------------------------------
# a3: z-statistics (scarf/datastore/graph_datastore.py:767-796, scarf/utils.py:143-153)
# --------------------------------------------------------------------------
def clean_array(x, fill_val: float = 0):
    """NaN -> 0, +-inf -> 0, then 0 -> ``fill_val`` (utils.py:143-153)."""
    x = np.nan_to_num(np.asarray(x, dtype=np.float64), copy=True)
    x[(x == np.inf) | (x == -np.inf)] = 0
    x[x == 0] = fill_val
    return x


def zstats(x: np.ndarray) -> Tuple[np.ndarray, np.ndarray]:
    """Population mean and std (ddof 0) with ``clean_array`` (graph_datastore.py:767-796)."""
    mu = clean_array(x.mean(axis=0))
    sigma = clean_array(x.std(axis=0), 1)
    return mu, sigma


# --------------------------------------------------------------------------
# a4: PCA (scarf/ann.py:207-256 driving scikit-learn IncrementalPCA)
# --------------------------------------------------------------------------
def svd_flip_v(v: np.ndarray, u: Optional[np.ndarray] = None):
    """scikit-learn ``svd_flip(u, v, u_based_decision=False)``: the entry of
    largest magnitude in each row of ``v`` is made positive."""
    pos = np.argmax(np.abs(v), axis=1)
    signs = np.sign(v[np.arange(v.shape[0]), pos])
    signs[signs == 0] = 1
    v = v * signs[:, None]
    if u is not None:
        u = u * signs[None, :]
    return u, v


class IncrementalPCARestated:
    """Sequential Karhunen-Loeve update as published for scikit-learn 1.6.1
    ``IncrementalPCA.partial_fit`` (Ross et al. 2008): the running mean and
    variance are merged with the batch, the previous components are stacked,
    scaled by their singular values, above the centred batch plus a
    mean-correction row, and the stack is re-decomposed by SVD."""

    def __init__(self, n_components: int):
        self.n_components = n_components
        self.components_ = None
        self.singular_values_ = None
        self.n_samples_seen_ = 0
        self.mean_ = 0.0
        self.var_ = 0.0
        self.explained_variance_ = None
        self.explained_variance_ratio_ = None

    @staticmethod
    def _merge_mean_var(X, last_mean, last_var, last_n):
        new_sum = X.sum(axis=0, dtype=np.float64)
        new_n = X.shape[0]
        upd_n = last_n + new_n
        last_sum = last_mean * last_n
        upd_mean = (last_sum + new_sum) / upd_n
        t = new_sum / new_n
        tmp = X - t
        correction = tmp.sum(axis=0)
        new_unnorm = (tmp ** 2).sum(axis=0) - correction ** 2 / new_n
        if last_n == 0:
            upd_unnorm = new_unnorm
        else:
            last_unnorm = last_var * last_n
            ratio = last_n / new_n
            upd_unnorm = last_unnorm + new_unnorm + ratio / upd_n * (last_sum / ratio - new_sum) ** 2
        return upd_mean, upd_unnorm / upd_n, upd_n

    def partial_fit(self, X: np.ndarray):
        X = np.array(X, dtype=np.float64, copy=True)
        n_samples, n_features = X.shape
        if self.n_components > n_samples:
            raise ValueError("n_components must be less or equal to the batch number of samples")
        col_mean, col_var, n_total = self._merge_mean_var(
            X, self.mean_, self.var_, self.n_samples_seen_)
        if self.n_samples_seen_ == 0:
            X -= col_mean
        else:
            batch_mean = X.mean(axis=0)
            X -= batch_mean
            corr = math.sqrt((self.n_samples_seen_ / n_total) * n_samples) * (self.mean_ - batch_mean)
            X = np.vstack((self.singular_values_.reshape(-1, 1) * self.components_, X, corr))
        U, S, Vt = np.linalg.svd(X, full_matrices=False)
        U, Vt = svd_flip_v(Vt, U)
        ev = S ** 2 / (n_total - 1)
        evr = S ** 2 / np.sum(col_var * n_total)
        nc = self.n_components
        self.n_samples_seen_ = n_total
        self.components_ = Vt[:nc]
        self.singular_values_ = S[:nc]
        self.mean_ = col_mean
        self.var_ = col_var
        self.explained_variance_ = ev[:nc]
        self.explained_variance_ratio_ = evr[:nc]
        return self


def fit_pca_reference_order(z_blocks, dims: int, use_for_pca=None):
    """Block order of ``AnnStream._fit_pca`` (ann.py:207-256): the first block
    big enough is held back (``end_reservoir``) and fitted last; blocks
    smaller than ``dims + 1`` rows are carried into the next one. Each block
    is already z-scaled. Returns ``(loadings h x dims, pca)`` with
    ``loadings = components_[:-1].T`` (ann.py:256)."""
    pca = IncrementalPCARestated(dims + 1)
    end_reservoir = None
    carry = None
    s = 0
    for blk in z_blocks:
        if use_for_pca is not None:
            e = s + blk.shape[0]
            blk = blk[use_for_pca[s:e]]
            s = e
        if carry is not None:
            blk = np.vstack((carry, blk))
            carry = None
        if len(blk) < dims + 1:
            carry = blk
            continue
        if end_reservoir is None:
            end_reservoir = blk
            continue
        try:
            pca.partial_fit(blk)
        except np.linalg.LinAlgError:
            carry = blk
    last = end_reservoir if carry is None else np.vstack((end_reservoir, carry))
    pca.partial_fit(last)
    return pca.components_[:-1, :].T, pca


def pca_exact(z: np.ndarray, n_components: int):
    """Exact FP64 PCA of the centred rows of ``z`` via the covariance
    eigendecomposition, sign convention of ``svd_flip`` (the value of largest
    magnitude of each component positive). Returns ``(components h x nc,
    eigenvalues descending)``; this is what the GPU path computes."""
    zc = z - z.mean(axis=0)
    cov = zc.T @ zc
    w, v = np.linalg.eigh(cov)
    order = np.argsort(w)[::-1][:n_components]
    comps = v[:, order].T
    _, comps = svd_flip_v(comps)
    return comps.T, w[order]


def reducer(x: np.ndarray, mu, sigma, loadings) -> np.ndarray:
    """``((x - mu) / sigma) . L`` with no PCA-mean centring (ann.py:129-138, :191-192)."""
    return ((x - mu) / sigma).dot(loadings)


def subspace_angles(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Principal angles (radians, descending) between the column spans of ``a`` and ``b``."""
    qa, _ = np.linalg.qr(a)
    qb, _ = np.linalg.qr(b)
    s = np.linalg.svd(qa.T @ qb, compute_uv=False)
    s = np.clip(s, -1.0, 1.0)
    return np.sort(np.arccos(s))[::-1]


# --------------------------------------------------------------------------
# a6/a7: kNN (scarf/ann.py:31-52, :194-205; scarf/knn_utils.py:23-76)
# --------------------------------------------------------------------------
def exact_knn(q: np.ndarray, r: np.ndarray, k: int, block: int = 4096,
              extra: int = 8) -> Tuple[np.ndarray, np.ndarray]:
    """Exact squared-L2 kNN in FP64, ordered by (distance, index).

    This stands in for ``hnswlib.Index(space='l2').knn_query`` (ann.py:201,
    :204), which returns squared Euclidean distances."""
    q = np.asarray(q, dtype=np.float64)
    r = np.asarray(r, dtype=np.float64)
    nq, nr = q.shape[0], r.shape[0]
    k = min(k, nr)
    kk = min(k + extra, nr)
    rn = (r * r).sum(1)
    out_i = np.empty((nq, k), dtype=np.int64)
    out_d = np.empty((nq, k), dtype=np.float64)
    for s in range(0, nq, block):
        qb = q[s:s + block]
        d2 = (qb * qb).sum(1)[:, None] + rn[None, :] - 2.0 * (qb @ r.T)
        if kk < nr:
            cand = np.argpartition(d2, kk - 1, axis=1)[:, :kk]
        else:
            cand = np.broadcast_to(np.arange(nr), (qb.shape[0], nr)).copy()
        diff = qb[:, None, :] - r[cand]
        ex = (diff * diff).sum(-1)
        order = np.lexsort((cand, ex), axis=1)
        ci = np.take_along_axis(cand, order, 1)[:, :k]
        cd = np.take_along_axis(ex, order, 1)[:, :k]
        out_i[s:s + block] = ci
        out_d[s:s + block] = cd
    return out_i, out_d


def fix_knn_query(indices: np.ndarray, distances: np.ndarray, ref_idx: np.ndarray):
    """Drop the self hit from a (k+1)-query (ann.py:31-52): column 0 when it is
    self; else the first self position; else the last column. Returns the
    fixed arrays and the number of rows whose first hit was not self."""
    ind = np.asarray(indices)
    dist = np.asarray(distances)
    fixed_i = ind[:, 1:].copy()
    fixed_d = dist[:, 1:].copy()
    mis = ind[:, 0] != ref_idx
    for n in np.where(mis)[0]:
        j, kv = ind[n], dist[n]
        p = np.where(j == ref_idx[n])[0]
        if len(p) > 0:
            p = p[0]
            fixed_i[n] = np.concatenate((j[:p], j[p + 1:]))
            fixed_d[n] = np.concatenate((kv[:p], kv[p + 1:]))
        else:
            fixed_i[n] = j[:-1]
            fixed_d[n] = kv[:-1]
    return fixed_i, fixed_d, int(mis.sum())


def self_query_knn(scores: np.ndarray, k: int, chunk_size: int = 1000):
    """``self_query_knn`` (knn_utils.py:23-76) with an exact index: per block of
    ``chunk_size`` rows query k+1, drop self, count misses. Returns
    ``(indices u8, distances f8, recall%)``; distances are rounded to float32
    as hnswlib returns them (ann.py:201-204)."""
    n = scores.shape[0]
    k = min(k, n - 1)
    idx_all, d_all = exact_knn(scores, scores, k + 1)
    out_i = np.empty((n, k), dtype=np.uint64)
    out_d = np.empty((n, k), dtype=np.float64)
    tnm = 0
    for s in range(0, n, chunk_size):
        e = min(n, s + chunk_size)
        fi, fd, nm = fix_knn_query(idx_all[s:e], d_all[s:e].astype(np.float32), np.arange(s, e))
        out_i[s:e] = fi
        out_d[s:e] = fd
        tnm += nm
    recall = 100.0 * (n - tnm) / n
    return out_i, out_d, recall


def recall_at_k(scores_q: np.ndarray, scores_r: np.ndarray, got_idx: np.ndarray,
                exact_kth: np.ndarray, rel: float = 1e-6) -> float:
    """Tie-aware recall@k: a returned neighbour is a hit when its exact FP64
    distance is within ``(1 + rel)`` of the exact k-th neighbour distance."""
    q = np.asarray(scores_q, dtype=np.float64)
    r = np.asarray(scores_r, dtype=np.float64)
    gi = np.asarray(got_idx, dtype=np.int64)
    diff = q[:, None, :] - r[gi]
    d = (diff * diff).sum(-1)
    thr = exact_kth[:, None] * (1.0 + rel) + 1e-12
    return float((d <= thr).mean())


# --------------------------------------------------------------------------
# a8: smoothing (scarf/knn_utils.py:89-159 -> umap-learn smooth_knn_dist,
#     compute_membership_strengths)
# --------------------------------------------------------------------------
def _seq_mean_f32(a: np.ndarray) -> np.float32:
    """The float32 accumulator of numba's ``np.mean`` (one float32 sum, in
    order); the caller divides by the element count in float64."""
    flat = np.ascontiguousarray(a, dtype=np.float32).ravel()
    if flat.size == 0:
        return np.float32(np.nan)
    return np.float32(np.cumsum(flat, dtype=np.float32)[-1])


def smooth_knn_dist(distances: np.ndarray, k: int, n_iter: int = 64,
                    local_connectivity: float = 1.0, bandwidth: float = 1.0):
    """umap-learn ``smooth_knn_dist``, vectorised over rows with the per-row
    arithmetic order of its numba loop (float32 ``psum``/``lo``/``hi``/``mid``).

    rho: distance to the ``local_connectivity``-th non-zero neighbour;
    sigma: bisection so that sum_{j>=1} exp(-max(0, d_ij - rho)/sigma) equals
    ``log2(k) * bandwidth`` within 1e-5 (the sum starts at column 1); then
    sigma is clamped from below by 1e-3 x the row mean (rho > 0) or 1e-3 x the
    mean over the whole chunk (rho == 0)."""
    d = np.ascontiguousarray(distances, dtype=np.float32)
    n, kc = d.shape
    target = np.log2(k) * bandwidth
    rho = np.zeros(n, dtype=np.float32)
    sum_all = _seq_mean_f32(d)
    lc = float(local_connectivity)
    index = int(math.floor(lc))
    interp = lc - index
    nz = d > 0.0
    nnz = nz.sum(1)
    # non-zero distances in row order, padded with +inf
    pos = np.cumsum(nz, axis=1) - 1
    nzv = np.full((n, kc + 1), np.inf, dtype=np.float32)
    rr, cc = np.nonzero(nz)
    nzv[rr, pos[rr, cc]] = d[rr, cc]
    has = nnz >= lc
    if index > 0:
        sel = has
        base = nzv[sel, index - 1]
        if interp > SMOOTH_K_TOLERANCE:
            base = base + np.float32(interp) * (nzv[sel, index] - nzv[sel, index - 1])
        rho[sel] = base
    else:
        rho[has] = np.float32(interp) * nzv[has, 0]
    some = (~has) & (nnz > 0)
    if some.any():
        rho[some] = np.where(nz[some], d[some], -np.inf).max(1)

    lo = np.zeros(n, dtype=np.float32)
    hi = np.full(n, np.inf, dtype=np.float32)
    mid = np.ones(n, dtype=np.float32)
    active = np.ones(n, dtype=bool)
    one = np.float32(1.0)
    for _ in range(n_iter):
        ia = np.nonzero(active)[0]
        if ia.size == 0:
            break
        m = mid[ia]
        rh = rho[ia]
        psum = np.zeros(ia.size, dtype=np.float32)
        for j in range(1, kc):
            dd = (d[ia, j] - rh).astype(np.float32)
            pos_ = dd > 0
            with np.errstate(over="ignore", under="ignore", divide="ignore", invalid="ignore"):
                ev = np.exp(-(dd / m)).astype(np.float32)
            psum = (psum + np.where(pos_, ev, one)).astype(np.float32)
        done = np.abs(psum.astype(np.float64) - target) < SMOOTH_K_TOLERANCE
        upd = ~done
        gt = upd & (psum > target)
        le = upd & ~(psum > target)
        hi_ia = hi[ia]
        lo_ia = lo[ia]
        mid_ia = m.copy()
        hi_ia[gt] = mid_ia[gt]
        mid_ia[gt] = ((lo_ia[gt] + hi_ia[gt]) / np.float32(2.0)).astype(np.float32)
        lo_ia[le] = mid_ia[le]
        inf_hi = le & np.isinf(hi_ia)
        fin_hi = le & ~np.isinf(hi_ia)
        mid_ia[inf_hi] = mid_ia[inf_hi] * np.float32(2.0)
        mid_ia[fin_hi] = ((lo_ia[fin_hi] + hi_ia[fin_hi]) / np.float32(2.0)).astype(np.float32)
        hi[ia] = hi_ia
        lo[ia] = lo_ia
        mid[ia] = mid_ia
        active[ia[done]] = False
    result = mid.copy()
    row_mean = (np.cumsum(d, axis=1, dtype=np.float32)[:, -1] if kc else np.zeros(n, np.float32))
    row_mean = row_mean.astype(np.float64) / kc
    posr = rho > 0.0
    lim_r = MIN_K_DIST_SCALE * row_mean
    # numba divides the float32 accumulator by the element count in float64
    lim_a = MIN_K_DIST_SCALE * (float(sum_all) / d.size if d.size else np.nan)
    low_r = posr & (result < lim_r)
    result[low_r] = lim_r[low_r].astype(np.float32)
    low_a = (~posr) & (result < lim_a)
    result[low_a] = np.float32(lim_a)
    return result, rho


def compute_membership_strengths(knn_indices: np.ndarray, knn_dists: np.ndarray,
                                 sigmas: np.ndarray, rhos: np.ndarray):
    """umap-learn ``compute_membership_strengths`` (non-bipartite): weight 0
    where the neighbour index equals the *chunk-local* row number (scarf passes
    global indices, knn_utils.py:128-134, so this fires on global index == local
    row), 1 where ``d - rho <= 0`` or ``sigma == 0``, else ``exp(-(d - rho)/sigma)``,
    all in float32. Returns ``(rows int32, cols, vals float32)``."""
    n, k = knn_indices.shape
    kd = np.asarray(knn_dists, dtype=np.float32)
    rows = np.repeat(np.arange(n, dtype=np.int32), k)
    cols = np.asarray(knn_indices).reshape(-1)
    dd = (kd - rhos[:, None]).astype(np.float32)
    with np.errstate(over="ignore", under="ignore", divide="ignore", invalid="ignore"):
        ev = np.exp(-(dd / sigmas[:, None])).astype(np.float32)
    one_mask = (dd <= 0.0) | (sigmas[:, None] == 0.0)
    vals = np.where(one_mask, np.float32(1.0), ev).astype(np.float32)
    self_mask = np.asarray(knn_indices).astype(np.int64) == np.arange(n, dtype=np.int64)[:, None]
    vals[self_mask] = np.float32(0.0)
    return rows, cols, vals.reshape(-1)


def smoothen_dists(z_idx: np.ndarray, z_dist: np.ndarray, lc: float, bw: float,
                   chunk_size: int):
    """``smoothen_dists`` (knn_utils.py:89-159): chunk-wise smoothing on float32
    distances, rows offset by the chunk start, then zero weights replaced by
    ``global_min`` = min(1, smallest non-zero weight of every chunk that holds
    a zero). Returns ``(edges (n*k, 2) u8, weights (n*k,) f8)``."""
    n, k = z_idx.shape
    edges = np.zeros((n * k, 2), dtype=np.uint64)
    weights = np.zeros(n * k, dtype=np.float64)
    last_row = 0
    vc = 0
    null_idx = []
    global_min = 1
    for i in range(0, n, chunk_size):
        ki = z_idx[i:min(n, i + chunk_size)]
        kv = np.asarray(z_dist[i:min(n, i + chunk_size)]).astype(np.float32)
        sig, rho = smooth_knn_dist(kv, k=k, local_connectivity=lc, bandwidth=bw)
        rows, cols, vals = compute_membership_strengths(ki, kv, sig, rho)
        rows = rows + last_row
        start, end = vc, vc + len(rows)
        last_row = rows[-1] + 1
        vc += len(rows)
        edges[start:end, 0] = rows
        edges[start:end, 1] = cols
        weights[start:end] = vals
        nidx = vals == 0
        if nidx.sum() > 0:
            mv = vals[~nidx].min()
            if mv < global_min:
                global_min = mv
        null_idx.extend(nidx)
    w = weights
    w[np.asarray(null_idx, dtype=bool)] = global_min
    return edges, w


# --------------------------------------------------------------------------
# a9: fuzzy union (scarf/datastore/graph_datastore.py:474-511, :1052-1055;
#     scarf/umap.py:118-123)
# --------------------------------------------------------------------------
def store_to_sparse(edges: np.ndarray, weights: np.ndarray, n_cells: int, k: int,
                    use_k: Optional[int] = None) -> sp.csr_matrix:
    """``_store_to_sparse`` (graph_datastore.py:474-511): keep the first
    ``use_k`` of every row's k edges, build CSR with duplicates summed."""
    if use_k is None:
        use_k = k
    use_k = max(1, min(use_k, k))
    w, e = weights, edges
    if use_k != k:
        keep = np.tile([True] * use_k + [False] * (k - use_k), n_cells)
        w, e = w[keep], e[keep]
    return sp.csr_matrix((w, (e[:, 0], e[:, 1])), shape=(n_cells, n_cells))


def symmetrize(g: sp.csr_matrix, upper_only: bool = False) -> sp.csr_matrix:
    """``load_graph(symmetric=True)``: ``G + G^T - G o G^T`` (graph_datastore.py:1052-1055),
    optionally ``triu`` (:1071-1072)."""
    t = g + g.T
    t = t - g.multiply(g.T)
    if upper_only:
        t = sp.triu(t)
    return t.tocsr()


def fuzzy_simplicial_set(g: sp.csr_matrix, set_op_mix_ratio: float = 1.0) -> sp.coo_matrix:
    """umap.py:118-123: ``mix*(G + G^T - G o G^T) + (1-mix)*(G o G^T)``, zeros eliminated."""
    tg = g.transpose()
    prod = g.multiply(tg)
    res = set_op_mix_ratio * (g + tg - prod) + (1.0 - set_op_mix_ratio) * prod
    res.eliminate_zeros()
    return res.tocoo()


# --------------------------------------------------------------------------
# a10: mapping (scarf/datastore/mapping_datastore.py:198-208,
#      scarf/mapping_utils.py:148-214)
# --------------------------------------------------------------------------
def align_target(indptr, indices, data, n_genes_t: int, t_idx: np.ndarray, sf: float = 1000,
                 log_transform: bool = True, renormalize_subset: bool = True,
                 n_counts=None) -> np.ndarray:
    """``align_features`` (mapping_utils.py:148-214): ``t_idx[j]`` is the
    target gene for reference feature j or -1. The target is normalised over
    its present genes (sorted), reordered to the reference order, and absent
    features are filled with 1.0 (mapping_utils.py:208)."""
    t_idx = np.asarray(t_idx)
    present = t_idx != -1
    sorted_t = np.array(sorted(t_idx[present]))
    x, _ = normed_csr(indptr, indices, data, n_genes_t, sorted_t, sf, log_transform,
                      renormalize_subset, n_counts)
    unsorter = np.argsort(np.argsort(t_idx[present]))
    out = np.ones((x.shape[0], len(t_idx)))
    out[:, np.where(present)[0]] = x[:, unsorter]
    return out


def map_queries(x_t: np.ndarray, mu, sigma, loadings, ref_scores: np.ndarray, save_k: int):
    """Per block ``reducer`` then ``knn_query(k=save_k)`` with no self fix
    (mapping_datastore.py:198-208)."""
    s = reducer(x_t, mu, sigma, loadings)
    i, d = exact_knn(s, ref_scores, save_k)
    return i, d, s


# --------------------------------------------------------------------------
# The whole path at oracle precision
# --------------------------------------------------------------------------
def make_graph(indptr, indices, data, n_genes: int, feat_idx, dims: int, k: int,
               batch_size: int = 1000, sf: float = 1000, lc: float = 1.0, bw: float = 1.5,
               pca: str = "exact"):
    """normalise -> z-stats -> PCA -> self-kNN -> smoothing, FP64 (the order of
    ``make_graph``, graph_datastore.py:747-999). ``pca='exact'`` uses the FP64
    covariance eigendecomposition (what the GPU path computes); ``pca='ipca'``
    runs the restated IncrementalPCA in the reference's block order."""
    x, scalar = normed_csr(indptr, indices, data, n_genes, feat_idx, sf)
    mu, sigma = zstats(x)
    z = (x - mu) / sigma
    if pca == "exact":
        comps, evals = pca_exact(z, dims + 1)
        loadings = comps[:, :-1]
    else:
        blocks = [z[s:s + batch_size] for s in range(0, z.shape[0], batch_size)]
        loadings, _ = fit_pca_reference_order(blocks, dims)
    scores = z.dot(loadings)
    ki, kd, recall = self_query_knn(scores, k, batch_size)
    edges, weights = smoothen_dists(ki, kd, lc, bw, batch_size)
    return dict(x=x, scalar=scalar, mu=mu, sigma=sigma, loadings=loadings, scores=scores,
                indices=ki, distances=kd, recall=recall, edges=edges, weights=weights)


# ---- f1: MiniBatchKMeans of make_graph (scarf/ann.py:328-346) ---------------

_M64 = (1 << 64) - 1


def kmeans_hash(seed: int, stream: int, i) -> np.ndarray:
    """The kernel's counter hash (SplitMix64's finaliser) of seed, stream and
    index, as uint64 (wrapping arithmetic)."""
    with np.errstate(over="ignore"):
        i = np.asarray(i, dtype=np.uint64)
        z = np.uint64(seed & _M64) + (np.uint64((stream << 32) & _M64) + i) * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def _kmeans_unit(seed: int, stream: int, i) -> np.ndarray:
    return (kmeans_hash(seed, stream, i) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def _sq_dists(x: np.ndarray, c: np.ndarray) -> np.ndarray:
    x64 = x.astype(np.float64)
    c64 = c.astype(np.float64)
    return ((x64[:, None, :] - c64[None, :, :]) ** 2).sum(-1)


def _kmeans_plusplus(x: np.ndarray, k: int, seed: int) -> np.ndarray:
    """Greedy k-means++ (sklearn _kmeans_plusplus, 2 + ln k local trials),
    draws from the counter hash: the first centre uniformly, round c's
    candidates at cumsum(D2) >= u * total."""
    rows = x.shape[0]
    trials = 2 + int(np.log(k))
    chosen = int(_kmeans_unit(seed, 1, 0) * rows) % rows
    centers = np.empty((k, x.shape[1]), dtype=np.float64)
    d2 = None
    for c in range(k):
        centers[c] = x[chosen]
        t = _sq_dists(x, x[chosen:chosen + 1])[:, 0]
        d2 = t if d2 is None else np.minimum(d2, t)
        if c + 1 == k:
            break
        csum = np.cumsum(d2)
        r = _kmeans_unit(seed, 2 + c, np.arange(trials)) * csum[-1]
        cid = np.minimum(np.searchsorted(csum, r, side="left"), rows - 1)
        pots = [np.minimum(d2, _sq_dists(x, x[j:j + 1])[:, 0]).sum() for j in cid]
        chosen = int(cid[int(np.argmin(pots))])
    return centers


def kmeans_minibatch(x: np.ndarray, k: int, block_rows: int, seed: int):
    """partial_fit over the row blocks of x in order, then predict
    (scarf/ann.py:328-346 with sklearn's MiniBatchKMeans semantics, see the
    module docstring). Returns (centres f64 k x d, labels int64)."""
    x = np.asarray(x, dtype=np.float32)
    n = x.shape[0]
    first = min(n, block_rows)
    if first < k:
        raise ValueError("the first block has fewer rows than k")
    centers = x[:k].astype(np.float64) if first == k else _kmeans_plusplus(x[:first], k, seed)
    w = np.zeros(k)
    since = 0
    for step, r0 in enumerate(range(0, n, block_rows)):
        xb = x[r0:r0 + block_rows]
        rows = xb.shape[0]
        # _random_reassign (checked before the update, counted in first-block sizes)
        since += first
        reassign = bool((w == 0).any()) or since >= 10 * k
        if reassign:
            since = 0
        lab = np.argmin(_sq_dists(xb, centers.astype(np.float32)), axis=1)
        for c in np.unique(lab):
            members = np.nonzero(lab == c)[0]
            v = centers[c] * w[c]
            for m in members:
                v = v + xb[m].astype(np.float64)
            w_new = w[c] + len(members)
            centers[c] = v * (1.0 / w_new)
            w[c] = w_new
        if not reassign:
            continue
        flagged = np.nonzero(w < 0.01 * w.max())[0]
        cap = int(0.5 * rows)
        if len(flagged) > cap:
            flagged = np.sort(flagged[np.argsort(w[flagged], kind="stable")][:cap])
        m = len(flagged)
        if m == 0:
            continue
        keys = (kmeans_hash(seed, 0x80000000 + step, np.arange(rows)) & np.uint64(~0xFFF & _M64)) | \
            np.arange(rows, dtype=np.uint64)
        pick = np.argsort(keys, kind="stable")[:m]
        rest = np.ones(k, dtype=bool)
        rest[flagged] = False
        centers[flagged] = xb[pick].astype(np.float64)
        w[flagged] = w[rest].min()
    c32 = centers.astype(np.float32)
    labels = np.concatenate([np.argmin(_sq_dists(x[a:a + 2048], c32), axis=1)
                             for a in range(0, n, 2048)]).astype(np.int64)
    return centers, labels


# ---- f4: shared neighbours and graph merging (scarf/knn_utils.py:195-274) ---


def calc_snn(indices: np.ndarray) -> np.ndarray:
    """scarf/knn_utils.py:195-211: |set(row i) & set(row of its j-th
    neighbour)| / (k - 1) for every edge."""
    n, k = indices.shape
    sets = [set(r.tolist()) for r in indices]
    snn = np.zeros((n, k))
    for i in range(n):
        for j in range(k):
            snn[i, j] = len(sets[i] & sets[int(indices[i, j])])
    return snn / (k - 1)


def weight_sort_indices(i: np.ndarray, w: np.ndarray, wn: np.ndarray, n: int):
    """scarf/knn_utils.py:214-233: order by wn, largest first, keep the first
    occurrence of each index, the first n. The reference reverses numpy's
    default (unstable) argsort, so tied wn values have no fixed order there;
    here ties put the later candidate first (a stable argsort, reversed)."""
    idx = np.argsort(wn, kind="stable")[::-1]
    i = i[idx]
    w = w[idx]
    _, first = np.unique(i, return_index=True)
    first = sorted(first)
    return i[first][:n], w[first][:n]


def merge_graphs(csr_mats):
    """scarf/knn_utils.py:236-274 (returns a scipy COO matrix)."""
    nk = int(csr_mats[0].indptr[1] - csr_mats[0].indptr[0])
    n = csr_mats[0].shape[0]
    snns = [calc_snn(m.indices.reshape(n, nk)) for m in csr_mats]
    col, data = [], []
    for r in range(n):
        mi = np.hstack([m.indices[m.indptr[r]:m.indptr[r + 1]] for m in csr_mats])
        mw = np.hstack([m.data[m.indptr[r]:m.indptr[r + 1]] for m in csr_mats])
        mwn = np.hstack([m.data[m.indptr[r]:m.indptr[r + 1]] + snns[g][r] for g, m in enumerate(csr_mats)])
        a, b = weight_sort_indices(mi, mw, mwn, nk)
        col.extend(a)
        data.extend(b)
    row = np.repeat(np.arange(n), nk)
    return sp.coo_matrix((data, (row, col)), shape=csr_mats[0].shape)


# ---- f3: the UMAP layout (scarf/umap.py:41-163 over umap-learn) --------------


def umap_find_ab_params(spread: float, min_dist: float):
    """umap-learn find_ab_params (scipy curve_fit of 1 / (1 + a x^(2b)))."""
    from scipy.optimize import curve_fit

    def curve(x, a, b):
        return 1.0 / (1.0 + a * x ** (2 * b))

    xv = np.linspace(0, spread * 3, 300)
    yv = np.zeros(xv.shape)
    yv[xv < min_dist] = 1.0
    yv[xv >= min_dist] = np.exp(-(xv[xv >= min_dist] - min_dist) / spread)
    params, _ = curve_fit(curve, xv, yv)
    return float(params[0]), float(params[1])


def umap_make_epochs_per_sample(weights: np.ndarray, n_epochs: int) -> np.ndarray:
    result = -1.0 * np.ones(weights.shape[0], dtype=np.float64)
    n_samples = n_epochs * (weights / weights.max())
    result[n_samples > 0] = float(n_epochs) / np.float64(n_samples[n_samples > 0])
    return result


def umap_negative_vertex(seed: int, epoch: int, edge: int, p: int, nv: int) -> int:
    """The negative sample p of edge ``edge`` in epoch ``epoch`` as the layout
    kernel draws it: SplitMix64's output function applied once per input
    (seed, then epoch, edge and sample number), modulo the vertex count."""
    def mix(z, v):
        z = (z + v * 0x9E3779B97F4A7C15) & _M64
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
        return z ^ (z >> 31)
    return mix(mix(mix(seed & _M64, epoch), edge), p) % nv


def umap_layout_sequential(y: np.ndarray, head, tail, eps, n_epochs: int, a: float, b: float, gamma: float = 1.0,
                           initial_alpha: float = 1.0, negative_sample_rate: float = 5.0, rand_vertex=None):
    """umap-learn optimize_layout_euclidean, one thread, move_other=True
    (umap/layouts.py of the 0.5 line): edges in order every epoch, with the
    arithmetic of its numba loop -- float32 coordinates and coordinate
    differences, squared distances, gradient coefficients, alpha and the
    sampling schedule in float64, every step rounded back to float32 when it
    is stored. ``rand_vertex(epoch, edge, p)`` draws the negative samples.
    Returns the float32 layout (small cases only: Python loops)."""
    y = np.array(y, dtype=np.float32)
    nv, dim = y.shape
    eps = np.asarray(eps, dtype=np.float64)
    eps_neg = eps / negative_sample_rate
    nxt = eps.copy()
    nxt_neg = eps_neg.copy()
    alpha = initial_alpha
    clip = lambda v: min(4.0, max(-4.0, v))  # noqa: E731
    f32 = np.float32

    def sq_dist(u, v):
        r = 0.0
        for d in range(dim):
            t = float(f32(u[d]) - f32(v[d]))
            r += t * t
        return r

    for n in range(n_epochs):
        for i in range(len(eps)):
            if eps[i] <= 0 or nxt[i] > n:
                continue
            j, k = int(head[i]), int(tail[i])
            cur, oth = y[j], y[k]
            d2 = sq_dist(cur, oth)
            gc = (-2.0 * a * b * d2 ** (b - 1.0) / (a * d2 ** b + 1.0)) if d2 > 0 else 0.0
            for d in range(dim):
                g = clip(gc * float(f32(cur[d]) - f32(oth[d])))
                cur[d] = f32(float(cur[d]) + g * alpha)
                oth[d] = f32(float(oth[d]) + (-g) * alpha)
            nxt[i] += eps[i]
            nneg = int((n - nxt_neg[i]) / eps_neg[i])
            for p in range(nneg):
                kk = int(rand_vertex(n, i, p)) % nv
                o = y[kk]
                e2 = sq_dist(cur, o)
                if e2 > 0:
                    rc = 2.0 * gamma * b / ((0.001 + e2) * (a * e2 ** b + 1.0))
                elif j == kk:
                    continue
                else:
                    rc = 0.0
                for d in range(dim):
                    g = clip(rc * float(f32(cur[d]) - f32(o[d]))) if rc > 0 else 4.0
                    cur[d] = f32(float(cur[d]) + g * alpha)
            nxt_neg[i] += nneg * eps_neg[i]
        alpha = initial_alpha * (1.0 - float(n) / float(n_epochs))
    return y
