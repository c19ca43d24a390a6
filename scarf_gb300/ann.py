"""AnnStream and the exact device kNN index that stands in for hnswlib.

Mirrors scarf/ann.py: ``AnnStream`` takes the same 24 constructor arguments
(scarf/ann.py:56-82) and exposes the attributes scarf's callers read
(``data``, ``k``, ``nCells``, ``nFeats``, ``dims``, ``loadings``, ``mu``,
``sigma``, ``method``, ``reducer``, ``annIdx``, ``kmeans``,
``clusterLabels``, ``harmonizedData``, ``_pca.explained_variance_ratio_``,
``transform_ann``). The PCA is the exact covariance eigendecomposition on the
GPU instead of IncrementalPCA, and the index answers exact squared-L2 queries
on the GPU instead of HNSW. Options of the reference that this build does not
carry raise ``NotImplementedError`` rather than falling back to the CPU.
"""
from __future__ import annotations

import logging
from dataclasses import dataclass
from typing import Optional

import numpy as np
import torch

from . import kernels as K

log = logging.getLogger("scarf_gb300")

__all__ = ["AnnStream", "GpuExactIndex", "NormalizedData", "instantiate_knn_index", "fix_knn_query"]


@dataclass
class NormalizedData:
    """Device-resident normalised matrix (n x ld float32, ``n_feats`` used columns)
    standing where scarf holds a dask array over the ``normed__*/data`` zarr."""
    x: torch.Tensor
    n_feats: int
    chunk_rows: int

    @property
    def shape(self):
        return (self.x.shape[0], self.n_feats)

    @property
    def chunksize(self):
        return (self.chunk_rows, self.n_feats)

    @property
    def numblocks(self):
        return ((self.x.shape[0] + self.chunk_rows - 1) // self.chunk_rows, 1)

    def to_numpy(self) -> np.ndarray:
        return self.x[:, : self.n_feats].double().cpu().numpy()


def _as_device_f32(a, device) -> torch.Tensor:
    t = a if isinstance(a, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(a))
    return t.to(device=device, dtype=torch.float32).contiguous()


class GpuExactIndex:
    """The hnswlib ``Index`` surface used by scarf (scarf/ann.py:14-28, :201-204,
    :322-325; graph_datastore.py:875-879) over exact device kNN: ``add_items``,
    ``knn_query`` (labels uint64, squared-L2 distances float32, as hnswlib's
    'l2' space returns), ``set_ef``/``set_num_threads`` (accepted, no effect:
    the search is exact), ``save_index``/``load_index``."""

    def __init__(self, space: str = "l2", dim: int = 0, precision: str = "plain", margin: Optional[int] = None,
                 device=None):
        if space != "l2":
            raise NotImplementedError(f"only the 'l2' space is built (got {space!r})")
        self.space = space
        self.dim = int(dim)
        self.precision = precision
        self.margin = margin
        self.device = torch.device(device or "cuda")
        self.ef = 0
        self.num_threads = 1
        self._rows = []
        self._scores: Optional[torch.Tensor] = None

    @property
    def ld(self) -> int:
        return K.round_up(max(self.dim, 1), 4)

    def init_index(self, max_elements: int = 0, ef_construction: int = 0, M: int = 0, random_seed: int = 0):
        return None

    def set_ef(self, ef: int):
        self.ef = int(ef)

    def set_num_threads(self, n: int):
        self.num_threads = int(n)

    def _padded(self, a) -> torch.Tensor:
        t = _as_device_f32(a, self.device)
        if t.dim() == 1:
            t = t[None, :]
        if t.shape[1] != self.ld:
            pad = torch.zeros((t.shape[0], self.ld), dtype=torch.float32, device=self.device)
            pad[:, : self.dim] = t[:, : self.dim]
            t = pad
        return t

    def add_items(self, data, ids=None):
        if ids is not None:
            raise NotImplementedError("custom labels are not supported; rows are numbered in insertion order")
        self._rows.append(self._padded(data))
        self._scores = None

    @property
    def scores(self) -> torch.Tensor:
        if self._scores is None:
            self._scores = torch.cat(self._rows) if len(self._rows) > 1 else self._rows[0]
            self._rows = [self._scores]
        return self._scores

    def get_current_count(self) -> int:
        return 0 if not self._rows else int(self.scores.shape[0])

    def knn_query(self, data, k: int = 1, self_offset: int = -1):
        q = self._padded(data)
        idx, dist, nm = K.knn(q, self.scores, self.dim, int(k) if self_offset < 0 else int(k) - 1,
                              self_offset=self_offset, margin=self._margin(), precision=self.precision)
        return idx.cpu().numpy().astype(np.uint64), dist.cpu().numpy(), int(nm.item())

    def _margin(self) -> int:
        if self.margin is not None:
            return self.margin
        return 16 if self.precision == "precision" else 0

    def save_index(self, path: str):
        np.save(path if path.endswith(".npy") else path + ".npy", self.scores[:, : self.dim].cpu().numpy())

    def load_index(self, path: str, max_elements: int = 0):
        a = np.load(path if path.endswith(".npy") else path + ".npy")
        self.dim = a.shape[1]
        self._rows = [self._padded(a)]
        self._scores = None


def instantiate_knn_index(space, dim, max_elements, ef_construction, M, random_seed, ef, num_threads,
                          precision: str = "plain"):
    """scarf/ann.py:14-28 with the exact device index."""
    idx = GpuExactIndex(space=space, dim=dim, precision=precision)
    idx.init_index(max_elements=max_elements, ef_construction=ef_construction, M=M, random_seed=random_seed)
    idx.set_ef(ef)
    idx.set_num_threads(num_threads)
    return idx


def fix_knn_query(indices: np.ndarray, distances: np.ndarray, ref_idx: np.ndarray):
    """scarf/ann.py:31-52 for results that already live on the host: drop the
    self hit of a (k+1)-query (column 0 if self, else the first self
    position, else the last column). The device path fuses this rule into
    ``sg_knn``; this host form exists for callers that pass arrays."""
    ind = np.asarray(indices)
    dist = np.asarray(distances)
    ref = np.asarray(ref_idx).astype(ind.dtype, copy=False)
    is_self = ind == ref[:, None]
    first = is_self[:, 0]
    has = is_self.any(1)
    pos = np.where(has, is_self.argmax(1), ind.shape[1] - 1)
    keep = np.ones_like(is_self)
    keep[np.arange(len(pos)), pos] = False
    k = ind.shape[1] - 1
    return ind[keep].reshape(-1, k), dist[keep].reshape(-1, k), int((~first).sum())


class _PcaInfo:
    def __init__(self, components, evals, evr, n_samples):
        self.components_ = components
        self.explained_variance_ = evals / max(1, n_samples - 1)
        self.explained_variance_ratio_ = evr
        self.n_samples_seen_ = n_samples


class KMeansResult:
    """What make_graph reads from the fitted MiniBatchKMeans: ``cluster_centers_`` (k x dims, float64) and
    ``labels_`` (the predicted label of every cell)."""

    def __init__(self, centers: np.ndarray, labels: np.ndarray):
        self.cluster_centers_ = centers
        self.labels_ = labels
        self.n_clusters = centers.shape[0]


class AnnStream:
    """scarf/ann.py:55-205 on the GPU (see the module docstring)."""

    def __init__(self, data, k: int, n_cluster: int, reduction_method: str, dims: int, loadings, use_for_pca,
                 mu, sigma, ann_metric: str, ann_efc: int, ann_ef: int, ann_m: int, nthreads: int,
                 ann_parallel: bool, rand_state: int, do_kmeans_fit: bool, disable_scaling: bool, ann_idx,
                 lsi_skip_first: bool, lsi_params: dict, harmonize: bool, harmonized_data=None, batches=None,
                 precision: str = "plain", margin: Optional[int] = None):
        if not isinstance(data, NormalizedData):
            arr = np.asarray(data, dtype=np.float32)
            t = torch.zeros((arr.shape[0], K.round_up(arr.shape[1], 4)), dtype=torch.float32, device="cuda")
            t[:, : arr.shape[1]] = torch.from_numpy(arr).cuda()
            data = NormalizedData(t, arr.shape[1], min(arr.shape[0], 1000))
        self.data = data
        self.precision = precision
        self.margin = margin
        self.k = k
        if self.k >= self.data.shape[0]:
            self.k = self.data.shape[0] - 1
        self.nClusters = max(n_cluster, 2)
        self.dims = dims
        self.loadings = loadings
        if self.dims is None and self.loadings is None:
            raise ValueError("ERROR: Provide either value for atleast one: 'dims' or 'loadings'")
        self.annMetric = ann_metric
        self.annEfc, self.annEf, self.annM = ann_efc, ann_ef, ann_m
        self.nthreads = nthreads
        self.annThreads = nthreads if ann_parallel else 1
        self.randState = rand_state
        self.batchSize = self._handle_batch_size()
        self.method = reduction_method
        self.nCells, self.nFeats = self.data.shape
        self.clusterLabels = np.repeat(-1, self.nCells)
        self.harmonize = harmonize
        self.harmonizedData = harmonized_data
        self.batches = batches
        self._pca = None
        if harmonize:
            raise NotImplementedError("harmonize=True (Harmony batch correction) is not part of the GPU path")
        if self.method == "lsi":
            raise NotImplementedError("reduction_method='lsi' (gensim LSI) is not part of the GPU path")
        if self.method not in ("pca", "custom"):
            raise ValueError(f"ERROR: Unknown reduction method: {self.method}")
        disable_reduction = self.dims < 1
        dev = self.data.x.device
        h = self.nFeats
        self.mu = np.asarray(mu, dtype=np.float64) if mu is not None and np.size(mu) == h else None
        self.sigma = np.asarray(sigma, dtype=np.float64) if sigma is not None and np.size(sigma) == h else None
        if self.method == "pca" and (self.mu is None or self.sigma is None):
            raise ValueError("mu and sigma of the normalised data are required for the 'pca' method")
        if self.method == "custom" or disable_scaling:
            self.mu = np.zeros(h) if self.mu is None or disable_scaling else self.mu
            self.sigma = np.ones(h) if self.sigma is None or disable_scaling else self.sigma
        self._mu32 = torch.from_numpy(self.mu.astype(np.float32)).to(dev)
        self._sg32 = torch.from_numpy(self.sigma.astype(np.float32)).to(dev)
        if self.method == "pca" and (self.loadings is None or len(self.loadings) == 0):
            if len(use_for_pca) != self.nCells:
                raise ValueError("ERROR: `use_for_pca` does not have sample length as nCells")
            if not disable_reduction:
                self._fit_pca(use_for_pca)
        elif self.loadings is not None and len(self.loadings) > 0:
            self.dims = self.loadings.shape[1]
        if disable_reduction or self.loadings is None:
            raise NotImplementedError("a reduction to dims >= 1 is required by the GPU path")
        self._l32 = torch.from_numpy(np.ascontiguousarray(self.loadings, dtype=np.float32)).to(dev)
        self.reducer = self._reduce
        self.scores = K.project(self.data.x, self._mu32, self._sg32, self._l32, self.dims, n_cols=h,
                                precision=self.precision)
        if ann_idx is None:
            self.annIdx = GpuExactIndex(self.annMetric, self.dims, precision=precision, margin=margin, device=dev)
            self.annIdx._rows = [self.scores]
        else:
            self.annIdx = ann_idx
            self.annIdx.set_ef(self.annEf)
            self.annIdx.set_num_threads(self.annThreads)
        self.kmeans = self._fit_kmeans(do_kmeans_fit)

    def _fit_kmeans(self, do_kmeans_fit: bool):
        """scarf/ann.py:328-346 on the GPU: MiniBatchKMeans(n_clusters, random_state, batch_size) partial_fit
        over the blocks of the reduced data, then predict (sg_kmeans_minibatch). Sets ``clusterLabels``."""
        if do_kmeans_fit is False:
            return None
        try:
            seed = 0 if self.randState is None else int(self.randState)
            centers, labels = K.kmeans(self.scores, self.dims, int(self.nClusters), int(self.batchSize), seed)
        except ValueError as e:  # sizes outside the kernel's limits: the seeding labels stay -1
            log.warning(f"k-means seeding skipped: {e}")
            return None
        self.clusterLabels = labels.cpu().numpy().astype(np.int64)
        return KMeansResult(centers.cpu().numpy(), self.clusterLabels)

    def _handle_batch_size(self):
        if self.dims is not None and self.dims > self.data.shape[0]:
            self.dims = self.data.shape[0]
        batch_size = self.data.chunksize[0]
        if self.dims is not None and self.dims >= batch_size:
            self.dims = batch_size - 1
            log.info(f"Number of PCA/LSI components reduced to batch size of {batch_size}")
        if self.nClusters > batch_size:
            self.nClusters = batch_size
        return batch_size

    def _fit_pca(self, use_for_pca):
        mask = None
        n_used = self.nCells
        use = np.asarray(use_for_pca, dtype=bool)
        if not use.all():
            mask = torch.from_numpy(use.astype(np.uint8)).to(self.data.x.device)
            n_used = int(use.sum())
        cov, zsum = K.covariance(self.data.x, self._mu32, self._sg32, n_cols=self.nFeats, row_mask=mask,
                                 precision=self.precision)
        comps, evals, evr, _ = K.pca_basis(cov, zsum, n_used, self.dims + 1, n_load=self.dims, ld_l=self.dims,
                                           eigh="filter" if self.precision == "precision" else "fp64")
        c = comps.cpu().numpy()
        self._pca = _PcaInfo(c.T, evals.cpu().numpy(), evr.cpu().numpy(), n_used)
        self.loadings = c[:, :-1]

    def transform_z(self, a: np.ndarray) -> np.ndarray:
        return (a - self.mu) / self.sigma

    def _reduce(self, a) -> np.ndarray:
        """((a - mu)/sigma) . L on the GPU for host or device rows."""
        t = _as_device_f32(a, self.data.x.device)
        if t.shape[1] % 4:
            t = torch.nn.functional.pad(t, (0, 4 - t.shape[1] % 4))
        s = K.project(t, self._mu32, self._sg32, self._l32, self.dims, n_cols=self.nFeats,
                      precision=self.precision)
        return s[:, : self.dims].double().cpu().numpy()

    def transform_ann(self, a, k: Optional[int] = None, self_indices: Optional[np.ndarray] = None):
        """scarf/ann.py:194-205: plain query, or a (k+1)-query with self removed
        for a contiguous range of reference rows."""
        if k is None:
            k = self.k
        if self_indices is None:
            i, d, _ = self.annIdx.knn_query(a, k=k)
            return i, d
        si = np.asarray(self_indices)
        if len(si) and not np.array_equal(si, np.arange(si[0], si[0] + len(si))):
            raise ValueError("self_indices must be a contiguous range of reference rows")
        i, d, nm = self.annIdx.knn_query(a, k=k + 1, self_offset=int(si[0]) if len(si) else 0)
        return i, d, nm
