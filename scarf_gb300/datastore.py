"""``DataStore`` with scarf's graph entry points on the GPU path.

``make_graph``, ``load_graph`` and ``run_mapping`` keep the reference's
keyword arguments, defaults (scarf/datastore/graph_datastore.py:139-149,
:272, :298-303), the parameter-named group hierarchy used as a step cache
(:738-745), the dataset names and dtypes, and the ``latest_*`` attributes
(:1003-1008), so downstream readers of the store see the layout they expect.
Counts are CSR (int32) instead of a dense zarr array; normalised data stays on
the device (its float64 ``data`` dataset is written only when
``persist_normed=True``).
"""
from __future__ import annotations

import os

import logging
from typing import Optional

import numpy as np
import scipy.sparse as sp
import torch

from . import kernels as K
from .ann import AnnStream, GpuExactIndex, NormalizedData
from .knn_utils import self_query_knn, smoothen_dists
from .pipeline import col_map as _col_map
from .pipeline import normalize_csr_host
from .store import Group, create_zarr_dataset

log = logging.getLogger("scarf_gb300")

__all__ = ["MetaData", "RNAassay", "DataStore"]

DEFAULTS = {"log_transform": True, "renormalize_subset": True, "dims": 11, "ann_metric": "l2", "rand_state": 4466,
            "k": 11, "n_centroids": 1000, "local_connectivity": 1.0, "bandwidth": 1.5}


def rescale_array(a: np.ndarray, frac: float = 0.9) -> np.ndarray:
    """scarf/utils.py:120-140: clamp to the frac and 1 - frac quantiles of a
    normal with the vector's (median-centred) location and standard deviation."""
    from scipy.stats import norm
    loc = (np.median(a) + np.median(a[::-1])) / 2
    dist = norm(loc, np.std(a))
    minv, maxv = dist.ppf(1 - frac), dist.ppf(frac)
    a[a < minv] = minv
    a[a > maxv] = maxv
    return a


def pca_fit_transform(x: np.ndarray, n_components: int) -> np.ndarray:
    """scikit-learn PCA(n_components).fit_transform on a small dense matrix:
    centred, SVD, signs by svd_flip on the components (the largest-magnitude
    entry of each component positive), scores = centred x . components^T."""
    xc = x - x.mean(0)
    _, _, vt = np.linalg.svd(xc, full_matrices=False)
    vt = vt[:n_components]
    signs = np.sign(vt[np.arange(vt.shape[0]), np.argmax(np.abs(vt), axis=1)])
    signs[signs == 0] = 1.0
    return xc @ (vt * signs[:, None]).T


class MetaData:
    """Column table of cells or features (the part of scarf/metadata.py the
    graph path reads: boolean keys, ``fetch``, ``active_index``)."""

    def __init__(self, n: int, ids=None):
        self.N = int(n)
        self._c = {"I": np.ones(self.N, dtype=bool)}
        if ids is not None:
            self._c["ids"] = np.asarray(ids)

    @property
    def columns(self):
        return list(self._c)

    def fetch_all(self, column: str) -> np.ndarray:
        return self._c[column]

    def fetch(self, column: str, key: str = "I") -> np.ndarray:
        return self._c[column][self._c[key]]

    def active_index(self, key: str) -> np.ndarray:
        v = self._c[key]
        if v.dtype != bool:
            raise ValueError(f"ERROR: column {key} is not boolean")
        return np.nonzero(v)[0]

    def get_dtype(self, column: str):
        return self._c[column].dtype

    def insert(self, column: str, values, fill_value=False, key: str = "I", overwrite: bool = False):
        if column in self._c and not overwrite:
            raise ValueError(f"ERROR: {column} exists; use overwrite=True")
        values = np.asarray(values)
        if len(values) == self.N:
            self._c[column] = values
        else:
            full = np.full(self.N, fill_value, dtype=values.dtype)
            full[self._c[key]] = values
            self._c[column] = full


class RNAassay:
    """CSR counts of one RNA assay with ``save_normalized_data`` on the GPU
    (scarf/assay.py:400-478, :780-828)."""

    def __init__(self, name: str, indptr, indices, data, n_genes: int, cells: MetaData, feats: MetaData,
                 z: Group, device="cuda"):
        self.name = name
        ip = np.ascontiguousarray(indptr, dtype=np.int64)
        ind = np.ascontiguousarray(indices, dtype=np.int32)
        dat = np.ascontiguousarray(data, dtype=np.int32)
        self._pinned = None
        if torch.device(device).type == "cuda" and torch.cuda.is_available() and len(ind):
            # page-locked copies, which the normalisation kernel reads over the
            # host link itself (no staging copy of the counts on the device);
            # when the host cannot lock that much memory the counts stay
            # pageable and are copied to the device instead
            try:
                self._pinned = [torch.from_numpy(a).pin_memory() for a in (ip, ind, dat)]
                ip, ind, dat = (t.numpy() for t in self._pinned)
            except RuntimeError as e:
                log.warning(f"counts stay in pageable memory ({e}); they are copied to the device per use")
                self._pinned = None
        self.indptr, self.indices, self.data = ip, ind, dat
        self.n_genes = int(n_genes)
        self.cells = cells
        self.feats = feats
        self.z = z
        self.attrs = z.attrs
        self.attrs.setdefault("size_factor", 1000)
        self.sf = int(self.attrs["size_factor"])
        self.device = torch.device(device)
        self._normed_cache = {}

    def n_counts(self) -> np.ndarray:
        lib = np.add.reduceat(self.data.astype(np.int64), self.indptr[:-1]) if len(self.data) else 0
        lib = np.where(np.diff(self.indptr) > 0, lib, 0)
        return lib.astype(np.float64)

    def _rows(self, cell_idx: np.ndarray):
        if len(cell_idx) == len(self.indptr) - 1:
            return self.indptr, self.indices, self.data
        m = sp.csr_matrix((self.data, self.indices, self.indptr), shape=(len(self.indptr) - 1, self.n_genes))
        s = m[cell_idx]
        return s.indptr.astype(np.int64), s.indices.astype(np.int32), s.data.astype(np.int32)

    def save_normalized_data(self, cell_key: str, feat_key: str, batch_size: int, location: str,
                             log_transform: bool, renormalize_subset: bool, update_keys: bool,
                             persist_normed: bool = False):
        fk = feat_key if feat_key == "I" else cell_key + "__" + feat_key
        cell_idx = self.cells.active_index(cell_key)
        feat_idx = self.feats.active_index(fk)
        subset_hash = hash((hash(tuple(cell_idx)), hash(tuple(feat_idx))))
        params = {"log_transform": bool(log_transform), "renormalize_subset": bool(renormalize_subset)}
        ck = (location, subset_hash, tuple(sorted(params.items())))
        if update_keys:
            self.attrs["latest_feat_key"] = feat_key
            self.attrs["latest_cell_key"] = cell_key
        if ck in self._normed_cache and location in self.z and self.z[location].attrs.get("subset_hash") == subset_hash:
            log.info(f"Using existing normalized data with cell key {cell_key} and feat key {feat_key}")
            return self._normed_cache[ck]
        g = self.z.create_group(location, overwrite=True)
        h = len(feat_idx)
        dev = self.device
        if self._pinned is not None and len(cell_idx) == len(self.indptr) - 1:
            rows = self._pinned     # read in place over the host link
        else:
            rows = [torch.from_numpy(a) for a in self._rows(cell_idx)]   # one copy to the device
        nc = None if renormalize_subset else self.n_counts()[cell_idx]
        x, cs, cq = normalize_csr_host(*rows, self.n_genes, feat_idx, size_factor=self.sf,
                                       log_transform=log_transform, renormalize_subset=renormalize_subset,
                                       n_counts=nc, chunk_cells=0, device=dev)
        nd = NormalizedData(x, h, batch_size)
        nd.colsum, nd.colsumsq = cs, cq
        if persist_normed:
            ds = create_zarr_dataset(g, "data", (batch_size,), "f8", nd.shape)
            ds[:, :] = nd.to_numpy()
        g.attrs["subset_hash"] = subset_hash
        g.attrs["subset_params"] = params
        self._normed_cache = {ck: nd}
        return nd


class DataStore:
    """Graph construction and mapping of scarf's DataStore on one GPU."""

    def __init__(self, indptr, indices, data, n_genes: int, gene_ids=None, cell_ids=None, store=None,
                 assay_name: str = "RNA", nthreads: int = 2, precision: str = "plain", device="cuda"):
        self.z = store if store is not None else Group()
        self.zw = self.z
        self.nthreads = nthreads
        self.precision = precision
        n_cells = len(indptr) - 1
        self.cells = MetaData(n_cells, cell_ids if cell_ids is not None else np.arange(n_cells).astype(str))
        feats = MetaData(n_genes, gene_ids if gene_ids is not None else np.arange(n_genes).astype(str))
        self._defaultAssay = assay_name
        self._assays = {assay_name: RNAassay(assay_name, indptr, indices, data, n_genes, self.cells, feats,
                                             self.z.require_group(assay_name), device)}
        setattr(self, assay_name, self._assays[assay_name])
        self._ann_cache = {}

    @classmethod
    def from_zarr(cls, store: str, assay_name: str = "RNA", precision: str = "plain", device="cuda",
                  **kw) -> "DataStore":
        """A DataStore over a scarf zarr directory store: the assay's count
        chunks (``{assay}/counts``, Blosc-LZ4) decoded and turned into CSR on
        the device, gene ids from ``{assay}/featureData/ids`` and cell ids
        from ``cellData/ids`` when present (scarf/writers.py:58-89, :164-204)."""
        from .zarr_io import read_counts_csr, read_strings
        ip, ind, dat, n_genes = read_counts_csr(store, f"{assay_name}/counts", device=device)
        gid = f"{assay_name}/featureData/ids"
        genes = read_strings(store, gid, device) if os.path.exists(os.path.join(store, gid, ".zarray")) else None
        cells = read_strings(store, "cellData/ids", device) \
            if os.path.exists(os.path.join(store, "cellData", "ids", ".zarray")) else None
        return cls(ip.cpu().numpy(), ind.cpu().numpy(), dat.cpu().numpy(), n_genes, gene_ids=genes, cell_ids=cells,
                   assay_name=assay_name, precision=precision, device=device, **kw)

    def to_zarr(self, store: str, chunk_size=(1000, 1000)) -> None:
        """The DataStore as a scarf zarr directory store, every chunk encoded
        on the device (Blosc-LZ4, bit shuffle): each assay's counts as a dense
        ``<u4`` array in chunks of ``chunk_size`` (scarf/writers.py:164-204),
        the cell and feature tables (``cellData/{column}``,
        ``{assay}/featureData/{column}``) and every group and dataset the graph
        path wrote. ``DataStore.from_zarr`` reads it back."""
        from .zarr_io import write_counts, write_group, write_table
        write_group(store, self.z, device=self.RNA.device if hasattr(self, "RNA") else "cuda")
        write_table(store, "cellData", self.cells)
        for name, a in self._assays.items():
            write_counts(store, f"{name}/counts", a.indptr, a.indices, a.data, a.n_genes, chunk_size, device=a.device)
            write_table(store, f"{name}/featureData", a.feats, device=a.device)

    def _get_assay(self, name: Optional[str]):
        return self._assays[name or self._defaultAssay]

    # -- cached-parameter resolution (graph_datastore.py:88-346) ------------
    def _set_graph_params(self, from_assay, cell_key, feat_key, log_transform, renormalize_subset, dims,
                          pca_cell_key, ann_metric, ann_efc, ann_ef, ann_m, rand_state, k, n_centroids,
                          local_connectivity, bandwidth, reduction_method="pca"):
        zw = self.zw
        normed_loc = f"{from_assay}/normed__{cell_key}__{feat_key}"
        if log_transform is None or renormalize_subset is None:
            sp_ = zw[normed_loc].attrs.get("subset_params") if normed_loc in zw else None
            if log_transform is None:
                log_transform = sp_["log_transform"] if sp_ else DEFAULTS["log_transform"]
            if renormalize_subset is None:
                renormalize_subset = sp_["renormalize_subset"] if sp_ else DEFAULTS["renormalize_subset"]
        if dims is None or pca_cell_key is None:
            c_dims = c_pck = None
            if normed_loc in zw and "latest_reduction" in zw[normed_loc].attrs:
                c_dims, c_pck = zw[normed_loc].attrs["latest_reduction"].rsplit("__", 2)[1:]
            if dims is None:
                dims = int(c_dims) if c_dims is not None else DEFAULTS["dims"]
            if pca_cell_key is None:
                pca_cell_key = c_pck if c_pck is not None else cell_key
        dims = int(dims)
        reduction_loc = f"{normed_loc}/reduction__{reduction_method}__{dims}__{pca_cell_key}"
        cached_ann = None
        if reduction_loc in zw and "latest_ann" in zw[reduction_loc].attrs:
            cached_ann = zw[reduction_loc].attrs["latest_ann"].rsplit("/", 1)[1].split("__")[1:]
        if ann_metric is None:
            ann_metric = cached_ann[0] if cached_ann else DEFAULTS["ann_metric"]
        if ann_m is None:
            ann_m = int(cached_ann[3]) if cached_ann else min(max(48, int(dims * 1.5)), 64)
        if rand_state is None:
            rand_state = int(cached_ann[4]) if cached_ann else DEFAULTS["rand_state"]
        if k is None:
            if cached_ann is not None:
                ann_loc = zw[reduction_loc].attrs["latest_ann"]
                k = int(zw[ann_loc].attrs["latest_knn"].rsplit("__", 1)[1])
            else:
                k = DEFAULTS["k"]
        k = int(k)
        if ann_ef is None:
            ann_ef = int(cached_ann[2]) if cached_ann else min(100, max(k * 3, 50))
        if ann_efc is None:
            ann_efc = int(cached_ann[1]) if cached_ann else min(100, max(k * 3, 50))
        if n_centroids is None:
            n_centroids = DEFAULTS["n_centroids"]
        ann_loc = f"{reduction_loc}/ann__{ann_metric}__{ann_efc}__{ann_ef}__{ann_m}__{rand_state}"
        knn_loc = f"{ann_loc}/knn__{k}"
        if local_connectivity is None or bandwidth is None:
            c_lc = c_bw = None
            if knn_loc in zw and "latest_graph" in zw[knn_loc].attrs:
                c_lc, c_bw = map(float, zw[knn_loc].attrs["latest_graph"].rsplit("/")[-1].split("__")[1:])
            if local_connectivity is None:
                local_connectivity = c_lc if c_lc is not None else DEFAULTS["local_connectivity"]
            if bandwidth is None:
                bandwidth = c_bw if c_bw is not None else DEFAULTS["bandwidth"]
        return (bool(log_transform), bool(renormalize_subset), dims, pca_cell_key, str(ann_metric), int(ann_efc),
                int(ann_ef), int(ann_m), int(rand_state), k, int(n_centroids), float(local_connectivity),
                float(bandwidth))

    # -- make_graph (graph_datastore.py:513-1020) ----------------------------
    def make_graph(self, from_assay: Optional[str] = None, cell_key: Optional[str] = None,
                   feat_key: Optional[str] = None, pca_cell_key: Optional[str] = None, reduction_method: str = "auto",
                   dims: Optional[int] = None, k: Optional[int] = None, ann_metric: Optional[str] = None,
                   ann_efc: Optional[int] = None, ann_ef: Optional[int] = None, ann_m: Optional[int] = None,
                   ann_parallel: bool = False, rand_state: Optional[int] = None, n_centroids: Optional[int] = None,
                   batch_size: Optional[int] = None, log_transform: Optional[bool] = None,
                   renormalize_subset: Optional[bool] = None, local_connectivity: Optional[float] = None,
                   bandwidth: Optional[float] = None, update_keys: bool = True, return_ann_object: bool = False,
                   custom_loadings: Optional[np.ndarray] = None, feat_scaling: bool = True,
                   lsi_skip_first: bool = True, harmonize: bool = False, batch_columns=None,
                   show_elbow_plot: bool = False, ann_index_fetcher=None, ann_index_saver=None,
                   persist_normed: bool = False):
        from_assay = from_assay or self._defaultAssay
        assay = self._get_assay(from_assay)
        if batch_size is None:
            batch_size = 1000
        cell_key = cell_key or "I"
        if feat_key is None:
            raise ValueError("ERROR: You have to choose which features that should be used for graph construction.")
        if harmonize:
            raise NotImplementedError("harmonize=True (Harmony batch correction) is not part of the GPU path")
        if reduction_method == "auto":
            reduction_method = "pca"
        if reduction_method not in ("pca", "custom"):
            raise NotImplementedError(f"reduction_method={reduction_method!r} is not part of the GPU path")
        if custom_loadings is not None:
            reduction_method = "custom"
            dims = custom_loadings.shape[1]
        (log_transform, renormalize_subset, dims, pca_cell_key, ann_metric, ann_efc, ann_ef, ann_m, rand_state, k,
         n_centroids, local_connectivity, bandwidth) = self._set_graph_params(
            from_assay, cell_key, feat_key, log_transform, renormalize_subset, dims, pca_cell_key, ann_metric,
            ann_efc, ann_ef, ann_m, rand_state, k, n_centroids, local_connectivity, bandwidth, reduction_method)
        zw = self.zw
        normed_loc = f"{from_assay}/normed__{cell_key}__{feat_key}"
        reduction_loc = f"{normed_loc}/reduction__{reduction_method}__{dims}__{pca_cell_key}"
        ann_loc = f"{reduction_loc}/ann__{ann_metric}__{ann_efc}__{ann_ef}__{ann_m}__{rand_state}"
        knn_loc = f"{ann_loc}/knn__{k}"
        kmeans_loc = f"{reduction_loc}/kmeans__{n_centroids}__{rand_state}"
        graph_loc = f"{knn_loc}/graph__{local_connectivity}__{bandwidth}"
        data = assay.save_normalized_data(cell_key, feat_key, batch_size, normed_loc.split("/", 1)[1],
                                          log_transform, renormalize_subset, update_keys, persist_normed)
        if custom_loadings is not None and data.shape[1] != custom_loadings.shape[0]:
            raise ValueError("Provided custom loadings do not match the number of features")
        n = data.shape[0]
        if "mu" in zw[normed_loc] and "sigma" in zw[normed_loc]:
            mu, sigma = zw[normed_loc]["mu"][:], zw[normed_loc]["sigma"][:]
        else:
            mu_t, sg_t, _, _ = K.zstats(data.colsum, data.colsumsq, n)
            mu, sigma = mu_t.cpu().numpy(), sg_t.cpu().numpy()
            create_zarr_dataset(zw[normed_loc], "mu", (100000,), "f8", mu.shape)[:] = mu
            create_zarr_dataset(zw[normed_loc], "sigma", (100000,), "f8", sigma.shape)[:] = sigma
        loadings = None
        if reduction_loc in zw and "reduction" in zw[reduction_loc]:
            loadings = zw[reduction_loc]["reduction"][:]
            if loadings.shape[0] != data.shape[1]:
                loadings = None
                del zw[reduction_loc]
        if custom_loadings is not None:
            loadings = np.asarray(custom_loadings, dtype=np.float64)
        use_for_pca = self.cells.fetch(pca_cell_key, key=cell_key) if pca_cell_key in self.cells.columns \
            else np.ones(n, dtype=bool)
        ann_obj = AnnStream(data=data, k=k, n_cluster=n_centroids, reduction_method=reduction_method, dims=dims,
                            loadings=loadings, use_for_pca=use_for_pca, mu=mu, sigma=sigma, ann_metric=ann_metric,
                            ann_efc=ann_efc, ann_ef=ann_ef, ann_m=ann_m, nthreads=self.nthreads,
                            ann_parallel=ann_parallel, rand_state=rand_state, do_kmeans_fit=kmeans_loc not in zw,
                            disable_scaling=not feat_scaling, ann_idx=None, lsi_skip_first=lsi_skip_first,
                            lsi_params={}, harmonize=harmonize, precision=self.precision)
        if reduction_loc not in zw or "reduction" not in zw[reduction_loc]:
            g = zw.create_group(reduction_loc, overwrite=reduction_loc not in zw)
            create_zarr_dataset(g, "reduction", data.chunksize, "f8", ann_obj.loadings.shape)[:, :] = ann_obj.loadings
        if ann_obj.kmeans is not None:
            # graph_datastore.py:958-975: centres and labels of the seeding k-means
            g = zw.create_group(kmeans_loc, overwrite=True)
            cc = ann_obj.kmeans.cluster_centers_
            create_zarr_dataset(g, "cluster_centers", (1000, 1000), "f8", cc.shape)[:, :] = cc
            create_zarr_dataset(g, "cluster_labels", (100000,), "f8", ann_obj.clusterLabels.shape)[:] = \
                ann_obj.clusterLabels
        if ann_loc not in zw:
            zw.create_group(ann_loc)
        if ann_index_saver is not None:
            try:
                ann_index_saver(ann_obj.annIdx, ann_loc)
            except Exception:
                log.warning("Custom `ann_index_saver` failed")
        if knn_loc in zw and graph_loc in zw and "indices" in zw[knn_loc]:
            log.info("KNN graph already exists will not recompute.")
        else:
            recall = None
            if knn_loc not in zw or "indices" not in zw[knn_loc]:
                recall = self_query_knn(ann_obj, zw.create_group(knn_loc, overwrite=True), batch_size, self.nthreads)
            smoothen_dists(zw.create_group(graph_loc, overwrite=True), zw[knn_loc]["indices"],
                           zw[knn_loc]["distances"], local_connectivity, bandwidth, batch_size)
            if recall is not None:
                log.info("ANN recall: %.2f%%" % recall)
                zw[knn_loc].attrs["recall"] = float(recall)
        zw[normed_loc].attrs["latest_reduction"] = reduction_loc
        zw[reduction_loc].attrs["latest_ann"] = ann_loc
        zw[reduction_loc].attrs["latest_kmeans"] = kmeans_loc
        zw[ann_loc].attrs["isHarmonized"] = harmonize
        zw[ann_loc].attrs["latest_knn"] = knn_loc
        zw[knn_loc].attrs["latest_graph"] = graph_loc
        self._ann_cache[ann_loc] = ann_obj
        if return_ann_object:
            return ann_obj
        return None

    def _get_latest_graph_loc(self, from_assay: str, cell_key: str, feat_key: str) -> str:
        normed_loc = f"{from_assay}/normed__{cell_key}__{feat_key}"
        reduction_loc = self.zw[normed_loc].attrs["latest_reduction"]
        ann_loc = self.zw[reduction_loc].attrs["latest_ann"]
        knn_loc = self.zw[ann_loc].attrs["latest_knn"]
        return self.zw[knn_loc].attrs["latest_graph"]

    # -- load_graph (graph_datastore.py:1022-1075) ---------------------------
    def load_graph(self, from_assay: Optional[str] = None, cell_key: Optional[str] = None,
                   feat_key: Optional[str] = None, symmetric: Optional[bool] = None,
                   upper_only: Optional[bool] = None, use_k: Optional[int] = None,
                   graph_loc: Optional[str] = None) -> sp.csr_matrix:
        from_assay = from_assay or self._defaultAssay
        assay = self._get_assay(from_assay)
        cell_key = cell_key or assay.attrs.get("latest_cell_key", "I")
        feat_key = feat_key or assay.attrs.get("latest_feat_key")
        if graph_loc is None:
            graph_loc = self._get_latest_graph_loc(from_assay, cell_key, feat_key)
        if graph_loc not in self.zw:
            raise ValueError(f"{graph_loc} not found in zarr location. Run `make_graph` for assay {from_assay}")
        n_cells, k = self.zw[graph_loc.rsplit("/", 1)[0]]["indices"].shape
        if use_k is None:
            use_k = k
        use_k = max(1, min(use_k, k))
        e = np.asarray(self.zw[graph_loc]["edges"][:]).astype(np.int64)
        w = np.asarray(self.zw[graph_loc]["weights"][:], dtype=np.float64)
        if symmetric:
            ip, ind, dat = K.fuzzy_union(torch.from_numpy(e).cuda(), torch.from_numpy(w).cuda(), n_cells, k,
                                         use_k=use_k, mix=1.0, upper_only=bool(upper_only))
            return sp.csr_matrix((dat.cpu().numpy(), ind.cpu().numpy(), ip.cpu().numpy()), shape=(n_cells, n_cells))
        if use_k != k:
            keep = np.tile([True] * use_k + [False] * (k - use_k), n_cells)
            e, w = e[keep], w[keep]
        return sp.csr_matrix((w, (e[:, 0], e[:, 1])), shape=(n_cells, n_cells))

    # -- UMAP (graph_datastore.py:427-457, :1218-1380) ---------------------------
    @staticmethod
    def _col_renamer(from_assay: str, cell_key: str, suffix: str) -> str:
        """base_datastore.py:404-420."""
        return "_".join(map(str, [from_assay, suffix] if cell_key == "I" else [from_assay, cell_key, suffix]))

    def _get_ini_embed(self, from_assay: str, cell_key: str, feat_key: str, n_comps: int) -> np.ndarray:
        """graph_datastore.py:427-457: PCA of the seeding k-means centres, each
        component edge-trimmed by ``rescale_array``, given to every cell by its
        cluster label."""
        normed_loc = f"{from_assay}/normed__{cell_key}__{feat_key}"
        reduction_loc = self.zw[normed_loc].attrs["latest_reduction"]
        kmeans_loc = self.zw[reduction_loc].attrs["latest_kmeans"]
        if kmeans_loc not in self.zw:
            raise KeyError(f"{kmeans_loc} not found: the seeding k-means was not fitted")
        pc = pca_fit_transform(np.asarray(self.zw[kmeans_loc]["cluster_centers"][:], dtype=np.float64), n_comps)
        for i in range(n_comps):
            pc[:, i] = rescale_array(pc[:, i])
        clusters = np.asarray(self.zw[kmeans_loc]["cluster_labels"][:]).astype(np.uint32)
        return np.array([pc[x] for x in clusters]).astype(np.float32, order="C")

    def run_umap(self, from_assay: Optional[str] = None, cell_key: Optional[str] = None,
                 feat_key: Optional[str] = None, symmetric_graph: Optional[bool] = False,
                 graph_upper_only: Optional[bool] = False, ini_embed: Optional[np.ndarray] = None,
                 umap_dims: int = 2, spread: float = 2.0, min_dist: float = 1, n_epochs: int = 300,
                 repulsion_strength: float = 1.0, initial_alpha: float = 1.0, negative_sample_rate: float = 5,
                 use_density_map: bool = False, dens_lambda: float = 2.0, dens_frac: float = 0.3,
                 dens_var_shift: float = 0.1, random_seed: int = 4444, label: str = "UMAP",
                 integrated_graph: Optional[str] = None, parallel: bool = False,
                 nthreads: Optional[int] = None) -> None:
        """graph_datastore.py:1218-1380 with the layout on the GPU
        (scarf_gb300.umap.fit_transform). densMAP and integrated graphs are not
        part of this build."""
        from .umap import fit_transform
        if use_density_map:
            raise NotImplementedError("densMAP is not part of the GPU path")
        if integrated_graph is not None:
            raise NotImplementedError("integrated graphs are not part of the GPU path")
        from_assay = from_assay or self._defaultAssay
        assay = self._get_assay(from_assay)
        cell_key = cell_key or assay.attrs.get("latest_cell_key", "I")
        feat_key = feat_key or assay.attrs.get("latest_feat_key")
        graph = self.load_graph(from_assay=from_assay, cell_key=cell_key, feat_key=feat_key,
                                symmetric=symmetric_graph, upper_only=graph_upper_only)
        if ini_embed is None:
            ini_embed = self._get_ini_embed(from_assay, cell_key, feat_key, umap_dims)
        t, a, b = fit_transform(graph=graph.tocoo(), ini_embed=ini_embed, spread=spread, min_dist=min_dist,
                                n_epochs=n_epochs, random_seed=random_seed, repulsion_strength=repulsion_strength,
                                initial_alpha=initial_alpha, negative_sample_rate=negative_sample_rate,
                                densmap_kwds={}, parallel=parallel, nthreads=nthreads or self.nthreads,
                                verbose=False)
        for i in range(umap_dims):
            self.cells.insert(self._col_renamer(from_assay, cell_key, f"{label}{i + 1}"), t[:, i], key=cell_key,
                              overwrite=True)
        return None

    # -- run_mapping (mapping_datastore.py:31-209) -----------------------------
    def run_mapping(self, target_assay: RNAassay, target_name: str, target_feat_key: str,
                    target_cell_key: str = "I", from_assay: Optional[str] = None, cell_key: str = "I",
                    feat_key: Optional[str] = None, save_k: int = 3, batch_size: int = 1000, ref_mu: bool = True,
                    ref_sigma: bool = True, run_coral: bool = False, exclude_missing: bool = False,
                    filter_null: bool = False, feat_scaling: bool = True, ann_index_fetcher=None,
                    ann_index_saver=None) -> None:
        from_assay = from_assay or self._defaultAssay
        source = self._get_assay(from_assay)
        feat_key = feat_key or source.attrs.get("latest_feat_key")
        if target_feat_key == feat_key:
            raise ValueError(f"ERROR: `target_feat_key` cannot be sample as `feat_key`: {feat_key}")
        if run_coral or exclude_missing or not ref_mu or not ref_sigma:
            raise NotImplementedError("run_coral, exclude_missing and target-derived mu/sigma are not part of "
                                      "the GPU mapping path")
        if target_assay.sf != source.sf:
            target_assay.sf = source.sf
        ann_obj = self.make_graph(from_assay=from_assay, cell_key=cell_key, feat_key=feat_key,
                                  return_ann_object=True, update_keys=False, feat_scaling=feat_scaling)
        if save_k > ann_obj.k:
            save_k = ann_obj.k
        ref_ids = source.feats.fetch("ids", key=cell_key + "__" + feat_key)
        norm_params = self.zw[f"{from_assay}/normed__{cell_key}__{feat_key}"].attrs["subset_params"]
        t_ids = target_assay.feats.fetch_all("ids")
        cmap, missing = align_col_map(ref_ids, t_ids)
        ip, ind, dat = target_assay._rows(target_assay.cells.active_index(target_cell_key))
        idx, dist = map_cells(ann_obj, ip, ind, dat, cmap, missing, save_k, target_assay.sf, norm_params)
        store = self.zw.require_group(f"{from_assay}/projections").create_group(target_name, overwrite=True)
        nc = len(ip) - 1
        create_zarr_dataset(store, "indices", (batch_size,), "u8", (nc, save_k))[:, :] = idx.astype(np.uint64)
        create_zarr_dataset(store, "distances", (batch_size,), "f8", (nc, save_k))[:, :] = dist.astype(np.float64)
        return None


def align_col_map(ref_ids: np.ndarray, target_ids: np.ndarray):
    """Target gene -> reference feature column (or -1), and the mask of
    reference features absent from the target (filled with 1.0 after
    normalisation, scarf/mapping_utils.py:148-214)."""
    pos = {v: j for j, v in enumerate(ref_ids)}
    cmap = np.full(len(target_ids), -1, dtype=np.int32)
    for g, v in enumerate(target_ids):
        j = pos.get(v)
        if j is not None:
            cmap[g] = j
    missing = np.ones(len(ref_ids), dtype=np.uint8)
    missing[cmap[cmap >= 0]] = 0
    return cmap, missing


def map_cells(ann_obj: AnnStream, indptr, indices, data, cmap: np.ndarray, missing: np.ndarray, k: int,
              size_factor: float, norm_params: dict):
    """Normalise target cells onto the reference features, project with the
    reference's mu/sigma/loadings and query the reference cells
    (mapping_datastore.py:198-208). Returns host (indices, distances)."""
    dev = ann_obj.data.x.device
    h = ann_obj.nFeats
    x = K.normalize_csr(torch.from_numpy(np.asarray(indptr, np.int64)).to(dev),
                        torch.from_numpy(np.asarray(indices, np.int32)).to(dev),
                        torch.from_numpy(np.asarray(data, np.int32)).to(dev), torch.from_numpy(cmap).to(dev), h,
                        size_factor=size_factor, log_transform=norm_params["log_transform"],
                        renormalize_subset=norm_params["renormalize_subset"],
                        missing_mask=torch.from_numpy(missing).to(dev), fill_value=1.0)
    s = K.project(x, ann_obj._mu32, ann_obj._sg32, ann_obj._l32, ann_obj.dims, n_cols=h,
                  precision=ann_obj.annIdx.precision)
    idx, dist, _ = K.knn(s, ann_obj.annIdx.scores, ann_obj.dims, k, self_offset=-1,
                         margin=ann_obj.annIdx._margin(), precision=ann_obj.annIdx.precision)
    return idx.cpu().numpy(), dist.cpu().numpy()
