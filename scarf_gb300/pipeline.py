"""The make_graph hot path on one GPU, from CSR counts to the smoothed graph.

normalise (+ column sums) -> z-statistics -> scatter -> FP64 eigh -> projection
-> exact self-kNN (+ self removal, recall) -> smoothing, all resident in HBM.
The CSR may be given as CUDA tensors, as page-locked host tensors (which the
normalisation kernel reads over the host link itself, with no staging copy)
or as other host arrays (copied in chunks of cells, the copy of chunk i+1
overlapping the normalisation of chunk i).

Step order and parameters follow DataStore.make_graph
(scarf/datastore/graph_datastore.py:513-1020).
"""
from __future__ import annotations

import threading
from dataclasses import dataclass, field
from typing import Optional

import numpy as np
import torch

from . import kernels as K

PLAIN_MARGIN = 0
# rows per FP32 slice of sg_normalize_csr's column statistics
STAT_ROWS = 256
PRECISION_MARGIN = 16
# covariance forms with a kernel in this build
COV_FORMS = ("plain", "precision")


@dataclass
class GraphResult:
    n_cells: int
    n_feats: int
    dims: int
    k: int
    x: Optional[torch.Tensor]          # normalised rows (n x ld), float32
    mu: torch.Tensor                   # float64
    sigma: torch.Tensor                # float64
    mu32: torch.Tensor
    sigma32: torch.Tensor
    components: torch.Tensor           # h x (dims+1) float64
    loadings32: torch.Tensor           # h x dims float32
    evals: torch.Tensor
    evr: torch.Tensor
    scores: torch.Tensor               # n x ld_s float32
    indices: torch.Tensor              # n x k int64
    distances: torch.Tensor            # n x k float32
    n_missed: torch.Tensor             # device int64
    edges: Optional[torch.Tensor] = None
    weights: Optional[torch.Tensor] = None
    timings: dict = field(default_factory=dict)

    @property
    def loadings(self) -> torch.Tensor:
        return self.components[:, : self.dims]

    def recall(self) -> float:
        return 100.0 * (self.n_cells - int(self.n_missed.item())) / self.n_cells


# page-locked host arrays that a queued kernel reads in place, each held until
# the event recorded after its launch has completed (a later call drops them)
_inflight = []
_inflight_lock = threading.Lock()


def _hold_until_done(tensors, dev):
    ev = torch.cuda.Event()
    ev.record(torch.cuda.current_stream(dev))
    with _inflight_lock:
        _inflight[:] = [(e, t) for e, t in _inflight if not e.query()]
        _inflight.append((ev, tuple(tensors)))


def _to_device(a, dtype, dev, stream=None):
    if isinstance(a, torch.Tensor):
        t = a
    else:
        t = torch.from_numpy(np.ascontiguousarray(a))
    if t.dtype != dtype:
        t = t.to(dtype)
    return t.to(dev, non_blocking=True)


def col_map(feat_idx, n_genes: int, device) -> torch.Tensor:
    m = np.full(n_genes, -1, dtype=np.int32)
    m[np.asarray(feat_idx)] = np.arange(len(feat_idx), dtype=np.int32)
    return torch.from_numpy(m).to(device)


def normalize_csr_host(indptr, indices, data, n_genes: int, feat_idx, *, size_factor=1000.0,
                       log_transform=True, renormalize_subset=True, n_counts=None, chunk_cells=None,
                       device="cuda", missing_mask=None, fill_value=1.0, cmap=None):
    """a1+a3 over host CSR arrays. Page-locked (pinned) ``indices`` and
    ``data`` tensors are read by the row kernel over the host link, with no
    staging copy and no device copy of the CSR: one launch, or one per
    ``chunk_cells`` rows. Other host arrays are streamed through device
    staging slots: chunk i+1 is copied on a side stream while chunk i is
    normalised, in about 8 chunks unless ``chunk_cells`` says otherwise (0:
    one copy). Chunks are whole multiples of the 256-row statistics slices,
    so every form gives the same bits. Returns ``(x, colsum, colsumsq)``."""
    dev = torch.device(device)
    h = len(feat_idx)
    n = len(indptr) - 1
    cmap = col_map(feat_idx, n_genes, dev) if cmap is None else cmap
    ld = K.round_up(h, 4)
    x = torch.empty((n, ld), dtype=torch.float32, device=dev)
    cs = torch.zeros(h, dtype=torch.float64, device=dev)
    cq = torch.zeros_like(cs)
    nc = None if n_counts is None else _to_device(n_counts, torch.float64, dev)
    mm = None if missing_mask is None else _to_device(missing_mask, torch.uint8, dev)
    ip_h = torch.as_tensor(np.asarray(indptr, dtype=np.int64)) if not isinstance(indptr, torch.Tensor) else indptr
    ind_h = torch.as_tensor(indices) if not isinstance(indices, torch.Tensor) else indices
    dat_h = torch.as_tensor(data) if not isinstance(data, torch.Tensor) else data
    if ind_h.dtype != torch.int32:
        ind_h = ind_h.to(torch.int32)
    if dat_h.dtype != torch.int32:
        dat_h = dat_h.to(torch.int32)
    host = ind_h.device.type == "cpu"
    pinned = host and ind_h.numel() > 0 and ind_h.is_pinned() and dat_h.is_pinned()
    if chunk_cells is None and host and not pinned:
        chunk_cells = max(16384, -(-n // 8))
    if chunk_cells:
        # whole slices of the column-statistics pass (256 rows): the streamed
        # sums then add the same FP32 slice partials as one pass over all rows
        chunk_cells = -(-int(chunk_cells) // STAT_ROWS) * STAT_ROWS
    if pinned:
        ipn = ip_h.numpy() if ip_h.device.type == "cpu" else ip_h.cpu().numpy()
        ip_r = ip_h if (ip_h.device.type == "cpu" and ip_h.is_pinned()) or ip_h.is_cuda else ip_h.to(dev)
        bounds = [0, n] if not chunk_cells or chunk_cells >= n else list(range(0, n, chunk_cells)) + [n]
        last = ind_h.numel() - 1
        for a, b in zip(bounds[:-1], bounds[1:]):
            # the chunk's entries start at indptr[a]; a chunk of empty rows at
            # the very end reads nothing, so any entry address serves it
            off = min(int(ipn[a] - ipn[0]), last)
            K.normalize_csr(ip_r[a:b + 1], ind_h[off:], dat_h[off:], cmap, h, size_factor=size_factor,
                            log_transform=log_transform, renormalize_subset=renormalize_subset,
                            n_counts=None if nc is None else nc[a:b], missing_mask=mm, fill_value=fill_value,
                            out=x[a:b], colsum=cs, colsumsq=cq, device=dev)
        _hold_until_done((ip_h, ind_h, dat_h), dev)
        return x, cs, cq
    if not chunk_cells or chunk_cells >= n:
        ip = ip_h.to(dev, non_blocking=True)
        ind = ind_h.to(dev, non_blocking=True)
        dat = dat_h.to(dev, non_blocking=True)
        K.normalize_csr(ip, ind, dat, cmap, h, size_factor=size_factor, log_transform=log_transform,
                        renormalize_subset=renormalize_subset, n_counts=nc, missing_mask=mm, fill_value=fill_value,
                        out=x, colsum=cs, colsumsq=cq)
        return x, cs, cq
    comp = torch.cuda.current_stream(dev)
    side = torch.cuda.Stream(dev)
    ipn = ip_h.numpy() if ip_h.device.type == "cpu" else ip_h.cpu().numpy()
    bounds = list(range(0, n, chunk_cells)) + [n]
    nch = len(bounds) - 1
    # a ring of three device staging slots sized for the largest chunk: the
    # copy of chunk i+1 (side stream) overlaps the normalisation of chunk i,
    # and a slot is refilled only after the normalisation that read it is done
    nnz_max = max(int(ipn[bounds[i + 1]] - ipn[bounds[i]]) for i in range(nch))
    rows_max = max(bounds[i + 1] - bounds[i] for i in range(nch))
    nslot = min(3, nch)
    slots = [(torch.empty(rows_max + 1, dtype=torch.int64, device=dev),
              torch.empty(max(1, nnz_max), dtype=torch.int32, device=dev),
              torch.empty(max(1, nnz_max), dtype=torch.int32, device=dev)) for _ in range(nslot)]
    freed = [None] * nslot          # event: the last normalisation that read the slot has finished
    landed = [None] * nch

    def stage(ci):
        a, b = bounds[ci], bounds[ci + 1]
        pa, pb = int(ipn[a] - ipn[0]), int(ipn[b] - ipn[0])
        sl = ci % nslot
        t_ip, t_ind, t_dat = slots[sl]
        with torch.cuda.stream(side):
            if freed[sl] is not None:
                side.wait_event(freed[sl])
            t_ip[:b - a + 1].copy_(ip_h[a:b + 1], non_blocking=True)
            t_ind[:pb - pa].copy_(ind_h[pa:pb], non_blocking=True)
            t_dat[:pb - pa].copy_(dat_h[pa:pb], non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(side)
        landed[ci] = ev

    for ci in range(min(nslot, nch)):
        stage(ci)
    for ci in range(nch):
        a, b = bounds[ci], bounds[ci + 1]
        pa, pb = int(ipn[a] - ipn[0]), int(ipn[b] - ipn[0])
        sl = ci % nslot
        t_ip, t_ind, t_dat = slots[sl]
        comp.wait_event(landed[ci])
        K.normalize_csr(t_ip[:b - a + 1], t_ind[:max(1, pb - pa)], t_dat[:max(1, pb - pa)], cmap, h,
                        size_factor=size_factor, log_transform=log_transform,
                        renormalize_subset=renormalize_subset,
                        n_counts=None if nc is None else nc[a:b], missing_mask=mm, fill_value=fill_value,
                        out=x[a:b], colsum=cs, colsumsq=cq)
        done = torch.cuda.Event()
        done.record(comp)
        freed[sl] = done
        if ci + nslot < nch:
            stage(ci + nslot)
    return x, cs, cq


def make_graph(indptr, indices, data, n_genes: int, feat_idx, dims: int = 11, k: int = 11, *,
               batch_size: int = 1000, precision: str = "plain", margin: Optional[int] = None,
               local_connectivity: float = 1.0, bandwidth: float = 1.5, size_factor: float = 1000.0,
               log_transform: bool = True, renormalize_subset: bool = True, n_counts=None,
               use_for_pca: Optional[np.ndarray] = None, chunk_cells: Optional[int] = None,
               smooth: bool = True, keep_x: bool = True, cov_form: Optional[str] = None,
               eigh: Optional[str] = None, autotune: bool = True, device="cuda") -> GraphResult:
    """The whole path on the device; returns device tensors.

    ``precision`` selects the form: "plain" (FP32 scatter, FP32 kNN, full FP64
    eigendecomposition) or "precision" (3xBF16 scatter, BF16 tcgen05 kNN with
    FP32 re-rank, Chebyshev-filtered FP32 subspace iteration refined by an
    FP64 Rayleigh-Ritz step). ``cov_form`` and ``eigh`` override the scatter
    form and the eigensolver ("fp64", "mixed" or "filter")."""
    dev = torch.device(device)
    n = len(indptr) - 1
    h = len(feat_idx)
    # AnnStream caps (scarf/ann.py:91-92, :173-185)
    k = min(k, n - 1)
    dims = min(dims, n, batch_size - 1, h - 1)
    x, cs, cq = normalize_csr_host(indptr, indices, data, n_genes, feat_idx, size_factor=size_factor,
                                   log_transform=log_transform, renormalize_subset=renormalize_subset,
                                   n_counts=n_counts, chunk_cells=chunk_cells, device=dev)
    mu, sigma, mu32, sigma32 = K.zstats(cs, cq, n)
    mask = None
    n_used = n
    if use_for_pca is not None and not np.all(use_for_pca):
        mask = _to_device(np.asarray(use_for_pca, dtype=np.uint8), torch.uint8, dev)
        n_used = int(np.count_nonzero(use_for_pca))
    if cov_form is None:
        cov_form = precision if precision in COV_FORMS else "plain"
    cov, zsum = K.covariance(x, mu32, sigma32, n_cols=h, row_mask=mask, precision=cov_form)
    if eigh is None:
        eigh = "filter" if precision == "precision" else "fp64"
    comps, evals, evr, l32 = K.pca_basis(cov, zsum, n_used, dims + 1, n_load=dims, ld_l=dims, eigh=eigh)
    scores = K.project(x, mu32, sigma32, l32, dims, n_cols=h, precision=precision)
    if margin is None:
        margin = PRECISION_MARGIN if precision == "precision" else PLAIN_MARGIN
    K.set_autotune(autotune, dev.index)
    idx, dist, nm = K.knn(scores, scores, dims, k, self_offset=0, margin=margin, precision=precision)
    res = GraphResult(n_cells=n, n_feats=h, dims=dims, k=k, x=x if keep_x else None, mu=mu, sigma=sigma,
                      mu32=mu32, sigma32=sigma32, components=comps, loadings32=l32, evals=evals, evr=evr,
                      scores=scores, indices=idx, distances=dist, n_missed=nm)
    if smooth:
        res.edges, res.weights = K.smooth(idx, dist, local_connectivity, bandwidth, batch_size)
    return res


def make_graphs(samples, n_genes: int, feat_idx, dims: int = 30, k: int = 15, *, precision: str = "precision",
                union: bool = True, n_streams: int = 16, device="cuda", **kw) -> list:
    """Graphs of many independent samples (for instance hundreds of samples of
    500-20,000 cells). ``samples`` is a sequence of ``(indptr, indices, data)``
    CSR triples sharing the gene space and the feature list. Each sample runs
    ``make_graph`` (and, with ``union``, the fuzzy union of its graph) on one
    of ``n_streams`` worker threads, each with its own CUDA stream and library
    handle, so that the launches of small samples overlap on the device.
    Returns ``[(GraphResult, (indptr, indices, data) or None), ...]`` in
    sample order; the result of a sample does not depend on the others."""
    import concurrent.futures as cf
    dev = torch.device(device)
    out = [None] * len(samples)
    streams = [torch.cuda.Stream(dev) for _ in range(max(1, n_streams))]
    local = {}
    lock = threading.Lock()

    def run(i):
        tid = threading.get_ident()
        with lock:              # each worker thread keeps one stream of its own
            if tid not in local:
                local[tid] = streams[len(local) % len(streams)]
            st = local[tid]
        ip, ind, dat = samples[i]
        with torch.cuda.stream(st):
            g = make_graph(ip, ind, dat, n_genes, feat_idx, dims, k, precision=precision, device=dev, **kw)
            u = K.fuzzy_union(g.edges, g.weights, g.n_cells, g.k) if union else None
        st.synchronize()
        out[i] = (g, u)

    with cf.ThreadPoolExecutor(max_workers=len(streams)) as ex:
        list(ex.map(run, range(len(samples))))
    return out
