"""torch-tensor wrappers over the C ABI (one call per hot-path kernel group).

Inputs and outputs are CUDA tensors; every call is issued on torch's current
stream of the tensors' device. These wrappers check shapes, dtypes and
contiguity and raise on any failure of the library (there is no CPU path).
"""
from __future__ import annotations

import ctypes as C
import threading
from typing import Optional, Tuple

import numpy as np
import torch

from . import _lib as L

_tls = threading.local()
_budget = {"bytes": 0}

PRECISIONS = {"plain": L.SG_PLAIN, "precision": L.SG_PRECISION}


def set_hbm_budget(nbytes: int) -> None:
    """Scratch budget of handles created after this call (0 = no limit)."""
    _budget["bytes"] = int(nbytes)


class Handle:
    """Owns one ``sg_handle`` (scratch arena + solver state) on one device."""

    def __init__(self, device: int, budget: int = 0):
        lib = L.load()
        self.device = device
        self.ptr = C.c_void_p()
        L.check(lib.sg_create(device, budget, C.byref(self.ptr)))

    def workspace_bytes(self) -> int:
        return int(L.load().sg_workspace_bytes(self.ptr))

    def close(self):
        if self.ptr:
            L.load().sg_destroy(self.ptr)
            self.ptr = C.c_void_p()

    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            self.close()
        except Exception:
            pass


def handle(device: Optional[int] = None) -> Handle:
    if not torch.cuda.is_available():
        raise RuntimeError("scarf_gb300 needs a CUDA GPU (GB300); none is visible")
    dev = torch.cuda.current_device() if device is None else int(device)
    hs = getattr(_tls, "handles", None)
    if hs is None:
        hs = _tls.handles = {}
    h = hs.get(dev)
    if h is None:
        h = hs[dev] = Handle(dev, _budget["bytes"])
    return h


def reset_handles() -> None:
    hs = getattr(_tls, "handles", {})
    for h in hs.values():
        h.close()
    _tls.handles = {}


def _p(t: Optional[torch.Tensor]):
    return None if t is None else C.c_void_p(t.data_ptr())


def _stream(device) -> C.c_void_p:
    return C.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def _need(t: torch.Tensor, name: str, dtype=None, ndim=None, contiguous=True, pinned_ok=False):
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name} must be a CUDA tensor")
    if not t.is_cuda and not (pinned_ok and t.device.type == "cpu" and t.is_pinned()):
        raise TypeError(f"{name} must be a CUDA tensor" + (" or page-locked host tensor" if pinned_ok else ""))
    if dtype is not None and t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype}, got {t.dtype}")
    if ndim is not None and t.dim() != ndim:
        raise ValueError(f"{name} must be {ndim}-D, got shape {tuple(t.shape)}")
    if contiguous and not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")


def round_up(x: int, m: int) -> int:
    return (x + m - 1) // m * m


# --------------------------------------------------------------------------
def normalize_csr(indptr, indices, data, col_map, n_cols: int, *, size_factor: float = 1000.0,
                  log_transform: bool = True, renormalize_subset: bool = True, n_counts=None,
                  missing_mask=None, fill_value: float = 1.0, out=None, out_dtype=torch.float32,
                  colsum=None, colsumsq=None, libsize=None, device=None) -> torch.Tensor:
    """a1: dense normalised rows (n_rows x ld) from CSR counts; see sg_normalize_csr.
    indptr/indices/data may be CUDA tensors or page-locked host tensors, which
    the kernel reads over the host link (``device`` then names the GPU; by
    default that of ``col_map``)."""
    _need(indptr, "indptr", torch.int64, 1, pinned_ok=True)
    _need(indices, "indices", torch.int32, 1, pinned_ok=True)
    _need(data, "data", torch.int32, 1, pinned_ok=True)
    _need(col_map, "col_map", torch.int32, 1)
    n_rows = indptr.numel() - 1
    dev = col_map.device if device is None else torch.device(device)
    if out is None:
        ld = round_up(n_cols, 4 if out_dtype == torch.float32 else 8)
        out = torch.empty((n_rows, ld), dtype=out_dtype, device=dev)
    _need(out, "out", out_dtype, 2, contiguous=False)
    if out.stride(1) != 1:
        raise ValueError("out must have unit column stride")
    flags = (L.SG_NORM_LOG1P if log_transform else 0) | (L.SG_NORM_RENORM_SUBSET if renormalize_subset else 0)
    if n_counts is not None:
        _need(n_counts, "n_counts", torch.float64, 1)
    if missing_mask is not None:
        _need(missing_mask, "missing_mask", torch.uint8, 1)
    if colsum is not None:
        _need(colsum, "colsum", torch.float64, 1)
        _need(colsumsq, "colsumsq", torch.float64, 1)
    if libsize is not None:
        _need(libsize, "libsize", torch.int64, 1)
    h = handle(dev.index)
    lib = L.load()
    L.check(lib.sg_normalize_csr(
        h.ptr, _p(indptr), _p(indices), _p(data), n_rows, _p(col_map), col_map.numel(), n_cols,
        _p(missing_mask), float(fill_value), _p(n_counts), float(size_factor), flags, _p(out),
        out.stride(0), L.SG_F32 if out_dtype == torch.float32 else L.SG_BF16, _p(libsize), _p(colsum),
        _p(colsumsq), _stream(dev)))
    return out


def zstats(colsum: torch.Tensor, colsumsq: torch.Tensor, n_rows: int):
    """a3: (mu, sigma) float64 with clean_array semantics, and float32 copies."""
    _need(colsum, "colsum", torch.float64, 1)
    _need(colsumsq, "colsumsq", torch.float64, 1)
    h = colsum.numel()
    dev = colsum.device
    mu = torch.empty(h, dtype=torch.float64, device=dev)
    sigma = torch.empty_like(mu)
    mu32 = torch.empty(h, dtype=torch.float32, device=dev)
    sigma32 = torch.empty_like(mu32)
    L.check(L.load().sg_zstats(handle(dev.index).ptr, _p(colsum), _p(colsumsq), int(n_rows), h, _p(mu),
                               _p(sigma), _p(mu32), _p(sigma32), _stream(dev)))
    return mu, sigma, mu32, sigma32


def covariance(x: torch.Tensor, mu32: torch.Tensor, sigma32: torch.Tensor, n_cols: Optional[int] = None,
               row_mask: Optional[torch.Tensor] = None, precision: str = "plain", cov=None, zsum=None):
    """a4: accumulate the scatter of the z-scaled rows (cov, zsum) in float64."""
    _need(x, "x", torch.float32, 2, contiguous=False)
    if x.stride(1) != 1:
        raise ValueError("x must have unit column stride")
    h = int(n_cols if n_cols is not None else mu32.numel())
    dev = x.device
    if cov is None:
        cov = torch.zeros((h, h), dtype=torch.float64, device=dev)
    if zsum is None:
        zsum = torch.zeros(h, dtype=torch.float64, device=dev)
    if row_mask is not None:
        _need(row_mask, "row_mask", torch.uint8, 1)
    L.check(L.load().sg_covariance(handle(dev.index).ptr, _p(x), x.shape[0], h, x.stride(0), _p(mu32),
                                   _p(sigma32), _p(row_mask), PRECISIONS[precision], _p(cov), _p(zsum),
                                   _stream(dev)))
    return cov, zsum


def pca_basis(cov: torch.Tensor, zsum: Optional[torch.Tensor], n_used: int, n_comp: int,
              n_load: Optional[int] = None, ld_l: Optional[int] = None, eigh: str = "fp64"):
    """a4: top ``n_comp`` principal axes on the device, svd_flip signs.
    ``eigh='fp64'``: FP64 partial eigendecomposition of the whole scatter;
    ``eigh='mixed'``: FP32 partial eigendecomposition + FP64 Rayleigh-Ritz;
    ``eigh='filter'``: Chebyshev-filtered FP32 subspace iteration + FP64
    Rayleigh-Ritz (see ``filter_residual``).

    Returns ``(comps h x n_comp f64, evals, evr, loadings32 h x ld_l)`` where
    loadings32 holds the first ``n_load`` (default n_comp - 1) components."""
    _need(cov, "cov", torch.float64, 2)
    h = cov.shape[0]
    dev = cov.device
    n_load = n_comp - 1 if n_load is None else n_load
    ld_l = max(1, n_load) if ld_l is None else ld_l
    comps = torch.empty((h, n_comp), dtype=torch.float64, device=dev)
    evals = torch.empty(n_comp, dtype=torch.float64, device=dev)
    evr = torch.empty(n_comp, dtype=torch.float64, device=dev)
    l32 = torch.empty((h, ld_l), dtype=torch.float32, device=dev)
    fn = {"fp64": L.load().sg_pca_basis, "mixed": L.load().sg_pca_basis_mixed,
          "filter": L.load().sg_pca_basis_filter}[eigh]
    L.check(fn(handle(dev.index).ptr, _p(cov), _p(zsum), int(n_used), h, n_comp, _p(comps), _p(evals), _p(evr),
               n_load, _p(l32), ld_l, _stream(dev)))
    return comps, evals, evr, l32


def set_autotune(enable: bool, device: Optional[int] = None) -> None:
    """Autotune the precision kNN's reference split count per shape bucket on
    this thread's handle (see sg_set_autotune)."""
    L.check(L.load().sg_set_autotune(handle(device).ptr, int(bool(enable))))


def knn_last_splits(device: Optional[int] = None) -> int:
    return int(L.load().sg_knn_last_splits(handle(device).ptr))


def knn_last_locality(device: Optional[int] = None) -> int:
    return int(L.load().sg_knn_last_locality(handle(device).ptr))


def filter_residual(device: Optional[int] = None) -> float:
    """Max relative FP64 residual of the wanted pairs of the last
    ``pca_basis(eigh='filter')`` on this thread's handle (NaN: dense route for
    a small matrix; inf: fell back to the mixed solver)."""
    return float(L.load().sg_pca_filter_residual(handle(device).ptr))


def project(x: torch.Tensor, mu32, sigma32, loadings32: torch.Tensor, d: int, n_cols: Optional[int] = None,
            ld_s: Optional[int] = None, bf16_ld: Optional[int] = None, precision: str = "plain"):
    """a5: scores = ((x - mu)/sigma) . L as float32 (n x ld_s), optionally a BF16
    copy; "plain" in FP32 SIMT, "precision" as 3xBF16 tcgen05 products."""
    _need(x, "x", torch.float32, 2, contiguous=False)
    _need(loadings32, "loadings32", torch.float32, 2)
    h = int(n_cols if n_cols is not None else mu32.numel())
    dev = x.device
    ld_s = round_up(d, 4) if ld_s is None else ld_s
    scores = torch.empty((x.shape[0], ld_s), dtype=torch.float32, device=dev)
    sb = None
    if bf16_ld:
        sb = torch.empty((x.shape[0], bf16_ld), dtype=torch.bfloat16, device=dev)
    L.check(L.load().sg_project(handle(dev.index).ptr, _p(x), x.shape[0], h, x.stride(0), _p(mu32), _p(sigma32),
                                _p(loadings32), d, loadings32.stride(0), _p(scores), ld_s, _p(sb),
                                bf16_ld or 0, PRECISIONS[precision], _stream(dev)))
    return (scores, sb) if bf16_ld else scores


def knn(queries: torch.Tensor, refs: torch.Tensor, d: int, k: int, self_offset: int = -1, margin: int = 0,
        precision: str = "plain", n_missed: Optional[torch.Tensor] = None):
    """a6/a7/a10: exact squared-L2 kNN (see sg_knn). Returns ``(idx int64, dist f32, n_missed)``."""
    _need(queries, "queries", torch.float32, 2)
    _need(refs, "refs", torch.float32, 2)
    if queries.shape[1] != refs.shape[1]:
        raise ValueError("queries and refs must share the row stride")
    dev = queries.device
    nq = queries.shape[0]
    idx = torch.empty((nq, k), dtype=torch.int64, device=dev)
    dist = torch.empty((nq, k), dtype=torch.float32, device=dev)
    if n_missed is None:
        n_missed = torch.zeros(1, dtype=torch.int64, device=dev)
    L.check(L.load().sg_knn(handle(dev.index).ptr, _p(queries), nq, _p(refs), refs.shape[0], d,
                            queries.shape[1], k, int(self_offset), int(margin), PRECISIONS[precision], _p(idx),
                            _p(dist), _p(n_missed), _stream(dev)))
    return idx, dist, n_missed


def smooth(idx: torch.Tensor, dist: torch.Tensor, local_connectivity: float, bandwidth: float,
           chunk_rows: int):
    """a8: (edges int64 (n*k, 2), weights float64 (n*k,)) as smoothen_dists writes them."""
    _need(idx, "idx", torch.int64, 2)
    _need(dist, "dist", torch.float32, 2)
    n, k = idx.shape
    dev = idx.device
    edges = torch.empty((n * k, 2), dtype=torch.int64, device=dev)
    w = torch.empty(n * k, dtype=torch.float64, device=dev)
    L.check(L.load().sg_smooth(handle(dev.index).ptr, _p(idx), _p(dist), n, k, float(local_connectivity),
                               float(bandwidth), int(chunk_rows), _p(edges), _p(w), _stream(dev)))
    return edges, w


def kmeans(x: torch.Tensor, d: int, n_clusters: int, block_rows: int, seed: int):
    """f1: MiniBatchKMeans of make_graph (see sg_kmeans_minibatch): partial_fit
    over the row blocks of ``x`` (n x ld float32, rows of ``d`` values) in
    order, then predict. Returns ``(centres float64 (k, d), labels int32 (n,))``."""
    _need(x, "x", torch.float32, 2)
    if x.stride(0) % 4:
        raise ValueError("x's row stride must be a multiple of 4 floats")
    dev = x.device
    centers = torch.empty((n_clusters, d), dtype=torch.float64, device=dev)
    labels = torch.empty(x.shape[0], dtype=torch.int32, device=dev)
    L.check(L.load().sg_kmeans_minibatch(handle(dev.index).ptr, _p(x), x.shape[0], d, x.stride(0), n_clusters,
                                         block_rows, C.c_uint64(int(seed) & ((1 << 64) - 1)), _p(centers),
                                         _p(labels), _stream(dev)))
    return centers, labels


def calc_snn(indices: torch.Tensor) -> torch.Tensor:
    """f4: shared-neighbour fractions of a kNN graph (see sg_calc_snn); ``indices`` n x k int64."""
    _need(indices, "indices", torch.int64, 2)
    n, k = indices.shape
    out = torch.empty((n, k), dtype=torch.float64, device=indices.device)
    L.check(L.load().sg_calc_snn(handle(indices.device.index).ptr, _p(indices), n, k, _p(out),
                                 _stream(indices.device)))
    return out


def merge_graphs(indices, weights, snns):
    """f4: merge of kNN graphs (see sg_merge_graphs). Each argument is a list
    of n x k CUDA tensors (int64, float64, float64), one per graph. Returns
    ``(indices int64 (n, k), weights float64 (n, k))``."""
    if not (len(indices) == len(weights) == len(snns)) or not indices:
        raise ValueError("one indices, weights and snn tensor per graph")
    n, k = indices[0].shape
    dev = indices[0].device
    for a, b, c in zip(indices, weights, snns):
        _need(a, "indices", torch.int64, 2)
        _need(b, "weights", torch.float64, 2)
        _need(c, "snn", torch.float64, 2)
        if a.shape != (n, k) or b.shape != (n, k) or c.shape != (n, k):
            raise ValueError("all graphs must have the same shape")
    g = len(indices)
    arr = lambda ts: (C.c_void_p * g)(*[t.data_ptr() for t in ts])
    out_i = torch.empty((n, k), dtype=torch.int64, device=dev)
    out_w = torch.empty((n, k), dtype=torch.float64, device=dev)
    L.check(L.load().sg_merge_graphs(handle(dev.index).ptr, g, arr(indices), arr(weights), arr(snns), n, k,
                                     _p(out_i), _p(out_w), _stream(dev)))
    return out_i, out_w


def umap_layout(head: torch.Tensor, tail: torch.Tensor, epochs_per_sample: torch.Tensor, embedding: torch.Tensor,
                n_epochs: int, a: float, b: float, gamma: float = 1.0, initial_alpha: float = 1.0,
                negative_sample_rate: float = 5.0, seed: int = 0, sequential: bool = False) -> torch.Tensor:
    """f3: UMAP layout epochs on ``embedding`` (n x dim float32, in place; see
    sg_umap_layout). ``head``/``tail`` int32 edge endpoints, ``epochs_per_sample``
    float64 per edge; ``sequential`` runs the deterministic one-thread loop."""
    _need(head, "head", torch.int32, 1)
    _need(tail, "tail", torch.int32, 1)
    _need(epochs_per_sample, "epochs_per_sample", torch.float64, 1)
    _need(embedding, "embedding", torch.float32, 2)
    dev = embedding.device
    L.check(L.load().sg_umap_layout(handle(dev.index).ptr, _p(head), _p(tail), _p(epochs_per_sample), head.numel(),
                                    embedding.shape[0], embedding.shape[1], _p(embedding), int(n_epochs), float(a),
                                    float(b), float(gamma), float(initial_alpha), float(negative_sample_rate),
                                    C.c_uint64(int(seed) & ((1 << 64) - 1)), int(bool(sequential)), _stream(dev)))
    return embedding


def fuzzy_union(edges: torch.Tensor, w: torch.Tensor, n: int, k: int, use_k: Optional[int] = None,
                mix: float = 1.0, upper_only: bool = False) -> Tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
    """a9: CSR (indptr int64, indices int32, data float64) of the fuzzy union."""
    _need(edges, "edges", torch.int64, 2)
    _need(w, "w", torch.float64, 1)
    dev = edges.device
    nnz = edges.shape[0]
    cap = max(1, 2 * nnz)
    indptr = torch.empty(n + 1, dtype=torch.int64, device=dev)
    ind = torch.empty(cap, dtype=torch.int32, device=dev)
    dat = torch.empty(cap, dtype=torch.float64, device=dev)
    L.check(L.load().sg_fuzzy_union(handle(dev.index).ptr, _p(edges), _p(w), nnz, int(n), int(k),
                                    int(k if use_k is None else use_k), float(mix),
                                    L.SG_UNION_UPPER_ONLY if upper_only else 0, _p(indptr), _p(ind), _p(dat), cap,
                                    _stream(dev)))
    nz = int(indptr[-1].item())
    return indptr, ind[:nz], dat[:nz]


# --------------------------------------------------------------------------
def kernel_launches() -> int:
    """Number of this library's kernels launched by the process so far."""
    return int(L.load().sg_kernel_launches())


def profile(enable: bool, device: Optional[int] = None) -> None:
    L.check(L.load().sg_profile(handle(device).ptr, 1 if enable else 0))


def profile_reset(device: Optional[int] = None) -> None:
    L.check(L.load().sg_profile_reset(handle(device).ptr))


def profile_query(name: str, device: Optional[int] = None) -> Tuple[float, int]:
    """(total device ms, launches) of the named kernel while profiling was on."""
    ms = C.c_double()
    cnt = C.c_longlong()
    L.check(L.load().sg_profile_query(handle(device).ptr, name.encode(), C.byref(ms), C.byref(cnt)))
    return ms.value, cnt.value


def blosc_decode(frames, out: torch.Tensor, out_starts) -> torch.Tensor:
    """f2: decode Blosc1/LZ4 frames (a list of host ``bytes``) into the device
    uint8 buffer ``out`` at the given byte offsets (see sg_blosc_decode)."""
    _need(out, "out", torch.uint8, 1)
    n = len(frames)
    offs = np.zeros(n + 1, dtype=np.int64)
    np.cumsum([len(f) for f in frames], out=offs[1:])
    buf = np.frombuffer(b"".join(frames), dtype=np.uint8) if n else np.zeros(1, np.uint8)
    starts = np.ascontiguousarray(out_starts, dtype=np.int64)
    if len(starts) != n:
        raise ValueError("one output offset per frame")
    dev = out.device
    L.check(L.load().sg_blosc_decode(handle(dev.index).ptr, buf.ctypes.data_as(C.c_void_p),
                                     offs.ctypes.data_as(C.c_void_p), n, _p(out), out.numel(),
                                     starts.ctypes.data_as(C.c_void_p), _stream(dev)))
    return out


def blosc_encode(src: torch.Tensor, chunk_offsets, typesize: int, shuffle: int = 2,
                 blocksize: int = 32768) -> list:
    """f2: one Blosc1/LZ4 frame (``bytes``) per chunk of the device uint8
    buffer ``src``; chunk c is src[chunk_offsets[c]:chunk_offsets[c + 1]]
    (see sg_blosc_encode). ``shuffle``: 2 bit, 1 byte, 0 none."""
    _need(src, "src", torch.uint8, 1)
    offs = np.ascontiguousarray(chunk_offsets, dtype=np.int64)
    n = len(offs) - 1
    if n < 0 or offs[0] < 0 or offs[-1] > src.numel() or np.any(np.diff(offs) < 0):
        raise ValueError("chunk offsets must be non-decreasing and inside the buffer")
    bs = max(typesize, min(32768, blocksize) // typesize * typesize)
    lib = L.load()
    cap = lib.sg_blosc_encode_bound(offs.ctypes.data_as(C.c_void_p), n, bs)
    if cap < 0:
        raise ValueError("bad chunk offsets or block size")
    out = np.empty(max(1, cap), dtype=np.uint8)
    fo = np.zeros(n + 1, dtype=np.int64)
    dev = src.device
    L.check(lib.sg_blosc_encode(handle(dev.index).ptr, _p(src), offs.ctypes.data_as(C.c_void_p), n, int(typesize),
                                int(shuffle), bs, out.ctypes.data_as(C.c_void_p), cap,
                                fo.ctypes.data_as(C.c_void_p), _stream(dev)))
    return [out[fo[c]:fo[c + 1]].tobytes() for c in range(n)]


def chunks_to_csr(chunks: torch.Tensor, n_rows: int, chunk_rows: int, chunk_cols: int, n_cols: int,
                  indptr_base: int = 0):
    """f2: CSR (indptr int64, indices int32, data int32) of one band of decoded
    dense uint32 chunks held as int32 in ``chunks`` (see sg_chunks_to_csr)."""
    _need(chunks, "chunks", torch.int32, 1)
    dev = chunks.device
    h = handle(dev.index)
    lib = L.load()
    indptr = torch.empty(n_rows + 1, dtype=torch.int64, device=dev)
    nnz = C.c_int64()
    L.check(lib.sg_chunks_to_csr(h.ptr, _p(chunks), n_rows, chunk_rows, chunk_cols, n_cols, indptr_base,
                                 _p(indptr), None, None, 0, C.byref(nnz), _stream(dev)))
    cap = max(1, nnz.value)
    ind = torch.empty(cap, dtype=torch.int32, device=dev)
    dat = torch.empty(cap, dtype=torch.int32, device=dev)
    L.check(lib.sg_chunks_to_csr(h.ptr, _p(chunks), n_rows, chunk_rows, chunk_cols, n_cols, indptr_base,
                                 _p(indptr), _p(ind), _p(dat), cap, C.byref(nnz), _stream(dev)))
    return indptr, ind[:nnz.value], dat[:nnz.value]
