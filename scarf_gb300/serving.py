"""Continuous-batching mapping service over a device-resident reference.

The service answers the query of ``run_mapping``
(scarf/datastore/mapping_datastore.py:198-208): normalise target cells onto
the reference features (missing features filled with 1.0,
scarf/mapping_utils.py:208), z-scale with the reference's mu/sigma, project
with its loadings, and return the k nearest reference cells.

Scheduling (``BatchScheduler``, pure host logic):
* requests are admitted in arrival order while the HBM they need (their CSR,
  normalised rows, scores and results) fits the budget; a request that cannot
  fit the budget alone is rejected with ``MemoryError``;
* an admitted request is handed to the uploader, which copies its CSR to the
  device once; it is ready for batching when that copy has landed;
* each GPU batch takes up to ``max_batch_rows`` rows from the ready requests,
  shortest remaining first (ties by arrival), so a large request is processed
  in row slices and a small request that arrives while it is on the GPU goes
  into the next batch instead of waiting for it to finish;
* a request completes when all its rows are back; its memory is released and
  the next queued requests are admitted.

Execution (``MappingServer``): uploader threads (smallest request first) copy
admitted requests to the device; ``n_workers``
host threads, each with its own CUDA stream and library handle, take batches
from the scheduler and assemble each batch's CSR on the device from the
resident requests. The copies and kernels of different batches overlap on the
device. Rows are independent, so a request's result does not depend on what it
was batched with.
"""
from __future__ import annotations

import collections
import heapq
import threading
import time
import warnings
from dataclasses import dataclass, field
from typing import Deque, List, Optional, Tuple

import numpy as np


@dataclass
class MapRequest:
    rid: int
    indptr: np.ndarray
    indices: np.ndarray
    data: np.ndarray
    k: int
    arrival: float
    n_cells: int = 0
    bytes_needed: int = 0
    next_row: int = 0
    rows_done: int = 0
    idx: Optional[np.ndarray] = None
    dist: Optional[np.ndarray] = None
    t_done: Optional[float] = None
    error: Optional[BaseException] = None
    done: threading.Event = field(default_factory=threading.Event)
    ready: bool = True                 # CSR resident where the batches read it
    dev: Optional[tuple] = None        # device (indptr, indices, data)
    t_admit: float = 0.0               # handed to the uploader

    def __post_init__(self):
        self.n_cells = len(self.indptr) - 1

    @property
    def latency_ms(self) -> Optional[float]:
        return None if self.t_done is None else (self.t_done - self.arrival) * 1e3

    def result(self, timeout: Optional[float] = None):
        if not self.done.wait(timeout):
            raise TimeoutError(f"request {self.rid} not done")
        if self.error is not None:
            raise self.error
        return self.idx, self.dist


Slice = Tuple[MapRequest, int, int]


class BatchScheduler:
    """HBM-budget admission and row-sliced continuous batching (host only)."""

    def __init__(self, hbm_budget_bytes: int, max_batch_rows: int, bytes_per_row: int, bytes_per_nnz: int = 8,
                 uploader=None):
        """``uploader(req)``, when given, is called (outside the lock) for each
        admitted request, which becomes ready when ``mark_ready`` is called."""
        self.uploader = uploader
        self.budget = int(hbm_budget_bytes)
        self.max_rows = int(max_batch_rows)
        self.bytes_per_row = int(bytes_per_row)
        self.bytes_per_nnz = int(bytes_per_nnz)
        self.queued: Deque[MapRequest] = collections.deque()
        self.active: List[MapRequest] = []
        self.in_use = 0
        self.lock = threading.Condition()
        self.closed = False

    def cost(self, req: MapRequest) -> int:
        return req.n_cells * self.bytes_per_row + int(req.indptr[-1] - req.indptr[0]) * self.bytes_per_nnz

    def submit(self, req: MapRequest) -> MapRequest:
        req.bytes_needed = self.cost(req)
        with self.lock:
            if req.bytes_needed > self.budget:
                req.error = MemoryError(f"request {req.rid} needs {req.bytes_needed} bytes of HBM, more than the "
                                        f"budget of {self.budget}")
                req.t_done = time.perf_counter()
                req.done.set()
                return req
            if req.n_cells == 0:
                req.idx = np.zeros((0, req.k), np.int64)
                req.dist = np.zeros((0, req.k), np.float32)
                req.t_done = time.perf_counter()
                req.done.set()
                return req
            self.queued.append(req)
            new = self._admit()
            self.lock.notify_all()
        self._upload(new)
        return req

    def _admit(self) -> List[MapRequest]:
        new = []
        while self.queued and self.in_use + self.queued[0].bytes_needed <= self.budget:
            r = self.queued.popleft()
            self.in_use += r.bytes_needed
            r.idx = np.empty((r.n_cells, r.k), np.int64)
            r.dist = np.empty((r.n_cells, r.k), np.float32)
            r.ready = self.uploader is None
            self.active.append(r)
            new.append(r)
        return new

    def _upload(self, reqs: List[MapRequest]):
        if self.uploader is not None:
            for r in reqs:
                self.uploader(r)

    def mark_ready(self, req: MapRequest, error: Optional[BaseException] = None):
        """The uploader's report: ``req`` is resident (or failed with ``error``)."""
        new = []
        with self.lock:
            if error is None:
                req.ready = True
            else:
                req.error = error
                if req in self.active:
                    self.active.remove(req)
                    self.in_use -= req.bytes_needed
                req.dev = None
                req.t_done = time.perf_counter()
                req.done.set()
                new = self._admit()
            self.lock.notify_all()
        self._upload(new)

    def _pending(self) -> List[MapRequest]:
        return [r for r in self.active if r.ready and r.next_row < r.n_cells]

    def next_batch(self, timeout: Optional[float] = None) -> List[Slice]:
        """Up to max_rows rows from the ready requests, shortest remaining
        first (ties: oldest first)."""
        with self.lock:
            end = None if timeout is None else time.perf_counter() + timeout
            while not self.closed and not self._pending():
                left = None if end is None else end - time.perf_counter()
                if left is not None and left <= 0:
                    return []
                self.lock.wait(left)
            batch: List[Slice] = []
            room = self.max_rows
            for r in sorted(self._pending(), key=lambda q: (q.n_cells - q.next_row, q.arrival, q.rid)):
                if room == 0:
                    break
                take = min(room, r.n_cells - r.next_row)
                batch.append((r, r.next_row, r.next_row + take))
                r.next_row += take
                room -= take
            return batch

    def complete(self, batch: List[Slice], idx: np.ndarray, dist: np.ndarray, error: Optional[BaseException] = None):
        """Scatter a finished batch back into its requests."""
        now = time.perf_counter()
        with self.lock:
            off = 0
            for r, a, b in batch:
                n = b - a
                if error is None:
                    r.idx[a:b] = idx[off:off + n]
                    r.dist[a:b] = dist[off:off + n]
                else:
                    r.error = error
                off += n
                r.rows_done += n
                if (r.rows_done == r.n_cells or error is not None) and not r.done.is_set():
                    if r in self.active:
                        self.active.remove(r)
                        self.in_use -= r.bytes_needed
                    r.dev = None
                    r.t_done = now
                    r.done.set()
            new = self._admit()
            self.lock.notify_all()
        self._upload(new)

    def close(self):
        with self.lock:
            self.closed = True
            self.lock.notify_all()


class Reference:
    """Device-resident mapping reference: z-scale statistics, loadings and the
    reference cells' scores, with the query form ("plain" or "precision").
    ``from_graph`` takes them from a ``pipeline.GraphResult``; an ``AnnStream``
    carries the same attributes and can be used in its place."""

    def __init__(self, mu32, sigma32, loadings32, dims: int, scores, n_feats: int, precision: str = "precision",
                 margin: Optional[int] = None):
        from .ann import GpuExactIndex, NormalizedData
        self._mu32, self._sg32, self._l32 = mu32, sigma32, loadings32
        self.dims = int(dims)
        self.nFeats = int(n_feats)
        self.data = NormalizedData(scores, n_feats, 1)  # only .x.device is read
        self.annIdx = GpuExactIndex("l2", dims, precision=precision, margin=margin, device=scores.device)
        self.annIdx._rows = [scores]

    @classmethod
    def from_graph(cls, g, precision: str = "precision", margin: Optional[int] = None) -> "Reference":
        return cls(g.mu32, g.sigma32, g.loadings32.contiguous(), g.dims, g.scores, g.n_feats, precision, margin)


class _Staging:
    """Pinned host buffers of one worker, grown on demand."""

    def __init__(self):
        self.bufs = {}

    def get(self, name, n, dtype):
        import torch
        b = self.bufs.get(name)
        if b is None or b.numel() < n:
            b = torch.empty(max(n, 1024) * 5 // 4, dtype=dtype, pin_memory=True)
            self.bufs[name] = b
        return b[:n]


class MappingServer:
    """GPU executor of the scheduler's batches (see the module docstring).

    ``reference`` is an ``AnnStream`` (device-resident scores, mu/sigma,
    loadings); ``target_gene_ids`` is the gene panel of the queries, aligned
    once to the reference features."""

    def __init__(self, reference, ref_feature_ids, target_gene_ids, k: int = 11, max_batch_rows: int = 16384,
                 hbm_budget_bytes: int = 8 << 30, n_workers: int = 2, size_factor: float = 1000.0,
                 log_transform: bool = True, renormalize_subset: bool = True, precision: Optional[str] = None,
                 n_uploaders: int = 2):
        import torch

        from .datastore import align_col_map
        self.ref = reference
        self.k = int(k)
        self.size_factor = float(size_factor)
        self.log_transform = log_transform
        self.renorm = renormalize_subset
        self.precision = precision or reference.annIdx.precision
        self.device = reference.data.x.device
        cmap, missing = align_col_map(np.asarray(ref_feature_ids), np.asarray(target_gene_ids))
        self.cmap = torch.from_numpy(cmap).to(self.device)
        self.missing = torch.from_numpy(missing).to(self.device)
        h = reference.nFeats
        ld = (h + 3) // 4 * 4
        lds = (reference.dims + 3) // 4 * 4
        per_row = 8 + ld * 4 + lds * 4 + self.k * 12
        self.sched = BatchScheduler(hbm_budget_bytes, max_batch_rows, per_row, bytes_per_nnz=8,
                                    uploader=self._enqueue_upload)
        self.n_workers = int(n_workers)
        self.n_uploaders = max(1, int(n_uploaders))
        # in-flight requests never exceed the admission budget
        self._upload_reserve = int(min(16 << 30, hbm_budget_bytes // self.n_uploaders))
        self._threads: List[threading.Thread] = []
        self._rid = 0
        self._rid_lock = threading.Lock()
        self._up_heap: list = []
        self._up_cv = threading.Condition()
        self._stopping = False
        self.batches_run = 0
        # (rows, seconds from batch taken to results on the host) per batch;
        # (cells, bytes, seconds queued for an uploader, seconds issuing the
        # copies, seconds until they landed) per request
        self.batch_log: List[Tuple[int, float]] = []
        self.upload_log: List[Tuple[int, int, float, float, float]] = []

    # -- client side ----------------------------------------------------------
    def submit(self, indptr, indices, data, arrival: Optional[float] = None) -> MapRequest:
        with self._rid_lock:
            rid = self._rid
            self._rid += 1
        req = MapRequest(rid, np.asarray(indptr, np.int64), np.asarray(indices, np.int32), np.asarray(data, np.int32),
                         self.k, arrival if arrival is not None else time.perf_counter())
        return self.sched.submit(req)

    def start(self):
        for i in range(self.n_uploaders):
            t = threading.Thread(target=self._uploader, name=f"sg-up-{i}", daemon=True)
            t.start()
            self._threads.append(t)
        for i in range(self.n_workers):
            t = threading.Thread(target=self._worker, name=f"sg-map-{i}", daemon=True)
            t.start()
            self._threads.append(t)
        return self

    def stop(self):
        self.sched.close()
        with self._up_cv:
            self._stopping = True
            self._up_cv.notify_all()
        for t in self._threads:
            t.join(timeout=30)
        self._threads = []

    def __enter__(self):
        return self.start()

    def __exit__(self, *exc):
        self.stop()

    # -- uploader side --------------------------------------------------------
    def _enqueue_upload(self, req: MapRequest):
        req.t_admit = time.perf_counter()
        with self._up_cv:
            heapq.heappush(self._up_heap, (req.n_cells, req.arrival, req.rid, req))
            self._up_cv.notify()

    def _uploader(self):
        # Copies go straight from the request's (pageable) arrays: on a
        # coherent CPU-GPU link they run at the copy engines' rate, where a
        # pass through a pinned staging buffer would add a host memcpy.
        import torch
        torch.cuda.set_device(self.device)
        stream = torch.cuda.Stream(self.device)
        # reserve device memory for this uploader's copies in torch's cache, so
        # that requests of new sizes split a cached segment instead of taking
        # a fresh allocation while kernels run
        with torch.cuda.stream(stream):
            torch.empty(self._upload_reserve, dtype=torch.uint8, device=self.device)
        stream.synchronize()
        while True:
            with self._up_cv:
                while not self._up_heap and not self._stopping:
                    self._up_cv.wait(0.05)
                if not self._up_heap:
                    return
                req = heapq.heappop(self._up_heap)[3]
            t0 = time.perf_counter()
            try:
                p0, p1 = int(req.indptr[0]), int(req.indptr[-1])
                hs = [req.indptr, req.indices[p0:p1], req.data[p0:p1]]
                nbytes = sum(int(a.nbytes) for a in hs)
                if p1 == p0:  # keep the device pointers valid for an all-empty request
                    hs[1], hs[2] = np.zeros(1, np.int32), np.zeros(1, np.int32)
                with torch.cuda.stream(stream), warnings.catch_warnings():
                    # read-only request arrays are only read here
                    warnings.filterwarnings("ignore", message="The given NumPy array is not writable")
                    dev = tuple(torch.from_numpy(np.ascontiguousarray(h)).to(self.device, non_blocking=True)
                                for h in hs)
                t1 = time.perf_counter()
                stream.synchronize()
                req.dev = dev
                t2 = time.perf_counter()
                self.upload_log.append((req.n_cells, nbytes, t0 - req.t_admit, t1 - t0, t2 - t1))
                self.sched.mark_ready(req)
            except BaseException as e:  # surfaces in MapRequest.result()
                self.sched.mark_ready(req, error=e)

    # -- worker side ----------------------------------------------------------
    def _batch_csr(self, batch: List[Slice], stage: "_Staging"):
        """The batch's CSR on the device: views of the request when the batch
        is one slice, else a device concatenation of the slices."""
        import torch
        if len(batch) == 1:
            r, a, b = batch[0]
            ip_d, ind_d, dat_d = r.dev
            return ip_d[a:b + 1], ind_d, dat_d, int(r.indptr[a] - r.indptr[0])
        ptrs, inds, dats = [np.zeros(1, np.int64)], [], []
        base = 0
        for r, a, b in batch:
            q0 = int(r.indptr[0])
            p0, p1 = int(r.indptr[a]) - q0, int(r.indptr[b]) - q0
            ptrs.append((r.indptr[a + 1:b + 1] - q0 - p0 + base).astype(np.int64))
            inds.append(r.dev[1][p0:p1])
            dats.append(r.dev[2][p0:p1])
            base += p1 - p0
        ip = np.concatenate(ptrs)
        h_ip = stage.get("ip", len(ip), torch.int64)
        h_ip.numpy()[:] = ip
        if base == 0:  # keep the device pointers valid for an all-empty batch
            inds, dats = [torch.zeros(1, dtype=torch.int32, device=self.device)], \
                [torch.zeros(1, dtype=torch.int32, device=self.device)]
        return h_ip.to(self.device, non_blocking=True), torch.cat(inds), torch.cat(dats), 0

    def _run_batch(self, K, t_ip, t_ind, t_dat, off):
        ref = self.ref
        h = ref.nFeats
        x = K.normalize_csr(t_ip, t_ind[off:], t_dat[off:], self.cmap, h, size_factor=self.size_factor,
                            log_transform=self.log_transform, renormalize_subset=self.renorm,
                            missing_mask=self.missing, fill_value=1.0)
        s = K.project(x, ref._mu32, ref._sg32, ref._l32, ref.dims, n_cols=h, precision=self.precision)
        return K.knn(s, ref.annIdx.scores, ref.dims, self.k, self_offset=-1, margin=ref.annIdx._margin(),
                     precision=self.precision)

    def _worker(self):
        import torch

        from . import kernels as K
        torch.cuda.set_device(self.device)
        stream = torch.cuda.Stream(self.device)
        stage = _Staging()
        # Size this worker's library scratch and torch's cache with one batch
        # of the largest shape first: growing them later synchronises the
        # whole device, which stalls every other stream (uploads included).
        with torch.cuda.stream(stream):
            rows = self.sched.max_rows
            z = torch.zeros(rows + 1, dtype=torch.int64, device=self.device)
            one = torch.zeros(1, dtype=torch.int32, device=self.device)
            self._run_batch(K, z, one, one, 0)
        stream.synchronize()
        while True:
            batch = self.sched.next_batch(timeout=0.05)
            if not batch:
                if self.sched.closed:
                    return
                continue
            t0 = time.perf_counter()
            try:
                with torch.cuda.stream(stream):
                    t_ip, t_ind, t_dat, off = self._batch_csr(batch, stage)
                    idx, dist, _ = self._run_batch(K, t_ip, t_ind, t_dat, off)
                    hi = stage.get("oi", idx.numel(), idx.dtype).view(idx.shape)
                    hd = stage.get("od", dist.numel(), dist.dtype).view(dist.shape)
                    hi.copy_(idx, non_blocking=True)
                    hd.copy_(dist, non_blocking=True)
                stream.synchronize()
                self.batches_run += 1
                self.batch_log.append((int(idx.shape[0]), time.perf_counter() - t0))
                self.sched.complete(batch, hi.numpy(), hd.numpy())
            except BaseException as e:  # surfaces in MapRequest.result()
                self.sched.complete(batch, None, None, error=e)


def _concat_rows(batch: List[Slice]):
    """One CSR of the batch's row slices (indptr rebased to 0)."""
    ptrs, inds, dats = [np.zeros(1, np.int64)], [], []
    base = 0
    for r, a, b in batch:
        p0, p1 = int(r.indptr[a]), int(r.indptr[b])
        seg = r.indptr[a + 1:b + 1] - p0 + base
        ptrs.append(seg.astype(np.int64))
        inds.append(r.indices[p0:p1])
        dats.append(r.data[p0:p1])
        base += p1 - p0
    ind = np.concatenate(inds) if inds else np.zeros(0, np.int32)
    dat = np.concatenate(dats) if dats else np.zeros(0, np.int32)
    if ind.size == 0:  # keep the device pointers valid for an all-empty batch
        ind = np.zeros(1, np.int32)
        dat = np.zeros(1, np.int32)
    return np.concatenate(ptrs), ind, dat


def latency_summary(requests: List[MapRequest]) -> dict:
    lat = np.array([r.latency_ms for r in requests if r.latency_ms is not None and r.error is None])
    cells = sum(r.n_cells for r in requests if r.error is None)
    if lat.size == 0:
        return {"requests": 0}
    return {"requests": int(lat.size), "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "max_ms": float(lat.max()), "cells": int(cells)}
