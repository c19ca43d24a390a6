#!/usr/bin/env python
"""make_graph throughput of scarf's graph-construction path on GB300.

Workload (default, ``--config c3``): 1,000,000 cells x 30,000 genes of seeded
negative-binomial counts (40 clusters), 2,000 HVGs, 50 PCs, k = 21, smoothing
chunks of 1,000 rows (``--config c2``: 100,000 cells, 20 clusters). One step =
normalise -> z-stats -> scatter -> FP64 eigh -> projection -> self-kNN (+ self
removal) -> smoothing over the whole matrix.

* ``value``: cells/s of the precision form (BF16 tcgen05 distances + FP32
  re-rank of k+1+16 candidates) with the CSR already resident in HBM.
* ``e2e``: the same through the public pipeline call with pinned HOST CSR,
  which the normalisation kernel reads over the host link in 50,000-cell
  chunks, and the device->host read of indices, distances, edges and weights
  inside every timed step.
* ``plain``: the all-FP32 form on the same input.
* ``--impl reference``: the CPU restatement of the reference path (the
  oracle), timed on a bounded sample of the same workload on the host cores.

Launch: ``python bench.py [--gpus N --steps K --warmup W]``; N > 1 runs under
torchrun as N independent replicas (the path is one GPU per graph).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONFIGS = {
    "c1": dict(name="C1: 10,000 cells x 20,000 genes NB (8 clusters), 2,000 HVGs, 30 PCs, k=11",
               n_cells=10_000, n_genes=20_000, n_clusters=8, n_hvg=2000, dims=30, k=11, lib_median=3000.0),
    "c2": dict(name="C2: 100,000 cells x 30,000 genes NB (20 clusters), 2,000 HVGs, 50 PCs, k=21",
               n_cells=100_000, n_genes=30_000, n_clusters=20, n_hvg=2000, dims=50, k=21, lib_median=3000.0),
    # C2's generator at 40,000 cells: the case the detailed profiler captures use
    # (inputs still larger than L2, a few GB on the device)
    "c2s": dict(name="C2-small: 40,000 cells x 30,000 genes NB (20 clusters), 2,000 HVGs, 50 PCs, k=21",
                n_cells=40_000, n_genes=30_000, n_clusters=20, n_hvg=2000, dims=50, k=21, lib_median=3000.0),
    "c3": dict(name="C3: 1,000,000 cells x 30,000 genes NB (40 clusters), 2,000 HVGs, 50 PCs, k=21, "
                    "50,000-cell chunks from pinned host memory",
               n_cells=1_000_000, n_genes=30_000, n_clusters=40, n_hvg=2000, dims=50, k=21, lib_median=2500.0,
               chunk=50_000),
}
BATCH = 1000
SEED = 4466
# kernel groups timed with CUDA events inside the library ("eigh" is the
# cuSOLVER call; every other name is a kernel of this repository)
PROFILED = ("normalize", "zsplit", "cov_tc", "cov_simt", "eigh", "project", "knn_tc", "knn_simt", "rerank",
            "smooth", "union")
# parts of the filtered eigensolver (inside "eigh")
EIG_PARTS = ("eig_filter", "eig_qr", "eig_rr32", "eig_rr64")


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(ms: float, device) -> float:
    """The job's step time: the slowest rank's (all-reduce MAX over the
    process group; the rank's own time outside one)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return ms
    t = torch.tensor([ms], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "sm_min_mhz": min(sm) if sm else None, "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
def make_input(cfg, device):
    from scarf_gb300 import synth
    csr = synth.nb_counts(cfg["n_cells"], cfg["n_genes"], cfg["n_clusters"], SEED, lib_median=cfg["lib_median"],
                          device=device, chunk=4096)
    feat = synth.select_hvgs(csr, cfg["n_hvg"])
    return csr, feat


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"],
                "bf16_tflops_sustained": d.get("bf16_tflops_sustained"), "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "source": "fallback"}


# DRAM bytes (read + write) per launch from one-pass ncu captures of the
# full-size C2 and C3 steps (dram__bytes_read.sum + dram__bytes_write.sum; the
# commands and per-kernel tables are kept under profiles/). At C2 "normalize"
# is the row pass, the column-statistics pass and the partial reductions
# together, and "smooth" the smoothing kernel with its two chunk kernels.
# Only the line's dominant kernel (knn_tc) feeds roofline.traffic; the zsplit
# and rerank figures were captured before their 16-byte-load forms.
DRAM_TRAFFIC = {
    "c2:normalize": 3_442_579_776, "c2:zsplit": 1_596_928_704, "c2:cov_tc": 1_729_305_792,
    "c2:project": 831_836_245, "c2:knn_tc": 25_911_808, "c2:rerank": 36_871_680, "c2:smooth": 36_306_773,
    "c3:zsplit": 18_312_334_720, "c3:cov_tc": 53_842_151_360, "c3:project": 8_341_655_616,
    "c3:knn_tc": 17_302_698_854, "c3:rerank": 4_295_605_350, "c3:smooth": 698_150_464,
}


def traffic_table():
    return DRAM_TRAFFIC


def kernel_work(cfg, nnz):
    """Algorithmic work of one launch of each kernel at this workload."""
    n, h, d, k = cfg["n_cells"], cfg["n_hvg"], cfg["dims"], cfg["k"]
    return {
        "normalize": ("hbm", 8.0 * nnz + 8.0 * (n + 1) + 4.0 * n * h),
        "zsplit": ("hbm", 4.0 * n * h + 4.0 * n * h),
        # the symmetric scatter: h(h+1)/2 entries x n multiply-adds, three
        # split products for the tensor-core form
        "cov_tc": ("tensor", 3 * 1.0 * n * h * (h + 1)),
        "cov_simt": ("fp32", 1.0 * n * h * (h + 1)),
        "project": ("fp32", 2.0 * n * h * d),
        "knn_tc": ("tensor", 2.0 * n * n * d),
        "knn_simt": ("fp32", 2.0 * n * n * d),
        "rerank": ("fp32", 2.0 * n * (k + 1 + 16) * d),
        "smooth": ("hbm", n * k * (8.0 + 4.0) + n * k * (16.0 + 8.0)),
        "union": ("hbm", 2.0 * n * k * 24 + 2 * 2 * 2.0 * n * k * 8 + 2.0 * n * k * 12),
    }


# ---------------------------------------------------------------------------
def _sample_rows(n, n_sample, seed, device):
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    return torch.randperm(n, generator=g)[:min(n_sample, n)].sort().values.to(device)


def _fp64_topk(S, rows, k, block=512):
    """Exact FP64 squared-L2 top-k (self removed) of the rows ``rows`` of S
    against all of S: (distances ascending, indices)."""
    import torch
    dl, il = [], []
    sn = (S * S).sum(1)
    for a in range(0, len(rows), block):
        r = rows[a:a + block]
        q = S[r]
        d2 = (q * q).sum(1, keepdim=True) + sn[None, :] - 2.0 * q @ S.T
        d2[torch.arange(len(r), device=S.device), r] = float("inf")
        v, i = torch.topk(d2, k, dim=1, largest=False)
        # exact differences for the winners
        diff = q[:, None, :] - S[i]
        v = (diff * diff).sum(-1)
        v, o = v.sort(1)
        dl.append(v)
        il.append(torch.gather(i, 1, o))
    return torch.cat(dl), torch.cat(il)


def smooth_fp64(dist, k, bandwidth=1.5, n_iter=64, tol=1e-5, min_scale=1e-3):
    """FP64 restatement of umap's smooth_knn_dist + membership strengths for
    rows whose nearest distance is non-zero (local_connectivity = 1): rho =
    the nearest distance, sigma by bisection on sum_{j>=1} exp(-(d_j - rho)/
    sigma) = log2(k) * bandwidth, clamped below by min_scale x the row mean."""
    import math
    import torch
    target = math.log2(k) * bandwidth
    rho = dist[:, 0]
    lo = torch.zeros_like(rho)
    hi = torch.full_like(rho, float("inf"))
    mid = torch.ones_like(rho)
    active = torch.ones_like(rho, dtype=torch.bool)
    dd = (dist[:, 1:] - rho[:, None])
    for _ in range(n_iter):
        ps = torch.where(dd > 0, torch.exp(-dd / mid[:, None]), torch.ones_like(dd)).sum(1)
        done = (ps - target).abs() < tol
        upd = active & ~done
        gt = upd & (ps > target)
        le = upd & ~(ps > target)
        hi = torch.where(gt, mid, hi)
        lo = torch.where(le, mid, lo)
        mid = torch.where(gt | (le & torch.isfinite(hi)), (lo + hi) / 2, torch.where(le, mid * 2, mid))
        active = upd
        if not bool(active.any()):
            break
    sigma = torch.maximum(mid, min_scale * dist.mean(1))
    e = dist - rho[:, None]
    return torch.where(e > 0, torch.exp(-e / sigma[:, None]), torch.ones_like(e))


def graph_check(res, batch, n_sample=2000, seed=0):
    """Sampled rows of one result against FP64 on its own scores: tie-aware
    recall@k and the max-abs error of the edge weights (row weights in rank
    order) against FP64 smoothing of the FP64 exact distances. Entries that
    the chunk-local self rule sets to the global minimum are left out."""
    import torch
    n, k = res.indices.shape
    rows = _sample_rows(n, n_sample, seed, res.scores.device)
    s = res.scores[:, :res.dims].double()
    dt, _ = _fp64_topk(s, rows, k)
    diff = s[rows][:, None, :] - s[res.indices[rows]]
    dg = (diff * diff).sum(-1)
    rec = float((dg <= dt[:, -1:] * (1 + 1e-6) + 1e-12).double().mean().item())
    keep = dt[:, 0] > 0
    wt = smooth_fp64(dt[keep], k)
    w = res.weights.view(n, k)[rows][keep]
    quirk = res.indices[rows][keep] == (rows[keep] % batch)[:, None]
    err = ((w - wt).abs() * (~quirk)).max()
    return rec, float(err.item())


def fp64_truth(K, pipeline, ip, ind, dat, G, feat, dims, k, results, n_sample=2000, seed=0, block=50_000):
    """The FP64 pipeline on this workload's normalised matrix: FP64 scatter of
    the z-scaled rows (torch FP64 GEMM), FP64 eigendecomposition, FP64 scores
    and exact FP64 kNN of sampled rows. Returns, per form, the max principal
    angle of its subspace against the FP64 one (leading 10 and all dims) and
    the tie-aware recall@k of its graph against the FP64 pipeline's kNN."""
    import torch
    x, cs, cq = pipeline.normalize_csr_host(ip, ind, dat, G, feat, device=ip.device)
    n = x.shape[0]
    h = len(feat)
    mu, sg, _, _ = K.zstats(cs, cq, n)
    dev = x.device
    cov = torch.zeros((h, h), dtype=torch.float64, device=dev)
    zs = torch.zeros(h, dtype=torch.float64, device=dev)
    for a in range(0, n, block):
        z = (x[a:a + block, :h].double() - mu[None, :h]) / sg[None, :h]
        cov += z.T @ z
        zs += z.sum(0)
    comps = K.pca_basis(cov, zs, n, dims + 1, n_load=dims, ld_l=dims, eigh="fp64")[0][:, :dims].contiguous()
    S = torch.empty((n, dims), dtype=torch.float64, device=dev)
    for a in range(0, n, block):
        S[a:a + block] = ((x[a:a + block, :h].double() - mu[None, :h]) / sg[None, :h]) @ comps
    del x
    rows = _sample_rows(n, n_sample, seed, dev)
    kth = _fp64_topk(S, rows, k)[0][:, -1]
    T = comps.cpu().numpy()

    def max_angle(A, B):
        qa, _ = np.linalg.qr(A)
        qb, _ = np.linalg.qr(B)
        sv = np.clip(np.linalg.svd(qa.T @ qb, compute_uv=False), -1.0, 1.0)
        return float(np.arccos(sv).max())

    out = {}
    for name, r in results.items():
        B = r.components[:, :dims].cpu().numpy()
        diff = S[rows][:, None, :] - S[r.indices[rows]]
        dg = (diff * diff).sum(-1)
        out[name] = {"max_angle_top10_rad": max_angle(B[:, :10], T[:, :10]),
                     "max_angle_all_rad": max_angle(B, T),
                     "recall_at_k_vs_fp64_pipeline": round(float((dg <= kth[:, None] * (1 + 1e-6) + 1e-12)
                                                                 .double().mean().item()), 5)}
    return out


def host_link(dev, nbytes=2 << 30, reps=3):
    """Pinned host <-> device copy bandwidth of this machine: one large copy each
    way (a single cudaMemcpyAsync of a pinned buffer), best of ``reps``,
    timed with CUDA events on the copying stream."""
    import torch
    hbuf = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    dbuf = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    st = torch.cuda.current_stream()
    out = {"bytes": nbytes}
    for name, (dst, src) in (("h2d_gbs", (dbuf, hbuf)), ("d2h_gbs", (hbuf, dbuf))):
        dst.copy_(src, non_blocking=True)
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            dst.copy_(src, non_blocking=True)
            e1.record(st)
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        out[name] = round(nbytes / (best * 1e-3) / 1e9, 1)
    del hbuf, dbuf
    return out


def datastore_e2e(csr, feat, cfg, reps=2):
    """``DataStore.make_graph`` (the drop-in surface) from host numpy CSR to
    the store's u8/f8 datasets, precision form, wall clock with the device
    synchronised on both sides; a fresh DataStore per call so nothing is
    cached. It includes what the reference's make_graph also does beyond the
    timed step: the k-means seeding and the host-side dataset writes."""
    import gc
    import torch
    from scarf_gb300.datastore import DataStore
    mask = np.zeros(csr.n_genes, dtype=bool)
    mask[feat] = True
    times = []
    for i in range(reps + 1):
        ds = DataStore(csr.indptr, csr.indices, csr.data, csr.n_genes, precision="precision")
        ds.RNA.feats.insert("I__hvgs", mask)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ds.make_graph(feat_key="hvgs", dims=cfg["dims"], k=cfg["k"], batch_size=BATCH)
        torch.cuda.synchronize()
        if i:
            times.append(time.perf_counter() - t0)
        del ds
        gc.collect()
        torch.cuda.empty_cache()
    ms = statistics.median(times) * 1e3
    return {"value": round(csr.n_cells / (ms * 1e-3), 1), "unit": "cells/s", "ms_per_step": round(ms, 1),
            "calls": reps, "note": "DataStore.make_graph from host numpy CSR to the store's datasets (indices u8, "
            "distances f8, edges u8, weights f8, the k-means group), wall clock"}


def run_gb300(args, cfg):
    import torch
    import torch.distributed as dist

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        dist.init_process_group("nccl")
    import __graft_entry__
    __graft_entry__.build()
    from scarf_gb300 import kernels as K
    from scarf_gb300 import pipeline

    dev = torch.device("cuda", local)
    csr, feat = make_input(cfg, dev)
    n, G = csr.n_cells, csr.n_genes
    dims, k = cfg["dims"], cfg["k"]
    chunk = cfg.get("chunk")
    ip_h = torch.from_numpy(csr.indptr).pin_memory()
    ind_h = torch.from_numpy(csr.indices).pin_memory()
    dat_h = torch.from_numpy(csr.data).pin_memory()
    ip_d, ind_d, dat_d = ip_h.to(dev), ind_h.to(dev), dat_h.to(dev)
    torch.cuda.synchronize()

    def step(form, host=False, outs=None):
        if host:
            res = pipeline.make_graph(ip_h, ind_h, dat_h, G, feat, dims, k, batch_size=BATCH, precision=form,
                                      chunk_cells=chunk, keep_x=False)
            # the step's result read back to the host
            for name in ("indices", "distances", "edges", "weights"):
                outs[name].copy_(getattr(res, name), non_blocking=True)
            return res
        return pipeline.make_graph(ip_d, ind_d, dat_d, G, feat, dims, k, batch_size=BATCH, precision=form,
                                   keep_x=False)

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            dist.barrier()
        torch.cuda.synchronize()

    def timed(form, steps, warmup, host=False, prof=False):
        outs = None
        if host:
            outs = {"indices": torch.empty((n, k), dtype=torch.int64).pin_memory(),
                    "distances": torch.empty((n, k), dtype=torch.float32).pin_memory(),
                    "edges": torch.empty((n * k, 2), dtype=torch.int64).pin_memory(),
                    "weights": torch.empty(n * k, dtype=torch.float64).pin_memory()}
        res = None
        for _ in range(warmup):
            res = step(form, host, outs)
        barrier()
        if prof:
            K.profile(True)
            K.profile_reset()
        l0 = K.kernel_launches()
        st = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(steps):
            res = step(form, host, outs)
        e1.record(st)
        barrier()
        launches = K.kernel_launches() - l0
        ms = e0.elapsed_time(e1) / steps
        prof_ms = {}
        if prof:
            for name in PROFILED:
                t, c = K.profile_query(name)
                if c:
                    prof_ms[name] = (t / c, c / steps)
            for name in EIG_PARTS:
                t, c = K.profile_query(name)
                if c:
                    eig_parts[name] = {"ms_per_step": round(t / steps, 3), "calls_per_step": c / steps}
            K.profile(False)
        ms = max_over_ranks(ms, dev)
        return ms, res, launches, prof_ms, outs

    eig_parts = {}
    sampler = ClockSampler(local)
    sampler.start()
    ms, res, launches, prof_ms, _ = timed("precision", args.steps, args.warmup, prof=True)
    clocks = sampler.stop()
    knn_layout = {"splits": K.knn_last_splits(), "locality_order": bool(K.knn_last_locality())}
    rec, werr = graph_check(res, BATCH)
    ann_recall = res.recall()
    sampler_e2e = ClockSampler(local)
    sampler_e2e.start()
    e2e_ms, res_h, _, _, outs = timed("precision", args.steps, args.warmup, host=True)
    clocks_e2e = sampler_e2e.stop()
    plain_ms, res_p, _, prof_p, _ = timed("plain", max(1, min(args.steps, 3)), 1, prof=True)
    rec_p, werr_p = graph_check(res_p, BATCH)
    truth = fp64_truth(K, pipeline, ip_d, ind_d, dat_d, G, feat, dims, k, {"precision": res, "plain": res_p})

    # the fuzzy union of the graph just built (load_graph(symmetric=True)), timed alone
    K.profile(True)
    K.profile_reset()
    for _ in range(3):
        K.fuzzy_union(res.edges, res.weights, n, k)
    torch.cuda.synchronize()
    t_u, c_u = K.profile_query("union")
    K.profile(False)
    if c_u:
        prof_ms["union"] = (t_u / c_u, 0.0)
    # the k-means seeding step of make_graph (MiniBatchKMeans, 1,000 centres,
    # blocks of the batch size), reported beside the step as the reference
    # does not count it in make_graph's graph time
    n_cent = min(1000, BATCH)
    K.kmeans(res.scores, dims, n_cent, BATCH, 4466)
    torch.cuda.synchronize()
    st_k = torch.cuda.current_stream()
    k0, k1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    k0.record(st_k)
    K.kmeans(res.scores, dims, n_cent, BATCH, 4466)
    k1.record(st_k)
    torch.cuda.synchronize()
    kmeans_info = {"ms": round(k0.elapsed_time(k1), 3), "n_clusters": n_cent, "block_rows": BATCH,
                   "note": "partial_fit per block of the scores, then predict; not part of ms_per_step"}
    eig = eigensolver_comparison(K, pipeline, ip_d, ind_d, dat_d, G, feat, n, dims)
    pk = peaks()
    work = kernel_work(cfg, csr.nnz)
    kernels = {}
    for name, (t, per_step) in prof_ms.items():
        kind, amount = work.get(name, (None, None))
        ent = {"ms": round(t, 4), "launches_per_step": per_step}
        if kind == "hbm":
            ent["GB/s"] = round(amount / (t * 1e-3) / 1e9, 1)
        elif kind in ("tensor", "fp32"):
            ent["TFLOP/s"] = round(amount / (t * 1e-3) / 1e12, 2)
        kernels[name] = ent
    own = {k_: v for k_, v in prof_ms.items() if k_ != "eigh"}
    top = max(own.items(), key=lambda kv: kv[1][0])[0] if own else None
    roof = None
    tt = traffic_table()
    if top is not None:
        kind, amount = work.get(top, ("tensor", 0.0))
        t = prof_ms[top][0] * 1e-3
        if kind == "hbm":
            ach, peak, unit = amount / t / 1e9, pk["hbm_gbs"], "GB/s"
        else:
            ach, peak, unit = amount / t / 1e12, pk["bf16_tflops"], "TFLOP/s"
        tr = tt.get(f"{args.config}:{top}")
        roof = {"kernel": top, "bound": "hbm" if kind == "hbm" else "tensor", "achieved": round(ach, 2),
                "peak": peak, "unit": unit, "frac": round(ach / peak, 4),
                "traffic": tr, "peak_source": pk["source"] + " (MEASURED_PEAKS.json, burst)",
                "work_per_launch": amount}
    h2d = int(ip_h.numel() * 8 + ind_h.numel() * 4 + dat_h.numel() * 4)
    d2h = int(sum(v.numel() * v.element_size() for v in outs.values()))
    del outs, res_h
    link = host_link(dev)
    # the normalisation reading the pinned CSR over the link itself (the e2e form)
    zc = []
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        pipeline.normalize_csr_host(ip_h, ind_h, dat_h, G, feat, chunk_cells=chunk, device=dev)
        e1.record()
        e1.synchronize()
        zc.append(e0.elapsed_time(e1))
    link["normalize_read_gbs"] = round(h2d / (min(zc) * 1e-3) / 1e9, 1)
    link["normalize_read_ms"] = round(min(zc), 3)
    # the step cannot beat the larger of its device time and its copies at the link's rate
    bound_ms = max(ms, h2d / (link["h2d_gbs"] * 1e9) * 1e3 + d2h / (link["d2h_gbs"] * 1e9) * 1e3)
    ds_e2e = None if args.no_datastore else datastore_e2e(csr, feat, cfg)
    serving = None
    if not args.no_serve:
        sv = serve_measure()
        serving = {k_: sv[k_] for k_ in ("p50_ms", "p99_ms", "p50_ms_requests_le_10k_cells",
                                          "p99_ms_requests_le_10k_cells", "requests", "cells", "cells_per_s",
                                          "gpu_batches", "batch_ms_p50", "batch_ms_p99",
                                          "recall_at_k_sampled_request")}
        serving["config"] = sv["config"]["workload"]
    cells = n * ws
    line = {
        "metric": "make_graph cells/s",
        "value": round(cells / (ms * 1e-3), 1),
        "unit": "cells/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "bf16",
        "data": "synthetic (seeded negative-binomial counts generated on the device)",
        "config": {"workload": cfg["name"], "form": "precision: 3xbf16 tcgen05 scatter, chebyshev-filtered f32 eigh + f64 "
                   "Rayleigh-Ritz, bf16 tcgen05 distances, f32 re-rank", "margin": 16, "batch_size": BATCH,
                   "nnz": csr.nnz, "l2": "inputs larger than L2 (CSR %.2f GB, normalised matrix %.2f GB)"
                   % (h2d / 1e9, n * cfg["n_hvg"] * 4 / 1e9), "parallelism": f"replicas x{ws}"},
        "recall_at_k": round(rec, 5),
        "edge_weight_max_abs_err": werr,
        "ann_recall_pct": round(ann_recall, 3),
        "vs_fp64_pipeline": truth["precision"],
        "accuracy_note": "recall_at_k and edge_weight_max_abs_err: 2,000 sampled rows against exact FP64 kNN and "
                         "FP64 smoothing of the result's own scores; vs_fp64_pipeline: principal angles against the "
                         "FP64 scatter + FP64 eigendecomposition, and recall@k against the kNN of its FP64 scores",
        "plain": {"value": round(cells / (plain_ms * 1e-3), 1), "ms_per_step": round(plain_ms, 3),
                  "recall_at_k": round(rec_p, 5), "edge_weight_max_abs_err": werr_p,
                  "vs_fp64_pipeline": truth["plain"], "speedup_precision_vs_plain": round(plain_ms / ms, 3),
                  "kernels_ms": {k_: round(v[0], 4) for k_, v in prof_p.items()}},
        "kernels": kernels,
        "knn_layout": knn_layout,
        "eigh_parts": eig_parts,
        "eigensolver": eig,
        "kmeans": kmeans_info,
        "e2e": {"value": round(cells / (e2e_ms * 1e-3), 1), "unit": "cells/s", "ms_per_step": round(e2e_ms, 3),
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "host_link": link,
                "bound_ms": round(bound_ms, 3), "frac_of_bound": round(bound_ms / e2e_ms, 4),
                "call": "pipeline.make_graph on pinned host CSR, read over the host link by the normalisation "
                        "kernel itself (%s), outputs read back"
                        % ("chunks of %d cells" % chunk if chunk else "one launch"), "clocks": clocks_e2e},
        "e2e_datastore": ds_e2e,
        "serving": serving,
        "roofline": roof,
        "clocks": clocks,
        "gpu_launches": int(launches),
    }
    if rank == 0 and ws == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(cfg, device=dev)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()


def eigensolver_comparison(K, pipeline, ip, ind, dat, G, feat, n, dims, reps=3):
    """FP64 partial eigendecomposition (the plain form's solver) against the
    mixed FP32 + FP64 Rayleigh-Ritz solver and the Chebyshev-filtered
    subspace iteration on this workload's scatter: device time of each and the
    principal angles between its leading subspace and the FP64 one."""
    import torch
    x, cs, cq = pipeline.normalize_csr_host(ip, ind, dat, G, feat, device=ip.device)
    mu, sg, mu32, sg32 = K.zstats(cs, cq, n)
    cov, zsum = K.covariance(x, mu32, sg32, n_cols=len(feat), precision="precision")
    del x
    out = {}
    comps = {}
    for method in ("fp64", "mixed", "filter"):
        K.pca_basis(cov, zsum, n, dims + 1, n_load=dims, ld_l=dims, eigh=method)
        torch.cuda.synchronize()
        st = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(reps):
            c, ev, _, _ = K.pca_basis(cov, zsum, n, dims + 1, n_load=dims, ld_l=dims, eigh=method)
        e1.record(st)
        torch.cuda.synchronize()
        out[f"{method}_ms"] = round(e0.elapsed_time(e1) / reps, 3)
        comps[method] = (c.cpu().numpy(), ev.cpu().numpy())
        if method == "filter":
            out["filter_residual"] = K.filter_residual()

    def angle(a, b):
        qa, _ = np.linalg.qr(a)
        qb, _ = np.linalg.qr(b)
        return float(np.arccos(np.clip(np.linalg.svd(qa.T @ qb, compute_uv=False), -1, 1)).max())
    a = comps["fp64"][0]
    for method in ("mixed", "filter"):
        b = comps[method][0]
        out[f"{method}_max_angle_top10_rad"] = angle(a[:, :10], b[:, :10])
        out[f"{method}_max_angle_all_rad"] = angle(a[:, :dims], b[:, :dims])
        out[f"{method}_max_eval_rel_diff"] = float(np.max(np.abs(comps["fp64"][1] - comps[method][1])
                                                          / np.abs(comps["fp64"][1])))
    return out


# ---------------------------------------------------------------------------
CPU_SAMPLE_CELLS = 10_000


def cpu_sample(cfg, n_cells=None, device=None):
    """A bounded sample of the workload for the CPU legs: ``n_cells`` cells
    drawn from the same seeded populations (genes, clusters, library sizes),
    with their own top-variance HVGs. At C1 the sample is the whole workload."""
    from scarf_gb300 import synth
    n = min(cfg["n_cells"], n_cells or CPU_SAMPLE_CELLS)
    csr = synth.nb_counts(n, cfg["n_genes"], cfg["n_clusters"], SEED, lib_median=cfg["lib_median"],
                          device=device or "cpu", chunk=4096)
    return csr, synth.select_hvgs(csr, cfg["n_hvg"])


def cpu_make_graph(csr, feat, cfg):
    """One make_graph of ``csr`` by the CPU restatement of the reference path
    (the oracle): normalise, z-statistics, the reference's IncrementalPCA in
    its block order, the reducer, self-kNN with the self fix (exact numpy kNN
    standing in for hnswlib) and smoothing, each stage timed. Returns
    ``(seconds, {stage: seconds})``."""
    import oracle
    dims, k = cfg["dims"], cfg["k"]
    t = {}
    t0 = time.perf_counter()
    x, _ = oracle.normed_csr(csr.indptr, csr.indices, csr.data, csr.n_genes, feat)
    mu, sg = oracle.zstats(x)
    t["normalise+stats"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    z = (x - mu) / sg
    blocks = [z[a:a + BATCH] for a in range(0, z.shape[0], BATCH)]
    load, _ = oracle.fit_pca_reference_order(blocks, dims)
    t["pca (IncrementalPCA)"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    s = oracle.reducer(x, mu, sg, load)
    t["projection"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    ki, kd, _ = oracle.self_query_knn(s, k, BATCH)
    t["exact kNN (stand-in for hnswlib)"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    oracle.smoothen_dists(ki, kd, 1.0, 1.5, BATCH)
    t["smoothing"] = time.perf_counter() - t0
    return sum(t.values()), t


def projected_cells_per_s(stage_s, n_sample, n_full):
    """The full workload's cells/s projected from one sample's stage times:
    every stage linear in cells, the exact kNN quadratic. A projection, not a
    measurement."""
    f = n_full / n_sample
    tot = sum(v * f for k_, v in stage_s.items() if not k_.startswith("exact kNN"))
    tot += sum(v * f * f for k_, v in stage_s.items() if k_.startswith("exact kNN"))
    return round(n_full / tot, 2)


def cpu_baseline(cfg, device=None):
    csr, feat = cpu_sample(cfg, device=device)
    cpu_make_graph(csr, feat, cfg)                    # warm-up (BLAS threads, page faults)
    secs, stages = cpu_make_graph(csr, feat, cfg)
    whole = csr.n_cells == cfg["n_cells"]
    return {"value": round(csr.n_cells / secs, 2), "unit": "cells/s", "cores": os.cpu_count(), "kind": "port",
            "sample": (f"the whole workload ({csr.n_cells} cells)" if whole else
                       f"make_graph of a {csr.n_cells}-cell sample drawn from the workload's populations "
                       f"({cfg['n_genes']} genes, {cfg['n_hvg']} HVGs, {cfg['dims']} PCs, k={cfg['k']}), "
                       f"measured") + "; oracle restatement: numpy/scipy, scikit-learn-order IncrementalPCA, "
                       "exact numpy kNN standing in for hnswlib; BLAS on all cores, the rest single-threaded",
            "seconds": round(secs, 3), "stage_seconds": {k_: round(v, 3) for k_, v in stages.items()},
            "projected_full_workload_cells_per_s": None if whole else
            projected_cells_per_s(stages, csr.n_cells, cfg["n_cells"])}


def run_reference(args, cfg):
    """The reference arm: the CPU restatement of the reference path (the
    oracle) on the host cores. Each step is one whole make_graph of a bounded
    sample of the workload (10,000 cells; at C1 the whole workload), timed by
    the wall clock; ``value`` is that sample's cells/s as measured."""
    ws, rank, local = dist_env()
    if rank != 0:
        return
    import torch
    csr, feat = cpu_sample(cfg, device="cuda" if torch.cuda.is_available() else "cpu")
    secs, stages = [], None
    for i in range(args.warmup + args.steps):
        t, st = cpu_make_graph(csr, feat, cfg)
        if i >= args.warmup:
            secs.append(t)
            stages = st
    med = statistics.median(secs)
    v = round(csr.n_cells / med, 2)
    whole = csr.n_cells == cfg["n_cells"]
    sample = (f"the whole workload ({csr.n_cells} cells) per step" if whole else
              f"per step one make_graph of a {csr.n_cells}-cell sample drawn from the workload's populations")
    print(json.dumps({
        "impl": "reference", "metric": "make_graph cells/s", "value": v, "unit": "cells/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(med * 1e3, 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (same seeded populations)",
        "config": {"workload": cfg["name"], "form": "reference CPU restatement (oracle)", "sample_cells":
                   csr.n_cells},
        "cpu_baseline": {"value": v, "unit": "cells/s", "cores": os.cpu_count(), "kind": "port",
                         "sample": sample + "; numpy/scipy, scikit-learn-order IncrementalPCA, exact numpy kNN "
                                   "standing in for hnswlib; BLAS on all cores"},
        "stage_seconds": {k_: round(x, 3) for k_, x in stages.items()},
        "projected_full_workload_cells_per_s": None if whole else
        projected_cells_per_s(stages, csr.n_cells, cfg["n_cells"]),
        "e2e": {"value": v, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="c3", choices=sorted(CONFIGS))
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline leg")
    ap.add_argument("--no-serve", action="store_true", help="skip the C4 serving figures in the default line")
    ap.add_argument("--no-datastore", action="store_true", help="skip the DataStore.make_graph e2e figure")
    ap.add_argument("--mode", default="full", choices=["full", "step", "serve", "knn", "union", "batched", "umap"],
                    help="step: warm-up steps then one make_graph step and nothing else (for profilers); "
                         "serve: the mapping service's latency under a Poisson request stream")
    ap.add_argument("--form", default="precision", choices=["precision", "plain"], help="form used by --mode step")
    ap.add_argument("--knn-queries", type=int, default=110_000, help="--mode knn: query rows")
    ap.add_argument("--knn-refs", type=int, default=1_000_000, help="--mode knn: reference rows")
    ap.add_argument("--knn-source", default=None, choices=sorted(CONFIGS),
                    help="--mode knn: self-kNN of this config's PCA scores instead of clustered points")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup) if args.impl == "gb300" else args.warmup
    cfg = CONFIGS[args.config]
    if args.impl == "reference":
        run_reference(args, cfg)
    elif args.mode == "step":
        run_step(args, cfg)
    elif args.mode == "serve":
        run_serve(args)
    elif args.mode == "knn":
        run_knn(args)
    elif args.mode == "union":
        run_union(args, cfg)
    elif args.mode == "batched":
        run_batched(args)
    elif args.mode == "umap":
        run_umap_layout(args)
    else:
        run_gb300(args, cfg)


SERVE = dict(name="C4: mapping service over a device-resident 500,000-cell reference (30,000 genes NB, 20 clusters, "
                   "2,000 HVGs, 50 PCs, BF16 projection); Poisson stream of query batches of log-uniform "
                   "100-50,000 cells drawn from the same populations with library sizes shifted to 2,200 UMIs; k=11",
             n_ref=500_000, n_genes=30_000, n_clusters=20, n_hvg=2000, dims=50, k=11, lib_median=3000.0,
             query_lib=2200.0, pool=60_000, n_requests=120, rate_hz=40.0, max_batch_rows=16384)


def run_serve(args):
    """p50/p99 request latency and cells/s of the continuous-batching mapper."""
    import __graft_entry__
    __graft_entry__.build()
    print(json.dumps(serve_measure()), flush=True)


def serve_measure():
    """The C4 serving workload: a 500,000-cell reference built by make_graph
    and kept on the device, 120 Poisson-arriving requests of log-uniform
    100-50,000 cells through MappingServer; latency percentiles, cells/s,
    batch and upload timings, and the recall of one request against exact
    FP64 kNN."""
    import torch
    from scarf_gb300 import pipeline, synth
    from scarf_gb300.serving import MappingServer, Reference, latency_summary
    c = SERVE
    dev = torch.device("cuda", 0)
    ref_csr = synth.nb_counts(c["n_ref"], c["n_genes"], c["n_clusters"], SEED, lib_median=c["lib_median"],
                              device=dev)
    feat = synth.select_hvgs(ref_csr, c["n_hvg"])
    ip, ind, dat = (torch.from_numpy(a).to(dev) for a in (ref_csr.indptr, ref_csr.indices, ref_csr.data))
    g = pipeline.make_graph(ip, ind, dat, ref_csr.n_genes, feat, c["dims"], c["k"], precision="precision",
                            smooth=False, keep_x=False)
    del ip, ind, dat
    ref = Reference.from_graph(g, precision="precision")
    pool = synth.nb_counts(c["pool"], c["n_genes"], c["n_clusters"], SEED, lib_median=c["query_lib"], device=dev,
                           cells_seed=SEED + 1)
    rng = np.random.default_rng(7)
    sizes = np.exp(rng.uniform(np.log(100), np.log(50_000), c["n_requests"])).astype(int)
    gaps = rng.exponential(1.0 / c["rate_hz"], c["n_requests"])
    starts = [int(rng.integers(0, c["pool"] - s + 1)) for s in sizes]
    genes = np.arange(c["n_genes"]).astype(str)

    def slice_rows(a, n):
        p0, p1 = int(pool.indptr[a]), int(pool.indptr[a + n])
        return pool.indptr[a:a + n + 1] - p0, pool.indices[p0:p1], pool.data[p0:p1]

    with MappingServer(ref, genes[feat], genes, k=c["k"], max_batch_rows=c["max_batch_rows"], n_workers=2,
                       hbm_budget_bytes=16 << 30) as srv:
        for s in (100, 5000, 20000):          # warm-up: handles, scratch, pinned staging
            srv.submit(*slice_rows(0, s)).result(timeout=120)
        reqs = []
        t0 = time.perf_counter()
        t = t0
        for s, a, gap in zip(sizes, starts, gaps):
            t += gap
            now = time.perf_counter()
            if t > now:
                time.sleep(t - now)
            reqs.append(srv.submit(*slice_rows(a, int(s)), arrival=t))
        for r in reqs:
            r.result(timeout=600)
        t_end = max(r.t_done for r in reqs)
        batches = srv.batches_run
        blog = np.array(srv.batch_log[3:], dtype=np.float64).reshape(-1, 2)
        ulog = np.array(srv.upload_log[3:], dtype=np.float64).reshape(-1, 5)
    summ = latency_summary(reqs)
    small = latency_summary([r for r in reqs if r.n_cells <= 10_000])
    # recall of one mid-size request against exact FP64 kNN on the device
    r = reqs[int(np.argsort(sizes)[len(sizes) // 2])]
    qi = r.idx
    a = starts[reqs.index(r)]
    from scarf_gb300 import kernels as K
    from scarf_gb300.datastore import align_col_map
    cmap, missing = align_col_map(genes[feat], genes)
    qp, qind, qdat = slice_rows(a, r.n_cells)
    x = K.normalize_csr(torch.from_numpy(qp).to(dev), torch.from_numpy(qind).to(dev), torch.from_numpy(qdat).to(dev),
                        torch.from_numpy(cmap).to(dev), len(feat), missing_mask=torch.from_numpy(missing).to(dev))
    qs = K.project(x, g.mu32, g.sigma32, g.loadings32.contiguous(), g.dims, n_cols=len(feat))[:, :g.dims].double()
    rs = g.scores[:, :g.dims].double()
    d2 = (qs * qs).sum(1, keepdim=True) + (rs * rs).sum(1)[None, :] - 2.0 * qs @ rs.T
    kth = torch.topk(d2, c["k"], dim=1, largest=False).values[:, -1]
    got = torch.from_numpy(qi).to(dev)
    dg = ((qs[:, None, :] - rs[got]) ** 2).sum(-1)
    rec = float((dg <= kth[:, None] * (1 + 1e-6) + 1e-12).double().mean().item())
    out = {
        "metric": "mapping latency p99 (ms)", "value": round(summ["p99_ms"], 3), "unit": "ms",
        "higher_is_better": False, "p50_ms": round(summ["p50_ms"], 3), "p99_ms": round(summ["p99_ms"], 3),
        "p99_ms_requests_le_10k_cells": round(small.get("p99_ms", float("nan")), 3),
        "p50_ms_requests_le_10k_cells": round(small.get("p50_ms", float("nan")), 3),
        "requests": summ["requests"], "cells": summ["cells"],
        "cells_per_s": round(summ["cells"] / (t_end - t0), 1), "gpu_batches": batches,
        "batch_rows_mean": round(float(blog[:, 0].mean()), 1) if len(blog) else None,
        "batch_ms_p50": round(float(np.percentile(blog[:, 1], 50)) * 1e3, 3) if len(blog) else None,
        "batch_ms_p99": round(float(np.percentile(blog[:, 1], 99)) * 1e3, 3) if len(blog) else None,
        "upload_ms_p50": round(float(np.percentile(ulog[:, 3:].sum(1), 50)) * 1e3, 3) if len(ulog) else None,
        "upload_ms_p99": round(float(np.percentile(ulog[:, 3:].sum(1), 99)) * 1e3, 3) if len(ulog) else None,
        "upload_queue_ms_p99": round(float(np.percentile(ulog[:, 2], 99)) * 1e3, 3) if len(ulog) else None,
        "slowest_uploads": [{"cells": int(u[0]), "MB": round(u[1] / 1e6, 1), "queued_ms": round(u[2] * 1e3, 2),
                             "issue_ms": round(u[3] * 1e3, 2), "land_ms": round(u[4] * 1e3, 2)}
                            for u in sorted(ulog.tolist(), key=lambda u: -(u[3] + u[4]))[:4]],
        "recall_at_k_sampled_request": round(rec, 5), "data": "synthetic",
        "config": {"workload": c["name"], "arrival_rate_hz": c["rate_hz"], "max_batch_rows": c["max_batch_rows"],
                   "workers": 2, "form": "precision"}}
    del g, ref, pool
    torch.cuda.empty_cache()
    return out


def run_umap_layout(args):
    """The UMAP layout alone (f3 case): seeded clustered points (20 centres,
    d = 50, N(0, 1) offsets) of --knn-refs rows, their precision self-kNN
    (k = 21), smoothing and fuzzy union, then 300 layout epochs of a random 2-D
    start, timed with CUDA events after a 10-epoch warm-up."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from scarf_gb300 import kernels as K
    from scarf_gb300 import umap as gu
    dev = torch.device("cuda", 0)
    n, d, k = args.knn_refs, 50, 21
    g = torch.Generator(device="cuda").manual_seed(3)
    centers = torch.randn((20, d), generator=g, device=dev) * 4.0
    lab = torch.randint(0, 20, (n,), generator=g, device=dev)
    x = torch.zeros((n, 52), device=dev)
    x[:, :d] = centers[lab] + torch.randn((n, d), generator=g, device=dev)
    idx, dist, _ = K.knn(x, x, d, k, self_offset=0, margin=16, precision="precision")
    edges, w = K.smooth(idx, dist, 1.0, 1.5, BATCH)
    ip, ind, dat = K.fuzzy_union(edges, w, n, k)
    nnz = int(ip[-1].item())
    rows = torch.repeat_interleave(torch.arange(n, device=dev, dtype=torch.int32), ip[1:] - ip[:-1])
    cols = ind[:nnz].contiguous()
    eps = torch.from_numpy(gu.make_epochs_per_sample(dat[:nnz].cpu().numpy(), 300).astype(np.float64)).to(dev)
    a, b = gu.find_ab_params(2.0, 1.0)
    y = (torch.randn((n, 2), generator=g, device=dev) * 10).contiguous()
    K.umap_layout(rows, cols, eps, y.clone(), 10, a, b, seed=1)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    K.umap_layout(rows, cols, eps, y, 300, a, b, seed=1)
    e1.record()
    torch.cuda.synchronize()
    print(json.dumps({"mode": "umap", "cells": n, "edges": nnz, "epochs": 300,
                      "layout_ms": round(e0.elapsed_time(e1), 3), "finite": bool(torch.isfinite(y).all().item())}))


def run_knn_scores(args):
    """The precision self-kNN on a config's PCA scores (--knn-source c1/c2/c3):
    make_graph's own scores, once with the queries being the references (the
    locality order applies) and once with a copy of them as the queries (it
    does not); W warm-up calls and one more of each, CUDA-event timed."""
    import torch
    from scarf_gb300 import kernels as K
    from scarf_gb300 import pipeline
    cfg = CONFIGS[args.knn_source]
    dev = torch.device("cuda", 0)
    csr, feat = make_input(cfg, dev)
    ip, ind, dat = (torch.from_numpy(a).to(dev) for a in (csr.indptr, csr.indices, csr.data))
    g = pipeline.make_graph(ip, ind, dat, csr.n_genes, feat, cfg["dims"], cfg["k"], batch_size=BATCH,
                            precision="precision", smooth=False, keep_x=False, autotune=False)
    del ip, ind, dat
    s = g.scores
    out = {"mode": "knn", "source": args.knn_source, "rows": int(s.shape[0])}
    for name, q in (("self_locality", s), ("copy_no_locality", s.clone())):
        for _ in range(args.warmup):
            K.knn(q, s, g.dims, g.k, self_offset=0, margin=16, precision="precision")
        K.profile(True)
        K.profile_reset()
        idx, _, nm = K.knn(q, s, g.dims, g.k, self_offset=0, margin=16, precision="precision")
        torch.cuda.synchronize()
        t, _ = K.profile_query("knn_tc")
        K.profile(False)
        out[name] = {"knn_tc_ms": round(t, 3), "splits": K.knn_last_splits(),
                     "locality_order": bool(K.knn_last_locality()), "missed": int(nm.item())}
        out.setdefault("_idx", []).append(idx)
    out["same_neighbours"] = bool(torch.equal(out["_idx"][0], out["_idx"][1]))
    del out["_idx"]
    print(json.dumps(out), flush=True)


def run_knn(args):
    """The kNN kernel alone (profiling case): seeded clustered points (40
    centres, N(0, 1) offsets, d = 50), the first --knn-queries rows against
    all --knn-refs rows, k = 21, margin 16, the precision form; W warm-up
    calls and one more. With --knn-source, a config's PCA scores instead
    (run_knn_scores)."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    if args.knn_source:
        return run_knn_scores(args)
    from scarf_gb300 import kernels as K
    dev = torch.device("cuda", 0)
    g = torch.Generator(device="cuda").manual_seed(3)
    n, d, ld = args.knn_refs, 50, 52
    centers = torch.randn((40, d), generator=g, device=dev) * 4.0
    lab = torch.randint(0, 40, (n,), generator=g, device=dev)
    refs = torch.zeros((n, ld), device=dev)
    refs[:, :d] = centers[lab] + torch.randn((n, d), generator=g, device=dev)
    # the first --knn-queries rows; all rows: the self-kNN of make_graph (the
    # same tensor as queries and references, so the locality order applies)
    q = refs if args.knn_queries >= n else refs[:args.knn_queries].contiguous()
    self_offset = 0 if args.knn_queries <= n else -1
    for _ in range(args.warmup):
        K.knn(q, refs, d, 21, self_offset=self_offset, margin=16, precision="precision")
    K.profile(True)
    K.profile_reset()
    idx, dist, nm = K.knn(q, refs, d, 21, self_offset=self_offset, margin=16, precision="precision")
    torch.cuda.synchronize()
    t, _ = K.profile_query("knn_tc")
    t2, _ = K.profile_query("rerank")
    K.profile(False)
    print(json.dumps({"mode": "knn", "queries": int(q.shape[0]), "refs": n, "knn_tc_ms": round(t, 3),
                      "rerank_ms": round(t2, 3), "missed": int(nm.item())}))


BATCHED = dict(name="C5: 256 independent samples of log-uniform 500-20,000 cells (20,000 genes NB, 8 clusters, "
                     "library sizes around 3,000: the C1 generator), 2,000 HVGs, 30 PCs, k=15; kNN + smoothing + "
                     "fuzzy union per sample",
               n_samples=256, lo=500, hi=20_000, n_genes=20_000, n_clusters=8, n_hvg=2000, dims=30, k=15)


def run_batched(args):
    """Cells/s of many small graphs: the precision form through
    pipeline.make_graphs (16 streams) against the plain form sample by sample."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from scarf_gb300 import pipeline, synth
    c = BATCHED
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(11)
    sizes = np.exp(rng.uniform(np.log(c["lo"]), np.log(c["hi"]), c["n_samples"])).astype(int)
    total = int(sizes.sum())
    pool = synth.nb_counts(total, c["n_genes"], c["n_clusters"], SEED, device=dev)
    feat = synth.select_hvgs(pool, c["n_hvg"])
    samples, a = [], 0
    for s_ in sizes:
        p0, p1 = int(pool.indptr[a]), int(pool.indptr[a + s_])
        samples.append((torch.from_numpy(pool.indptr[a:a + s_ + 1] - p0).to(dev),
                        torch.from_numpy(pool.indices[p0:p1]).to(dev), torch.from_numpy(pool.data[p0:p1]).to(dev)))
        a += s_
    del pool
    kw = dict(keep_x=False, batch_size=BATCH)
    pipeline.make_graphs(samples[:8], c["n_genes"], feat, c["dims"], c["k"], **kw)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = pipeline.make_graphs(samples, c["n_genes"], feat, c["dims"], c["k"], **kw)
    torch.cuda.synchronize()
    t_prec = time.perf_counter() - t0
    rec = float(np.mean([graph_check(g, BATCH, n_sample=200)[0] for g, _ in res[::16]]))
    # the plain form, one sample after another on one stream
    for smp in samples[:4]:
        pipeline.make_graph(*smp, c["n_genes"], feat, c["dims"], c["k"], precision="plain", **kw)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for smp in samples:
        g = pipeline.make_graph(*smp, c["n_genes"], feat, c["dims"], c["k"], precision="plain", **kw)
        K_union(g)
    torch.cuda.synchronize()
    t_plain = time.perf_counter() - t0
    print(json.dumps({"metric": "batched make_graph + union cells/s", "value": round(total / t_prec, 1),
                      "unit": "cells/s", "higher_is_better": True, "samples": len(samples), "cells": total,
                      "seconds": round(t_prec, 3), "plain_sequential_seconds": round(t_plain, 3),
                      "speedup_vs_plain_sequential": round(t_plain / t_prec, 3), "sampled_recall_at_k": round(rec, 5),
                      "data": "synthetic", "config": {"workload": c["name"], "streams": 16}}), flush=True)


def K_union(g):
    from scarf_gb300 import kernels as K
    return K.fuzzy_union(g.edges, g.weights, g.n_cells, g.k)


def run_union(args, cfg):
    """The fuzzy union (load_graph(symmetric=True)) of one precision graph of
    the config, W warm-up calls and one more (profiling case)."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from scarf_gb300 import kernels as K
    from scarf_gb300 import pipeline
    dev = torch.device("cuda", 0)
    csr, feat = make_input(cfg, dev)
    ip, ind, dat = (torch.from_numpy(a).to(dev) for a in (csr.indptr, csr.indices, csr.data))
    res = pipeline.make_graph(ip, ind, dat, csr.n_genes, feat, cfg["dims"], cfg["k"], batch_size=BATCH,
                              precision="precision", keep_x=False)
    del ip, ind, dat
    for _ in range(args.warmup):
        K.fuzzy_union(res.edges, res.weights, res.n_cells, res.k)
    K.profile(True)
    K.profile_reset()
    indptr, _, _ = K.fuzzy_union(res.edges, res.weights, res.n_cells, res.k)
    torch.cuda.synchronize()
    t, _ = K.profile_query("union")
    K.profile(False)
    print(json.dumps({"mode": "union", "config": args.config, "union_ms": round(t, 3),
                      "nnz": int(indptr[-1].item())}))


def run_step(args, cfg):
    """W warm-up steps and one step of one form, CSR resident on the device."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from scarf_gb300 import pipeline
    dev = torch.device("cuda", 0)
    csr, feat = make_input(cfg, dev)
    ip, ind, dat = (torch.from_numpy(a).to(dev) for a in (csr.indptr, csr.indices, csr.data))
    for _ in range(args.warmup + 1):
        res = pipeline.make_graph(ip, ind, dat, csr.n_genes, feat, cfg["dims"], cfg["k"], batch_size=BATCH,
                                  precision=args.form, keep_x=False)
    torch.cuda.synchronize()
    print(json.dumps({"mode": "step", "config": args.config, "form": args.form, "ann_recall_pct": res.recall()}))


if __name__ == "__main__":
    main()
