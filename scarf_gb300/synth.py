"""Seeded synthetic single-cell counts (CSR int32) for benchmarks and tests.

Negative-binomial counts drawn as gamma-Poisson mixtures: per-gene mean
log-normal (mu=-1, sigma=1.5), dispersion 0.5 (gamma shape 2, mean 1), per-cell
library size log-normal around a median number of UMIs, and ``n_clusters``
cluster programmes that each scale the means of 100 random genes by U(2, 4).
The highly variable genes are the top genes by variance of log1p-normalised
values (a fixed stand-in for the LOWESS-detrended selection upstream of
make_graph). Generation runs in torch on the requested device (chunks of
cells), so large matrices are drawn on the GPU.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Optional

import numpy as np
import torch


@dataclass
class CountsCSR:
    indptr: np.ndarray   # int64 (n_cells + 1)
    indices: np.ndarray  # int32 (nnz)
    data: np.ndarray     # int32 (nnz)
    n_cells: int
    n_genes: int
    labels: np.ndarray   # int32 cluster of each cell
    # per-gene sums of log1p(1000 c / library size) and of its square, taken
    # while the counts were drawn (what select_hvgs ranks by)
    gene_s1: Optional[np.ndarray] = None
    gene_s2: Optional[np.ndarray] = None

    @property
    def nnz(self) -> int:
        return int(self.indptr[-1])


def nb_counts(n_cells: int, n_genes: int, n_clusters: int, seed: int, lib_median: float = 3000.0,
              lib_sigma: float = 0.35, dispersion: float = 0.5, genes_per_cluster: int = 100,
              device: str = "cpu", chunk: int = 4096, cells_seed: Optional[int] = None) -> CountsCSR:
    """``seed`` fixes the population (gene means, cluster programmes);
    ``cells_seed`` (default: the same) fixes the cells drawn from it, so that
    query cells of the same populations can be drawn apart from a reference."""
    dev = torch.device(device)
    g = torch.Generator(device=dev)
    g.manual_seed(int(seed))
    f32 = torch.float32
    gene_mu = torch.exp(torch.randn(n_genes, generator=g, device=dev, dtype=torch.float64) * 1.5 - 1.0)
    prog = torch.ones((n_clusters, n_genes), dtype=torch.float64, device=dev)
    for c in range(n_clusters):
        idx = torch.randperm(n_genes, generator=g, device=dev)[:genes_per_cluster]
        prog[c, idx] = 2.0 + 2.0 * torch.rand(idx.numel(), generator=g, device=dev, dtype=torch.float64)
    prob = gene_mu[None, :] * prog
    prob = (prob / prob.sum(1, keepdim=True)).to(f32)
    if cells_seed is not None and cells_seed != seed:
        g.manual_seed(int(cells_seed) * 7919 + 17)
    labels = torch.randint(0, n_clusters, (n_cells,), generator=g, device=dev)
    lib = torch.exp(math.log(lib_median) + lib_sigma * torch.randn(n_cells, generator=g, device=dev))
    shape = 1.0 / dispersion
    ptr_parts, ind_parts, dat_parts = [], [], []
    counts_per_row = []
    s1 = torch.zeros(n_genes, dtype=torch.float64, device=dev)
    s2 = torch.zeros(n_genes, dtype=torch.float64, device=dev)
    for s in range(0, n_cells, chunk):
        e = min(n_cells, s + chunk)
        mu = lib[s:e, None] * prob[labels[s:e]]
        gam = torch._standard_gamma(torch.full_like(mu, shape), generator=g) / shape
        cnt = torch.poisson(mu * gam, generator=g).to(torch.int32)
        tot = cnt.sum(1, keepdim=True).clamp_min(1).double()
        xl = torch.log1p(1000.0 * cnt.double() / tot)
        s1 += xl.sum(0)
        s2 += (xl * xl).sum(0)
        del xl, tot
        nz = cnt.nonzero()
        ind_parts.append(nz[:, 1].to(torch.int32).cpu())
        dat_parts.append(cnt[nz[:, 0], nz[:, 1]].cpu())
        counts_per_row.append(torch.bincount(nz[:, 0], minlength=e - s).cpu())
        del mu, gam, cnt, nz
    per_row = torch.cat(counts_per_row).numpy().astype(np.int64)
    indptr = np.zeros(n_cells + 1, dtype=np.int64)
    np.cumsum(per_row, out=indptr[1:])
    return CountsCSR(indptr=indptr, indices=torch.cat(ind_parts).numpy(), data=torch.cat(dat_parts).numpy(),
                     n_cells=n_cells, n_genes=n_genes, labels=labels.cpu().numpy().astype(np.int32),
                     gene_s1=s1.cpu().numpy(), gene_s2=s2.cpu().numpy())


def select_hvgs(csr: CountsCSR, n_top: int, size_factor: float = 1000.0) -> np.ndarray:
    """Sorted indices of the ``n_top`` genes of largest variance of
    log1p(size_factor * c / library size) (library size over all genes)."""
    if csr.gene_s1 is not None and size_factor == 1000.0:
        var = csr.gene_s2 / csr.n_cells - (csr.gene_s1 / csr.n_cells) ** 2
        return np.sort(np.argsort(-var, kind="stable")[:n_top]).astype(np.int64)
    lib = np.diff(np.concatenate([[0], np.cumsum(csr.data, dtype=np.int64)])[csr.indptr])
    lib = np.maximum(lib, 1).astype(np.float64)
    rows = np.repeat(np.arange(csr.n_cells), np.diff(csr.indptr))
    x = np.log1p(size_factor * csr.data / lib[rows])
    s1 = np.bincount(csr.indices, weights=x, minlength=csr.n_genes)
    s2 = np.bincount(csr.indices, weights=x * x, minlength=csr.n_genes)
    var = s2 / csr.n_cells - (s1 / csr.n_cells) ** 2
    top = np.argsort(-var, kind="stable")[:n_top]
    return np.sort(top).astype(np.int64)


def col_map_for(feat_idx: np.ndarray, n_genes: int) -> np.ndarray:
    """gene -> output column (position in the ascending feature list) or -1."""
    m = np.full(n_genes, -1, dtype=np.int32)
    m[np.asarray(feat_idx)] = np.arange(len(feat_idx), dtype=np.int32)
    return m
