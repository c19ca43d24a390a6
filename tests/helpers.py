"""Shared helpers of the test suite (seeded inputs, device transfers)."""
import numpy as np
import scipy.sparse as sp


def small_counts(n_cells=1500, n_genes=3000, n_clusters=6, seed=0, empty_rows=(3, 700)):
    """Seeded NB-like CSR counts (numpy, fast) with a few empty rows."""
    rng = np.random.default_rng(seed)
    mu = np.exp(rng.normal(-1.0, 1.5, n_genes))
    prog = np.ones((n_clusters, n_genes))
    for c in range(n_clusters):
        prog[c, rng.choice(n_genes, 60, replace=False)] = rng.uniform(2, 4, 60)
    p = mu * prog
    p /= p.sum(1, keepdims=True)
    lab = rng.integers(0, n_clusters, n_cells)
    lib = np.exp(np.log(1500) + 0.4 * rng.normal(size=n_cells))
    lam = lib[:, None] * p[lab] * rng.gamma(2.0, 0.5, size=(n_cells, n_genes))
    cnt = rng.poisson(lam).astype(np.int32)
    for r in empty_rows:
        if r < n_cells:
            cnt[r] = 0
    m = sp.csr_matrix(cnt)
    m.sort_indices()
    return m.indptr.astype(np.int64), m.indices.astype(np.int32), m.data.astype(np.int32), n_genes, lab


def top_var_genes(indptr, indices, data, n_genes, n_top):
    n = len(indptr) - 1
    lib = np.add.reduceat(data.astype(np.int64), indptr[:-1]) if len(data) else np.zeros(n)
    lib[np.diff(indptr) == 0] = 0
    lib = np.maximum(lib, 1)
    rows = np.repeat(np.arange(n), np.diff(indptr))
    x = np.log1p(1000.0 * data / lib[rows])
    s1 = np.bincount(indices, weights=x, minlength=n_genes)
    s2 = np.bincount(indices, weights=x * x, minlength=n_genes)
    var = s2 / n - (s1 / n) ** 2
    return np.sort(np.argsort(-var, kind="stable")[:n_top])


def clustered_points(n, d, n_clusters=8, seed=0, spread=0.6, dup=()):
    rng = np.random.default_rng(seed)
    centers = rng.normal(0, 4, size=(n_clusters, d))
    lab = rng.integers(0, n_clusters, n)
    x = centers[lab] + spread * rng.normal(size=(n, d))
    for a, b in dup:
        x[b] = x[a]
    return x.astype(np.float32)


def umap_graph(n, d, n_clusters, k, seed):
    """Clustered points, their labels and the fused UMAP graph of their exact
    kNN (oracle smoothing + fuzzy union) as COO arrays (head, tail, weight)."""
    import oracle
    rng = np.random.default_rng(seed)
    centers = rng.normal(0, 6, size=(n_clusters, d))
    lab = rng.integers(0, n_clusters, n)
    x = (centers[lab] + rng.normal(size=(n, d))).astype(np.float32)
    ki, kd = oracle.exact_knn(x, x, k + 1)
    fi, fd, _ = oracle.fix_knn_query(ki, kd.astype(np.float32), np.arange(n))
    edges, w = oracle.smoothen_dists(fi.astype(np.uint64), fd.astype(np.float64), 1.0, 1.5, 1000)
    import scipy.sparse as sp
    g = sp.csr_matrix((w, (edges[:, 0].astype(np.int64), edges[:, 1].astype(np.int64))), shape=(n, n))
    u = oracle.fuzzy_simplicial_set(g, 1.0).tocsr()
    u.sort_indices()
    u = u.tocoo()
    return x, lab, g, u.row.astype(np.int64), u.col.astype(np.int64), u.data


def embedding_purity(y, lab, k=10):
    """Fraction of each point's k nearest embedded neighbours in its cluster."""
    d = ((y[:, None, :] - y[None, :, :]) ** 2).sum(-1)
    np.fill_diagonal(d, np.inf)
    nn = np.argsort(d, axis=1)[:, :k]
    return float((lab[nn] == lab[:, None]).mean())


def multirank_worker(rank, ws, port, q):
    """One rank of a CPU (gloo) process group: reports bench.max_over_ranks of
    a rank-dependent step time."""
    import os
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    q.put((rank, bench.max_over_ranks(10.0 + rank, torch.device("cpu")), bench.dist_env()))
    dist.barrier()
    dist.destroy_process_group()
