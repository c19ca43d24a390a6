"""The benchmark's full-size workloads, checked through properties that need no
FP64 pipeline of the same size (the sampled FP64 comparisons of the bench
line cover the rest): 100,000 and 1,000,000 cells of seeded negative-binomial
counts (30,000 genes; 20 and 40 clusters; library sizes around 3,000 and
2,500 UMIs), 2,000 HVGs, 50 PCs, k = 21, precision form through
``pipeline.make_graph`` (DataStore.make_graph, scarf/datastore/
graph_datastore.py:513-1020).

* a1/a3: normalised rows finite and non-negative; mu and sigma against FP64
  sums of sampled columns of the normalised matrix;
* a4: at 100,000 cells the well separated leading axes and the span of the
  first 10 against an FP64 eigendecomposition of the FP64 scatter (the
  oracle's exact PCA);
* a6/a7: distances ascending along each row, no self, indices in range,
  (nearly) every cell's first hit itself; tie-aware recall@k >= 0.995 on 500 sampled
  rows against exact FP64 kNN of the graph's own scores;
* a8: weights in [0, 1], the nearest non-zero-distance neighbour of a row at
  weight 1 (umap-learn's rho);
* a9 at 100,000 cells: the fuzzy union symmetric bit for bit, values in (0, 1];
* at 1,000,000 cells the page-locked host CSR, read over the host link in
  50,000-cell launches, gives the graph of the device-resident CSR bit for bit.
"""
import numpy as np
import pytest
import scipy.sparse as sp

import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

SIZES = {
    "100k": dict(n_cells=100_000, n_clusters=20, lib_median=3000.0, seed=2718),
    "1M": dict(n_cells=1_000_000, n_clusters=40, lib_median=2500.0, seed=2718),
}
N_GENES, N_HVG, DIMS, K, BATCH = 30_000, 2000, 50, 21, 1000


def _workload(size):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from scarf_gb300 import synth
    c = SIZES[size]
    csr = synth.nb_counts(c["n_cells"], N_GENES, c["n_clusters"], c["seed"], lib_median=c["lib_median"],
                          device="cuda", chunk=4096)
    return csr, synth.select_hvgs(csr, N_HVG)


def _check_graph(res, n, rng):
    h = res.n_feats
    x = res.x[:, :h]
    # a1/a3
    assert bool(torch.isfinite(x).all()) and float(x.min()) >= 0.0
    cols = torch.from_numpy(np.sort(rng.choice(h, 64, replace=False))).cuda()
    xs = x[:, cols].double()
    mu = xs.mean(0)
    sd = (xs * xs).mean(0).sub(mu * mu).clamp_min(0).sqrt()
    assert torch.allclose(res.mu[cols], mu, rtol=5e-6, atol=1e-8)
    assert torch.allclose(res.sigma[cols], torch.where(sd > 0, sd, torch.ones_like(sd)), rtol=1e-5, atol=1e-8)
    # a6/a7
    idx = res.indices
    dist = res.distances
    k = idx.shape[1]
    assert int(idx.min()) >= 0 and int(idx.max()) < n
    assert not bool((idx == torch.arange(n, device=idx.device)[:, None]).any())
    assert bool((dist[:, 1:] >= dist[:, :-1]).all())
    assert res.recall() >= 99.9                 # cells whose first hit is themselves, in %
    rows = np.sort(rng.choice(n, 500, replace=False))
    s = res.scores[:, :res.dims].double().cpu().numpy()
    _, ed = oracle.exact_knn(s[rows], s, k + 1)
    # the exact list holds the query itself first; the graph has self removed
    rec = oracle.recall_at_k(s[rows], s, idx[rows].cpu().numpy(), ed[:, -1], rel=1e-5)
    assert rec >= 0.995, f"recall@k {rec}"
    # a8
    w = res.weights.view(n, k)
    assert float(w.min()) >= 0.0 and float(w.max()) <= 1.0
    top = (w.max(1).values >= 1.0 - 1e-6).double().mean().item()
    assert top >= 0.999, f"rows whose rho neighbour has weight 1: {top}"
    return s


@pytest.fixture(scope="module")
def c100k():
    return _workload("100k")


def test_100k_cells_make_graph_properties(c100k):
    from scarf_gb300 import kernels
    from scarf_gb300 import pipeline
    csr, feat = c100k
    n = csr.n_cells
    dev = [torch.from_numpy(a).cuda() for a in (csr.indptr, csr.indices, csr.data)]
    res = pipeline.make_graph(*dev, csr.n_genes, feat, DIMS, K, batch_size=BATCH, precision="precision")
    torch.cuda.synchronize()
    rng = np.random.default_rng(5)
    _check_graph(res, n, rng)
    # a4: the leading, well separated axes against the oracle's FP64 PCA of the same z-scores
    z = ((res.x[:, :res.n_feats].double() - res.mu) / res.sigma).cpu().numpy()
    want, evals = oracle.pca_exact(z, 11)
    del z
    rel = (evals[:-1] - evals[1:]) / evals[0]
    m = max([i + 1 for i, r in enumerate(rel) if r > 0.02] or [1])
    got = res.loadings.cpu().numpy()
    ang = oracle.subspace_angles(got[:, :m], want[:, :m]).max()
    assert ang < 1e-4, f"principal angle {ang} over the first {m} axes"
    ang10 = oracle.subspace_angles(got[:, :10], want[:, :10]).max()
    assert ang10 < 1e-4, f"principal angle {ang10} over the first 10 axes"
    # a9: the fuzzy union is symmetric, values in (0, 1]
    ip, ind, val = kernels.fuzzy_union(res.edges, res.weights, n, res.k)
    u = sp.csr_matrix((val.cpu().numpy(), ind.cpu().numpy(), ip.cpu().numpy()), shape=(n, n))
    assert (u != u.T).nnz == 0
    assert u.data.min() > 0.0 and u.data.max() <= 1.0


def test_1m_cells_make_graph_properties_and_host_path():
    from scarf_gb300 import pipeline
    csr, feat = _workload("1M")
    n = csr.n_cells
    dev = [torch.from_numpy(a).cuda() for a in (csr.indptr, csr.indices, csr.data)]
    res = pipeline.make_graph(*dev, csr.n_genes, feat, DIMS, K, batch_size=BATCH, precision="precision")
    torch.cuda.synchronize()
    del dev
    _check_graph(res, n, np.random.default_rng(6))
    keep = (res.indices.clone(), res.weights.clone(), res.mu.clone())
    del res
    pin = [torch.from_numpy(a).pin_memory() for a in (csr.indptr, csr.indices, csr.data)]
    hres = pipeline.make_graph(*pin, csr.n_genes, feat, DIMS, K, batch_size=BATCH, precision="precision",
                               chunk_cells=50_000, keep_x=False)
    torch.cuda.synchronize()
    assert torch.equal(hres.indices, keep[0]) and torch.equal(hres.weights, keep[1])
    assert torch.allclose(hres.mu, keep[2], rtol=1e-14, atol=0)
