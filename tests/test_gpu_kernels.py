"""Parity of each CUDA kernel group (through the C ABI) with the CPU oracle.

Tolerances: integer, index and edge outputs are compared bit-exactly; FP32
values against the FP64 oracle to the bounds stated in each test; the fuzzy
union, computed in FP64 with scipy's operation order, bit-exactly.
"""
import os

import numpy as np
import pytest
import scipy.sparse as sp

import oracle
from helpers import clustered_points, small_counts, top_var_genes

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def K():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from scarf_gb300 import kernels
    return kernels


def cu(a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a))
    if dtype is not None:
        t = t.to(dtype)
    return t.cuda()


@pytest.fixture(scope="module")
def counts():
    indptr, indices, data, G, lab = small_counts()
    feat = top_var_genes(indptr, indices, data, G, 400)
    return indptr, indices, data, G, feat


def _normalize(K, counts, **kw):
    indptr, indices, data, G, feat = counts
    cmap = np.full(G, -1, np.int32)
    cmap[feat] = np.arange(len(feat), dtype=np.int32)
    h = len(feat)
    cs = torch.zeros(h, dtype=torch.float64, device="cuda")
    cq = torch.zeros_like(cs)
    lib = torch.zeros(len(indptr) - 1, dtype=torch.int64, device="cuda")
    x = K.normalize_csr(cu(indptr), cu(indices), cu(data), cu(cmap), h, colsum=cs, colsumsq=cq, libsize=lib, **kw)
    torch.cuda.synchronize()
    return x, cs, cq, lib


def test_normalize_and_stats(K, counts):
    indptr, indices, data, G, feat = counts
    x, cs, cq, lib = _normalize(K, counts)
    want, scal = oracle.normed_csr(indptr, indices, data, G, feat)
    got = x[:, :len(feat)].double().cpu().numpy()
    assert np.abs(got - want).max() <= 4e-7 * max(1.0, np.abs(want).max())
    assert np.array_equal(lib.cpu().numpy(), scal.astype(np.int64))          # integer library sizes, exact
    assert np.allclose(cs.cpu().numpy(), want.sum(0), rtol=2e-6, atol=1e-6)
    assert np.allclose(cq.cpu().numpy(), (want ** 2).sum(0), rtol=2e-6, atol=1e-6)
    mu, sg, mu32, sg32 = K.zstats(cs, cq, len(indptr) - 1)
    omu, osg = oracle.zstats(want)
    assert np.allclose(mu.cpu().numpy(), omu, rtol=2e-6, atol=1e-7)
    assert np.allclose(sg.cpu().numpy(), osg, rtol=2e-6, atol=1e-7)


def test_normalize_is_deterministic(K, counts):
    a = _normalize(K, counts)
    b = _normalize(K, counts)
    assert torch.equal(a[0], b[0]) and torch.equal(a[1], b[1]) and torch.equal(a[2], b[2])


def test_normalize_modes(K, counts):
    indptr, indices, data, G, feat = counts
    ncounts = np.add.reduceat(data.astype(np.int64), indptr[:-1]).astype(np.float64)
    ncounts[np.diff(indptr) == 0] = 0
    ncounts[ncounts == 0] = 1.0
    x, *_ = _normalize(K, counts, renormalize_subset=False, n_counts=cu(ncounts), log_transform=False)
    want, _ = oracle.normed_csr(indptr, indices, data, G, feat, log_transform=False, renormalize_subset=False,
                                n_counts=ncounts)
    got = x[:, :len(feat)].double().cpu().numpy()
    assert np.allclose(got, want, rtol=4e-7, atol=1e-6)
    # missing features take the fill value (mapping_utils.py:208 fills 1.0)
    miss = np.zeros(len(feat), np.uint8)
    miss[[0, 7, 100]] = 1
    x2, *_ = _normalize(K, counts, missing_mask=cu(miss), fill_value=1.0)
    g2 = x2[:, :len(feat)].cpu().numpy()
    assert np.all(g2[:, [0, 7, 100]] == 1.0)
    # bf16 output is the rounding of the float32 values
    x3, *_ = _normalize(K, counts, out_dtype=torch.bfloat16)
    x1, *_ = _normalize(K, counts)
    assert torch.equal(x3[:, :len(feat)], x1[:, :len(feat)].to(torch.bfloat16))


def _zscaled(counts):
    indptr, indices, data, G, feat = counts
    want, _ = oracle.normed_csr(indptr, indices, data, G, feat)
    mu, sg = oracle.zstats(want)
    return want, mu, sg, (want - mu) / sg


def test_covariance_plain(K, counts):
    x, cs, cq, _ = _normalize(K, counts)
    mu, sg, mu32, sg32 = K.zstats(cs, cq, x.shape[0])
    xw, omu, osg, z = _zscaled(counts)
    h = z.shape[1]
    cov, zsum = K.covariance(x, mu32, sg32, n_cols=h)
    torch.cuda.synchronize()
    want = z.T @ z
    got = cov.cpu().numpy()
    assert np.abs(got - want).max() <= 2e-5 * np.abs(want).max()
    assert np.allclose(got, got.T)
    assert np.abs(zsum.cpu().numpy() - z.sum(0)).max() < 1e-2
    # row mask
    mask = (np.arange(x.shape[0]) % 3 != 0).astype(np.uint8)
    cov2, zs2 = K.covariance(x, mu32, sg32, n_cols=h, row_mask=cu(mask))
    zm = z[mask.astype(bool)]
    assert np.abs(cov2.cpu().numpy() - zm.T @ zm).max() <= 2e-5 * np.abs(want).max()
    assert np.allclose(zs2.cpu().numpy(), zm.sum(0), atol=1e-2)


def test_covariance_precision(K, counts):
    # 3xBF16 split products on the tensor cores, FP32 accumulation, FP64 reduction
    x, cs, cq, _ = _normalize(K, counts)
    mu, sg, mu32, sg32 = K.zstats(cs, cq, x.shape[0])
    xw, omu, osg, z = _zscaled(counts)
    h = z.shape[1]
    cov, zsum = K.covariance(x, mu32, sg32, n_cols=h, precision="precision")
    torch.cuda.synchronize()
    want = z.T @ z
    got = cov.cpu().numpy()
    assert np.abs(got - want).max() <= 1e-4 * np.abs(want).max()
    assert np.array_equal(got, got.T)
    assert np.abs(zsum.cpu().numpy() - z.sum(0)).max() < 1e-2
    mask = (np.arange(x.shape[0]) % 3 != 0).astype(np.uint8)
    cov2, _ = K.covariance(x, mu32, sg32, n_cols=h, row_mask=cu(mask), precision="precision")
    zm = z[mask.astype(bool)]
    assert np.abs(cov2.cpu().numpy() - zm.T @ zm).max() <= 1e-4 * np.abs(want).max()
    # the leading principal axes agree with the FP64 oracle
    comps, evals, _, _ = K.pca_basis(cov, zsum, x.shape[0], 11, n_load=10, ld_l=10)
    ocomp, oev = oracle.pca_exact(z, 11)
    assert oracle.subspace_angles(comps.cpu().numpy()[:, :5], ocomp[:, :5]).max() < 1e-3


def test_covariance_long_accumulation(K):
    # 600,000 rows of sparse columns: the zero entries of a column give one
    # repeated z value, whose products all round the same way in a long FP32
    # accumulation. Both scatters stay within their bounds of an FP64 scatter
    # of the same z = (x - mu32)/sigma32.
    g = torch.Generator(device="cuda").manual_seed(11)
    n, h = 600_000, 512
    dens = torch.linspace(0.05, 0.9, h, device="cuda", dtype=torch.float64)
    x = torch.empty((n, h), dtype=torch.float32, device="cuda")
    for a in range(0, n, 100_000):
        u = torch.rand((100_000, h), generator=g, device="cuda", dtype=torch.float64)
        v = torch.log1p(20.0 * torch.rand((100_000, h), generator=g, device="cuda", dtype=torch.float64))
        x[a:a + 100_000] = torch.where(u < dens[None, :], v, torch.zeros_like(v)).float()
    mu = x.double().mean(0)
    sg = x.double().std(0, unbiased=False)
    mu32, sg32 = mu.float(), sg.float()
    want = torch.zeros((h, h), dtype=torch.float64, device="cuda")
    zs = torch.zeros(h, dtype=torch.float64, device="cuda")
    for a in range(0, n, 100_000):
        z = (x[a:a + 100_000].double() - mu32.double()) / sg32.double()
        want += z.T @ z
        zs += z.sum(0)
    scale = float(want.abs().max())
    err = {}
    for form in ("plain", "precision"):
        cov, zsum = K.covariance(x, mu32, sg32, n_cols=h, precision=form)
        torch.cuda.synchronize()
        err[form] = float((cov - want).abs().max()) / scale
        assert float((zsum - zs).abs().max()) < 1.0
    print("relative max-abs scatter error", err)
    assert err["precision"] <= 1.2e-5
    assert err["plain"] <= 1.2e-4


def _spiked_cov(h, n_cells, n_spikes, seed):
    # Z^T Z of n_cells rows: n_spikes strong directions over a Marchenko-Pastur bulk
    g = torch.Generator(device="cuda").manual_seed(seed)
    z = torch.randn((n_cells, h), generator=g, device="cuda", dtype=torch.float64)
    idx = torch.randperm(h, generator=g, device="cuda")[:n_spikes]
    scale = torch.linspace(4.0, 1.3, n_spikes, device="cuda", dtype=torch.float64)
    z[:, idx] *= scale[None, :]
    return z.T @ z, z.sum(0)


@pytest.mark.parametrize("h,n_cells,n_comp", [(2000, 40_000, 51), (1200, 20_000, 31)])
def test_pca_basis_filter_matches_fp64(K, h, n_cells, n_comp):
    # 18 spikes over a Marchenko-Pastur bulk: components 19.. sit in the bulk,
    # where the FP32 rounding of the scatter alone moves single eigenvectors
    # by ~1e-4 rad; the FP64 Rayleigh-Ritz step keeps the eigenvalues to
    # second order in that error
    cov, zsum = _spiked_cov(h, n_cells, 18, seed=h)
    a = K.pca_basis(cov, zsum, n_cells, n_comp, n_load=n_comp - 1, ld_l=n_comp - 1)
    b = K.pca_basis(cov, zsum, n_cells, n_comp, n_load=n_comp - 1, ld_l=n_comp - 1, eigh="filter")
    r = K.filter_residual()
    ca, cb = a[0].cpu().numpy(), b[0].cpu().numpy()
    ea, eb = a[1].cpu().numpy(), b[1].cpu().numpy()
    ang = oracle.subspace_angles(ca[:, :n_comp - 1], cb[:, :n_comp - 1]).max()
    ang18 = oracle.subspace_angles(ca[:, :18], cb[:, :18]).max()
    ev = np.abs(ea - eb).max() / np.abs(ea).max()
    spike = np.abs(ca[:, :5] - cb[:, :5]).max()
    print(f"filter residual {r:.2e}, angle all {ang:.2e}, spikes {ang18:.2e}, evals {ev:.2e}, top-5 {spike:.2e}")
    assert np.isfinite(r) and r <= 1e-4           # the filtered route ran and converged
    assert ang < 5e-4 and ang18 < 1e-5
    assert ev < 1e-8
    assert spike < 1e-5                            # separated spikes agree one by one, signs included
    assert np.allclose(a[2].cpu().numpy(), b[2].cpu().numpy(), rtol=1e-7)


def test_pca_basis_filter_small_matrix_takes_dense_route(K, counts):
    x, cs, cq, _ = _normalize(K, counts)
    mu, sg, mu32, sg32 = K.zstats(cs, cq, x.shape[0])
    cov, zsum = K.covariance(x, mu32, sg32, n_cols=len(counts[4]))
    b = K.pca_basis(cov, zsum, x.shape[0], 120, n_load=119, ld_l=119, eigh="filter")
    assert np.isnan(K.filter_residual())           # block wider than half the matrix
    a = K.pca_basis(cov, zsum, x.shape[0], 120, n_load=119, ld_l=119, eigh="mixed")
    assert np.array_equal(a[0].cpu().numpy(), b[0].cpu().numpy())


def test_pca_basis_mixed_matches_fp64(K, counts):
    x, cs, cq, _ = _normalize(K, counts)
    mu, sg, mu32, sg32 = K.zstats(cs, cq, x.shape[0])
    cov, zsum = K.covariance(x, mu32, sg32, n_cols=len(counts[4]))
    a = K.pca_basis(cov, zsum, x.shape[0], 21, n_load=20, ld_l=20)
    b = K.pca_basis(cov, zsum, x.shape[0], 21, n_load=20, ld_l=20, eigh="mixed")
    ca, cb = a[0].cpu().numpy(), b[0].cpu().numpy()
    assert np.allclose(a[1].cpu().numpy(), b[1].cpu().numpy(), rtol=1e-5)
    assert oracle.subspace_angles(ca[:, :20], cb[:, :20]).max() < 1e-3
    for j in range(3):                      # separated leading components agree one by one, signs included
        assert np.abs(ca[:, j] - cb[:, j]).max() < 1e-4


def test_pca_basis_and_projection(K, counts):
    x, cs, cq, _ = _normalize(K, counts)
    mu, sg, mu32, sg32 = K.zstats(cs, cq, x.shape[0])
    xw, omu, osg, z = _zscaled(counts)
    h = z.shape[1]
    dims = 20
    cov, zsum = K.covariance(x, mu32, sg32, n_cols=h)
    comps, evals, evr, l32 = K.pca_basis(cov, zsum, x.shape[0], dims + 1, n_load=dims, ld_l=dims)
    ocomp, oev = oracle.pca_exact(z, dims + 1)
    ang = oracle.subspace_angles(comps.cpu().numpy()[:, :dims], ocomp[:, :dims])
    assert ang.max() < 1e-3
    assert np.allclose(evals.cpu().numpy(), oev, rtol=1e-4)
    # svd_flip convention: the largest-magnitude entry of each component is positive
    c = comps.cpu().numpy()
    assert np.all(c[np.argmax(np.abs(c), 0), np.arange(c.shape[1])] > 0)
    # leading, well separated components agree one by one
    for j in range(3):
        assert np.abs(c[:, j] - ocomp[:, j]).max() < 1e-3
    scores = K.project(x, mu32, sg32, l32, dims, n_cols=h)
    torch.cuda.synchronize()
    want = oracle.reducer(xw, omu, osg, c[:, :dims])
    got = scores[:, :dims].cpu().numpy()
    assert np.abs(got - want).max() <= 1e-4 * max(1.0, np.abs(want).max())
    assert torch.all(scores[:, dims:] == 0)


@pytest.mark.parametrize("form,n_cells,dims,ld_s,bf16_ld", [("plain", 6000, 30, 32, 40),
                                                          ("precision", 6000, 30, 32, 40),
                                                          ("precision", 1000, 50, 52, 72),
                                                          ("precision", 131, 7, 8, 0)])
def test_projection_forms(K, form, n_cells, dims, ld_s, bf16_ld):
    """The reducer in both forms against the oracle's on the same basis: the
    plain form in FP32 SIMT, the precision form as 3xBF16 tcgen05 products of
    the uncentred rows with the centring as a per-column shift (several
    tiles, a ragged last tile and feature chunk, d up to 50). Both pad with
    zeros and write the optional BF16 copy."""
    indptr, indices, data, G, _ = small_counts(n_cells=n_cells, seed=3)
    feat = top_var_genes(indptr, indices, data, G, 300)
    counts = (indptr, indices, data, G, feat)
    x, cs, cq, _ = _normalize(K, counts)
    mu, sg, mu32, sg32 = K.zstats(cs, cq, x.shape[0])
    xw, omu, osg, z = _zscaled(counts)
    h = z.shape[1]
    cov, zsum = K.covariance(x, mu32, sg32, n_cols=h)
    comps, _, _, l32 = K.pca_basis(cov, zsum, x.shape[0], dims + 1, n_load=dims, ld_l=dims)
    out = K.project(x, mu32, sg32, l32, dims, n_cols=h, ld_s=ld_s, bf16_ld=bf16_ld, precision=form)
    scores, sb = out if bf16_ld else (out, None)
    torch.cuda.synchronize()
    want = oracle.reducer(xw, omu, osg, comps.cpu().numpy()[:, :dims])
    got = scores[:, :dims].cpu().numpy()
    tol = 2e-5 if form == "plain" else 1e-4
    assert np.abs(got - want).max() <= tol * max(1.0, np.abs(want).max())
    assert torch.all(scores[:, dims:] == 0)
    if sb is not None:
        assert torch.all(sb[:, dims:].float() == 0)
        assert torch.equal(sb[:, :dims], scores[:, :dims].to(torch.bfloat16))


def _self_knn(K, pts, k, **kw):
    t = cu(np.pad(pts, ((0, 0), (0, (-pts.shape[1]) % 4))))
    idx, dist, nm = K.knn(t, t, pts.shape[1], k, self_offset=0, **kw)
    torch.cuda.synchronize()
    return idx.cpu().numpy(), dist.cpu().numpy(), int(nm.item())


@pytest.mark.parametrize("n,d,k", [(3000, 30, 11), (1234, 50, 21), (700, 7, 3)])
def test_self_knn_plain(K, n, d, k):
    pts = clustered_points(n, d, seed=n, dup=((5, 6), (10, 11), (10, 12)))
    gi, gd, nm = _self_knn(K, pts, k)
    oi, od, rec = oracle.self_query_knn(pts, k, chunk_size=1000)
    # the self-removal rule counts the same misses (duplicates make self non-first)
    assert nm == round((100 - rec) * n / 100)
    # tie-aware recall against the FP64 exact neighbours
    _, ed = oracle.exact_knn(pts.astype(np.float64), pts.astype(np.float64), k + 1)
    r = oracle.recall_at_k(pts, pts, gi, od[:, -1])
    assert r >= 0.999
    assert np.abs(gd - od).max() <= 1e-4 * max(1.0, od.max())
    # indices agree except where distances tie within float32 resolution
    diff = gi != oi
    if diff.any():
        assert np.all(np.abs(gd[diff] - od[diff]) <= 1e-4 * np.maximum(1.0, od[diff]))


@pytest.mark.parametrize("n,d,k", [(6000, 50, 21), (2345, 30, 11), (700, 7, 3)])
def test_self_knn_precision(K, n, d, k):
    # BF16 tcgen05 candidates + FP32 exact re-rank of k+1+16 per query
    pts = clustered_points(n, d, seed=n + 1, dup=((5, 6), (10, 11), (10, 12)))
    gi, gd, nm = _self_knn(K, pts, k, precision="precision", margin=16)
    oi, od, rec = oracle.self_query_knn(pts, k, chunk_size=1000)
    assert nm == round((100 - rec) * n / 100)
    r = oracle.recall_at_k(pts, pts, gi, od[:, -1])
    assert r >= 0.995
    # distances are the exact FP32 ones of the neighbours found
    diff = pts[:, None, :].astype(np.float64) - pts[gi].astype(np.float64)
    assert np.abs(gd - (diff * diff).sum(-1)).max() <= 1e-4 * max(1.0, od.max())


def test_knn_precision_query_splits(K):
    refs = clustered_points(40000, 50, seed=21)
    q = clustered_points(300, 50, seed=22)
    tr, tq = cu(np.pad(refs, ((0, 0), (0, 2)))), cu(np.pad(q, ((0, 0), (0, 2))))
    idx, dist, _ = K.knn(tq, tr, 50, 11, precision="precision", margin=16)
    torch.cuda.synchronize()
    oi, od = oracle.exact_knn(q, refs, 11)
    assert oracle.recall_at_k(q, refs, idx.cpu().numpy(), od[:, -1]) >= 0.995


def test_knn_plain_and_precision_agree(K):
    pts = clustered_points(5000, 50, seed=31)
    a = _self_knn(K, pts, 21)
    b = _self_knn(K, pts, 21, precision="precision", margin=16)
    same = (a[0] == b[0]).mean()
    assert same >= 0.99


def test_self_knn_precision_locality_order(K):
    # From 32,768 rows the precision self-kNN sorts the rows by their nearest
    # pilot row and starts each CTA's reference scan at its own tile; the
    # neighbours must be those of the exact FP32 plain form all the same.
    n, d, k = 40000, 50, 21
    pts = clustered_points(n, d, n_clusters=20, seed=77, dup=((5, 6), (10, 11), (10, 12), (30000, 39999)))
    pi, pd, pm = _self_knn(K, pts, k)
    gi, gd, gm = _self_knn(K, pts, k, precision="precision", margin=16)
    assert gm == pm
    assert (gi == pi).mean() >= 0.999
    assert np.abs(gd - pd).max() <= 1e-5 * max(1.0, pd.max())
    rows = np.random.default_rng(0).choice(n, 1500, replace=False)
    _, ed = oracle.exact_knn(pts[rows], pts, k + 1)
    # the k+1-th exact distance bounds the k kept after the self hit is dropped
    assert oracle.recall_at_k(pts[rows], pts, gi[rows], ed[:, -1]) >= 0.995


def test_knn_query_mapping(K):
    refs = clustered_points(5000, 30, seed=1)
    q = clustered_points(333, 30, seed=2)
    tr = cu(np.pad(refs, ((0, 0), (0, 2))))
    tq = cu(np.pad(q, ((0, 0), (0, 2))))
    idx, dist, _ = K.knn(tq, tr, 30, 7)
    torch.cuda.synchronize()
    oi, od = oracle.exact_knn(q, refs, 7)
    assert oracle.recall_at_k(q, refs, idx.cpu().numpy(), od[:, -1]) >= 0.999
    assert np.abs(dist.cpu().numpy() - od).max() <= 1e-4 * max(1.0, od.max())


def test_knn_edges(K):
    # k + 1 == n, a single query, ragged sizes
    pts = clustered_points(9, 5, seed=3)
    gi, gd, nm = _self_knn(K, pts, 8)
    oi, od, rec = oracle.self_query_knn(pts, 8)
    assert np.array_equal(np.sort(gi, 1), np.sort(oi.astype(np.int64), 1))
    refs = clustered_points(131, 5, seed=4)
    q = refs[:1].copy()
    idx, dist, _ = K.knn(cu(np.pad(q, ((0, 0), (0, 3)))), cu(np.pad(refs, ((0, 0), (0, 3)))), 5, 4)
    oi, od = oracle.exact_knn(q, refs, 4)
    assert np.array_equal(idx.cpu().numpy(), oi)
    with pytest.raises(ValueError):
        K.knn(cu(np.pad(q, ((0, 0), (0, 3)))), cu(np.pad(refs, ((0, 0), (0, 3)))), 5, 200)


def test_knn_many_splits(K):
    # few queries against many references: the reference range is split across CTAs
    refs = clustered_points(60000, 16, seed=5)
    q = clustered_points(50, 16, seed=6)
    idx, dist, _ = K.knn(cu(q), cu(refs), 16, 11)
    oi, od = oracle.exact_knn(q, refs, 11)
    assert oracle.recall_at_k(q, refs, idx.cpu().numpy(), od[:, -1]) >= 0.999


def test_smooth_known_answer(K, golden_dir):
    kat = np.load(os.path.join(golden_dir, "pbmc1k_knn.npz"))
    idx = cu(kat["indices"].astype(np.int64))
    dist = cu(kat["distances"].astype(np.float32))
    edges, w = K.smooth(idx, dist, 1.0, 1.5, 1000)
    torch.cuda.synchronize()
    n, k = kat["indices"].shape
    e = edges.cpu().numpy()
    assert np.array_equal(e[:, 0], np.repeat(np.arange(n), k))
    assert np.array_equal(e[:, 1], kat["indices"].ravel().astype(np.int64))
    assert np.abs(w.cpu().numpy() - kat["weights"]).max() < 1e-5


def test_smooth_chunked_global_min(K, golden_dir):
    ref = np.load(os.path.join(golden_dir, "ref_functions.npz"))
    idx = cu(ref["smooth_idx"].astype(np.int64))
    dist = cu(ref["smooth_dist"].astype(np.float32))
    edges, w = K.smooth(idx, dist, 1.0, 1.5, int(ref["smooth_chunk"]))
    torch.cuda.synchronize()
    assert np.array_equal(edges.cpu().numpy(), ref["smooth_edges"].astype(np.int64))
    got = w.cpu().numpy()
    want = ref["smooth_w"]
    # the same zero weights were replaced by the global minimum (its value is
    # within the weight tolerance, not bit-equal)
    assert np.array_equal(got == got.min(), want == want.min())
    assert np.abs(got - want).max() < 1e-5


def test_smooth_vs_oracle_random(K):
    pts = clustered_points(2500, 12, seed=9, dup=((1, 2),))
    oi, od, _ = oracle.self_query_knn(pts, 15)
    for chunk in (1000, 333):
        edges, w = K.smooth(cu(oi.astype(np.int64)), cu(od.astype(np.float32)), 1.0, 1.5, chunk)
        e, ow = oracle.smoothen_dists(oi, od, 1.0, 1.5, chunk)
        assert np.array_equal(edges.cpu().numpy(), e.astype(np.int64))
        assert np.abs(w.cpu().numpy() - ow).max() < 1e-5


def _csr(ref, p):
    return ref[p + "_indptr"], ref[p + "_indices"], ref[p + "_data"]


def test_fuzzy_union_bit_exact(K, golden_dir):
    ref = np.load(os.path.join(golden_dir, "ref_functions.npz"))
    n = int(ref["union_n"])
    edges = np.stack([ref["union_rows"], ref["union_cols"]], 1).astype(np.int64)
    k = edges.shape[0] // n
    for mix, p in ((1.0, "sym"), (1.0, "fss"), (0.7, "fss07")):
        ip, ind, dat = K.fuzzy_union(cu(edges), cu(ref["union_w"]), n, k, mix=mix)
        for got, want in zip((ip, ind, dat), _csr(ref, p)):
            assert np.array_equal(got.cpu().numpy(), want)


def test_fuzzy_union_use_k_upper_and_hubs(K):
    rng = np.random.default_rng(11)
    n, k = 3000, 9
    cols = rng.integers(0, n, size=(n, k))
    cols[:, 0] = 17              # a hub: in-degree 3000 exercises the CTA sorter
    cols[::5, 1] = 999           # a second, smaller hub
    w = rng.random(n * k).astype(np.float32).astype(np.float64)
    edges = np.stack([np.repeat(np.arange(n), k), cols.ravel()], 1).astype(np.int64)
    for use_k, upper in ((k, False), (4, False), (k, True)):
        g = oracle.store_to_sparse(edges, w, n, k, use_k)
        want = oracle.symmetrize(g, upper_only=upper)
        want.sort_indices()
        ip, ind, dat = K.fuzzy_union(cu(edges), cu(w), n, k, use_k=use_k, upper_only=upper)
        assert np.array_equal(ip.cpu().numpy(), want.indptr)
        assert np.array_equal(ind.cpu().numpy(), want.indices)
        assert np.array_equal(dat.cpu().numpy(), want.data)


@pytest.mark.gpu
@pytest.mark.parametrize("n,d,k,block,clusters", [(1500, 10, 500, 500, 12), (20000, 16, 100, 1000, 30),
                                                  (5000, 30, 64, 777, 8)])
def test_kmeans_minibatch_matches_oracle(K, n, d, k, block, clusters):
    """sg_kmeans_minibatch against the oracle's restatement (same draws from
    the counter hash): rows-in-order init (k = block) and k-means++ init with
    reassignment and a ragged last block. FP32 assignment distances on the GPU
    against FP64 in the oracle can split a near-tie, so labels must agree on
    99.9% of rows and the centres' inertia to 1e-6."""
    x = clustered_points(n, d, n_clusters=clusters, seed=n + d)
    ld = -(-d // 4) * 4
    t = torch.zeros((n, ld), dtype=torch.float32, device="cuda")
    t[:, :d] = cu(x)
    centers, labels = K.kmeans(t, d, k, block, 4466)
    torch.cuda.synchronize()
    c_o, l_o = oracle.kmeans_minibatch(x, k, block, 4466)
    got_c = centers.cpu().numpy()
    got_l = labels.cpu().numpy().astype(np.int64)
    assert got_c.shape == (k, d) and got_l.shape == (n,)
    assert np.mean(got_l == l_o) >= 0.999
    inertia = lambda c, l: float(((x.astype(np.float64) - c[l]) ** 2).sum())
    assert abs(inertia(got_c, got_l) / inertia(c_o, l_o) - 1.0) < 1e-6
    assert np.abs(got_c - c_o).max() <= 1e-5 * max(1.0, np.abs(c_o).max())


@pytest.mark.gpu
def test_kmeans_minibatch_rejects_bad_sizes(K):
    t = torch.zeros((100, 8), dtype=torch.float32, device="cuda")
    with pytest.raises(ValueError):
        K.kmeans(t, 8, 200, 100, 1)   # first block smaller than k
    with pytest.raises(ValueError):
        K.kmeans(t, 8, 10, 5000, 1)   # block above the kernel's limit


@pytest.mark.gpu
def test_calc_snn_and_merge_graphs_golden(K, golden_dir):
    """sg_calc_snn and sg_merge_graphs against the reference's calc_snn and
    merge_graphs run on the same two graphs (bit-exact), and the knn_utils
    surface that mirrors merge_graphs."""
    import scipy.sparse as sps
    from scarf_gb300 import knn_utils
    ref = np.load(os.path.join(golden_dir, "ref_functions.npz"))
    n, k = int(ref["merge_n"]), int(ref["merge_k"])
    idx = [cu(ref[f"merge_g{g}_indices"].astype(np.int64)) for g in range(2)]
    w = [cu(ref[f"merge_g{g}_data"].reshape(n, k)) for g in range(2)]
    snn = [K.calc_snn(i) for i in idx]
    torch.cuda.synchronize()
    for g in range(2):
        assert np.array_equal(snn[g].cpu().numpy(), ref[f"merge_g{g}_snn"])
    oi, ow = K.merge_graphs(idx, w, snn)
    torch.cuda.synchronize()
    assert np.array_equal(oi.cpu().numpy().ravel(), ref["merge_col"])
    assert np.array_equal(ow.cpu().numpy().ravel(), ref["merge_data"])
    mats = [sps.csr_matrix((ref[f"merge_g{g}_data"], ref[f"merge_g{g}_indices"].ravel(),
                            np.arange(0, n * k + 1, k)), shape=(n, n)) for g in range(2)]
    m = knn_utils.merge_graphs(mats)
    assert np.array_equal(m.row, ref["merge_row"]) and np.array_equal(m.col, ref["merge_col"])
    assert np.array_equal(m.data, ref["merge_data"])


@pytest.mark.gpu
def test_merge_graphs_three_graphs_with_ties(K):
    """Three graphs with shared neighbours and tied weight + snn values (the
    tie rule of the restatement: the later candidate first) against the oracle."""
    rng = np.random.default_rng(11)
    n, k = 500, 12
    base = np.stack([rng.choice(n, k, replace=False) for _ in range(n)])
    idx_np, w_np = [], []
    for g in range(3):
        mi = base.copy()
        swap = rng.random((n, k)) < 0.4
        mi[swap] = rng.integers(0, n, swap.sum())
        # keep each row's neighbours distinct
        for r in range(n):
            _, first = np.unique(mi[r], return_index=True)
            dup = np.setdiff1d(np.arange(k), first)
            pool = np.setdiff1d(np.arange(n), mi[r])
            mi[r, dup] = rng.choice(pool, len(dup), replace=False)
        idx_np.append(mi)
        w_np.append(np.round(rng.random((n, k)) * 4) / 4)   # quarter steps: many ties
    idx = [cu(a.astype(np.int64)) for a in idx_np]
    w = [cu(a) for a in w_np]
    snn = [K.calc_snn(i) for i in idx]
    oi, ow = K.merge_graphs(idx, w, snn)
    torch.cuda.synchronize()
    mats = [sp.csr_matrix((w_np[g].ravel(), idx_np[g].ravel(), np.arange(0, n * k + 1, k)), shape=(n, n))
            for g in range(3)]
    want = oracle.merge_graphs(mats)
    assert np.array_equal(oi.cpu().numpy().ravel(), want.col)
    assert np.array_equal(ow.cpu().numpy().ravel(), want.data)


@pytest.mark.gpu
def test_umap_layout_matches_sequential_restatement_in_quality(K):
    """sg_umap_layout (all edges of an epoch concurrently) against the
    restated single-threaded optimize_layout_euclidean on the same fused graph
    and start: both separate the clusters, and their neighbourhood purity
    agrees within 0.1 (the two are samples of one stochastic process; the
    concurrent epochs apply a vertex's steps from one stale position, and the
    atomic sums make the GPU layout differ from run to run)."""
    from helpers import umap_graph, embedding_purity
    x, lab, _, head, tail, w = umap_graph(400, 10, 5, 10, seed=6)
    a, b = oracle.umap_find_ab_params(2.0, 1.0)
    eps = oracle.umap_make_epochs_per_sample(w, 60)
    y0 = (np.random.default_rng(1).normal(size=(400, 2)) * 10).astype(np.float32)
    y = cu(y0.copy())
    K.umap_layout(cu(head.astype(np.int32)), cu(tail.astype(np.int32)), cu(eps.astype(np.float64)), y, 60, a, b,
                  seed=3)
    torch.cuda.synchronize()
    got = y.cpu().numpy()
    assert np.isfinite(got).all()
    rnd = np.random.default_rng(2)
    want = oracle.umap_layout_sequential(y0, head, tail, eps, 60, a, b,
                                         rand_vertex=lambda n, i, p: rnd.integers(1 << 30))
    pg, pw = embedding_purity(got, lab), embedding_purity(want, lab)
    assert embedding_purity(y0, lab) < 0.5
    assert pw > 0.95 and pg > 0.85
    assert pg >= pw - 0.1


@pytest.mark.gpu
def test_umap_layout_sequential_mode_pins_the_restatement(K):
    """The deterministic mode of sg_umap_layout (one thread, edges in order,
    umap-learn's float64 gradient arithmetic on float32 coordinates and its
    float64 sampling schedule) follows the oracle's restatement of
    optimize_layout_euclidean step for step when both draw the same negative
    samples (the kernel's counter hash, restated in the oracle): the same
    trajectory to float32 rounding after 40 epochs on a 300-point graph."""
    from helpers import umap_graph
    x, lab, _, head, tail, w = umap_graph(300, 10, 4, 10, seed=9)
    a, b = (float(np.float32(v)) for v in oracle.umap_find_ab_params(1.0, 0.1))
    eps = oracle.umap_make_epochs_per_sample(w, 40)
    y0 = (np.random.default_rng(4).normal(size=(300, 2)) * 10).astype(np.float32)
    seed = 12345
    y = cu(y0.copy())
    K.umap_layout(cu(head.astype(np.int32)), cu(tail.astype(np.int32)), cu(eps.astype(np.float64)), y, 40, a, b,
                  seed=seed, sequential=True)
    torch.cuda.synchronize()
    got = y.cpu().numpy()
    want = oracle.umap_layout_sequential(y0, head, tail, eps, 40, a, b,
                                         rand_vertex=lambda n, i, p: oracle.umap_negative_vertex(seed, n, i, p, 300))
    assert np.isfinite(got).all()
    err = np.abs(got - want).max()
    assert err <= 1e-3 * max(1.0, np.abs(want).max()), f"sequential layout differs by {err}"
    # most coordinates agree bit for bit (the two pow implementations may round differently)
    assert np.mean(got == want) > 0.9


@pytest.mark.gpu
def test_umap_fit_transform_surface(K):
    """scarf_gb300.umap.fit_transform (scarf/umap.py:126-163): the GPU fuzzy
    union equals the reference's scipy union, and the layout separates the
    clusters from scarf's default parameters."""
    from helpers import umap_graph, embedding_purity
    from scarf_gb300 import umap as gu
    x, lab, g, head, tail, w = umap_graph(500, 10, 4, 10, seed=8)
    rows, cols, vals = gu.fuzzy_simplicial_set(g, 1.0)
    assert np.array_equal(rows.cpu().numpy(), head) and np.array_equal(cols.cpu().numpy(), tail)
    assert np.array_equal(vals.cpu().numpy(), w)
    y0 = (np.random.default_rng(3).normal(size=(500, 2)) * 10).astype(np.float32)
    emb, a, b = gu.fit_transform(g, y0, 2.0, 1.0, 100, 4444, 1.0, 1.0, 5, {}, False, 1, False)
    assert emb.shape == (500, 2) and np.isfinite(emb).all()
    assert embedding_purity(emb, lab) > 0.85
    with pytest.raises(NotImplementedError):
        gu.fit_transform(g, y0, 2.0, 1.0, 10, 4444, 1.0, 1.0, 5, {"lambda": 2.0}, False, 1, False)
