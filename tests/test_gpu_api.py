"""The reference-facing surface on the GPU: DataStore.make_graph / load_graph /
run_mapping, AnnStream, knn_utils and the mapping server, against the oracle
and against the reference's store layout and dtypes."""
import numpy as np
import pytest
import scipy.sparse as sp

import oracle
from helpers import small_counts, top_var_genes

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ds():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from scarf_gb300.datastore import DataStore
    indptr, indices, data, G, _ = small_counts(n_cells=1800, n_genes=3000, seed=7)
    feat = top_var_genes(indptr, indices, data, G, 300)
    d = DataStore(indptr, indices, data, G, gene_ids=np.array([f"g{i}" for i in range(G)]))
    mask = np.zeros(G, dtype=bool)
    mask[feat] = True
    d.RNA.feats.insert("I__hvgs", mask)
    d.make_graph(feat_key="hvgs", dims=15, k=11, batch_size=500)
    return d, (indptr, indices, data, G, feat)


def test_make_graph_layout_and_dtypes(ds):
    d, _ = ds
    loc = d._get_latest_graph_loc("RNA", "I", "hvgs")
    assert loc == "RNA/normed__I__hvgs/reduction__pca__15__I/ann__l2__50__50__48__4466/knn__11/graph__1.0__1.5"
    knn = d.zw[loc.rsplit("/", 1)[0]]
    assert knn["indices"].dtype == np.uint64 and knn["indices"].shape == (1800, 11)
    assert knn["distances"].dtype == np.float64
    g = d.zw[loc]
    assert g["edges"].dtype == np.uint64 and g["edges"].shape == (1800 * 11, 2)
    assert g["weights"].dtype == np.float64
    red = d.zw["RNA/normed__I__hvgs/reduction__pca__15__I"]
    assert red["reduction"].shape == (300, 15) and red["reduction"].dtype == np.float64
    assert d.zw["RNA/normed__I__hvgs"]["mu"].dtype == np.float64
    assert d.zw["RNA/normed__I__hvgs"].attrs["subset_params"] == {"log_transform": True, "renormalize_subset": True}


def test_make_graph_matches_oracle(ds):
    d, (indptr, indices, data, G, feat) = ds
    want = oracle.make_graph(indptr, indices, data, G, feat, dims=15, k=11, batch_size=500)
    red = d.zw["RNA/normed__I__hvgs/reduction__pca__15__I"]["reduction"][:]
    assert oracle.subspace_angles(red[:, :5], want["loadings"][:, :5]).max() < 1e-3
    assert np.allclose(d.zw["RNA/normed__I__hvgs"]["mu"][:], want["mu"], rtol=1e-5, atol=1e-7)
    loc = d._get_latest_graph_loc("RNA", "I", "hvgs")
    knn = d.zw[loc.rsplit("/", 1)[0]]
    gi, gd = knn["indices"][:].astype(np.int64), knn["distances"][:]
    # the scores the graph was built on, recomputed by the oracle from the GPU loadings
    s = oracle.reducer(want["x"], want["mu"], want["sigma"], red)
    _, ed = oracle.exact_knn(s, s, 12)
    assert oracle.recall_at_k(s, s, gi, ed[:, -1], rel=1e-4) >= 0.995
    _, w = oracle.smoothen_dists(gi, gd, 1.0, 1.5, 500)
    assert np.abs(d.zw[loc]["weights"][:] - w).max() < 1e-5


def test_make_graph_cache_and_load_graph(ds):
    d, _ = ds
    loc = d._get_latest_graph_loc("RNA", "I", "hvgs")
    before = d.zw[loc]["weights"][:].copy()
    d.make_graph(feat_key="hvgs")            # cached parameters and steps are reused
    assert d._get_latest_graph_loc("RNA", "I", "hvgs") == loc
    assert np.array_equal(d.zw[loc]["weights"][:], before)
    e = d.zw[loc]["edges"][:].astype(np.int64)
    w = d.zw[loc]["weights"][:]
    g = sp.csr_matrix((w, (e[:, 0], e[:, 1])), shape=(1800, 1800))
    for upper in (False, True):
        got = d.load_graph(feat_key="hvgs", symmetric=True, upper_only=upper)
        want = oracle.symmetrize(g, upper_only=upper)
        want.sort_indices()
        assert np.array_equal(got.indptr, want.indptr) and np.array_equal(got.indices, want.indices)
        assert np.array_equal(got.data, want.data)
    plain = d.load_graph(feat_key="hvgs", symmetric=False, use_k=5)
    assert plain.nnz == 1800 * 5


def test_run_mapping_self_map(ds):
    d, _ = ds
    d.run_mapping(target_assay=d.RNA, target_name="selfmap", target_feat_key="hvgs_self", save_k=3)
    p = d.zw["RNA/projections/selfmap"]
    idx, dist = p["indices"][:], p["distances"][:]
    assert idx.shape == (1800, 3) and idx.dtype == np.uint64
    # every cell maps onto itself at distance 0 (ties with duplicates aside)
    assert np.mean(dist[:, 0] <= 1e-6) > 0.99


def test_annstream_transform_ann(ds):
    d, _ = ds
    ann = d._ann_cache[d.zw["RNA/normed__I__hvgs/reduction__pca__15__I"].attrs["latest_ann"]]
    s = ann.annIdx.scores[:100, : ann.dims].cpu().numpy()
    i, dd = ann.transform_ann(s, k=4)
    assert i.dtype == np.uint64 and dd.dtype == np.float32 and np.array_equal(i[:, 0], np.arange(100))
    fi, fd, nm = ann.transform_ann(s, k=4, self_indices=np.arange(100))
    assert fi.shape == (100, 4) and nm <= 2


def test_mapping_server_alone_equals_mixed(ds):
    from scarf_gb300.serving import MappingServer, latency_summary
    d, (indptr, indices, data, G, feat) = ds
    ann = d._ann_cache[d.zw["RNA/normed__I__hvgs/reduction__pca__15__I"].attrs["latest_ann"]]
    ref_ids = d.RNA.feats.fetch("ids", key="I__hvgs")
    rng = np.random.default_rng(1)
    sizes = [5, 300, 1, 1200, 77]
    reqs, picks = [], []
    m = sp.csr_matrix((data, indices, indptr), shape=(len(indptr) - 1, G))
    for n in sizes:
        rows = rng.choice(m.shape[0], n, replace=False)
        s = m[rows]
        picks.append(rows)
        reqs.append((s.indptr.astype(np.int64), s.indices.astype(np.int32), s.data.astype(np.int32)))
    genes = d.RNA.feats.fetch_all("ids")
    alone = []
    with MappingServer(ann, ref_ids, genes, k=5, max_batch_rows=256, n_workers=1) as srv:
        for r in reqs:
            alone.append(srv.submit(*r).result(timeout=60))
    with MappingServer(ann, ref_ids, genes, k=5, max_batch_rows=256, n_workers=2,
                       hbm_budget_bytes=10_000_000) as srv:
        mixed = [srv.submit(*r) for r in reqs]
        outs = [q.result(timeout=60) for q in mixed]
        summ = latency_summary(mixed)
    assert summ["requests"] == len(sizes)
    for (ia, da), (ib, db) in zip(alone, outs):
        assert np.array_equal(ia, ib)
        assert np.abs(da - db).max() <= 1e-6
    # and the service answers what run_mapping stores for the same cells
    d.run_mapping(target_assay=d.RNA, target_name="selfmap5", target_feat_key="hvgs_self5", save_k=5)
    full_i = d.zw["RNA/projections/selfmap5"]["indices"][:].astype(np.int64)
    full_d = d.zw["RNA/projections/selfmap5"]["distances"][:]
    for (ia, da), rows in zip(alone, picks):
        assert np.abs(da - full_d[rows]).max() <= 1e-5
        assert np.mean(ia == full_i[rows]) > 0.99


def test_mapping_server_rejects_over_budget(ds):
    from scarf_gb300.serving import MappingServer
    d, (indptr, indices, data, G, feat) = ds
    ann = d._ann_cache[d.zw["RNA/normed__I__hvgs/reduction__pca__15__I"].attrs["latest_ann"]]
    with MappingServer(ann, d.RNA.feats.fetch("ids", key="I__hvgs"), d.RNA.feats.fetch_all("ids"), k=5,
                       hbm_budget_bytes=1000) as srv:
        r = srv.submit(indptr[:101] - indptr[0], indices[: indptr[100]], data[: indptr[100]])
        with pytest.raises(MemoryError):
            r.result(timeout=10)


def test_make_graphs_equals_one_by_one():
    # many small graphs on 3 streams give what each gives alone
    from helpers import small_counts, top_var_genes
    from scarf_gb300 import pipeline
    indptr, indices, data, G, _ = small_counts()
    feat = top_var_genes(indptr, indices, data, G, 300)
    cuts = [0, 300, 700, 1500]
    samples = []
    for a, b in zip(cuts[:-1], cuts[1:]):
        p0, p1 = int(indptr[a]), int(indptr[b])
        samples.append((torch.from_numpy((indptr[a:b + 1] - p0).astype(np.int64)).cuda(),
                        torch.from_numpy(indices[p0:p1].astype(np.int32)).cuda(),
                        torch.from_numpy(data[p0:p1].astype(np.int32)).cuda()))
    many = pipeline.make_graphs(samples, G, feat, 20, 10, n_streams=3)
    for (g, u), smp in zip(many, samples):
        one = pipeline.make_graph(*smp, G, feat, 20, 10, precision="precision")
        assert np.array_equal(g.indices.cpu().numpy(), one.indices.cpu().numpy())
        assert np.array_equal(g.weights.cpu().numpy(), one.weights.cpu().numpy())
        ui, uj, uv = (t.cpu().numpy() for t in u)
        from scarf_gb300 import kernels as K
        oi, oj, ov = (t.cpu().numpy() for t in K.fuzzy_union(one.edges, one.weights, one.n_cells, one.k))
        assert np.array_equal(ui, oi) and np.array_equal(uj, oj) and np.array_equal(uv, ov)


def test_make_graph_writes_kmeans_and_run_umap(ds):
    """make_graph writes the seeding k-means group (graph_datastore.py:958-975);
    run_umap builds its start from it (_get_ini_embed) and writes UMAP1/UMAP2
    for every cell (graph_datastore.py:1218-1380)."""
    d, (indptr, indices, data, G, feat) = ds
    red = d.zw["RNA/normed__I__hvgs"].attrs["latest_reduction"]
    km = d.zw[red].attrs["latest_kmeans"]
    centres = np.asarray(d.zw[km]["cluster_centers"][:])
    labels = np.asarray(d.zw[km]["cluster_labels"][:])
    assert centres.shape[1] == 15 and 2 <= centres.shape[0] <= 1000 and labels.shape == (1800,)
    assert labels.min() >= 0 and labels.max() < centres.shape[0]
    ini = d._get_ini_embed("RNA", "I", "hvgs", 2)
    assert ini.shape == (1800, 2) and ini.dtype == np.float32
    d.run_umap(feat_key="hvgs", n_epochs=50)
    u1, u2 = d.cells.fetch("RNA_UMAP1"), d.cells.fetch("RNA_UMAP2")
    assert u1.shape == (1800,) and np.isfinite(u1).all() and np.isfinite(u2).all()
    assert np.std(u1) > 0 and np.std(u2) > 0


def test_streamed_host_csr_equals_device_csr():
    """Host CSR gives the graph of the same CSR on the device, in every form:
    page-locked arrays read by the row kernel over the host link (one launch,
    or one per chunk; indptr pinned or not), and pageable arrays streamed in
    chunks through the three-slot staging ring (the copy of chunk i+1
    overlapping the normalisation of chunk i). Ragged last chunk, an empty
    row. The chunks are whole 256-row slices of the column statistics, so only
    the FP64 order of adding the slice partials differs."""
    from scarf_gb300 import pipeline
    indptr, indices, data, G, _ = small_counts(n_cells=2300, seed=5)
    feat = top_var_genes(indptr, indices, data, G, 300)
    pin = [torch.from_numpy(a).pin_memory() for a in (indptr, indices, data)]
    pageable = [torch.from_numpy(a.copy()) for a in (indptr, indices, data)]
    mixed = [pageable[0], pin[1], pin[2]]
    dev = [t.cuda() for t in pin]
    b = pipeline.make_graph(*dev, G, feat, 20, 10, precision="precision")
    for arrays, chunks in ((pin, (None, 500, 777, 2300)), (mixed, (None, 1000)), (pageable, (500, 777, None))):
        for chunk in chunks:
            a = pipeline.make_graph(*arrays, G, feat, 20, 10, precision="precision", chunk_cells=chunk)
            torch.cuda.synchronize()
            assert torch.equal(a.x, b.x)
            assert torch.allclose(a.mu, b.mu, rtol=1e-14, atol=0)
            assert torch.allclose(a.sigma, b.sigma, rtol=1e-14, atol=0)
            assert torch.equal(a.mu32, b.mu32) and torch.equal(a.sigma32, b.sigma32)
            assert torch.equal(a.indices, b.indices) and torch.equal(a.weights, b.weights)


def test_pinned_csr_trailing_empty_rows_and_pageable_refusal():
    """Page-locked CSR whose last chunk holds only empty rows, and a CSR that
    starts at a non-zero indptr[0], normalise like the device copy; the C ABI
    refuses pageable host pointers before any launch."""
    from scarf_gb300 import _lib as L
    from scarf_gb300 import kernels as K
    from scarf_gb300 import pipeline
    indptr, indices, data, G, _ = small_counts(n_cells=1000, seed=9)
    n = len(indptr) - 1
    feat = top_var_genes(indptr, indices, data, G, 200)
    indptr = np.concatenate([indptr, np.full(600, indptr[-1], dtype=indptr.dtype)])  # 600 empty rows
    ip = torch.from_numpy(indptr).pin_memory()
    ind, dat = torch.from_numpy(indices).pin_memory(), torch.from_numpy(data).pin_memory()
    xd, sd, qd = pipeline.normalize_csr_host(ip.cuda(), ind.cuda(), dat.cuda(), G, feat)
    for chunk in (None, 512, 256):
        x, s, q = pipeline.normalize_csr_host(ip, ind, dat, G, feat, chunk_cells=chunk)
        torch.cuda.synchronize()
        assert torch.equal(x, xd) and torch.allclose(s, sd, rtol=1e-14, atol=0)
    assert torch.count_nonzero(x[n:]) == 0
    # rows 300.. on their own: indptr starts at indptr[300], the entries at that offset
    a = 300
    off = int(indptr[a])
    x2, _, _ = pipeline.normalize_csr_host(ip[a:], ind[off:], dat[off:], G, feat)
    torch.cuda.synchronize()
    assert torch.equal(x2, xd[a:])
    cmap = pipeline.col_map(feat, G, "cuda")
    out = torch.empty((n, K.round_up(len(feat), 4)), dtype=torch.float32, device="cuda")
    with pytest.raises(ValueError, match="pageable"):
        L.check(L.load().sg_normalize_csr(
            K.handle(0).ptr, indptr.ctypes.data, indices.ctypes.data, data.ctypes.data, n, cmap.data_ptr(), G,
            len(feat), None, 1.0, None, 1000.0, L.SG_NORM_LOG1P | L.SG_NORM_RENORM_SUBSET, out.data_ptr(),
            out.stride(0), L.SG_F32, None, None, None, None))
