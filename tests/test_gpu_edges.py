"""Edge cases of the graph path through DataStore.make_graph, both forms,
against the oracle: the smallest graph AnnStream allows (k = n - 1 after the
caps of scarf/ann.py:91-92, :173-185), duplicate cells (zero distances and
ties, where the self rule of fix_knn_query, scarf/ann.py:31-52, and rho of
smooth_knn_dist matter), cells without any count in the selected features
(library size 0 -> 1, scarf/assay.py:54-64) and a feature that is constant
over the cells (sigma 0 -> 1, clean_array, scarf/utils.py:143-153)."""
import numpy as np
import pytest
import scipy.sparse as sp

import oracle
from helpers import small_counts, top_var_genes

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _graph(indptr, indices, data, G, feat, form, dims, k, batch):
    from scarf_gb300.datastore import DataStore
    ds = DataStore(indptr, indices, data, G, precision=form)
    mask = np.zeros(G, dtype=bool)
    mask[feat] = True
    ds.RNA.feats.insert("I__hvgs", mask)
    ds.make_graph(feat_key="hvgs", dims=dims, k=k, batch_size=batch)
    loc = ds._get_latest_graph_loc("RNA", "I", "hvgs")
    knn = ds.zw[loc.rsplit("/", 1)[0]]
    g = ds.zw[loc]
    red = ds.zw["RNA/normed__I__hvgs"].attrs["latest_reduction"]
    ann = ds._ann_cache[ds.zw[red].attrs["latest_ann"]]
    return ds, knn, g, ann


def _check(indptr, indices, data, G, feat, form, dims, k, batch, want_k=None):
    ds, knn, g, ann = _graph(indptr, indices, data, G, feat, form, dims, k, batch)
    n = len(indptr) - 1
    gi = knn["indices"][:].astype(np.int64)
    gd = knn["distances"][:]
    kk = gi.shape[1]
    if want_k is not None:
        assert kk == want_k
    d = ann.dims
    s = ann.annIdx.scores[:, :d].double().cpu().numpy()
    # the neighbours: tie-aware recall against exact FP64 kNN of the graph's own scores
    _, ed = oracle.exact_knn(s, s, kk + 1)
    rec = oracle.recall_at_k(s, s, gi, ed[:, -1], rel=1e-5)
    assert rec >= 0.995, f"{form}: recall {rec}"
    assert np.all((gi >= 0) & (gi < n))
    # the weights: the oracle's smoothing of the same neighbours, edges bit for bit
    e_want, w_want = oracle.smoothen_dists(gi.astype(np.uint64), gd, 1.0, 1.5, batch)
    assert np.array_equal(g["edges"][:], e_want)
    assert np.abs(g["weights"][:] - w_want).max() <= 1e-5
    assert np.all(np.isfinite(g["weights"][:]))
    # the union, bit for bit
    gm = sp.csr_matrix((g["weights"][:], (g["edges"][:, 0].astype(np.int64), g["edges"][:, 1].astype(np.int64))),
                       shape=(n, n))
    u_want = oracle.symmetrize(gm)
    u_want.sort_indices()
    u = ds.load_graph(feat_key="hvgs", symmetric=True)
    assert np.array_equal(u.indptr, u_want.indptr) and np.array_equal(u.indices, u_want.indices)
    assert np.array_equal(u.data, u_want.data)
    return ds, gi, gd


@pytest.fixture(scope="module")
def gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


@pytest.mark.parametrize("form", ["plain", "precision"])
def test_smallest_graph(gpu, form):
    # 14 cells, k = 21 asked: AnnStream caps k at n - 1 = 13 and dims at n
    indptr, indices, data, G, _ = small_counts(n_cells=14, n_genes=400, seed=3)
    feat = top_var_genes(indptr, indices, data, G, 50)
    _check(indptr, indices, data, G, feat, form, dims=10, k=21, batch=14, want_k=13)


@pytest.mark.parametrize("form", ["plain", "precision"])
def test_duplicate_cells_and_empty_feature_rows(gpu, form):
    indptr, indices, data, G, _ = small_counts(n_cells=900, n_genes=1500, seed=8)
    m = sp.csr_matrix((data, indices, indptr), shape=(len(indptr) - 1, G)).tolil()
    feat = top_var_genes(indptr, indices, data, G, 120)
    other = np.setdiff1d(np.arange(G), feat)
    # cells 10..14 copy cell 5; cells 20..27 have counts only outside the features
    for r in range(10, 15):
        m[r] = m[5]
    for r in range(20, 28):
        m[r] = 0
        m[r, other[r]] = 4
    # a feature no cell has a count of: constant over the cells, sigma 0
    m[:, feat[0]] = 0
    c = m.tocsr()
    c.sort_indices()
    ds, gi, gd = _check(c.indptr.astype(np.int64), c.indices.astype(np.int32), c.data.astype(np.int32), G, feat,
                        form, dims=15, k=11, batch=300)
    # the copies of cell 5 find one another at distance 0
    for r in (5, 10, 11, 12, 13, 14):
        dup = {5, 10, 11, 12, 13, 14} - {r}
        assert dup <= set(gi[r].tolist()), (r, gi[r])
        assert np.all(gd[r][np.isin(gi[r], list(dup))] <= 1e-6)
    # the cells without feature counts (and the empty cells 3 and 700) are identical in the reduced
    # space: one zero-distance clique of 10, within every member's 11 neighbours
    zero = set(range(20, 28)) | {3, 700}
    for r in sorted(zero):
        assert zero - {r} <= set(gi[r].tolist()), (r, gi[r])
    sig = ds.zw["RNA/normed__I__hvgs"]["sigma"][:]
    assert np.all(np.isfinite(sig)) and np.all(sig > 0)


@pytest.mark.parametrize("d,k,margin", [(30, 10, 0), (30, 28, 16), (40, 40, 16), (64, 21, 16), (62, 5, 8)])
def test_knn_list_lengths_and_unfolded_norms(gpu, d, k, margin):
    """Every candidate-list length of the tensor-core kNN (16, 48, 64 slots)
    and the dimensions above 61, where the reference norms are added in the
    epilogue instead of folded into the MMA, against exact FP64 kNN, beside
    a self-kNN of 9,220 rows, whose last reference split (of nine, 1,152 rows
    each) holds four rows."""
    from helpers import clustered_points
    from scarf_gb300 import kernels as K
    for n in (3000, 9220):
        pts = clustered_points(n, d, seed=n + d)
        ld = (d + 3) // 4 * 4
        t = torch.zeros((n, ld), dtype=torch.float32, device="cuda")
        t[:, :d] = torch.from_numpy(pts).cuda()
        idx, dist, nm = K.knn(t, t, d, k, self_offset=0, margin=margin, precision="precision")
        torch.cuda.synchronize()
        gi = idx.cpu().numpy()
        assert np.all((gi >= 0) & (gi < n))
        _, od = oracle.exact_knn(pts, pts, k + 1)
        assert oracle.recall_at_k(pts, pts, gi, od[:, -1]) >= 0.995
        diff = pts[:, None, :].astype(np.float64) - pts[gi].astype(np.float64)
        assert np.abs(dist.cpu().numpy() - (diff * diff).sum(-1)).max() <= 1e-4 * max(1.0, od.max())


def test_normalize_wide_output(gpu):
    """More than 32,767 selected features: the column map stays int32 (the
    narrow int16 map covers the usual widths) and each dense row buffer takes
    most of a CTA's shared memory; values, library sizes and the column
    statistics against the oracle."""
    from scarf_gb300 import kernels as K
    indptr, indices, data, G, _ = small_counts(n_cells=300, n_genes=42_000, seed=12)
    feat = np.sort(np.random.default_rng(1).choice(G, 40_000, replace=False))
    cmap = np.full(G, -1, np.int32)
    cmap[feat] = np.arange(len(feat), dtype=np.int32)
    h = len(feat)
    cs = torch.zeros(h, dtype=torch.float64, device="cuda")
    cq = torch.zeros_like(cs)
    lib = torch.zeros(len(indptr) - 1, dtype=torch.int64, device="cuda")
    x = K.normalize_csr(*(torch.from_numpy(a).cuda() for a in (indptr, indices, data, cmap)), h, colsum=cs,
                        colsumsq=cq, libsize=lib)
    torch.cuda.synchronize()
    want, libw = oracle.normed_csr(indptr, indices, data, G, feat)
    got = x[:, :h].double().cpu().numpy()
    assert np.abs(got - want).max() <= 4e-7 * max(1.0, np.abs(want).max())
    assert np.array_equal(lib.cpu().numpy(), np.asarray(libw).astype(np.int64))
    assert np.allclose(cs.cpu().numpy(), want.sum(0), rtol=2e-6, atol=1e-6)
    assert np.allclose(cq.cpu().numpy(), (want * want).sum(0), rtol=2e-6, atol=1e-6)


@pytest.mark.parametrize("lc,bw", [(0.5, 1.5), (1.5, 1.0), (2.0, 2.5), (3.0, 1.5)])
def test_smoothing_connectivity_and_bandwidth(gpu, lc, bw):
    """make_graph's local_connectivity and bandwidth (rho interpolated between
    non-zero distances, smooth_knn_dist's target log2(k) * bandwidth) against
    the oracle, duplicates (zero distances) included."""
    from helpers import clustered_points
    from scarf_gb300 import kernels as K
    pts = clustered_points(2000, 10, seed=31, dup=((1, 2), (3, 4), (3, 5)))
    oi, od, _ = oracle.self_query_knn(pts, 11)
    for chunk in (2000, 700):
        edges, w = K.smooth(torch.from_numpy(oi.astype(np.int64)).cuda(), torch.from_numpy(od.astype(np.float32)).cuda(),
                            lc, bw, chunk)
        e, ow = oracle.smoothen_dists(oi, od, lc, bw, chunk)
        assert np.array_equal(edges.cpu().numpy(), e.astype(np.int64))
        assert np.abs(w.cpu().numpy() - ow).max() < 1e-5, (lc, bw, chunk)


@pytest.mark.parametrize("mix", [1.0, 0.5, 0.0])
def test_union_mix_duplicates_self_loops_and_zeros(gpu, mix):
    """The fuzzy union (umap.py:118-123, set_op_mix_ratio) of a graph with
    repeated (row, column) pairs (summed, as the reference's CSR build does),
    self loops and zero weights, bit for bit against scipy, zeros removed."""
    from scarf_gb300 import kernels as K
    rng = np.random.default_rng(2)
    n, k = 500, 7
    cols = rng.integers(0, n, size=(n, k))
    cols[:, 3] = cols[:, 2]                      # the same neighbour twice in a row
    cols[::7, 4] = np.arange(0, n, 7)            # self loops
    w = rng.random(n * k).astype(np.float32).astype(np.float64)
    w[::11] = 0.0                                # zero weights
    edges = np.stack([np.repeat(np.arange(n), k), cols.ravel()], 1).astype(np.int64)
    g = oracle.store_to_sparse(edges, w, n, k)
    want = oracle.fuzzy_simplicial_set(g, mix).tocsr()
    want.sort_indices()
    ip, ind, dat = K.fuzzy_union(torch.from_numpy(edges).cuda(), torch.from_numpy(w).cuda(), n, k, mix=mix)
    torch.cuda.synchronize()
    assert np.array_equal(ip.cpu().numpy(), want.indptr)
    assert np.array_equal(ind.cpu().numpy(), want.indices)
    assert np.array_equal(dat.cpu().numpy(), want.data)


def test_kmeans_one_centre_per_row(gpu):
    """k = n = block rows: scikit-learn's k-means++ then picks every row, so
    each row is its own centre and its own label."""
    from scarf_gb300 import kernels as K
    pts = np.random.default_rng(4).normal(size=(300, 12)).astype(np.float32)
    x = torch.zeros((300, 12), dtype=torch.float32, device="cuda")
    x[:] = torch.from_numpy(pts).cuda()
    c, lab = K.kmeans(x, 12, 300, 300, 7)
    torch.cuda.synchronize()
    assert np.array_equal(lab.cpu().numpy(), np.arange(300))
    assert np.array_equal(c.cpu().numpy(), pts.astype(np.float64))


@pytest.mark.parametrize("k", [2, 3])
def test_smoothing_few_neighbours(gpu, k):
    """Very short rows (k = 2 and 3): the bisection sums from column 1 only."""
    from helpers import clustered_points
    from scarf_gb300 import kernels as K
    pts = clustered_points(1200, 8, seed=5, dup=((1, 2),))
    oi, od, _ = oracle.self_query_knn(pts, k)
    edges, w = K.smooth(torch.from_numpy(oi.astype(np.int64)).cuda(), torch.from_numpy(od.astype(np.float32)).cuda(),
                        1.0, 1.5, 500)
    e, ow = oracle.smoothen_dists(oi, od, 1.0, 1.5, 500)
    assert np.array_equal(edges.cpu().numpy(), e.astype(np.int64))
    assert np.abs(w.cpu().numpy() - ow).max() < 1e-5


@pytest.mark.parametrize("precision", ["plain", "precision"])
@pytest.mark.parametrize("nr", [12, 40, 129])
def test_query_against_a_tiny_reference(gpu, precision, nr):
    """Mapping queries (no self rule) against references fewer than a
    candidate list's slots: every returned neighbour is a real reference."""
    from helpers import clustered_points
    from scarf_gb300 import kernels as K
    refs = clustered_points(nr, 20, seed=nr)
    q = clustered_points(700, 20, seed=nr + 1)
    tr = torch.from_numpy(refs).cuda()
    tq = torch.from_numpy(q).cuda()
    k = min(11, nr)
    idx, dist, _ = K.knn(tq, tr, 20, k, margin=16, precision=precision)
    torch.cuda.synchronize()
    gi = idx.cpu().numpy()
    assert np.all((gi >= 0) & (gi < nr))
    _, od = oracle.exact_knn(q, refs, k)
    assert oracle.recall_at_k(q, refs, gi, od[:, -1]) >= 0.995
    for row in gi:
        assert len(set(row.tolist())) == k


@pytest.mark.parametrize("h,dims", [(40, 20), (300, 64)])
def test_projection_narrow_features_and_widest_basis(gpu, h, dims):
    """The tensor-core projection with fewer features than one 64-feature
    chunk (the rest of the box reads as zeros) and with the widest basis it
    takes (64 scores), against the oracle's reducer; the plain form beside it."""
    from scarf_gb300 import kernels as K
    indptr, indices, data, G, _ = small_counts(n_cells=2000, n_genes=1500, seed=6)
    feat = top_var_genes(indptr, indices, data, G, h)
    cmap = np.full(G, -1, np.int32)
    cmap[feat] = np.arange(h, dtype=np.int32)
    cs = torch.zeros(h, dtype=torch.float64, device="cuda")
    cq = torch.zeros_like(cs)
    x = K.normalize_csr(*(torch.from_numpy(a).cuda() for a in (indptr, indices, data, cmap)), h, colsum=cs,
                        colsumsq=cq)
    mu, sg, mu32, sg32 = K.zstats(cs, cq, x.shape[0])
    cov, zsum = K.covariance(x, mu32, sg32, n_cols=h)
    comps, _, _, l32 = K.pca_basis(cov, zsum, x.shape[0], dims + 1, n_load=dims, ld_l=dims)
    xw, _ = oracle.normed_csr(indptr, indices, data, G, feat)
    omu, osg = oracle.zstats(xw)
    want = oracle.reducer(xw, omu, osg, comps.cpu().numpy()[:, :dims])
    for form, tol in (("plain", 2e-5), ("precision", 1e-4)):
        s = K.project(x, mu32, sg32, l32, dims, n_cols=h, ld_s=(dims + 3) // 4 * 4, precision=form)
        torch.cuda.synchronize()
        got = s[:, :dims].cpu().numpy()
        assert np.abs(got - want).max() <= tol * max(1.0, np.abs(want).max()), form


@pytest.mark.parametrize("h", [300, 257])
def test_covariance_precision_unaligned_rows_equal_aligned(gpu, h):
    """The 3xBF16 scatter reads its rows as 16-byte vectors when every row
    starts on a 16-byte boundary and element by element otherwise (an odd row
    stride, or a matrix starting one float in): both give the same bits, also
    with a row mask and a ragged last tile."""
    from scarf_gb300 import kernels as K
    g = torch.Generator(device="cuda").manual_seed(h)
    n = 5_000 + 37
    base = torch.rand((n, h), generator=g, device="cuda") * torch.rand(h, generator=g, device="cuda")
    base[base < 0.6] = 0.0
    aligned = torch.zeros((n, K.round_up(h, 4)), device="cuda")
    aligned[:, :h] = base
    odd = torch.zeros((n, h + 1), device="cuda")          # row stride h + 1: rows not 16-byte aligned
    odd[:, :h] = base
    shifted = torch.zeros(n * (h + 4) + 1, device="cuda")[1:].view(n, h + 4)   # starts one float in
    shifted[:, :h] = base
    mu = base.double().mean(0).float()
    sg = base.double().std(0).float()
    sg = torch.where(sg > 0, sg, torch.ones_like(sg))    # all-zero columns: sigma 1, as clean_array sets it
    mask = torch.from_numpy((np.arange(n) % 5 != 2).astype(np.uint8)).cuda()
    for rm in (None, mask):
        want = K.covariance(aligned, mu, sg, n_cols=h, row_mask=rm, precision="precision")
        for x in (odd, shifted):
            got = K.covariance(x, mu, sg, n_cols=h, row_mask=rm, precision="precision")
            torch.cuda.synchronize()
            assert torch.equal(got[0], want[0]) and torch.equal(got[1], want[1])
