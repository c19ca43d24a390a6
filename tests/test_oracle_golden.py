"""Pin the CPU oracle against the reference's own fixtures and functions.

``pbmc1k_knn.npz`` is the reference's test data (scarf/tests/datasets,
checked by scarf/tests/test_datastore.py:66-79); ``ref_functions.npz`` holds
outputs of the reference's own functions executed from its source by
``tests/golden/make_golden.py``.
"""
import os

import numpy as np
import pytest
import scipy.sparse as sp

import oracle


@pytest.fixture(scope="module")
def kat(golden_dir):
    return np.load(os.path.join(golden_dir, "pbmc1k_knn.npz"))


@pytest.fixture(scope="module")
def ref(golden_dir):
    return np.load(os.path.join(golden_dir, "ref_functions.npz"))


def test_smoothing_known_answer(kat):
    # test_graph_weights (test_datastore.py:76-79), made two-sided
    edges, w = oracle.smoothen_dists(kat["indices"], kat["distances"], 1.0, 1.5, 1000)
    assert np.abs(w - kat["weights"]).max() < 1e-5
    n, k = kat["indices"].shape
    assert np.array_equal(edges[:, 0], np.repeat(np.arange(n), k))
    assert np.array_equal(edges[:, 1], kat["indices"].ravel())
    # the first weight of every row is exactly 1.0 (rho is the first distance)
    assert np.all(w.reshape(n, k)[:, 0] == 1.0)


def test_smoothing_column0_is_skipped(kat):
    # including column 0 in the sigma sum breaks the known answer
    d = kat["distances"].astype(np.float32)
    sig, rho = oracle.smooth_knn_dist(d, 11, local_connectivity=1.0, bandwidth=1.5)
    d2 = np.concatenate([np.zeros((d.shape[0], 1), np.float32), d], axis=1)
    sig2, _ = oracle.smooth_knn_dist(d2, 11, local_connectivity=1.0, bandwidth=1.5)
    assert not np.allclose(sig, sig2)


def test_smoothen_dists_chunk_loop(ref):
    edges, w = oracle.smoothen_dists(ref["smooth_idx"], ref["smooth_dist"], 1.0, 1.5,
                                     int(ref["smooth_chunk"]))
    assert np.array_equal(edges, ref["smooth_edges"])
    assert np.array_equal(w, ref["smooth_w"])
    # the chunk-local self check of compute_membership_strengths fires in later chunks
    assert (ref["smooth_w"] == ref["smooth_w"].min()).sum() >= 1


def test_clean_array(ref):
    assert np.array_equal(oracle.clean_array(ref["clean_in"]), ref["clean_out0"])
    assert np.array_equal(oracle.clean_array(ref["clean_in"], 1), ref["clean_out1"])


def test_norm_lib_size_log(ref):
    c = ref["norm_counts"]
    m = sp.csr_matrix(c)
    x, _ = oracle.normed_csr(m.indptr, m.indices, m.data.astype(np.int32), c.shape[1],
                             np.arange(c.shape[1]))
    assert np.array_equal(x, ref["norm_log"])


def test_fix_knn_query(ref):
    fi, fd, nm = oracle.fix_knn_query(ref["fix_ind"], ref["fix_dist"], ref["fix_ref"])
    assert np.array_equal(fi, ref["fix_out_i"])
    assert np.array_equal(fd, ref["fix_out_d"])
    assert nm == int(ref["fix_nmis"])


def test_self_query_knn(ref):
    pts = ref["sqk_points"]
    k = int(ref["sqk_k"])
    i, d, rec = oracle.self_query_knn(pts, k, int(ref["sqk_chunk"]))
    assert np.array_equal(i, ref["sqk_indices"])
    assert np.array_equal(d, ref["sqk_distances"])
    assert rec == pytest.approx(float(ref["sqk_recall"]))


def _csr(ref, p):
    return ref[p + "_indptr"], ref[p + "_indices"], ref[p + "_data"]


def test_symmetrize_and_fuzzy_union(ref):
    n = int(ref["union_n"])
    edges = np.stack([ref["union_rows"], ref["union_cols"]], 1)
    k = len(ref["union_rows"]) // n
    g = oracle.store_to_sparse(edges, ref["union_w"], n, k)
    s = oracle.symmetrize(g)
    s.sort_indices()
    for got, want in zip((s.indptr, s.indices, s.data), _csr(ref, "sym")):
        assert np.array_equal(got, want)
    for mix, p in ((1.0, "fss"), (0.7, "fss07")):
        u = oracle.fuzzy_simplicial_set(g, mix).tocsr()
        u.sort_indices()
        for got, want in zip((u.indptr, u.indices, u.data), _csr(ref, p)):
            assert np.array_equal(got, want)


def test_incremental_pca_block_order(ref):
    x = ref["pca_x"]
    mu, sd = ref["pca_mu"], ref["pca_sigma"]
    z = (x - mu) / sd
    b = int(ref["pca_batch"])
    blocks = [z[s:s + b] for s in range(0, z.shape[0], b)]
    load, pca = oracle.fit_pca_reference_order(blocks, int(ref["pca_dims"]), ref["pca_use"])
    want = ref["pca_loadings"]
    assert load.shape == want.shape
    assert np.abs(load - want).max() < 1e-8
    assert np.abs(pca.explained_variance_ratio_ - ref["pca_evr"]).max() < 1e-10


def test_incremental_pca_vs_sklearn():
    skd = pytest.importorskip("sklearn.decomposition")
    rng = np.random.default_rng(3)
    z = rng.normal(size=(500, 30)) @ rng.normal(size=(30, 30))
    ours = oracle.IncrementalPCARestated(8)
    theirs = skd.IncrementalPCA(n_components=8)
    for s in range(0, 500, 120):
        ours.partial_fit(z[s:s + 120])
        theirs.partial_fit(z[s:s + 120])
    assert np.abs(ours.components_ - theirs.components_).max() < 1e-8


def test_exact_pca_spans_ipca_subspace():
    rng = np.random.default_rng(4)
    base = rng.normal(size=(2000, 5)) * np.array([9, 7, 5, 4, 3.0])
    z = np.hstack([base, 0.1 * rng.normal(size=(2000, 15))]) @ np.linalg.qr(rng.normal(size=(20, 20)))[0]
    comps, _ = oracle.pca_exact(z, 6)
    blocks = [z[s:s + 300] for s in range(0, 2000, 300)]
    load, _ = oracle.fit_pca_reference_order(blocks, 5)
    ang = oracle.subspace_angles(comps[:, :5], load)
    assert ang.max() < 1e-3


def test_exact_knn_tie_order():
    pts = np.array([[0.0], [1.0], [1.0], [2.0], [5.0]])
    i, d = oracle.exact_knn(pts, pts, 4)
    assert i[0].tolist() == [0, 1, 2, 3]
    assert i[1].tolist() == [1, 2, 0, 3]
    assert i[2].tolist() == [1, 2, 0, 3]


def _sklearn_minibatch(x, k, block, seed):
    cluster = pytest.importorskip("sklearn.cluster")
    import warnings
    km = cluster.MiniBatchKMeans(n_clusters=k, random_state=seed, batch_size=block, n_init=3)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        for r0 in range(0, len(x), block):
            km.partial_fit(x[r0:r0 + block].astype(np.float64))
    return km.cluster_centers_, km.predict(x.astype(np.float64))


@pytest.mark.parametrize("n,d,k,clusters,seed", [(1500, 10, 500, 12, 5), (1000, 12, 300, 9, 11)])
def test_kmeans_minibatch_matches_sklearn_when_it_draws_nothing(n, d, k, clusters, seed):
    """k = block rows: k-means++ picks every row of the first block (in a
    random order) and no centre is ever light enough to be reassigned, so
    scikit-learn's MiniBatchKMeans is deterministic up to the order of its
    centres, and the restatement reproduces it exactly (the second case ends
    on a ragged block of 100 rows)."""
    from helpers import clustered_points
    x = clustered_points(n, d, n_clusters=clusters, seed=seed)
    c_o, l_o = oracle.kmeans_minibatch(x, k, k, 4466)
    c_s, l_s = _sklearn_minibatch(x, k, k, 4466)
    d = ((c_o[:, None, :] - c_s[None, :, :]) ** 2).sum(-1)
    perm = d.argmin(1)
    assert len(np.unique(perm)) == k
    assert np.sqrt(d.min(1)).max() == 0.0
    assert np.array_equal(perm[l_o], l_s)


def test_kmeans_minibatch_quality_with_kmeans_plusplus_and_reassignment():
    """k < block rows (k-means++ on the first block) over 20 blocks, where the
    periodic reassignment check runs: the draws differ from numpy's, so the
    result is compared by inertia."""
    from helpers import clustered_points
    x = clustered_points(20000, 16, n_clusters=30, seed=7)
    c_o, l_o = oracle.kmeans_minibatch(x, 100, 1000, 4466)
    c_s, l_s = _sklearn_minibatch(x, 100, 1000, 4466)
    inertia = lambda c, l: float(((x.astype(np.float64) - c[l]) ** 2).sum())
    assert abs(inertia(c_o, l_o) / inertia(c_s, l_s) - 1.0) < 0.05
    # every label is the nearest centre
    d = ((x[:, None, :].astype(np.float64) - c_o[None].astype(np.float32).astype(np.float64)) ** 2).sum(-1)
    assert np.array_equal(d.argmin(1), l_o)


def test_kmeans_hash_is_the_splitmix64_finaliser():
    """The counter hash both the kernel and the restatement draw from:
    SplitMix64's output function of seed + (stream * 2^32 + i) * golden."""
    def ref(seed, stream, i):
        m = (1 << 64) - 1
        z = (seed + ((stream << 32) + i) * 0x9E3779B97F4A7C15) & m
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & m
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & m
        return z ^ (z >> 31)
    for seed, stream, i in ((4466, 1, 0), (0, 2, 7), ((1 << 64) - 5, 0x80000000 + 3, 4095)):
        assert int(oracle.kmeans_hash(seed, stream, i)) == ref(seed, stream, i)


def _merge_inputs(ref):
    n, k = int(ref["merge_n"]), int(ref["merge_k"])
    mats = [sp.csr_matrix((ref[f"merge_g{g}_data"], ref[f"merge_g{g}_indices"].ravel(),
                           np.arange(0, n * k + 1, k)), shape=(n, n)) for g in range(2)]
    return n, k, mats


def test_calc_snn_and_merge_graphs(ref):
    """calc_snn and merge_graphs (knn_utils.py:195-274) against the reference's
    own functions run on the same two graphs."""
    n, k, mats = _merge_inputs(ref)
    for g in range(2):
        assert np.array_equal(oracle.calc_snn(ref[f"merge_g{g}_indices"]), ref[f"merge_g{g}_snn"])
    m = oracle.merge_graphs(mats)
    assert np.array_equal(m.row, ref["merge_row"])
    assert np.array_equal(m.col, ref["merge_col"])
    assert np.array_equal(m.data, ref["merge_data"])


def test_umap_find_ab_params_published_values():
    """umap-learn's curve parameters for its defaults (spread 1, min_dist 0.1)
    are the published a = 1.577, b = 0.895; the GPU module's copy agrees."""
    a, b = oracle.umap_find_ab_params(1.0, 0.1)
    assert abs(a - 1.577) < 1e-3 and abs(b - 0.895) < 1e-3
    from scarf_gb300 import umap as gu
    assert np.allclose(gu.find_ab_params(2.0, 1.0), oracle.umap_find_ab_params(2.0, 1.0))
    w = np.array([1.0, 0.5, 0.25, 0.0])
    assert np.allclose(oracle.umap_make_epochs_per_sample(w, 200), [1.0, 2.0, 4.0, -1.0])
    assert np.allclose(gu.make_epochs_per_sample(w, 200), [1.0, 2.0, 4.0, -1.0])


def test_umap_layout_sequential_separates_clusters():
    """The restated sequential layout pulls a random start apart into its
    clusters (a property check: umap-learn is not installed to pin against)."""
    from helpers import umap_graph, embedding_purity
    x, lab, _, head, tail, w = umap_graph(150, 8, 3, 8, seed=4)
    a, b = oracle.umap_find_ab_params(2.0, 1.0)
    eps = oracle.umap_make_epochs_per_sample(w, 40)
    y0 = np.random.default_rng(1).normal(size=(150, 2)) * 10
    rnd = np.random.default_rng(2)
    y = oracle.umap_layout_sequential(y0, head, tail, eps, 40, a, b, rand_vertex=lambda n, i, p: rnd.integers(1 << 30))
    assert embedding_purity(y0, lab) < 0.6
    assert embedding_purity(y, lab) > 0.95


def test_rescale_array_and_ini_embed_pca(ref):
    """The host steps of _get_ini_embed (graph_datastore.py:427-457):
    rescale_array against the reference's own function (utils.py:120-140),
    and the PCA of the k-means centres against scikit-learn's PCA."""
    from scarf_gb300 import datastore
    assert np.array_equal(datastore.rescale_array(ref["rescale_in"].copy()), ref["rescale_out"])
    skd = pytest.importorskip("sklearn.decomposition")
    rng = np.random.default_rng(9)
    c = rng.normal(size=(300, 20)) @ rng.normal(size=(20, 20))
    ours = datastore.pca_fit_transform(c, 2)
    theirs = skd.PCA(n_components=2).fit_transform(c)
    assert np.abs(ours - theirs).max() < 1e-9 * max(1.0, np.abs(theirs).max())
