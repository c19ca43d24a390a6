"""Parity at the benchmark's CPU-runnable configuration and for mapping.

* C1: 10,000 cells x 20,000 genes of seeded negative-binomial counts (8
  clusters), 2,000 HVGs, 30 PCs, k = 11, through ``DataStore.make_graph`` in
  both numeric forms against the oracle (scarf/datastore/graph_datastore.py:
  513-1020 restated): library sizes bit-exact; normalised values, mu and
  sigma to FP32 rounding; the separated principal components; tie-aware
  recall@k of the graph against exact FP64 kNN of its own scores; edges bit
  for bit and edge weights within 1e-5 of the oracle's smoothing of the same
  neighbours; the fuzzy union's CSR bit for bit against scipy's. At 10,000
  cells the precision form splits the references over many CTAs, so each
  query has more candidate lists than the re-rank's bitonic path takes and
  the list-merge re-rank runs.
* run_mapping on a target whose genes come in another order with some of
  the reference's features absent (filled with 1.0 after normalisation,
  scarf/mapping_utils.py:148-214), against the oracle's align_target +
  map_queries (scarf/datastore/mapping_datastore.py:198-208).
"""
import numpy as np
import pytest
import scipy.sparse as sp

import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

C1 = dict(n_cells=10_000, n_genes=20_000, n_clusters=8, n_hvg=2000, dims=30, k=11, batch=1000)


@pytest.fixture(scope="module")
def c1():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from scarf_gb300 import synth
    csr = synth.nb_counts(C1["n_cells"], C1["n_genes"], C1["n_clusters"], 4466, lib_median=3000.0, device="cuda")
    feat = synth.select_hvgs(csr, C1["n_hvg"])
    want = oracle.make_graph(csr.indptr, csr.indices, csr.data, csr.n_genes, feat, dims=C1["dims"], k=C1["k"],
                             batch_size=C1["batch"])
    z = (want["x"] - want["mu"]) / want["sigma"]
    _, evals = oracle.pca_exact(z, C1["dims"] + 1)
    return csr, feat, want, evals


def _separated(evals, gap=0.02):
    """Number of leading components whose eigenvalue gap to the next one is
    above ``gap`` of the largest eigenvalue (their subspace is well defined)."""
    rel = (evals[:-1] - evals[1:]) / evals[0]
    m = 0
    for i, r in enumerate(rel):
        if r > gap:
            m = i + 1
    return max(m, 1)


@pytest.mark.parametrize("form", ["plain", "precision"])
def test_c1_make_graph_matches_oracle(c1, form):
    from scarf_gb300 import kernels as K
    from scarf_gb300.datastore import DataStore
    csr, feat, want, evals = c1
    n, G, dims, k, batch = csr.n_cells, csr.n_genes, C1["dims"], C1["k"], C1["batch"]
    ds = DataStore(csr.indptr, csr.indices, csr.data, G, precision=form)
    mask = np.zeros(G, dtype=bool)
    mask[feat] = True
    ds.RNA.feats.insert("I__hvgs", mask)
    ds.make_graph(feat_key="hvgs", dims=dims, k=k, batch_size=batch)
    zw = ds.zw
    normed = zw["RNA/normed__I__hvgs"]

    # a1: library sizes bit-exact, values to FP32 rounding
    dev = torch.device("cuda")
    lib = torch.empty(n, dtype=torch.int64, device=dev)
    cmap = np.full(G, -1, dtype=np.int32)
    cmap[feat] = np.arange(len(feat), dtype=np.int32)
    x = K.normalize_csr(torch.from_numpy(csr.indptr).to(dev), torch.from_numpy(csr.indices).to(dev),
                        torch.from_numpy(csr.data).to(dev), torch.from_numpy(cmap).to(dev), len(feat), libsize=lib)
    assert np.array_equal(lib.cpu().numpy(), want["scalar"].astype(np.int64))
    xg = x[:, :len(feat)].double().cpu().numpy()
    assert np.abs(xg - want["x"]).max() <= 4e-7 * max(1.0, np.abs(want["x"]).max())
    # a3: mu / sigma
    assert np.allclose(normed["mu"][:], want["mu"], rtol=2e-6, atol=1e-9)
    assert np.allclose(normed["sigma"][:], want["sigma"], rtol=2e-6, atol=1e-9)

    # a4: the separated components against the FP64 eigendecomposition
    red = zw["RNA/normed__I__hvgs/reduction__pca__30__I"]["reduction"][:]
    m = _separated(evals)
    assert m >= 3
    ang = oracle.subspace_angles(red[:, :m], want["loadings"][:, :m]).max()
    assert ang < 1e-3, f"{form}: principal angle {ang} over the first {m} components"

    # a6/a7: tie-aware recall@k against exact FP64 kNN of the graph's own scores
    loc = ds._get_latest_graph_loc("RNA", "I", "hvgs")
    knn = zw[loc.rsplit("/", 1)[0]]
    gi = knn["indices"][:].astype(np.int64)
    gd = knn["distances"][:]
    ann = ds._ann_cache[zw["RNA/normed__I__hvgs/reduction__pca__30__I"].attrs["latest_ann"]]
    s = ann.annIdx.scores[:, :dims].double().cpu().numpy()
    _, ed = oracle.exact_knn(s, s, k + 1)
    rec = oracle.recall_at_k(s, s, gi, ed[:, -1], rel=1e-5)
    assert rec >= (0.995 if form == "precision" else 0.999), f"{form}: recall@k {rec}"
    # self removal and the reference's recall figure: every cell finds itself
    assert not np.any(gi == np.arange(n)[:, None])
    assert knn.attrs["recall"] > 99.0

    # a8: edges bit for bit, weights within 1e-5 of the oracle's smoothing of the same neighbours
    e_want, w_want = oracle.smoothen_dists(gi.astype(np.uint64), gd, 1.0, 1.5, batch)
    g = zw[loc]
    assert np.array_equal(g["edges"][:], e_want)
    werr = np.abs(g["weights"][:] - w_want).max()
    assert werr <= 1e-5, f"{form}: edge weights off by {werr}"

    # a9: the fuzzy union bit for bit against scipy
    gm = sp.csr_matrix((g["weights"][:], (g["edges"][:, 0].astype(np.int64), g["edges"][:, 1].astype(np.int64))),
                       shape=(n, n))
    u_want = oracle.symmetrize(gm)
    u_want.sort_indices()
    u = ds.load_graph(feat_key="hvgs", symmetric=True)
    assert np.array_equal(u.indptr, u_want.indptr) and np.array_equal(u.indices, u_want.indices)
    assert np.array_equal(u.data, u_want.data)


@pytest.fixture(scope="module")
def mapped():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from helpers import small_counts, top_var_genes
    from scarf_gb300.datastore import DataStore
    indptr, indices, data, G, _ = small_counts(n_cells=2000, n_genes=3000, seed=7)
    feat = top_var_genes(indptr, indices, data, G, 300)
    ids = np.array([f"g{i}" for i in range(G)])
    ref = DataStore(indptr, indices, data, G, gene_ids=ids, precision="precision")
    mask = np.zeros(G, dtype=bool)
    mask[feat] = True
    ref.RNA.feats.insert("I__hvgs", mask)
    ref.make_graph(feat_key="hvgs", dims=20, k=11, batch_size=500)
    # target: other cells of the same populations, genes shuffled, 30 of the 300 features absent
    tp, ti, tv, _, _ = small_counts(n_cells=700, n_genes=3000, seed=7, empty_rows=(5,))
    rng = np.random.default_rng(3)
    drop = rng.choice(feat, 30, replace=False)
    order = rng.permutation(np.setdiff1d(np.arange(G), drop))
    tm = sp.csr_matrix((tv, ti, tp), shape=(700, G))[:, order].tocsr()
    tm.sort_indices()
    target = DataStore(tm.indptr.astype(np.int64), tm.indices.astype(np.int32), tm.data.astype(np.int32),
                       len(order), gene_ids=ids[order])
    ref.run_mapping(target_assay=target.RNA, target_name="panel", target_feat_key="hvgs_panel", save_k=5)
    return ref, target, tm, ids[order], feat


def test_run_mapping_target_panel_matches_oracle(mapped):
    from scarf_gb300 import kernels as K
    from scarf_gb300.datastore import align_col_map
    ref, target, tm, t_ids, feat = mapped
    zw = ref.zw
    ref_feat_ids = ref.RNA.feats.fetch("ids", key="I__hvgs")
    pos = {g: j for j, g in enumerate(t_ids)}
    t_idx = np.array([pos.get(g, -1) for g in ref_feat_ids])
    assert (t_idx == -1).sum() == 30
    want_x = oracle.align_target(tm.indptr, tm.indices, tm.data, len(t_ids), t_idx)
    # the aligned, normalised target rows: absent features are 1.0
    cmap, missing = align_col_map(ref_feat_ids, t_ids)
    dev = torch.device("cuda")
    x = K.normalize_csr(torch.from_numpy(tm.indptr.astype(np.int64)).to(dev),
                        torch.from_numpy(tm.indices.astype(np.int32)).to(dev),
                        torch.from_numpy(tm.data.astype(np.int32)).to(dev), torch.from_numpy(cmap).to(dev),
                        len(ref_feat_ids), missing_mask=torch.from_numpy(missing).to(dev), fill_value=1.0)
    xg = x[:, :len(ref_feat_ids)].double().cpu().numpy()
    assert np.all(xg[:, t_idx == -1] == 1.0)
    assert np.abs(xg - want_x).max() <= 4e-7 * max(1.0, np.abs(want_x).max())
    # per-block reducer -> knn_query(k=save_k), no self fix, against the reference cells' scores
    norm = zw["RNA/normed__I__hvgs"]
    red = zw["RNA/normed__I__hvgs/reduction__pca__20__I"]["reduction"][:]
    ann = ref._ann_cache[zw["RNA/normed__I__hvgs/reduction__pca__20__I"].attrs["latest_ann"]]
    rs = ann.annIdx.scores[:, :20].double().cpu().numpy()
    oi, od, qs = oracle.map_queries(want_x, norm["mu"][:], norm["sigma"][:], red, rs, 5)
    p = zw["RNA/projections/panel"]
    gi, gd = p["indices"][:], p["distances"][:]
    assert gi.shape == (700, 5) and gi.dtype == np.uint64 and gd.dtype == np.float64
    rec = oracle.recall_at_k(qs, rs, gi.astype(np.int64), od[:, -1], rel=1e-4)
    assert rec >= 0.999, f"mapping recall@k {rec}"
    assert np.abs(gd - od).max() <= 1e-4 * max(1.0, od.max())
    # the empty target row maps like every other row (library size 0 -> 1)
    assert np.all(np.isfinite(gd[5]))
