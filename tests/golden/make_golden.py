"""Generate the golden fixtures under tests/golden from the scarf reference.

Run here, where the reference source tree is present:

    python tests/golden/make_golden.py /root/reference

Two kinds of fixtures are written:

* ``pbmc1k_knn.npz`` -- the reference's own test vectors
  (``scarf/tests/datasets/knn_indices.npy``, ``knn_distances.npy``,
  ``knn_weights.npy``; checked by ``scarf/tests/test_datastore.py:66-79``),
  re-saved compressed. ``knn_weights`` is a known answer for the smoothing
  step given the indices and distances (one chunk of 808 rows, k=11,
  lc=1.0, bw=1.5).
* ``zarr_chunks.npz`` -- Blosc-LZ4 chunks of the reference's test store and
  the cell totals that pin their decoding (see ``zarr_chunks``).
* ``ref_functions.npz`` -- seeded small inputs and the outputs of the
  reference's own functions, executed from its source files. scarf's package
  import pulls dask/zarr/numba, which are absent, so each function is lifted
  out of its module with ``ast`` and executed in a namespace holding numpy,
  scipy and scikit-learn (and, for ``smoothen_dists``, the oracle's
  restatement of the two umap-learn functions it calls, so that the chunk
  loop and the ``global_min`` fix of the reference are what is pinned;
  ``calc_snn`` runs without its numba ``jit`` decorator).

The fixtures are committed; this script is the recipe that made them.
"""

from __future__ import annotations

import ast
import sys
import types
from pathlib import Path

import numpy as np
import scipy.sparse as sp

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

import oracle  # noqa: E402


def lift(src_file: Path, qualname: str, ns: dict):
    """Execute the definition ``qualname`` (``func`` or ``Class.method`` or
    ``func.inner``) from ``src_file`` in ``ns`` and return the object."""
    tree = ast.parse(src_file.read_text())
    text = src_file.read_text()
    parts = qualname.split(".")
    node = None
    body = tree.body
    for p in parts:
        node = next(n for n in body if isinstance(n, (ast.FunctionDef, ast.ClassDef)) and n.name == p)
        body = node.body
    import textwrap
    # the segment's first line starts at the node's column; restore it, then
    # de-indent methods and nested functions to module level
    seg = textwrap.dedent(" " * node.col_offset + ast.get_source_segment(text, node))
    exec(compile(seg, f"{src_file}:{node.lineno}", "exec"), ns)
    return ns[parts[-1]]


class _Blocks:
    """Minimal stand-in for a dask array's ``.blocks`` iteration."""

    def __init__(self, arr, chunk):
        self.arr, self.chunk = arr, chunk

    def __iter__(self):
        for s in range(0, self.arr.shape[0], self.chunk):
            yield _Computable(self.arr[s:s + self.chunk])


class _Computable:
    def __init__(self, a):
        self.a = a

    def compute(self):
        return self.a.copy()


class _FakeDask:
    def __init__(self, arr, chunk):
        self.arr = arr
        self.shape = arr.shape
        self.chunksize = (chunk, arr.shape[1])
        self.numblocks = ((arr.shape[0] + chunk - 1) // chunk, 1)
        self.blocks = _Blocks(arr, chunk)


class _ExactIndex:
    """hnswlib-like index answering exactly (float32 distances, uint64 labels)."""

    def __init__(self, data):
        self.data = np.asarray(data, dtype=np.float32)

    def knn_query(self, a, k):
        i, d = oracle.exact_knn(np.asarray(a, dtype=np.float32), self.data, k)
        return i.astype(np.uint64), d.astype(np.float32)


def zarr_chunks(ds: Path):
    """``zarr_chunks.npz``: Blosc-LZ4 chunks of the reference's own test store
    (``1K_pbmc_citeseq.zarr.tar.gz``, written by scarf's create_zarr_dataset,
    scarf/writers.py:58-89): the first and last RNA count chunks (bit shuffle,
    split streams, a ragged last block), the one ADT count chunk and the cell
    ids (byte shuffle). The oracle's decoder is pinned here on the whole RNA
    matrix: its per-cell totals and non-zero counts must equal the reference's
    ``RNA_nCounts`` / ``RNA_nFeatures`` in ``cell_attributes.csv`` for every
    listed cell (and ``assay2_*`` for the ADT chunk)."""
    import csv
    import hashlib
    import json
    import tarfile
    import tempfile
    from oracle import blosc
    with tempfile.TemporaryDirectory() as tmp:
        with tarfile.open(ds / "1K_pbmc_citeseq.zarr.tar.gz") as tf:
            tf.extractall(tmp, filter="data")
        root = Path(tmp)
        rna_meta = json.loads((root / "RNA" / "counts" / ".zarray").read_text())
        adt_meta = json.loads((root / "assay2" / "counts" / ".zarray").read_text())
        ids_meta = json.loads((root / "cellData" / "ids" / ".zarray").read_text())
        n_cells, n_genes = rna_meta["shape"]
        cr, cc = rna_meta["chunks"]
        nchunk = -(-n_genes // cc)
        frames = {f"rna_0_{c}": (root / "RNA" / "counts" / f"0.{c}").read_bytes() for c in (0, nchunk - 1)}
        frames["adt_0_0"] = (root / "assay2" / "counts" / "0.0").read_bytes()
        frames["cell_ids_0"] = (root / "cellData" / "ids" / "0").read_bytes()
        ids = np.frombuffer(blosc.decompress(frames["cell_ids_0"]), dtype=ids_meta["dtype"])[:n_cells]
        tot = np.zeros(n_cells, np.int64)
        nz = np.zeros(n_cells, np.int64)
        for c in range(nchunk):
            b = blosc.decode_chunk((root / "RNA" / "counts" / f"0.{c}").read_bytes(), (cr, cc), "<u4")[:n_cells]
            w = min(cc, n_genes - c * cc)
            tot += b[:, :w].sum(1, dtype=np.int64)
            nz += (b[:, :w] > 0).sum(1)
        adt = blosc.decode_chunk(frames["adt_0_0"], tuple(adt_meta["chunks"]), "<u4")[:n_cells, :adt_meta["shape"][1]]
    rows = list(csv.DictReader(open(ds / "cell_attributes.csv")))
    pos = {v: i for i, v in enumerate(ids)}
    sel = np.array([pos[r["ids"]] for r in rows])
    col = lambda k: np.array([float(r[k]) for r in rows])  # noqa: E731
    assert np.array_equal(tot[sel], col("RNA_nCounts")) and np.array_equal(nz[sel], col("RNA_nFeatures"))
    assert np.array_equal(adt.sum(1)[sel], col("assay2_nCounts"))
    assert np.array_equal((adt > 0).sum(1)[sel], col("assay2_nFeatures"))
    out = {k: np.frombuffer(v, dtype=np.uint8) for k, v in frames.items()}
    out.update({f"sha256_{k}": np.array(hashlib.sha256(blosc.decompress(v)).hexdigest()) for k, v in frames.items()})
    out.update(rna_zarray=np.array(json.dumps(rna_meta)), adt_zarray=np.array(json.dumps(adt_meta)),
               ids_zarray=np.array(json.dumps(ids_meta)), csv_ids=np.array([r["ids"] for r in rows]),
               csv_rna_ncounts=col("RNA_nCounts"), csv_rna_nfeatures=col("RNA_nFeatures"),
               csv_adt_ncounts=col("assay2_nCounts"), csv_adt_nfeatures=col("assay2_nFeatures"),
               rna_totals_all_chunks=tot, rna_nnz_all_chunks=nz, rna_last_chunk=np.int64(nchunk - 1))
    np.savez_compressed(HERE / "zarr_chunks.npz", **out)


def main(ref_root: str):
    ref = Path(ref_root) / "scarf"
    ds = ref / "tests" / "datasets"
    zarr_chunks(ds)
    np.savez_compressed(
        HERE / "pbmc1k_knn.npz",
        indices=np.load(ds / "knn_indices.npy"),
        distances=np.load(ds / "knn_distances.npy"),
        weights=np.load(ds / "knn_weights.npy"),
    )

    rng = np.random.default_rng(20240611)
    out = {}

    # --- clean_array (utils.py:143) -----------------------------------------
    ns = {"np": np}
    clean_array = lift(ref / "utils.py", "clean_array", ns)
    ca_in = rng.normal(size=64)
    ca_in[[1, 5, 9]] = [np.nan, np.inf, -np.inf]
    ca_in[[2, 3]] = 0.0
    out["clean_in"] = ca_in
    out["clean_out0"] = clean_array(ca_in.copy())
    out["clean_out1"] = clean_array(ca_in.copy(), 1)

    # --- norm_lib_size_log (assay.py:54) on a dense count block ------------
    ns = {"np": np, "daskArrayType": np.ndarray}
    nll = lift(ref / "assay.py", "norm_lib_size_log", ns)
    counts = rng.negative_binomial(2, 0.7, size=(40, 30)).astype(np.uint32)
    counts[3] = 0
    scalar = counts.sum(axis=1)
    scalar[scalar == 0] = 1
    fake_assay = types.SimpleNamespace(sf=1000, scalar=scalar)
    out["norm_counts"] = counts
    out["norm_log"] = nll(fake_assay, counts)

    # --- fix_knn_query (ann.py:31) ------------------------------------------
    ns = {"np": np}
    fix = lift(ref / "ann.py", "fix_knn_query", ns)
    n, kq = 50, 8
    ind = np.stack([rng.permutation(200)[:kq] for _ in range(n)]).astype(np.uint64)
    ref_idx = np.arange(100, 100 + n)
    ind[:20, 0] = ref_idx[:20]                    # self first
    ind[20:30, 3] = ref_idx[20:30]                # self in the middle
    dist = np.sort(rng.random((n, kq)), axis=1)
    fi, fd, nm = fix(ind, dist, ref_idx)
    out.update(fix_ind=ind, fix_dist=dist, fix_ref=ref_idx, fix_out_i=fi, fix_out_d=fd,
               fix_nmis=np.int64(nm))

    # --- symmetrize (graph_datastore.py:1052) and fuzzy_simplicial_set (umap.py:118)
    ns = {"np": np}
    sym = lift(ref / "datastore" / "graph_datastore.py", "GraphDataStore.load_graph.symmetrize", ns)
    fss = lift(ref / "umap.py", "fuzzy_simplicial_set", ns)
    ng, kg = 300, 7
    gi = np.stack([rng.choice(ng, kg, replace=False) for _ in range(ng)])
    gw = rng.random(ng * kg).astype(np.float32).astype(np.float64)
    rows = np.repeat(np.arange(ng), kg)
    g = sp.csr_matrix((gw, (rows, gi.ravel())), shape=(ng, ng))
    s = sym(g).tocsr()
    s.sort_indices()
    u = fss(g, 1.0).tocsr()
    u.sort_indices()
    u2 = fss(g, 0.7).tocsr()
    u2.sort_indices()
    out.update(union_rows=rows, union_cols=gi.ravel(), union_w=gw, union_n=np.int64(ng),
               sym_indptr=s.indptr, sym_indices=s.indices, sym_data=s.data,
               fss_indptr=u.indptr, fss_indices=u.indices, fss_data=u.data,
               fss07_indptr=u2.indptr, fss07_indices=u2.indices, fss07_data=u2.data)

    # --- smoothen_dists (knn_utils.py:89) with a 3-chunk split --------------
    store = {}

    def create_zarr_dataset(g_, name, chunks, dtype, shape, overwrite=True):
        if isinstance(dtype, tuple):
            dtype = dtype[0]
        store[name] = np.zeros(shape, dtype=dtype)
        return store[name]

    umap_mod = types.ModuleType("umap")
    umap_sub = types.ModuleType("umap.umap_")
    umap_sub.smooth_knn_dist = oracle.smooth_knn_dist

    def _cms(ki, kv, sig, rho):
        r, c, v = oracle.compute_membership_strengths(ki, kv, sig, rho)
        return r, c, v, None

    umap_sub.compute_membership_strengths = _cms
    umap_mod.umap_ = umap_sub
    umap_mod.__version__ = "0.5.7"
    sys.modules["umap"] = umap_mod
    sys.modules["umap.umap_"] = umap_sub
    ns = {"np": np, "create_zarr_dataset": create_zarr_dataset, "tqdmbar": lambda x, **kw: x,
          "_is_umap_version_new": lambda: True}
    smd = lift(ref / "knn_utils.py", "smoothen_dists", ns)
    ns_, ks_ = 260, 9
    sq = rng.normal(size=(ns_, 6)).astype(np.float32)
    sq[17] = sq[16]                               # a duplicate cell -> zero distance
    si, sd = oracle.exact_knn(sq, sq, ks_ + 1)
    si2, sd2, _ = oracle.fix_knn_query(si, sd.astype(np.float32), np.arange(ns_))
    smd(None, si2.astype(np.uint64), sd2.astype(np.float64), 1.0, 1.5, 100)
    out.update(smooth_idx=si2.astype(np.uint64), smooth_dist=sd2.astype(np.float64),
               smooth_chunk=np.int64(100), smooth_edges=store["edges"], smooth_w=store["weights"])

    # --- self_query_knn (knn_utils.py:23) + AnnStream.transform_ann (ann.py:194)
    store.clear()
    ns = {"np": np, "create_zarr_dataset": create_zarr_dataset, "tqdmbar": lambda x, **kw: x,
          "controlled_compute": lambda a, n: a.compute(), "fix_knn_query": fix}
    sqk = lift(ref / "knn_utils.py", "self_query_knn", ns)
    tra = lift(ref / "ann.py", "AnnStream.transform_ann", ns)
    pts = rng.normal(size=(230, 5)).astype(np.float32)
    pts[40] = pts[41]
    pts[120] = pts[121] = pts[122]
    ann = types.SimpleNamespace(data=_FakeDask(pts, 64), harmonizedData=None,
                                reducer=lambda x: x, nCells=pts.shape[0], k=6,
                                annIdx=_ExactIndex(pts))
    ann.transform_ann = lambda a, k=None, self_indices=None: tra(ann, a, k, self_indices)
    rec = sqk(ann, None, 64, 1)
    out.update(sqk_points=pts, sqk_k=np.int64(6), sqk_chunk=np.int64(64),
               sqk_indices=store["indices"], sqk_distances=store["distances"], sqk_recall=rec)

    # --- AnnStream._fit_pca (ann.py:207) with scikit-learn IncrementalPCA ----
    import logging
    ns = {"np": np, "logger": logging.getLogger("golden")}
    fitp = lift(ref / "ann.py", "AnnStream._fit_pca", ns)
    zp = rng.normal(size=(700, 40)) @ rng.normal(size=(40, 40))
    zp[:, :5] *= 4.0
    mu_p, sd_p = zp.mean(0), zp.std(0)
    use = np.ones(700, dtype=bool)
    use[rng.choice(700, 50, replace=False)] = False
    blocks = _FakeDask(zp, 150)
    fake = types.SimpleNamespace(dims=6, batchSize=150, nCells=700, mu=mu_p, sigma=sd_p)
    fake.transform_z = lambda a: (a - fake.mu) / fake.sigma
    fake.iter_blocks = lambda msg="": (b.compute() for b in blocks.blocks)
    fitp(fake, False, use)
    out.update(pca_x=zp, pca_mu=mu_p, pca_sigma=sd_p, pca_use=use, pca_dims=np.int64(6),
               pca_batch=np.int64(150), pca_loadings=fake.loadings,
               pca_evr=fake._pca.explained_variance_ratio_)

    # --- calc_snn, weight_sort_indices, merge_graphs (knn_utils.py:195-274) --
    ns = {"np": np, "jit": lambda **kw: (lambda f: f), "tqdmbar": lambda x, **kw: x,
          "csr_matrix": sp.csr_matrix, "coo_matrix": sp.coo_matrix, "List": list, "Tuple": tuple}
    snn_f = lift(ref / "knn_utils.py", "calc_snn", ns)
    lift(ref / "knn_utils.py", "weight_sort_indices", ns)
    merge_f = lift(ref / "knn_utils.py", "merge_graphs", ns)
    nm, km = 240, 7
    mats = []
    for gidx in range(2):
        mi = np.stack([rng.choice(nm, km, replace=False) for _ in range(nm)])
        if gidx == 1:
            mi[:, :3] = mats[0].indices.reshape(nm, km)[:, :3]   # neighbours shared by both graphs
        mw = rng.random(nm * km).astype(np.float32).astype(np.float64)
        mats.append(sp.csr_matrix((mw, mi.ravel(), np.arange(0, nm * km + 1, km)), shape=(nm, nm)))
        out[f"merge_g{gidx}_indices"] = mi
        out[f"merge_g{gidx}_data"] = mw
        out[f"merge_g{gidx}_snn"] = snn_f(mi)
    mg = merge_f(mats)
    out.update(merge_n=np.int64(nm), merge_k=np.int64(km), merge_row=mg.row, merge_col=mg.col, merge_data=mg.data)

    # --- rescale_array (utils.py:120-140), used by _get_ini_embed ----------
    ns = {"np": np}
    rescale = lift(ref / "utils.py", "rescale_array", ns)
    ra = rng.standard_t(3, size=500) * 2.0 + 1.0
    out["rescale_in"] = ra.copy()
    out["rescale_out"] = rescale(ra.copy())

    np.savez_compressed(HERE / "ref_functions.npz", **out)
    print("wrote", sorted(out))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the scarf source tree>")
    main(sys.argv[1])
