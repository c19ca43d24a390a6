"""The mapping service through the C ABI (sg_serve_*), called with ctypes as a
non-Python host would: the same answers as the Python MappingServer for the
same reference and requests (run_mapping's query,
scarf/datastore/mapping_datastore.py:198-208), requests of every size
including empty ones served in row slices across batches, and a request
larger than the HBM budget refused with SG_ERR_BUDGET."""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp

from helpers import small_counts, top_var_genes

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from scarf_gb300.datastore import DataStore
    indptr, indices, data, G, _ = small_counts(n_cells=1800, n_genes=3000, seed=11)
    feat = top_var_genes(indptr, indices, data, G, 300)
    ids = np.array([f"g{i}" for i in range(G)])
    d = DataStore(indptr, indices, data, G, gene_ids=ids, precision="precision")
    mask = np.zeros(G, dtype=bool)
    mask[feat] = True
    d.RNA.feats.insert("I__hvgs", mask)
    d.make_graph(feat_key="hvgs", dims=15, k=11, batch_size=500)
    ann = d._ann_cache[d.zw["RNA/normed__I__hvgs/reduction__pca__15__I"].attrs["latest_ann"]]
    return d, ann, ids, feat, (indptr, indices, data, G)


def _requests(counts, ids, sizes, seed):
    """Requests drawn from the reference cells with the genes in another order
    and 10 of the features absent."""
    indptr, indices, data, G = counts
    rng = np.random.default_rng(seed)
    m = sp.csr_matrix((data, indices, indptr), shape=(len(indptr) - 1, G))
    keep = np.setdiff1d(np.arange(G), rng.choice(G, 10, replace=False))
    order = rng.permutation(keep)
    out = []
    for n in sizes:
        rows = rng.choice(m.shape[0], n, replace=False)
        s = m[rows][:, order].tocsr()
        s.sort_indices()
        out.append((s.indptr.astype(np.int64), s.indices.astype(np.int32), s.data.astype(np.int32)))
    return out, ids[order]


class NativeServer:
    def __init__(self, lib, ann, ref_ids, target_ids, k, max_rows, budget, workers):
        from scarf_gb300.datastore import align_col_map
        self.lib = lib
        self.k = k
        cmap, missing = align_col_map(np.asarray(ref_ids), np.asarray(target_ids))
        self._keep = (np.ascontiguousarray(cmap, np.int32), np.ascontiguousarray(missing, np.uint8))
        sc = ann.annIdx.scores
        self.h = C.c_void_p()
        rc = lib.sg_serve_create(0, C.c_void_p(ann._mu32.data_ptr()), C.c_void_p(ann._sg32.data_ptr()),
                                 C.c_void_p(ann._l32.data_ptr()), ann.nFeats, ann.dims, ann._l32.stride(0),
                                 C.c_void_p(sc.data_ptr()), sc.shape[0], sc.stride(0),
                                 self._keep[0].ctypes.data_as(C.c_void_p), len(cmap),
                                 self._keep[1].ctypes.data_as(C.c_void_p), k, 1, 1000.0, 3, max_rows, budget,
                                 workers, C.byref(self.h))
        assert rc == 0, lib.sg_last_error().decode()
        self.held = {}

    def submit(self, ip, ind, dat):
        rid = C.c_int64()
        rc = self.lib.sg_serve_submit(self.h, ip.ctypes.data_as(C.c_void_p), ind.ctypes.data_as(C.c_void_p),
                                      dat.ctypes.data_as(C.c_void_p), len(ip) - 1, C.byref(rid))
        assert rc == 0, self.lib.sg_last_error().decode()
        self.held[rid.value] = (ip, ind, dat)   # the arrays stay alive until the request is done
        return rid.value

    def result(self, rid, n):
        rc = self.lib.sg_serve_wait(self.h, rid, 60_000)
        assert rc == 0, self.lib.sg_last_error().decode()
        done = C.c_int32()
        assert self.lib.sg_serve_poll(self.h, rid, C.byref(done)) == 0 and done.value == 1
        idx = np.empty((n, self.k), np.int64)
        dist = np.empty((n, self.k), np.float32)
        rc = self.lib.sg_serve_result(self.h, rid, idx.ctypes.data_as(C.c_void_p), dist.ctypes.data_as(C.c_void_p))
        self.held.pop(rid)
        return rc, idx, dist

    def close(self):
        self.lib.sg_serve_destroy(self.h)


def test_native_server_equals_python_server(ref):
    from scarf_gb300 import _lib
    from scarf_gb300.serving import MappingServer
    d, ann, ids, feat, counts = ref
    lib = _lib.load()
    ref_ids = d.RNA.feats.fetch("ids", key="I__hvgs")
    reqs, t_ids = _requests(counts, ids, [5, 300, 1, 1200, 0, 77, 640], seed=2)
    with MappingServer(ann, ref_ids, t_ids, k=5, max_batch_rows=256, n_workers=1) as srv:
        want = [srv.submit(*r).result(timeout=60) for r in reqs]
    nat = NativeServer(lib, ann, ref_ids, t_ids, k=5, max_rows=256, budget=1 << 30, workers=2)
    try:
        rids = [nat.submit(*r) for r in reqs]          # all in flight at once: batches mix requests
        for rid, r, (wi, wd) in zip(rids, reqs, want):
            rc, gi, gd = nat.result(rid, len(r[0]) - 1)
            assert rc == 0
            assert np.array_equal(gi, wi)
            assert np.array_equal(gd, wd)
        batches, rows = C.c_int64(), C.c_int64()
        assert lib.sg_serve_stats(nat.h, C.byref(batches), C.byref(rows)) == 0
        assert rows.value == sum(len(r[0]) - 1 for r in reqs)
        assert batches.value >= rows.value // 256           # the 1,200-cell request went in slices
    finally:
        nat.close()


def test_native_server_refuses_over_budget(ref):
    from scarf_gb300 import _lib
    d, ann, ids, feat, counts = ref
    lib = _lib.load()
    ref_ids = d.RNA.feats.fetch("ids", key="I__hvgs")
    reqs, t_ids = _requests(counts, ids, [400, 3], seed=4)
    nat = NativeServer(lib, ann, ref_ids, t_ids, k=5, max_rows=128, budget=200_000, workers=1)
    try:
        big, small = nat.submit(*reqs[0]), nat.submit(*reqs[1])
        rc, _, _ = nat.result(big, 400)
        assert rc == _lib.SG_ERR_BUDGET
        assert b"budget" in lib.sg_last_error()
        rc, gi, gd = nat.result(small, 3)
        assert rc == 0 and np.all(gi >= 0) and np.all(np.isfinite(gd))
        # an unknown request is an argument error, not a hang
        assert lib.sg_serve_wait(nat.h, 12345, 10) == _lib.SG_ERR_ARG
    finally:
        nat.close()
