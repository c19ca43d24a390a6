"""sg_smooth_noalloc: smoothing for callers that cannot let the library
allocate device memory (they own the HBM budget through their own pool, or
cannot take cudaMalloc's device-wide synchronisation). The entry point keeps
its scratch in a fixed static device array; this file checks it against the
allocating sg_smooth on two calls in a row through the C ABI. It is collected
last so that a failure here comes after every other test has run.
"""
import ctypes as C
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _noalloc(lib, idx, dist, lc, bw, chunk):
    n, k = idx.shape
    edges = torch.empty((n * k, 2), dtype=torch.int64, device="cuda")
    w = torch.empty(n * k, dtype=torch.float64, device="cuda")
    rc = lib.sg_smooth_noalloc(_ptr(idx), _ptr(dist), n, k, lc, bw, chunk, _ptr(edges), _ptr(w),
                               C.c_void_p(torch.cuda.current_stream().cuda_stream))
    return rc, edges, w


def _random_knn(n, k, seed):
    rng = np.random.default_rng(seed)
    idx = rng.integers(0, n, size=(n, k)).astype(np.int64)
    idx[::7, 3] = np.arange(0, n, 7) % 333          # neighbour == chunk-local row: weight 0, then global_min
    d = np.sort(rng.gamma(2.0, 1.0, size=(n, k)), axis=1).astype(np.float32)
    d[::11, 0] = 0.0                                  # zero distances (duplicate cells)
    return idx, d


def test_noalloc_matches_allocating_entry_point(golden_dir):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from scarf_gb300 import _lib, kernels as K
    lib = _lib.load()
    kat = np.load(os.path.join(golden_dir, "pbmc1k_knn.npz"))
    cases = [(kat["indices"].astype(np.int64), kat["distances"].astype(np.float32), 1000),
             (*_random_knn(20000, 15, 5), 333)]
    for idx_np, dist_np, chunk in cases:     # two calls in a row share the static array
        idx = torch.from_numpy(idx_np).cuda()
        dist = torch.from_numpy(dist_np).cuda()
        rc, e_na, w_na = _noalloc(lib, idx, dist, 1.0, 1.5, chunk)
        assert rc == 0, lib.sg_last_error().decode()
        e_ref, w_ref = K.smooth(idx, dist, 1.0, 1.5, chunk)
        torch.cuda.synchronize()
        # the same kernels on the same inputs: bit for bit the same outputs
        assert torch.equal(e_na, e_ref)
        assert torch.equal(w_na, w_ref)
    # the known answer of the reference holds through this entry point too
    idx = torch.from_numpy(kat["indices"].astype(np.int64)).cuda()
    dist = torch.from_numpy(kat["distances"].astype(np.float32)).cuda()
    rc, _, w = _noalloc(lib, idx, dist, 1.0, 1.5, 1000)
    torch.cuda.synchronize()
    assert rc == 0 and np.abs(w.cpu().numpy() - kat["weights"]).max() < 1e-5


def test_noalloc_rejects_sizes_beyond_its_limit():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from scarf_gb300 import _lib
    lib = _lib.load()
    n, k = (1 << 14) + 1, 4                          # one chunk more than the 2^14 the array holds
    idx = torch.zeros((n, k), dtype=torch.int64, device="cuda")
    dist = torch.ones((n, k), dtype=torch.float32, device="cuda")
    rc, _, _ = _noalloc(lib, idx, dist, 1.0, 1.5, 1)
    assert rc == _lib.SG_ERR_ARG
    assert "fixed scratch limit" in lib.sg_last_error().decode()
    # a row count whose edge count would overflow is refused before any work
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.sg_smooth_noalloc(_ptr(idx), _ptr(dist), 1 << 62, 16, 1.0, 1.5, 1 << 50, _ptr(idx), _ptr(dist), st)
    assert rc == _lib.SG_ERR_ARG
