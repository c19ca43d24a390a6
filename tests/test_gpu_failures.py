"""Failure handling on the GPU without a GPU fault.

A tensor-core kernel whose mbarrier waits run out must report SG_ERR_TIMEOUT
through the C ABI, leave no work in flight and the context usable, so that
the next call on the same handle gives the right answer. The test shortens
the poll limit of the waits (sg_set_wait_limit) and keeps the MMA issuer of
one precision kNN launch idle (sg_test_idle_mma): its copy and epilogue
warps then wait on barriers that nothing arrives at, which is the flag that
nothing sets.
"""
import time

import numpy as np
import pytest

from helpers import clustered_points

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_expired_wait_returns_timeout_and_the_next_call_succeeds():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from scarf_gb300 import _lib as L
    from scarf_gb300 import kernels as K
    lib = L.load()
    d, k = 30, 10
    pts = clustered_points(3000, d, seed=4)
    x = torch.zeros((3000, 32), dtype=torch.float32)
    x[:, :d] = torch.from_numpy(pts)
    x = x.cuda()
    want_i, want_d, want_m = K.knn(x, x, d, k, self_offset=0, margin=16, precision="precision")
    torch.cuda.synchronize()
    h = K.handle(0)
    L.check(lib.sg_set_wait_limit(h.ptr, 1 << 12))
    L.check(lib.sg_test_idle_mma(h.ptr))
    t0 = time.perf_counter()
    with pytest.raises(L.GpuError) as ei:
        K.knn(x, x, d, k, self_offset=0, margin=16, precision="precision")
    waited = time.perf_counter() - t0
    assert ei.value.status == L.SG_ERR_TIMEOUT
    assert "expired" in str(ei.value)
    assert waited < 30.0
    # the context is usable and the handle answers correctly again
    L.check(lib.sg_set_wait_limit(h.ptr, 0))
    got_i, got_d, got_m = K.knn(x, x, d, k, self_offset=0, margin=16, precision="precision")
    torch.cuda.synchronize()
    assert torch.equal(got_i, want_i) and torch.equal(got_d, want_d)
    assert int(got_m.item()) == int(want_m.item())
    # and other kernels run on the same stream afterwards
    e, w = K.smooth(got_i, got_d, 1.0, 1.5, 1000)
    torch.cuda.synchronize()
    assert bool(torch.isfinite(w).all())
    assert np.all(e[:, 0].cpu().numpy() == np.repeat(np.arange(3000), k))
