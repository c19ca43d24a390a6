"""Host logic of the continuous-batching scheduler (no GPU)."""
import threading
import time

import numpy as np
import pytest

from scarf_gb300.serving import BatchScheduler, MapRequest


def req(rid, n, nnz_per_row=3, k=5):
    ip = np.arange(0, (n + 1) * nnz_per_row, nnz_per_row, dtype=np.int64)
    return MapRequest(rid, ip, np.zeros(n * nnz_per_row, np.int32), np.ones(n * nnz_per_row, np.int32), k,
                      time.perf_counter())


def finish(s, batch):
    n = sum(b - a for _, a, b in batch)
    rows = np.concatenate([np.arange(a, b) for _, a, b in batch]) if batch else np.zeros(0)
    idx = np.repeat(rows[:, None], 5, 1).astype(np.int64)
    s.complete(batch, idx, np.zeros((n, 5), np.float32))


def test_budget_admission_is_fifo_and_releases_on_completion():
    s = BatchScheduler(hbm_budget_bytes=2 * (100 * 10 + 300 * 8), max_batch_rows=1000, bytes_per_row=10)
    r = [s.submit(req(i, 100)) for i in range(3)]
    assert [x.rid for x in s.active] == [0, 1] and [x.rid for x in s.queued] == [2]
    b = s.next_batch(timeout=0)
    assert [(x.rid, a, e) for x, a, e in b] == [(0, 0, 100), (1, 0, 100)]
    finish(s, b)
    assert r[0].done.is_set() and r[1].done.is_set() and [x.rid for x in s.active] == [2]
    assert s.in_use == r[2].bytes_needed


def test_large_requests_are_sliced_and_later_requests_join():
    s = BatchScheduler(hbm_budget_bytes=1 << 40, max_batch_rows=16, bytes_per_row=1)
    big = s.submit(req(0, 40))
    b1 = s.next_batch(timeout=0)
    assert [(a, e) for _, a, e in b1] == [(0, 16)]
    small = s.submit(req(1, 4))          # arrives while the big request is on the GPU
    b2 = s.next_batch(timeout=0)         # shortest remaining first: the small one leads
    assert [(x.rid, a, e) for x, a, e in b2] == [(1, 0, 4), (0, 16, 28)]
    b3 = s.next_batch(timeout=0)
    assert [(x.rid, a, e) for x, a, e in b3] == [(0, 28, 40)]
    for b in (b1, b2, b3):
        finish(s, b)
    assert big.done.is_set() and small.done.is_set()
    assert np.array_equal(big.idx[:, 0], np.arange(40)) and np.array_equal(small.idx[:, 0], np.arange(4))


def test_request_larger_than_budget_is_rejected():
    s = BatchScheduler(hbm_budget_bytes=100, max_batch_rows=16, bytes_per_row=10)
    r = s.submit(req(0, 50))
    with pytest.raises(MemoryError):
        r.result(timeout=1)


def test_empty_request_completes_at_once():
    s = BatchScheduler(hbm_budget_bytes=1000, max_batch_rows=16, bytes_per_row=1)
    r = s.submit(req(0, 0))
    i, d = r.result(timeout=1)
    assert i.shape == (0, 5)


def test_errors_reach_the_caller():
    s = BatchScheduler(hbm_budget_bytes=1 << 20, max_batch_rows=16, bytes_per_row=1)
    r = s.submit(req(0, 8))
    b = s.next_batch(timeout=0)
    s.complete(b, None, None, error=RuntimeError("kernel failed"))
    with pytest.raises(RuntimeError):
        r.result(timeout=1)
    assert s.in_use == 0


def test_next_batch_waits_for_work_and_close_wakes_it():
    s = BatchScheduler(hbm_budget_bytes=1 << 20, max_batch_rows=16, bytes_per_row=1)
    got = []
    t = threading.Thread(target=lambda: got.append(s.next_batch()))
    t.start()
    time.sleep(0.05)
    s.submit(req(0, 3))
    t.join(timeout=2)
    assert got and got[0][0][2] == 3
    s.close()
    assert s.next_batch(timeout=0.1) == []


def test_requests_wait_for_their_upload():
    uploads = []
    s = BatchScheduler(hbm_budget_bytes=1 << 20, max_batch_rows=16, bytes_per_row=1, uploader=uploads.append)
    a = s.submit(req(0, 5))
    b = s.submit(req(1, 3))
    assert [r.rid for r in uploads] == [0, 1]
    assert s.next_batch(timeout=0) == []          # nothing resident yet
    s.mark_ready(b)
    assert [(x.rid, lo, hi) for x, lo, hi in s.next_batch(timeout=0)] == [(1, 0, 3)]
    s.mark_ready(a, error=IOError("copy failed"))
    with pytest.raises(IOError):
        a.result(timeout=1)
    assert s.in_use == b.bytes_needed


def test_failed_upload_admits_the_next_request():
    uploads = []
    cost = 10 * 1 + 30 * 8
    s = BatchScheduler(hbm_budget_bytes=cost, max_batch_rows=16, bytes_per_row=1, uploader=uploads.append)
    a = s.submit(req(0, 10))
    b = s.submit(req(1, 10))
    assert [r.rid for r in uploads] == [0] and [r.rid for r in s.queued] == [1]
    s.mark_ready(a, error=RuntimeError("no memory"))
    assert [r.rid for r in uploads] == [0, 1] and [r.rid for r in s.active] == [1]
