"""Host-side argument checks of the scarf-facing functions (no GPU needed)."""
import numpy as np
import pytest
import scipy.sparse as sp


def _graph(n, k, seed):
    rng = np.random.default_rng(seed)
    idx = np.stack([rng.choice(n, k, replace=False) for _ in range(n)])
    return sp.csr_matrix((rng.random(n * k), idx.ravel(), np.arange(0, n * k + 1, k)), shape=(n, n))


def test_merge_graphs_rejects_mismatched_graphs():
    """merge_graphs refuses graphs of different shapes or edge counts, with
    the reference's messages (scarf/knn_utils.py:249-256), before any device
    work."""
    from scarf_gb300 import knn_utils
    with pytest.raises(ValueError, match="same shape"):
        knn_utils.merge_graphs([_graph(20, 3, 0), _graph(21, 3, 1)])
    with pytest.raises(ValueError, match="same number of edges"):
        knn_utils.merge_graphs([_graph(20, 3, 0), _graph(20, 4, 1)])


def test_kmeans_hash_streams_are_distinct():
    """The k-means draws: different streams and indices give different words."""
    import oracle
    a = oracle.kmeans_hash(4466, 1, np.arange(1000))
    b = oracle.kmeans_hash(4466, 2, np.arange(1000))
    assert len(np.unique(a)) == 1000 and len(np.unique(np.concatenate([a, b]))) == 2000
