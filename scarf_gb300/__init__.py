"""GB300-native (sm_103a) graph-construction path of scarf.

Hot path: CSR normalisation -> z-statistics -> PCA -> exact self-kNN ->
UMAP smoothing -> fuzzy union, as hand-written CUDA kernels behind the C ABI
of ``include/scarf_gb300.h``, with scarf's own Python surface
(``DataStore.make_graph``, ``AnnStream``, ``knn_utils``) on top.
"""
__version__ = "0.1.0"
