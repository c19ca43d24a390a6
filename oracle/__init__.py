"""CPU oracle for scarf's graph-construction path -- TEST INFRASTRUCTURE ONLY.

This package restates, in numpy/scipy, what the reference computes on the path
normalise -> z-stats -> PCA -> self-kNN -> smoothing -> fuzzy union, and the
mapping query of ``run_mapping``. Every function cites the reference file:line
it follows (paths are relative to the scarf project root).

Who may use it: ``tests/`` (as the checker), ``__graft_entry__.smoke()`` (as the
checker) and ``bench.py`` (its ``cpu_baseline`` leg and ``--impl reference``
arm, as the timed CPU restatement). The product package ``scarf_gb300`` never
imports it; the product path fails loudly when its CUDA library is missing.

Pinning: ``tests/golden`` holds the reference's own kNN/graph fixtures and
vectors produced by executing the reference's own numpy/scipy functions
(``tests/golden/make_golden.py``); ``tests/test_oracle_golden.py`` checks this
package against them.
"""

from .restate import *  # noqa: F401,F403
from .restate import __all__  # noqa: F401
