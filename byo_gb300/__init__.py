"""byo_gb300: GB300-native (sm_103a) implementation of BYO's data-parallel hot
path -- the GBBS edgeMap/vertexSubset traversal engine with BFS, connectivity,
PageRank and triangle counting, and the batched insert/delete of a packed
(CPMA-style) graph container -- behind a C ABI (include/byo_gpu.h).

The compute lives in byo_gb300/lib/libbyo_gpu.so (built from byo_gb300/csrc
by byo_gb300.build); this package is the Python view of that ABI.
"""
from . import _abi  # noqa: F401
from ._abi import ByoError  # noqa: F401
from .graph import (BFS, BFS_ComponentLabel_F, BFS_F, BFS_multi, Context, Graph, PR_Delta_F, PR_F,  # noqa: F401
                    PageRank, PageRank_edgeMap, PageRankDelta, SimpleUnionAsync, Test_Map, Test_Map_Remote,
                    Triangle_degree_ordering, UINT_E_MAX, bfs_cc, edgeMap, vertexFilter, vertexMap, vertexSubset)

__version__ = "0.1.0"
