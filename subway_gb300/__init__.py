"""GB300-native out-of-HBM graph engine with Subway's application interface.

The compute path is libsubwaygb.so (hand-written sm_103a CUDA kernels behind
the C ABI of include/subway_gb300.h); `subway_gb300.native` binds it.
"""
from . import native  # noqa: F401
from .native import ALGOS, ASYNC, BFS, CC, INF, MODES, PR, SSSP, SSWP, SYNC, Engine, Graph  # noqa: F401
