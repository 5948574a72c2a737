"""GB300-native random-walk engine with PTWalker's app surface.

The walker-update path (neighbour pick, geometric / fixed-length
termination, visit counting, endpoint and path recording) runs as
hand-written sm_103a CUDA kernels in libptw.so behind the C ABI in
include/ptw.h; this package is the Python host mirror of that ABI.
"""
from ._capi import PTWError, load as load_library, lib_path  # noqa: F401
from .api import (  # noqa: F401
    Graph,
    Tune,
    WalkStats,
    pagerank,
    ppr,
    rwr,
    deepwalk,
    node2vec,
    PageRankApp,
    PPRApp,
    RWRApp,
    DeepWalkApp,
    Solver,
    walk,
    probe_gather,
    trim_memory,
    pagerank_submit,
    pagerank_wait,
)

from .batch import (BatchResult, BatchTune, autotune_batch, get_batch_tune, ppr_batch,  # noqa: F401,E402
                    ppr_batch_resumable, set_batch_tune)
from .serving import Server, open_loop  # noqa: F401,E402

__version__ = "0.1.0"
