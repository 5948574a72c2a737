"""CPU oracle for the walker-update path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package, and only as a checker.  The GPU engine in
``ptwalker_gb300`` never imports it.

Contents
  * ``oracle.c`` (built to ``oracle/_build/liboracle.so``): Philox4x32-10,
    raw R-MAT edges, walker replay for counts / endpoints / paths, and
    second-order (node2vec) paths.
  * ``partitioned.c``: the same count walks scheduled the reference's way
    (partition sweeps, per-partition walker pools); the timed CPU baseline.
  * ``graph.py``: canonical graph layout (names, CSR in index space) and the
    R-MAT clean-up pipeline, restating the reference loader's semantics.
  * ``power.py``: FP64 power iteration and the exact expected-visit formulas.
  * ``mlp.py``: FP64 forward / backward / Adam of the learned-budget MLP.

Parity pins: Philox is checked against the three published SC'11
known-answer vectors, and the GPU's draws equal this file's bit for bit
through every replay test; the walker semantics are checked statistically
against the reference binary built from its own sources (``oracle/ref``) and
against the FP64 expectation, and the node2vec replay against the transition
law of the reference's node2vec test.
"""
from .lib import load_lib, build_lib  # noqa: F401
from .graph import (  # noqa: F401
    CanonicalGraph,
    canonical_from_edges,
    rmat_raw_edges,
    rmat_clean_edges,
    rmat_clean_csr,
    rmat_thresholds,
    read_edge_file,
    write_text_edges,
    write_binary_edges,
)
from .replay import (  # noqa: F401
    philox4x32_10,
    replay_counts,
    replay_pairs,
    replay_paths,
    replay_node2vec,
    n2v_thresholds,
    n2v_fold,
    simple_symmetric,
    partitioned_counts,
    sp_threshold,
    TAG_WALK,
    TAG_START,
    TAG_RMAT,
)
from .power import (  # noqa: F401
    ppr_vector,
    expected_visits_from_source,
    expected_visits_per_vertex_start,
    expected_endpoint_from_source,
)
