"""Python wrappers over the C walker replay (test infrastructure).

The semantics are documented at the top of ``oracle/oracle.c``.  All
results are in canonical index space (see ``oracle/graph.py``).
"""
import ctypes

import numpy as np

from .lib import load_lib

TAG_WALK = 0x57414C4B
TAG_START = 0x53545254
TAG_RMAT = 0x524D4154

START_PER_VERTEX, START_UNIFORM, START_SOURCES = 0, 1, 2


def sp_threshold(sp):
    """Stop after a move iff the 32-bit draw is below floor(sp * 2^32)."""
    return min(int(sp * 4294967296.0), 1 << 32)


def _p(arr, ctype):
    if arr is None:
        return None
    return arr.ctypes.data_as(ctypes.POINTER(ctype))


def philox4x32_10(ctr, key):
    lib = load_lib()
    c = np.asarray(ctr, dtype=np.uint32)
    k = np.asarray(key, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    lib.ora_philox4x32_10(_p(c, ctypes.c_uint32), _p(k, ctypes.c_uint32), _p(out, ctypes.c_uint32))
    return out


def _sources_arg(g, start_mode, sources):
    if start_mode != START_SOURCES:
        return None, 0
    idx = g.name_to_index(sources)
    return np.ascontiguousarray(idx, dtype=np.uint32), int(idx.shape[0])


def replay_counts(g, w_begin, w_end, sp, seed, start_mode=START_PER_VERTEX,
                  sources=None, max_moves=0, threads=1):
    """Visit counts over vertex indices and the total number of moves."""
    lib = load_lib()
    counts = np.zeros(g.n, dtype=np.uint32)
    src_arr, n_src = _sources_arg(g, start_mode, sources)
    total = lib.ora_replay_walks(
        _p(g.row_ptr, ctypes.c_uint64), _p(g.col, ctypes.c_uint32), g.n,
        w_begin, w_end, sp_threshold(sp), seed, start_mode,
        _p(src_arr, ctypes.c_uint32), n_src, max_moves,
        _p(counts, ctypes.c_uint32), None, None, threads)
    return counts, int(total)


def replay_pairs(g, w_begin, w_end, sp, seed, start_mode=START_PER_VERTEX,
                 sources=None, max_moves=0, threads=1):
    """(start, end) vertex indices per walker and the move count per walker."""
    lib = load_lib()
    nw = w_end - w_begin
    pairs = np.zeros((nw, 2), dtype=np.uint32)
    moves = np.zeros(nw, dtype=np.uint32)
    src_arr, n_src = _sources_arg(g, start_mode, sources)
    lib.ora_replay_walks(
        _p(g.row_ptr, ctypes.c_uint64), _p(g.col, ctypes.c_uint32), g.n,
        w_begin, w_end, sp_threshold(sp), seed, start_mode,
        _p(src_arr, ctypes.c_uint32), n_src, max_moves,
        None, _p(pairs, ctypes.c_uint32), _p(moves, ctypes.c_uint32), threads)
    return pairs, moves


def replay_paths(g, w_begin, w_end, L, seed, start_mode=START_PER_VERTEX,
                 sources=None, threads=1):
    """[walkers, L] int32 vertex indices (-1 after a dead end)."""
    lib = load_lib()
    nw = w_end - w_begin
    paths = np.zeros((nw, L), dtype=np.int32)
    src_arr, n_src = _sources_arg(g, start_mode, sources)
    lib.ora_replay_paths(
        _p(g.row_ptr, ctypes.c_uint64), _p(g.col, ctypes.c_uint32), g.n,
        w_begin, w_end, L, seed, start_mode, _p(src_arr, ctypes.c_uint32), n_src,
        _p(paths, ctypes.c_int32), threads)
    return paths


def replay_node2vec(g, w_begin, w_end, L, seed, p, q, start_mode=START_PER_VERTEX,
                    sources=None, threads=1, fold=None):
    """Second-order (node2vec) walks, ora_replay_node2vec: ([walkers, L] int32
    vertex indices, -1 after a dead end; number of candidate draws).  The
    outlier folding for a small p applies on simple symmetric graphs;
    ``fold=False`` turns it off (a test's comparison)."""
    lib = load_lib()
    nw = w_end - w_begin
    paths = np.zeros((nw, L), dtype=np.int32)
    src_arr, n_src = _sources_arg(g, start_mode, sources)
    trials = lib.ora_replay_node2vec(
        _p(g.row_ptr, ctypes.c_uint64), _p(g.col, ctypes.c_uint32), g.n,
        w_begin, w_end, L, seed, float(p), float(q), start_mode, _p(src_arr, ctypes.c_uint32), n_src,
        int(simple_symmetric(g) if fold is None else fold), _p(paths, ctypes.c_int32), threads)
    return paths, int(trials)


def simple_symmetric(g):
    """True iff no row of g repeats a neighbour and every edge has its
    reverse (ora_csr_simple_symmetric); cached on g."""
    cached = getattr(g, "_simple_symmetric", None)
    if cached is None:
        lib = load_lib()
        cached = bool(lib.ora_csr_simple_symmetric(_p(g.row_ptr, ctypes.c_uint64), _p(g.col, ctypes.c_uint32),
                                                   g.n))
        g._simple_symmetric = cached
    return cached


def n2v_fold(p, q):
    """(thresholds against M', a_fx) of the folded draw, or None when the
    return weight is not the only largest one (ora_n2v_fold)."""
    lib = load_lib()
    thr = np.zeros(4, dtype=np.uint64)
    if not lib.ora_n2v_fold(float(p), float(q), _p(thr, ctypes.c_uint64)):
        return None
    return [int(x) for x in thr[:3]], int(thr[3])


def n2v_thresholds(p, q):
    """Acceptance thresholds (return, neighbour of the previous vertex,
    other) of the node2vec rejection draw, ora_n2v_thresholds."""
    lib = load_lib()
    thr = np.zeros(3, dtype=np.uint64)
    lib.ora_n2v_thresholds(float(p), float(q), _p(thr, ctypes.c_uint64))
    return [int(x) for x in thr]


def degree_relabelled(g, threads=None):
    """The graph relabelled by descending degree (ties by index), rows
    keeping the canonical order of their neighbours: (perm, row_ptr, col)
    with perm[canonical index] = new id (ora_degree_relabel).  Cached on g:
    it is graph-load work, kept out of the timed region as the reference's
    own relabelling is."""
    cached = getattr(g, "_degree_relabelled", None)
    if cached is not None:
        return cached
    import os
    lib = load_lib()
    perm = np.empty(g.n, dtype=np.uint32)
    row_ptr = np.empty(g.n + 1, dtype=np.uint64)
    col = np.empty(g.m, dtype=np.uint32)
    rc = lib.ora_degree_relabel(_p(g.row_ptr, ctypes.c_uint64), _p(g.col, ctypes.c_uint32), g.n,
                                _p(perm, ctypes.c_uint32), _p(row_ptr, ctypes.c_uint64), _p(col, ctypes.c_uint32),
                                threads or os.cpu_count() or 1)
    if rc:
        raise MemoryError("degree relabelling: host memory ran out")
    g._degree_relabelled = (perm, row_ptr, col)
    return g._degree_relabelled


def partitioned_counts(g, w_begin, w_end, sp, seed, start_mode=START_PER_VERTEX, sources=None, max_moves=0,
                       threads=1, part_bytes=1 << 20):
    """The same visit counts as replay_counts, computed the way the reference
    schedules its walkers (degree-sorted relabelling, partition sweeps with
    per-(thread, partition) pools, partitioned.c): the timed CPU baseline.
    Returns (counts by canonical index, moves, info) with info =
    {partitions, sweeps, migrations}."""
    lib = load_lib()
    perm, row_ptr, col = degree_relabelled(g)
    counts = np.zeros(g.n, dtype=np.uint32)
    src_arr, n_src = _sources_arg(g, start_mode, sources)
    if src_arr is not None:
        src_arr = np.ascontiguousarray(perm[src_arr], dtype=np.uint32)
    info = np.zeros(3, dtype=np.uint64)
    total = lib.ora_partitioned_walks(
        _p(row_ptr, ctypes.c_uint64), _p(col, ctypes.c_uint32), g.n, _p(perm, ctypes.c_uint32), w_begin, w_end,
        sp_threshold(sp), seed, start_mode, _p(src_arr, ctypes.c_uint32), n_src, max_moves, int(part_bytes),
        _p(counts, ctypes.c_uint32), threads, _p(info, ctypes.c_uint64))
    if total == (1 << 64) - 1:
        raise MemoryError("partitioned walk: host memory ran out")
    return counts[perm], int(total), {"partitions": int(info[0]), "sweeps": int(info[1]),
                                      "migrations": int(info[2])}
