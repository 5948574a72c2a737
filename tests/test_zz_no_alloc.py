"""GPU test of ptw_pagerank_noalloc, the count walk that allocates nothing.

Callers that cannot allocate device memory when they run (their pool
allocator owns the GPU, or allocation is not allowed where they issue work)
pass a loaded graph and their own output buffer; the walk's counters live in
a fixed array inside the library.  Its results must equal ptw_pagerank_dev's
bit for bit (integer counts, the tolerance every count test here uses), and
stay equal on back-to-back calls, since every call reuses that array.

This file is named so pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cfg(C, W, sp, seed, start, first=0, max_moves=0):
    cfg = C.WalkCfg()
    cfg.n_walkers = W
    cfg.sp = sp
    cfg.seed = seed
    cfg.start_mode = start
    cfg.first_walker = first
    cfg.max_moves = max_moves
    return cfg


def test_noalloc_equals_existing_entry_point_twice(gpu):
    import torch
    from ptwalker_gb300 import _capi as C

    lib = C.load()
    G = gpu.Graph.rmat(16, 16, 0.57, 0.19, 0.19, seed=1, clean=True)
    try:
        assert G.n <= C.PTW_NOALLOC_MAX_VERTICES
        stream = torch.cuda.Stream()  # a caller's stream (not the legacy default stream 0)
        # back-to-back calls: on a caller's stream, then on the graph's own
        # stream (None), ending walks by the draw, by max_moves and by sp = 1
        cases = [(G.n, 0.15, 31, C.PTW_START_PER_VERTEX, 0, 0, stream),
                 (3 * G.n + 7, 0.2, 32, C.PTW_START_UNIFORM, 1 << 33, 0, stream),
                 (2 * G.n, 0.05, 33, C.PTW_START_PER_VERTEX, 5, 5, None),
                 (G.n + 1, 1.0, 34, C.PTW_START_UNIFORM, 0, 0, None)]
        for W, sp, seed, start, first, max_moves, st in cases:
            cfg = _cfg(C, W, sp, seed, start, first, max_moves)
            ref = torch.zeros(G.id_bound, dtype=torch.int32, device="cuda")
            torch.cuda.synchronize()
            C.check(lib.ptw_pagerank_dev(G.handle, ctypes.byref(cfg), ctypes.c_void_p(ref.data_ptr()),
                                         None))
            G.sync()
            out = torch.full((G.id_bound,), -1, dtype=torch.int32, device="cuda")
            torch.cuda.synchronize()
            C.check(lib.ptw_pagerank_noalloc(G.handle, ctypes.byref(cfg),
                                             ctypes.c_void_p(out.data_ptr()),
                                             ctypes.c_void_p(st.cuda_stream) if st is not None else None))
            if st is None:
                G.sync()
            torch.cuda.synchronize()
            a = out.cpu().numpy().view(np.uint32)
            b = ref.cpu().numpy().view(np.uint32)
            assert np.array_equal(a, b)
            assert int(a.sum()) > W  # every walker counted its start and moved
            if sp == 1.0:
                assert int(a.astype(np.uint64).sum()) <= 2 * W  # one move at most
            if max_moves:
                assert int(a.astype(np.uint64).sum()) <= (max_moves + 1) * W
    finally:
        G.close()


def test_noalloc_rejects_too_many_vertices_and_sources(gpu):
    from ptwalker_gb300 import _capi as C

    lib = C.load()
    # R-MAT scale 23 keeps more than 2^22 non-isolated vertices
    G = gpu.Graph.rmat(23, 16, 0.57, 0.19, 0.19, seed=1, clean=True)
    try:
        assert G.n > C.PTW_NOALLOC_MAX_VERTICES
        cfg = _cfg(C, 10, 0.15, 1, C.PTW_START_PER_VERTEX)
        rc = lib.ptw_pagerank_noalloc(G.handle, ctypes.byref(cfg), ctypes.c_void_p(1), None)
        assert rc == C.PTW_EINVAL
        assert b"at most 4194304" in lib.ptw_last_error()
    finally:
        G.close()
    G = gpu.Graph.rmat(10, 8, seed=2, clean=True)
    try:
        src = (ctypes.c_uint32 * 1)(0)
        cfg = _cfg(C, 10, 0.15, 1, C.PTW_START_SOURCES)
        cfg.h_sources = src
        cfg.n_sources = 1
        rc = lib.ptw_pagerank_noalloc(G.handle, ctypes.byref(cfg), ctypes.c_void_p(1), None)
        assert rc == C.PTW_EINVAL
    finally:
        G.close()
