"""GPU node2vec paths (k_node2vec) against the oracle replay.

Paths must equal ora_replay_node2vec bit for bit under the same Philox
stream, and so must the number of candidate draws, for every (p, q), start
mode, walker-id offset and launch tune; on a small
undirected graph the GPU paths also follow the node2vec transition law that
the reference's test checks (src/test/debug/test_node2vec.cpp,
third_party/knightking/test_node2vec.hpp:47-80).
"""
import ctypes

import numpy as np
import pytest

import oracle
from oracle.replay import START_PER_VERTEX, START_SOURCES, START_UNIFORM

pytestmark = pytest.mark.gpu

MODES = {"per_vertex": START_PER_VERTEX, "uniform": START_UNIFORM, "sources": START_SOURCES}


@pytest.fixture(scope="module")
def G16(gpu):
    G = gpu.Graph.rmat(16, 16, 0.57, 0.19, 0.19, seed=1, clean=True)
    yield G
    G.close()


def as_names(canon, idx_paths):
    out = np.where(idx_paths >= 0, canon.names[np.maximum(idx_paths, 0)].astype(np.int64), -1)
    return out.astype(np.int32)


@pytest.mark.parametrize("p,q", [(0.5, 2.0), (2.0, 0.5), (1.0, 1.0), (0.25, 4.0), (4.0, 0.25),
                                 (32.0, 1.0 / 32.0), (1.0, 1024.0)])
def test_node2vec_paths_bit_exact(gpu, G16, s16_canon, p, q):
    W, L = G16.n, 40
    got, st = gpu.node2vec(G16, W, L, p, q, seed=21, stats=True)
    want, trials = oracle.replay_node2vec(s16_canon, 0, W, L, 21, p, q, threads=8)
    assert np.array_equal(got, want)
    assert st.moves == int((want[:, 1:] >= 0).sum())
    assert st.trials == trials
    if p == 1.0 and q == 1.0:
        assert st.trials == st.moves and st.checks == 0 and st.probes == 0


@pytest.mark.parametrize("start,W,L,first", [("uniform", 5000, 33, 0), ("uniform", 777, 17, (1 << 33) + 5),
                                             ("per_vertex", 4097, 7, 123), ("sources", 3001, 25, 0),
                                             ("per_vertex", 31, 1, 0), ("per_vertex", 100, 2, 0),
                                             ("uniform", 400_000, 1, 7), ("uniform", 300_000, 2, 0)])
def test_node2vec_start_modes_and_offsets(gpu, G16, s16_canon, start, W, L, first):
    sources = [0, 17, 4242] if start == "sources" else None
    got = gpu.node2vec(G16, W, L, 0.5, 2.0, seed=5, start=start, sources=sources, first_walker=first)
    want, _ = oracle.replay_node2vec(s16_canon, first, first + W, L, 5, 0.5, 2.0, MODES[start], sources,
                                     threads=8)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("paths_ilp,hints", [(1, 0), (2, 1), (4, 0), (4, 1)])
def test_node2vec_any_tune(gpu, G16, s16_canon, paths_ilp, hints):
    saved = G16.tune
    try:
        t = G16.tune
        t.paths_ilp = paths_ilp
        t.cache_hints = hints
        G16.tune = t
        for W, L in ((G16.n, 24), (4096 + 33, 7), (65, 33)):
            got = gpu.node2vec(G16, W, L, 2.0, 0.5, seed=9)
            want, _ = oracle.replay_node2vec(s16_canon, 0, W, L, 9, 2.0, 0.5, threads=8)
            assert np.array_equal(got, want)
    finally:
        G16.tune = saved


def test_node2vec_multigraph_dead_ends_sparse_names(gpu):
    # duplicate edges, self-loops, a sink (name 900) and names far apart
    rng = np.random.default_rng(4)
    src = rng.integers(0, 40, 400).astype(np.uint32) * 7 + 3
    dst = rng.integers(0, 40, 400).astype(np.uint32) * 7 + 3
    src = np.concatenate([src, [3, 3, 10, 10]]).astype(np.uint32)
    dst = np.concatenate([dst, [3, 900, 10, 10]]).astype(np.uint32)
    canon = oracle.canonical_from_edges(src, dst)
    with gpu.Graph.from_edges(src, dst) as G:
        for p, q in ((0.5, 2.0), (3.0, 0.3)):
            got = gpu.node2vec(G, 3000, 30, p, q, seed=3, start="uniform")
            want, _ = oracle.replay_node2vec(canon, 0, 3000, 30, 3, p, q, START_UNIFORM)
            assert np.array_equal(got, as_names(canon, want))
            assert (got == -1).any()  # some walkers reached the sink


def _undirected(v_num, e_num, seed):
    rng = np.random.default_rng(seed)
    pairs = set()
    while len(pairs) < e_num // 2:
        a, b = (int(x) for x in rng.integers(0, v_num, 2))
        if a != b:
            pairs.add((min(a, b), max(a, b)))
    src = np.array([a for a, b in pairs], dtype=np.uint32)
    dst = np.array([b for a, b in pairs], dtype=np.uint32)
    return src, dst


@pytest.mark.parametrize("p,q", [(0.5, 2.0), (2.0, 0.5)])
def test_node2vec_follows_transition_law(gpu, p, q):
    """The reference's check (test_node2vec.hpp:82-143) restated: every step is
    an edge and the empirical second-order transitions match the exact ones."""
    src, dst = _undirected(120, 800, seed=11)
    canon = oracle.canonical_from_edges(src, dst, as_undirected=True)
    with gpu.Graph.from_edges(src, dst, as_undirected=True) as G:
        W, L = canon.m * 60, 60
        paths = gpu.node2vec(G, W, L, p, q, seed=77, start="uniform")
    idx = np.searchsorted(canon.names, paths)
    rows = [set(canon.col[canon.row_ptr[i]:canon.row_ptr[i + 1]].tolist()) for i in range(canon.n)]
    a, b = idx[:, :-1].ravel(), idx[:, 1:].ravel()
    assert all(int(y) in rows[int(x)] for x, y in set(zip(a.tolist(), b.tolist())))
    t, v, x = idx[:, :-2].ravel(), idx[:, 1:-1].ravel(), idx[:, 2:].ravel()
    key = (t.astype(np.int64) * canon.n + v) * canon.n + x
    uk, cnt = np.unique(key, return_counts=True)
    emp = {}
    for k, c in zip(uk.tolist(), cnt.tolist()):
        tv, xx = divmod(k, canon.n)
        emp.setdefault(divmod(tv, canon.n), {})[xx] = c
    variance, worst_z = 0.0, 0.0
    for tt in range(canon.n):
        for vv in rows[tt]:
            w = {xx: (1.0 / p if xx == tt else 1.0 if xx in rows[tt] else 1.0 / q) for xx in rows[vv]}
            s = sum(w.values())
            seen = emp.get((tt, vv), {})
            total = sum(seen.values())
            assert set(seen) == set(w)
            for xx, wx in w.items():
                pr = wx / s
                f = seen[xx] / total
                variance += (f - pr) ** 2
                if pr < 1.0:
                    worst_z = max(worst_z, abs(f - pr) / np.sqrt(pr * (1 - pr) / total))
    assert variance < 1.0  # the reference's bound is 10.0
    assert worst_z < 6.0


def test_node2vec_device_output_and_app_mirror(gpu, G16, s16_canon):
    import torch

    W, L = 9000, 20
    out = torch.empty((W, L), dtype=torch.int32, device="cuda")
    gpu.node2vec(G16, W, L, 0.5, 2.0, seed=2, out=out)
    want, _ = oracle.replay_node2vec(s16_canon, 0, W, L, 2, 0.5, 2.0, threads=8)
    assert np.array_equal(out.cpu().numpy(), want)
    solver = gpu.Solver(G16)
    solver.set_node2vec(0.5, 2.0)
    app = gpu.DeepWalkApp(L, G16, start="per_vertex", seed=2)
    gpu.walk(solver, W, L, 0, app)
    assert np.array_equal(app.paths, want)


def test_node2vec_host_delivery_in_chunks(gpu, G16, s16_canon):
    """More than 2^20 walkers: chunks walked with overlapping copies; paths
    and the draw count equal one replay of all walkers."""
    W, L, w0 = 2_300_000, 5, 77
    got, st = gpu.node2vec(G16, W, L, 0.5, 2.0, seed=12, start="uniform", first_walker=w0, stats=True)
    want, trials = oracle.replay_node2vec(s16_canon, w0, w0 + W, L, 12, 0.5, 2.0, START_UNIFORM, threads=8)
    assert np.array_equal(got, want)
    assert st.trials == trials and st.moves == int((want[:, 1:] >= 0).sum())


def test_node2vec_rejects_bad_p_q(gpu, G16):
    from ptwalker_gb300 import _capi as C

    lib = C.load()
    cfg = C.WalkCfg()
    cfg.n_walkers = 10
    cfg.seed = 1
    buf = np.zeros(10 * 5, dtype=np.int32)
    ptr = buf.ctypes.data_as(ctypes.c_void_p)
    for p, q in ((0.0, 1.0), (1.0, -2.0), (float("inf"), 1.0), (1.0, float("nan")), (2048.0, 1.0),
                 (1.0, 1.0 / 2048.0), (0.03, 33.0)):
        rc = lib.ptw_node2vec(G16.handle, ctypes.byref(cfg), 5, p, q, ptr, None)
        assert rc == C.PTW_EINVAL, (p, q)
