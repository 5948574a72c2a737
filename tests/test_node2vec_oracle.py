"""CPU tests of the node2vec replay (oracle/oracle.c, ora_replay_node2vec).

The law is the one the reference's node2vec test checks
(src/test/debug/test_node2vec.cpp with the transition matrix of
third_party/knightking/test_node2vec.hpp:47-80): on a graph of undirected
edges, the walker that came from t to v moves to a neighbour x of v with
weight 1/p if x == t, 1 if x is a neighbour of t and 1/q otherwise.  The
test restates that check: every consecutive pair of a path is an edge, the
empirical second-order transitions have exactly the support of the exact
matrix, and they agree with it (the reference's bound on the summed squared
error, and a per-entry binomial bound)."""
import numpy as np
import pytest

import oracle


def test_thresholds():
    two32 = 1 << 32
    assert oracle.n2v_thresholds(1.0, 1.0) == [two32, two32, two32]
    assert oracle.n2v_thresholds(0.5, 2.0) == [two32, 1 << 31, 1 << 30]
    assert oracle.n2v_thresholds(2.0, 0.5) == [1 << 30, 1 << 31, two32]
    assert oracle.n2v_thresholds(4.0, 1.0) == [1 << 30, two32, two32]


def undirected_graph(v_num, e_num, seed):
    """e_num directed entries of a simple undirected graph on v_num vertices
    (no self-loops, no duplicates), every vertex with an edge."""
    rng = np.random.default_rng(seed)
    pairs = set()
    while len(pairs) < e_num // 2:
        a, b = (int(x) for x in rng.integers(0, v_num, 2))
        if a != b:
            pairs.add((min(a, b), max(a, b)))
    src = np.array([a for a, b in pairs], dtype=np.uint32)
    dst = np.array([b for a, b in pairs], dtype=np.uint32)
    return oracle.canonical_from_edges(src, dst, as_undirected=True)


def exact_transitions(g, p, q):
    """{(t, v): {x: probability}} over every directed edge t -> v."""
    rows = [set(g.col[g.row_ptr[i]:g.row_ptr[i + 1]].tolist()) for i in range(g.n)]
    out = {}
    for t in range(g.n):
        for v in rows[t]:
            w = {}
            for x in g.col[g.row_ptr[v]:g.row_ptr[v + 1]].tolist():
                w[x] = w.get(x, 0.0) + (1.0 / p if x == t else 1.0 if x in rows[t] else 1.0 / q)
            s = sum(w.values())
            out[(t, v)] = {x: c / s for x, c in w.items()}
    return out


def test_fold_thresholds():
    two32 = 1 << 32
    assert oracle.n2v_fold(2.0, 0.5) is None      # return weight not the largest
    assert oracle.n2v_fold(1.0, 1.0) is None      # not the only largest
    assert oracle.n2v_fold(0.5, 0.5) is None      # ties with the other weight
    assert oracle.n2v_fold(0.5, 2.0) == ([two32, two32, 1 << 31], 1 << 20)   # M' = 1, a = 1
    assert oracle.n2v_fold(0.25, 0.5) == ([two32, 1 << 31, two32], 1 << 20)  # M' = 2, a = 1
    assert oracle.n2v_fold(0.1, 4.0) == ([two32, two32, 1 << 30], 9 << 20)


def test_simple_symmetric_detection():
    g = undirected_graph(40, 200, seed=1)
    assert oracle.simple_symmetric(g)
    src, dst = np.array([0, 1, 1], np.uint32), np.array([1, 0, 2], np.uint32)
    assert not oracle.simple_symmetric(oracle.canonical_from_edges(src, dst))      # 1 -> 2 has no reverse
    src, dst = np.array([0, 0, 1], np.uint32), np.array([1, 1, 0], np.uint32)
    assert not oracle.simple_symmetric(oracle.canonical_from_edges(src, dst))      # repeated neighbour
    src, dst = np.array([0, 2], np.uint32), np.array([1, 2], np.uint32)
    # symmetrising doubles the self-loop (2, 2): a repeated neighbour
    assert not oracle.simple_symmetric(oracle.canonical_from_edges(src, dst, as_undirected=True))
    src, dst = np.array([0, 1, 2], np.uint32), np.array([1, 0, 2], np.uint32)
    assert oracle.simple_symmetric(oracle.canonical_from_edges(src, dst))          # one self-loop is its own reverse


@pytest.mark.parametrize("e_num", [64, 232, 800])
@pytest.mark.parametrize("p,q", [(0.5, 2.0), (2.0, 0.5), (10.0, 10.0), (0.25, 4.0), (0.25, 0.5)])
def test_replay_follows_node2vec_law(e_num, p, q):
    v_num = min(e_num // 2, 100 + e_num // 9)
    g = undirected_graph(v_num, e_num, seed=e_num)
    L = 60
    W = g.m * 40
    paths, trials = oracle.replay_node2vec(g, 0, W, L, seed=17, p=p, q=q, threads=4)
    assert np.all(paths >= 0)  # no dead ends on an undirected graph
    moves = W * (L - 1)
    assert trials >= moves
    # every consecutive pair is an edge
    edge = set(zip(np.repeat(np.arange(g.n), np.diff(g.row_ptr).astype(np.int64)).tolist(), g.col.tolist()))
    a, b = paths[:, :-1].ravel(), paths[:, 1:].ravel()
    assert all((int(x), int(y)) in edge for x, y in set(zip(a.tolist(), b.tolist())))
    # empirical second-order transitions
    t, v, x = paths[:, :-2].ravel(), paths[:, 1:-1].ravel(), paths[:, 2:].ravel()
    key = (t.astype(np.int64) * g.n + v) * g.n + x
    uk, cnt = np.unique(key, return_counts=True)
    emp = {}
    for k, c in zip(uk.tolist(), cnt.tolist()):
        tv, xx = divmod(k, g.n)
        emp.setdefault(divmod(tv, g.n), {})[xx] = c
    exact = exact_transitions(g, p, q)
    variance = 0.0
    worst_z = 0.0
    for tv, probs in exact.items():
        seen = emp.get(tv, {})
        total = sum(seen.values())
        assert total > 0, tv
        assert set(seen) == set(probs), tv  # same support
        for xx, pr in probs.items():
            f = seen[xx] / total
            variance += (f - pr) ** 2
            if pr < 1.0:
                worst_z = max(worst_z, abs(f - pr) / np.sqrt(pr * (1 - pr) / total))
    assert variance < 1.0  # the reference's check allows 10.0
    assert worst_z < 6.0


@pytest.mark.parametrize("p,q", [(0.5, 2.0), (0.25, 4.0)])
def test_folding_keeps_the_law_with_fewer_draws(p, q):
    g = undirected_graph(80, 600, seed=7)
    assert oracle.simple_symmetric(g)
    W, L = g.m * 20, 40
    folded, t_fold = oracle.replay_node2vec(g, 0, W, L, 3, p, q, threads=4)
    plain, t_plain = oracle.replay_node2vec(g, 0, W, L, 3, p, q, threads=4, fold=False)
    assert t_fold < 0.75 * t_plain
    # the same law: second-order transition frequencies agree within noise
    def freq(paths):
        t, v, x = paths[:, :-2].ravel(), paths[:, 1:-1].ravel(), paths[:, 2:].ravel()
        back = (x == t).mean()
        return back
    assert abs(freq(folded) - freq(plain)) < 0.01


def test_p_q_one_accepts_every_first_candidate():
    g = undirected_graph(50, 300, seed=3)
    W, L = 2000, 20
    paths, trials = oracle.replay_node2vec(g, 0, W, L, seed=5, p=1.0, q=1.0)
    assert trials == W * (L - 1)


def test_dead_ends_and_multigraph():
    # directed multigraph with a self-loop, a duplicate edge and a sink (name 9)
    src = np.array([0, 0, 0, 1, 1, 2, 2, 3, 3, 5], dtype=np.uint32)
    dst = np.array([1, 1, 2, 2, 0, 2, 3, 0, 9, 3], dtype=np.uint32)
    g = oracle.canonical_from_edges(src, dst)
    paths, _ = oracle.replay_node2vec(g, 0, 500, 12, seed=9, p=0.25, q=4.0, start_mode=oracle.replay.START_UNIFORM)
    sink = int(np.searchsorted(g.names, 9))
    edge = set(zip(np.repeat(np.arange(g.n), np.diff(g.row_ptr).astype(np.int64)).tolist(), g.col.tolist()))
    hit_sink = 0
    for row in paths:
        alive = row[row >= 0]
        assert np.all(row[len(alive):] == -1)  # padding only after the walk ended
        for a, b in zip(alive[:-1], alive[1:]):
            assert (int(a), int(b)) in edge
        if len(alive) < len(row):
            assert alive[-1] == sink
            hit_sink += 1
    assert hit_sink > 0
