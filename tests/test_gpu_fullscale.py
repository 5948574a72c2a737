"""Parity at the benchmark's own sizes.

R-MAT scale 22 (2.4 M vertices, 128 M CSR entries) and scale 24 (8.9 M
vertices, 521 M CSR entries: the headline workload) are both built by the
oracle's C pipeline in seconds and replayed on all host threads, so the GPU
graph, full one-walker-per-vertex count walks, DeepWalk path samples and
batched queries are compared with the replay bit for bit.  At scale 24 the
count walk is checked under the launch configurations the bench runs (the
autotuned one with the 8.3 GB extended column copy, and the plain-column
alternative), and the DeepWalk samples start at walker ids above 2^23 and
2^32 so the start map and the column offsets are exercised over the whole
id and edge range; so do node2vec samples, which also read the edge
filter.  Size-independent properties (every position counted
once, walker shards summing to the whole run) are checked as well.
"""
import os

import numpy as np
import pytest

import oracle
from oracle.replay import START_PER_VERTEX, START_SOURCES, START_UNIFORM

pytestmark = pytest.mark.gpu
NT = os.cpu_count() or 1


@pytest.fixture(scope="module")
def s22(gpu):
    G = gpu.Graph.rmat(22, 16, 0.57, 0.19, 0.19, seed=1, clean=True)
    canon = oracle.rmat_clean_csr(22, 16, 0.57, 0.19, 0.19, 1)
    yield G, canon
    G.close()


def test_s22_graph_equals_oracle(s22):
    G, canon = s22
    names, row_ptr, col = G.export_csr()
    assert G.n == canon.n and G.m == canon.m
    assert np.array_equal(names, canon.names)
    assert np.array_equal(row_ptr, canon.row_ptr)
    assert np.array_equal(col, canon.col)


def test_s22_pagerank_bit_exact(gpu, s22):
    G, canon = s22
    got, st = gpu.pagerank(G, G.n, 0.15, 31, "per_vertex", stats=True)
    want, moves = oracle.replay_counts(canon, 0, G.n, 0.15, 31, START_PER_VERTEX, threads=NT)
    assert st.moves == moves
    assert np.array_equal(got, want)


def test_s22_deepwalk_sample_bit_exact(gpu, s22):
    G, canon = s22
    W, L = 8192, 80
    got = gpu.deepwalk(G, W, L, 5, "per_vertex", first_walker=1_000_000)
    want = oracle.replay_paths(canon, 1_000_000, 1_000_000 + W, L, 5, START_PER_VERTEX, threads=NT)
    assert np.array_equal(got, want)


def test_s22_batched_queries_bit_exact(gpu, s22):
    """Budgets up to 1e6 put the large queries on dense count arrays and the
    small ones on hash tables; each must equal its query replayed alone."""
    G, canon = s22
    rng = np.random.default_rng(3)
    nq = 24
    src = rng.integers(0, G.n, nq).astype(np.uint32)
    bud = np.exp(rng.uniform(np.log(1e3), np.log(1e6), nq)).astype(np.int64)
    bud[0], bud[1] = 1_000_000, 500
    qids = np.arange(nq, dtype=np.uint32) + 7
    for top_k in (0, 100):
        res = gpu.ppr_batch(G, src, bud, sp=0.2, seed=9, query_ids=qids, top_k=top_k)
        for i in range(nq):
            w0 = int(qids[i]) << 32
            dense, _ = oracle.replay_counts(canon, w0, w0 + int(bud[i]), 0.2, 9, START_SOURCES, [int(src[i])],
                                            threads=NT)
            nz = np.nonzero(dense)[0]
            if top_k:
                nz = nz[np.lexsort((nz, -dense[nz].astype(np.int64)))][:top_k]
            names, counts = res.query(i)
            assert np.array_equal(names, nz.astype(np.uint32)), (top_k, i)
            assert np.array_equal(counts, dense[nz]), (top_k, i)
        if not top_k:
            assert int(res.counts.astype(np.uint64).sum()) == res.walkers + res.moves
        res.close()


# Launch configurations of the scale-24 bench: the autotuned pick (block 512,
# ILP 4, chunk 64, 8192 hot counters, L2 hints, extended columns for walks
# and paths), the runner-up (block 1024, ILP 2, plain columns) and the
# library default.
S24_TUNES = {
    "bench": dict(block=512, ilp=4, chunk=64, hot_k=8192, cache_hints=1, ext_columns=3, paths_ilp=2),
    "plain_1024x2": dict(block=1024, ilp=2, chunk=256, hot_k=8192, cache_hints=1, ext_columns=0,
                         paths_ilp=2, paths_named=1),
    "default": dict(),
}


@pytest.fixture(scope="module")
def s24(gpu):
    G = gpu.Graph.rmat(24, 16, 0.57, 0.19, 0.19, seed=1, clean=True)
    canon = oracle.rmat_clean_csr(24, 16, 0.57, 0.19, 0.19, 1, NT)
    yield G, canon
    G.close()


def _set_tune(gpu, G, name):
    G.tune = gpu.Tune(**S24_TUNES[name])


def test_s24_graph_equals_oracle(s24):
    G, canon = s24
    names, row_ptr, col = G.export_csr()
    assert G.n == canon.n and G.m == canon.m
    assert G.m > 500_000_000 and G.n > 2 ** 23
    assert np.array_equal(names, canon.names)
    assert np.array_equal(row_ptr, canon.row_ptr)
    assert np.array_equal(col, canon.col)


@pytest.mark.parametrize("tune", sorted(S24_TUNES))
def test_s24_pagerank_bit_exact(gpu, s24, tune):
    """The headline workload itself: W = |V| walkers, one per vertex, sp 0.15."""
    G, canon = s24
    _set_tune(gpu, G, tune)
    got, st = gpu.pagerank(G, G.n, 0.15, 41, "per_vertex", stats=True)
    want, moves = oracle.replay_counts(canon, 0, G.n, 0.15, 41, START_PER_VERTEX, threads=NT)
    assert st.moves == moves
    assert np.array_equal(got, want)


@pytest.mark.parametrize("tune", ["bench", "plain_1024x2"])
def test_s24_uniform_starts_high_ids_bit_exact(gpu, s24, tune):
    """Uniform starts (start vertex = mulhi(draw, n) over 8.9 M vertices) for
    a million walkers whose ids lie above 2^32."""
    G, canon = s24
    _set_tune(gpu, G, tune)
    W, w0 = 1_000_000, (1 << 32) + 12_345
    got, st = gpu.pagerank(G, W, 0.2, 43, "uniform", first_walker=w0, stats=True)
    want, moves = oracle.replay_counts(canon, w0, w0 + W, 0.2, 43, START_UNIFORM, threads=NT)
    assert st.moves == moves
    assert np.array_equal(got, want)


@pytest.mark.parametrize("tune", ["bench", "plain_1024x2"])
def test_s24_deepwalk_sample_bit_exact(gpu, s24, tune):
    """L = 80 path samples of 8,192 walkers at several walker-id offsets:
    the start, past 2^23, wrapping past |V| (per-vertex starts take the id
    modulo |V|) and above 2^33."""
    G, canon = s24
    _set_tune(gpu, G, tune)
    W, L = 8192, 80
    for w0 in (0, 4_000_000, (1 << 23) + 777, G.n - 3000, (1 << 33) + 5):
        got = gpu.deepwalk(G, W, L, 6, "per_vertex", first_walker=w0)
        want = oracle.replay_paths(canon, w0, w0 + W, L, 6, START_PER_VERTEX, threads=NT)
        assert np.array_equal(got, want), w0


@pytest.mark.parametrize("p,q", [(2.0, 0.5), (0.5, 2.0)])
def test_s24_node2vec_sample_bit_exact(gpu, s24, p, q):
    """Second-order path samples on the 8.3 GB extended columns and the 1 GB
    edge filter, at walker offsets past 2^23 and 2^33."""
    G, canon = s24
    _set_tune(gpu, G, "bench")
    W, L = 8192, 80
    for w0 in (0, (1 << 23) + 777, (1 << 33) + 5):
        got, st = gpu.node2vec(G, W, L, p, q, 8, "per_vertex", first_walker=w0, stats=True)
        want, trials = oracle.replay_node2vec(canon, w0, w0 + W, L, 8, p, q, START_PER_VERTEX, threads=NT)
        assert np.array_equal(got, want), w0
        assert st.trials == trials


def test_s24_count_walk_properties(gpu, s24):
    import torch
    G, _ = s24
    _set_tune(gpu, G, "bench")
    n = G.n
    full = torch.empty(G.id_bound, dtype=torch.int32, device="cuda")
    _, st = gpu.pagerank(G, n, 0.15, 77, "per_vertex", out=full, stats=True)
    f = full.cpu().numpy().view(np.uint32)
    assert int(f.astype(np.uint64).sum()) == n + st.moves   # every position counted once
    assert int(f.min()) >= 1                                  # every start counted
    # two walker shards, summed, equal the whole run
    a = torch.empty_like(full)
    b = torch.empty_like(full)
    half = n // 2
    gpu.pagerank(G, half, 0.15, 77, "per_vertex", out=a)
    gpu.pagerank(G, n - half, 0.15, 77, "per_vertex", out=b, first_walker=half)
    assert torch.equal(a.to(torch.int64) + b.to(torch.int64), full.to(torch.int64))
