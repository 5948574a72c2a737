"""Parity at the benchmark's own sizes.

R-MAT scale 22 (2.4 M vertices, 128 M CSR entries) is small enough for the
oracle's C pipeline to build and replay in seconds, so the GPU graph, count
walk, DeepWalk paths and batched queries are compared with it bit for bit.
At scale 24 (the headline workload) the checks are size-independent
properties: every position counted once (sum of counts = walkers + moves),
every start vertex visited, and walker shards summing to the whole run.
"""
import os

import numpy as np
import pytest

import oracle
from oracle.replay import START_PER_VERTEX, START_SOURCES

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


def test_s24_count_walk_properties(gpu):
    import torch
    with gpu.Graph.rmat(24, 16, 0.57, 0.19, 0.19, seed=1, clean=True) as G:
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
