"""Serving loop: continuous batching must not change any result.

Each query's sparse counts from the server equal the oracle replay of that
query alone, whether it ran alone or mixed with queries that arrived while
it was on the GPU, in CUDA-graph or plain-launch mode, under a small table
arena that forces admission to wait for memory, and when a table overflows.
"""
import numpy as np
import pytest

import oracle
from oracle.replay import START_SOURCES

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G16(gpu):
    G = gpu.Graph.rmat(16, 16, 0.57, 0.19, 0.19, seed=1, clean=True)
    yield G
    G.close()


def replay(canon, src, qid, budget, sp, seed, app="visits"):
    w0 = qid << 32
    if app == "visits":
        c, _ = oracle.replay_counts(canon, w0, w0 + budget, sp, seed, START_SOURCES, [src])
        return c
    pairs, _ = oracle.replay_pairs(canon, w0, w0 + budget, sp, seed, START_SOURCES, [src])
    return np.bincount(pairs[:, 1], minlength=canon.n).astype(np.uint32)


def check(r, canon, sp, seed, app="visits"):
    want = replay(canon, r["source"], r["query_id"], r["budget"], sp, seed, app)
    nz = np.nonzero(want)[0].astype(np.uint32)
    assert np.array_equal(r["names"], nz), r["query_id"]
    assert np.array_equal(r["counts"], want[nz]), r["query_id"]


@pytest.mark.parametrize("use_graph", [True, False])
def test_alone_and_in_the_mix(gpu, G16, s16_canon, use_graph):
    sp, seed = 0.2, 31
    # alone
    with gpu.Server(G16, sp=sp, seed=seed, tick_walkers=4096, use_graph=use_graph) as srv:
        srv.submit(1234, 20000, 7)
        alone = srv.drain()
    assert len(alone) == 1
    check(alone[0], s16_canon, sp, seed)
    # in a mix: the same query arrives while others are running and others
    # arrive while it runs (tick_walkers 4096 spreads it over several ticks)
    rng = np.random.default_rng(2)
    with gpu.Server(G16, sp=sp, seed=seed, tick_walkers=4096, use_graph=use_graph) as srv:
        got = {}
        for k in range(5):
            srv.submit(int(rng.integers(0, G16.n)), int(rng.integers(100, 30000)), 100 + k)
        for r in srv.step():
            got[r["query_id"]] = r
        srv.submit(1234, 20000, 7)
        for k in range(5, 40):
            srv.submit(int(rng.integers(0, G16.n)), int(rng.integers(100, 30000)), 100 + k)
            for r in srv.step():
                got[r["query_id"]] = r
        for r in srv.drain():
            got[r["query_id"]] = r
    assert len(got) == 41
    assert np.array_equal(got[7]["names"], alone[0]["names"])
    assert np.array_equal(got[7]["counts"], alone[0]["counts"])
    for qid in (100, 104, 120, 139):
        check(got[qid], s16_canon, sp, seed)
    assert got[7]["submit_s"] <= got[7]["admit_s"] <= got[7]["done_s"]


def test_admission_waits_for_table_memory(gpu, G16, s16_canon):
    seed = 5
    n = G16.n
    # Arena of 2^17 64-bit slots.  A 5000-walker query at sp 0.25 would need a
    # 2^16-slot hash table, so it counts into a dense array of n 32-bit
    # counters instead ((n + 1) / 2 slots, a 2^15 buddy block): four fit at
    # once.  A 1300-walker query at sp 0.5 keeps a 2^13-slot hash table (dense
    # would be more than twice its size): sixteen fit at once.  Both budgets
    # exceed a tick's smallest share (1024 walkers), so queries stay active
    # across ticks.
    assert 2 ** 14 < (n + 1) // 2 <= 2 ** 15
    for budget, fit, nq, sp in ((5000, 4, 8, 0.25), (1300, 16, 24, 0.5)):
        with gpu.Server(G16, sp=sp, seed=seed, tick_walkers=8192, table_bytes=8 << 17) as srv:
            for k in range(nq):
                srv.submit(100 + k, budget, k)
            seen_active, seen_pending = [], []
            res = []
            while True:
                res += srv.step()
                seen_active.append(srv.n_active)
                seen_pending.append(srv.n_pending)
                if srv.n_active == 0 and srv.n_pending == 0:
                    break
        assert max(seen_active) == fit and max(seen_pending) > 0
        assert len(res) == nq
        for r in res:
            check(r, s16_canon, sp, seed)


def test_overflow_and_endpoint_app(gpu, G16, s16_canon):
    with gpu.Server(G16, sp=0.2, seed=8, tick_walkers=50000, table_factor=0.001) as srv:
        for k in range(3):
            srv.submit(7 * k, 40000, k)
        res = srv.drain()
    assert len(res) == 3
    for r in res:
        check(r, s16_canon, 0.2, 8)
    with gpu.Server(G16, sp=0.5, seed=9, app="endpoint", tick_walkers=3000) as srv:
        srv.submit(42, 10000, 3)
        srv.submit(43, 777, 4)
        res = srv.drain()
    for r in res:
        check(r, s16_canon, 0.5, 9, "endpoint")


def test_submit_errors_and_open_loop(gpu, G16):
    with gpu.Server(G16, sp=0.2) as srv:
        with pytest.raises(gpu.PTWError):
            srv.submit(10 ** 8, 10, 0)
        with pytest.raises(gpu.PTWError):
            srv.submit(1, 0, 0)
        with pytest.raises(gpu.PTWError):
            srv.submit(1, (1 << 28) + 1, 0)
        rng = np.random.default_rng(0)
        out = gpu.open_loop(srv, rng.integers(0, G16.n, 200), rng.integers(1000, 5000, 200), rate=2000.0)
    assert out["n"] == 200 and out["p99_ms"] >= out["p50_ms"] > 0 and out["qps"] > 0


def test_chung_lu_graph(gpu):
    with gpu.Graph.chung_lu(20000, 2.1, 16.0, seed=3) as G:
        names, row_ptr, col = G.export_csr()
        deg = np.diff(row_ptr)
        assert deg.min() >= 1 and G.n <= 20000
        assert deg.max() > 20 * deg.mean()  # heavy tail
        s, d = G.export_edges()
        fwd = np.sort((s.astype(np.uint64) << np.uint64(32)) | d)
        rev = np.sort((d.astype(np.uint64) << np.uint64(32)) | s)
        assert np.array_equal(fwd, rev) and np.all(s != d)  # symmetric, no loops
        with gpu.Graph.chung_lu(20000, 2.1, 16.0, seed=3) as G2:
            assert np.array_equal(G2.export_csr()[2], col)  # deterministic


def test_untaken_results_survive_later_ticks_and_stats(gpu, G16, s16_canon):
    """Results wait in pinned staging blocks; later ticks must not overwrite a
    block that an untaken result still refers to."""
    sp, seed = 0.2, 77
    rng = np.random.default_rng(9)
    budgets = rng.integers(200, 20000, 30)
    with gpu.Server(G16, sp=sp, seed=seed, tick_walkers=8192) as srv:
        for k in range(30):
            srv.submit(int(rng.integers(0, G16.n)), int(budgets[k]), k)
            srv.step(take=False)
        while srv.n_active or srv.n_pending:
            srv.step(take=False)
        st = srv.stats()
        res = srv.results()
        assert srv.results() == []
    assert len(res) == 30
    for r in res:
        check(r, s16_canon, sp, seed)
    assert st["completed"] == 30 and st["walkers"] == int(budgets.sum())
    assert st["entries"] == sum(len(r["names"]) for r in res)
    assert st["moves"] > 0 and st["ticks"] >= 30 and st["retries"] == 0
    assert st["device_ms"] > 0 and st["step_ms"] >= st["collect_ms"] > 0
    assert st["active"] == 0 and st["pending"] == 0 and st["pinned_bytes"] >= 8 << 20


def test_serving_top_k(gpu, G16, s16_canon):
    sp, seed, k = 0.2, 13, 25
    rng = np.random.default_rng(4)
    with gpu.Server(G16, sp=sp, seed=seed, tick_walkers=8192, top_k=k) as srv:
        for q in range(12):
            srv.submit(int(rng.integers(0, G16.n)), int(rng.integers(1, 20000)), q)
        res = srv.drain()
    assert len(res) == 12
    for r in res:
        dense = replay(s16_canon, r["source"], r["query_id"], r["budget"], sp, seed)
        nz = np.nonzero(dense)[0]
        order = np.lexsort((nz, -dense[nz].astype(np.int64)))
        keep = nz[order][:k]
        assert np.array_equal(r["names"], keep.astype(np.uint32)), r["query_id"]
        assert np.array_equal(r["counts"], dense[keep]), r["query_id"]


def test_result_views_without_copy(gpu, G16, s16_canon):
    """step(copy=False) hands out read-only views of the page-locked staging:
    they hold the same lists as the replay until the next step."""
    with gpu.Server(G16, sp=0.2, seed=6) as srv:
        for i, (s, b) in enumerate([(3, 3000), (77, 5000), (1024, 2000), (46000, 4000)]):
            srv.submit(s, b, 40 + i)
        got = 0
        while got < 4:
            for r in srv.step(copy=False):
                assert not r["names"].flags.writeable and not r["counts"].flags.writeable
                check(r, s16_canon, 0.2, 6)   # before the next step
                got += 1
