"""Batched PPR / RWR: per-query sparse counts vs the oracle replay of each
query alone (bit-exact), independence from batch composition and wave
sizing, table-overflow recovery, and the device FP64 L1 oracle vs the CPU
FP64 oracle."""
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


def replay_query(canon, src, qid, budget, sp, seed, app, max_moves=0):
    w0 = qid << 32
    if app == "visits":
        c, _ = oracle.replay_counts(canon, w0, w0 + budget, sp, seed, START_SOURCES, [src],
                                    max_moves=max_moves)
        return c
    pairs, _ = oracle.replay_pairs(canon, w0, w0 + budget, sp, seed, START_SOURCES, [src],
                                   max_moves=max_moves)
    return np.bincount(pairs[:, 1], minlength=canon.n).astype(np.uint32)


def sparse_equal(res, i, dense):
    names, counts = res.query(i)
    nz = np.nonzero(dense)[0]
    return np.array_equal(names, nz.astype(np.uint32)) and np.array_equal(counts, dense[nz])


@pytest.mark.parametrize("app", ["visits", "endpoint"])
def test_batch_bit_exact_per_query(gpu, G16, s16_canon, app):
    rng = np.random.default_rng(5)
    nq = 24
    sources = rng.integers(0, G16.n, nq)
    budgets = rng.integers(1, 20000, nq)
    budgets[0] = 1
    qids = rng.permutation(1000)[:nq]
    res = gpu.ppr_batch(G16, sources, budgets, sp=0.2, seed=9, app=app, query_ids=qids)
    assert res.nq == nq and res.walkers == int(budgets.sum())
    tot_moves = 0
    for i in range(nq):
        want = replay_query(s16_canon, int(sources[i]), int(qids[i]), int(budgets[i]), 0.2, 9, app)
        assert sparse_equal(res, i, want), i
        if app == "visits":
            tot_moves += int(want.sum()) - int(budgets[i])
    if app == "visits":
        assert res.moves == tot_moves


def test_large_batches_one_after_another(gpu, G16, s16_canon):
    """Batches large enough for host result arrays sized, faulted in and
    page-locked before the walk (8 M entries and up) and for copies
    overlapping compaction range by range (16 M entries and up): a batch run
    after another one was freed must still equal the replay in every range,
    and results still held are not touched by later batches."""
    rng = np.random.default_rng(17)
    nq = 700  # about 25 K distinct vertices per query: 17 M entries written
    sources = rng.integers(0, G16.n, nq)
    budgets = np.full(nq, 60000)
    first = gpu.ppr_batch(G16, sources, budgets, sp=0.2, seed=3)
    keep = [first.query(i) for i in (0, 1)]
    kept = [(a.copy(), b.copy()) for a, b in keep]
    first.close()
    second = gpu.ppr_batch(G16, sources, budgets, sp=0.2, seed=4)
    held = gpu.ppr_batch(G16, sources[:40], budgets[:40], sp=0.2, seed=5)
    assert second.entries >= 16 << 20
    for i in (0, 57, 180, 349, 420, 555, nq - 1):
        want = replay_query(s16_canon, int(sources[i]), i, int(budgets[i]), 0.2, 4, "visits")
        assert sparse_equal(second, i, want), i
    second.close()
    third = gpu.ppr_batch(G16, sources, budgets, sp=0.2, seed=3)    # same as the first
    for i in (0, 1):
        names, counts = third.query(i)
        assert np.array_equal(names, kept[i][0]) and np.array_equal(counts, kept[i][1])
    want = replay_query(s16_canon, int(sources[7]), 7, int(budgets[7]), 0.2, 5, "visits")
    assert sparse_equal(held, 7, want)
    third.close()
    held.close()
    gpu.trim_memory()


def test_query_alone_equals_query_in_batch_and_across_waves(gpu, G16):
    sources = [3, 77, 77, 1024, 46000]
    budgets = [5000, 3000, 3000, 7000, 100]
    full = gpu.ppr_batch(G16, sources, budgets, sp=0.15, seed=4, query_ids=[10, 11, 12, 13, 14])
    alone = gpu.ppr_batch(G16, [1024], [7000], sp=0.15, seed=4, query_ids=[13])
    assert np.array_equal(full.dense(3), alone.dense(0))
    # one table per wave: every query in its own wave
    waves = gpu.ppr_batch(G16, sources, budgets, sp=0.15, seed=4, query_ids=[10, 11, 12, 13, 14],
                          table_bytes=1)
    for i in range(5):
        assert np.array_equal(full.dense(i), waves.dense(i))
    # the same source under two query ids draws two different walker streams
    assert not np.array_equal(full.dense(1), full.dense(2))
    # a query equals the single-source PPR call with first_walker = qid << 32
    single = gpu.ppr(G16, 1024, 7000, 0.15, 4, query_id=13)
    assert np.array_equal(single, alone.dense(0))


def test_table_overflow_rerun_is_exact(gpu, G16, s16_canon):
    # tiny tables force the probe limit; the rerun with 2n slots must give
    # the same counts as the replay
    sources = [0, 5, 9]
    budgets = [20000, 20000, 20000]
    res = gpu.ppr_batch(G16, sources, budgets, sp=0.2, seed=3, query_ids=[0, 1, 2], table_factor=0.001)
    for i in range(3):
        want = replay_query(s16_canon, sources[i], i, budgets[i], 0.2, 3, "visits")
        assert sparse_equal(res, i, want)


def test_batch_max_moves_and_errors(gpu, G16, s16_canon):
    res = gpu.ppr_batch(G16, [8, 9], [3000, 4000], sp=0.0001, seed=2, query_ids=[1, 2], max_moves=3)
    for i, (s, b, q) in enumerate(((8, 3000, 1), (9, 4000, 2))):
        want = replay_query(s16_canon, s, q, b, 0.0001, 2, "visits", max_moves=3)
        assert sparse_equal(res, i, want)
    with pytest.raises(gpu.PTWError):
        gpu.ppr_batch(G16, [10 ** 8], [10])
    with pytest.raises(gpu.PTWError):
        gpu.ppr_batch(G16, [1], [0])
    with pytest.raises(gpu.PTWError):
        gpu.ppr_batch(G16, [1], [(1 << 28) + 1])   # above the largest budget
    with pytest.raises(gpu.PTWError):
        gpu.ppr_batch(G16, [1], [10], sp=0.0)
    empty = gpu.ppr_batch(G16, [], [])
    assert empty.nq == 0 and empty.entries == 0


@pytest.mark.parametrize("app", ["visits", "endpoint"])
def test_device_fp64_l1_matches_cpu_oracle(gpu, G16, s16_canon, app):
    sp = 0.2
    sources = [0, 17, 500, 46878]
    res = gpu.ppr_batch(G16, sources, [20000] * 4, sp=sp, seed=12, app=app)
    l1_dev = res.l1(tol=1e-12)
    from oracle.power import _transition_T
    PT = _transition_T(s16_canon)
    for i, s in enumerate(sources):
        idx = s16_canon.name_to_index([s])[0]
        if app == "visits":
            exp = oracle.expected_visits_from_source(s16_canon, sp, idx, tol=1e-13, PT=PT)
        else:
            exp = oracle.expected_endpoint_from_source(s16_canon, sp, idx, tol=1e-13, PT=PT)
        c = res.dense(i).astype(np.float64)
        l1_cpu = np.abs(c / c.sum() - exp / exp.sum()).sum()
        assert abs(l1_dev[i] - l1_cpu) < 1e-8, (i, l1_dev[i], l1_cpu)
        assert 0.0 < l1_dev[i] < 2.0


def top_k_of(dense, k):
    """Oracle top-k: nonzero entries by count descending, then name ascending."""
    nz = np.nonzero(dense)[0]
    order = np.lexsort((nz, -dense[nz].astype(np.int64)))
    keep = nz[order][:k]
    return keep.astype(np.uint32), dense[keep]


@pytest.mark.parametrize("k", [1, 37, 1 << 30])
def test_batch_top_k_selection(gpu, G16, s16_canon, k):
    rng = np.random.default_rng(17)
    nq = 40
    src = rng.integers(0, G16.n, nq).astype(np.uint32)
    bud = rng.integers(1, 30000, nq)
    bud[0] = 1                                   # a single walker: few entries
    res = gpu.ppr_batch(G16, src, bud, sp=0.2, seed=12, top_k=k)
    for i in range(nq):
        want_n, want_c = top_k_of(replay_query(s16_canon, int(src[i]), i, int(bud[i]), 0.2, 12, "visits"), k)
        names, counts = res.query(i)
        assert np.array_equal(names, want_n) and np.array_equal(counts, want_c), i
    with pytest.raises(gpu.PTWError):
        res.l1()                                 # truncated lists have no L1 against the oracle
    res.close()


def test_top_k_with_wide_names_takes_the_two_sort_path(gpu, s16_canon):
    """Names near 2^31 leave no room for (query, count, name) in one 64-bit key,
    so compaction sorts by name and then by count; results must not change."""
    c = s16_canon
    rng = np.random.default_rng(23)
    big = np.sort(rng.choice(np.arange(1 << 30, (1 << 31) - 1, dtype=np.int64), c.n, replace=False)).astype(np.uint32)
    k, nq = 9, 40
    with gpu.Graph.from_csr(c.row_ptr, c.col, big) as G:
        src_idx = rng.integers(0, c.n, nq)
        bud = rng.integers(1, 20000, nq)
        res = gpu.ppr_batch(G, big[src_idx], bud, sp=0.2, seed=3, top_k=k)
        for i in range(nq):
            dense = replay_query(c, int(src_idx[i]), i, int(bud[i]), 0.2, 3, "visits")
            want_idx, want_c = top_k_of(dense, k)
            names, counts = res.query(i)
            assert np.array_equal(names, big[want_idx]) and np.array_equal(counts, want_c), i
        res.close()


@pytest.mark.parametrize("app", ["visits", "endpoint"])
def test_batch_and_serving_with_extended_columns(gpu, G16, s16_canon, app):
    """The walk kernel's one-gather path (row records carried with the
    column entries) must not change any query's counts."""
    saved = G16.tune
    try:
        t = G16.tune
        t.ext_columns = 1
        G16.tune = t
        rng = np.random.default_rng(31)
        nq = 30
        src = rng.integers(0, G16.n, nq).astype(np.uint32)
        bud = rng.integers(1, 40000, nq)
        res = gpu.ppr_batch(G16, src, bud, sp=0.25, seed=4, app=app)
        for i in range(nq):
            assert sparse_equal(res, i, replay_query(s16_canon, int(src[i]), i, int(bud[i]), 0.25, 4, app)), i
        res.close()
        with gpu.Server(G16, sp=0.25, seed=4, app=app, tick_walkers=8192) as srv:
            for i in range(8):
                srv.submit(int(src[i]), int(bud[i]), i)
            got = {r["query_id"]: r for r in srv.drain()}
        for i in range(8):
            want = replay_query(s16_canon, int(src[i]), i, int(bud[i]), 0.25, 4, app)
            nz = np.nonzero(want)[0].astype(np.uint32)
            assert np.array_equal(got[i]["names"], nz) and np.array_equal(got[i]["counts"], want[nz]), i
    finally:
        G16.tune = saved


@pytest.mark.parametrize("case", range(6))
def test_random_batches_equal_replay(gpu, G16, s16_canon, case):
    """Random batch shapes through compaction: hash and dense tables mixed,
    full lists and top-k, visit and endpoint apps, tiny and large budgets,
    repeated sources; every query equals its replay alone."""
    rng = np.random.default_rng(100 + case)
    nq = int(rng.integers(1, 120))
    app = ["visits", "endpoint"][case % 2]
    k = [0, 1, 7, 100, 0, 0][case]
    src = rng.integers(0, G16.n, nq).astype(np.uint32)
    src[rng.random(nq) < 0.2] = src[0]                        # some queries share a source
    bud = np.exp(rng.uniform(0, np.log(60000), nq)).astype(np.int64)
    qids = rng.permutation(1 << 20)[:nq].astype(np.uint32)
    sp = float(rng.choice([0.1, 0.2, 0.5]))
    res = gpu.ppr_batch(G16, src, bud, sp=sp, seed=case, app=app, query_ids=qids, top_k=k)
    for i in rng.choice(nq, min(nq, 12), replace=False):
        dense = replay_query(s16_canon, int(src[i]), int(qids[i]), int(bud[i]), sp, case, app)
        if k:
            want_n, want_c = top_k_of(dense, k)
            names, counts = res.query(i)
            assert np.array_equal(names, want_n) and np.array_equal(counts, want_c), (case, i)
        else:
            assert sparse_equal(res, i, dense), (case, i)
    res.close()
