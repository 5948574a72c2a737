"""GPU walker-update path vs the oracle replay under the same Philox stream.

Integer results must match bit for bit: visit counts (pagerank / PPR), the
(start, end) pairs of RWR and the DeepWalk paths, for every start mode,
walker-id offset, termination setting and launch configuration.
"""
import numpy as np
import pytest

import oracle
from oracle.replay import START_PER_VERTEX, START_SOURCES, START_UNIFORM

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G16(gpu):
    G = gpu.Graph.rmat(16, 16, 0.57, 0.19, 0.19, seed=1, clean=True)
    yield G
    G.close()


def by_name(canon, counts_idx, id_bound):
    out = np.zeros(id_bound, dtype=np.uint32)
    out[canon.names] = counts_idx
    return out


MODES = {"per_vertex": START_PER_VERTEX, "uniform": START_UNIFORM, "sources": START_SOURCES}


@pytest.mark.parametrize("W_mult,extra,start,sp,seed,max_moves", [
    (1, 0, "per_vertex", 0.15, 1, 0),
    (3, 17, "per_vertex", 0.15, 2, 0),
    (1, 5, "uniform", 0.15, 3, 0),
    (0, 4099, "uniform", 0.2, 0xDEADBEEFCAFEF00D, 0),
    (1, 0, "per_vertex", 1.0, 4, 0),
    (1, 0, "per_vertex", 0.001, 5, 7),
])
def test_pagerank_counts_bit_exact(gpu, G16, s16_canon, W_mult, extra, start, sp, seed, max_moves):
    W = W_mult * G16.n + extra
    got, st = gpu.pagerank(G16, W, sp, seed, start, max_moves=max_moves, stats=True)
    want, moves = oracle.replay_counts(s16_canon, 0, W, sp, seed, MODES[start], max_moves=max_moves)
    assert np.array_equal(got, want)
    assert st.moves == moves and st.visits == W + moves and st.walkers == W


@pytest.mark.parametrize("sources,W,qid", [
    ([0], 5000, 0),
    ([12345], 7777, 9),
    ([3, 99, 46878, 17, 17], 20000, 0),
])
def test_ppr_sources_and_query_ids(gpu, G16, s16_canon, sources, W, qid):
    got, st = gpu.pagerank(G16, W, 0.2, 11, "sources", sources, first_walker=qid << 32, stats=True)
    w0 = qid << 32
    want, moves = oracle.replay_counts(s16_canon, w0, w0 + W, 0.2, 11, START_SOURCES, sources)
    assert np.array_equal(got, want) and st.moves == moves
    if len(sources) == 1:
        got2 = gpu.ppr(G16, sources[0], W, 0.2, 11, query_id=qid)
        assert np.array_equal(got2, want)


@pytest.mark.parametrize("tune", [
    dict(block=32, ilp=1, chunk=1, hot_k=0),
    dict(block=128, ilp=2, chunk=33, hot_k=1024),
    dict(block=256, ilp=4, chunk=4096, hot_k=0),
    dict(block=1024, ilp=2, chunk=256, hot_k=40000),
    dict(block=512, ilp=4, chunk=64, hot_k=8192, blocks_per_sm=1),
    dict(block=512, ilp=4, chunk=256, hot_k=8192, min_blocks=2),
    dict(block=256, ilp=1, chunk=64, hot_k=0, min_blocks=2),
    dict(block=128, ilp=2, chunk=7, hot_k=100, min_blocks=2),
    dict(block=512, ilp=4, chunk=256, hot_k=8192, cache_hints=1),
    dict(block=256, ilp=2, chunk=64, hot_k=0, min_blocks=2, cache_hints=1),
    dict(block=512, ilp=4, chunk=256, hot_k=8192, cache_hints=1, ext_columns=1),
    dict(block=256, ilp=1, chunk=5, hot_k=0, cache_hints=0, ext_columns=1),
    dict(block=128, ilp=2, chunk=64, hot_k=300, min_blocks=2, ext_columns=1),
    dict(block=512, ilp=4, chunk=64, hot_k=0, min_blocks=2, ext_columns=1),
    dict(block=256, ilp=2, chunk=64, hot_k=8192, gather_slots=16),
    dict(block=128, ilp=2, chunk=7, hot_k=0, gather_slots=8),
    dict(block=64, ilp=1, chunk=256, hot_k=100, gather_slots=8, cache_hints=0),
    dict(block=256, ilp=4, chunk=4096, hot_k=10000, gather_slots=16),
    dict(block=512, ilp=4, chunk=64, hot_k=8192, cache_hints=1, ext_columns=1, warp_agg=1),
    dict(block=1024, ilp=2, chunk=256, hot_k=8192, cache_hints=1, warp_agg=1),
    dict(block=96, ilp=1, chunk=3, hot_k=0, warp_agg=1),
    dict(block=256, ilp=2, chunk=64, hot_k=50, cache_hints=0, ext_columns=1, warp_agg=1),
])
def test_launch_parameters_do_not_change_results(gpu, G16, s16_canon, tune):
    saved = G16.tune
    try:
        G16.tune = gpu.Tune(**tune)
        got = gpu.pagerank(G16, 2 * G16.n + 3, 0.15, 21, "uniform")
    finally:
        G16.tune = saved
    want, _ = oracle.replay_counts(s16_canon, 0, 2 * G16.n + 3, 0.15, 21, START_UNIFORM)
    assert np.array_equal(got, want)


def test_invalid_tune_rejected(gpu, G16):
    with pytest.raises(gpu.PTWError):
        G16.tune = gpu.Tune(block=100)
    with pytest.raises(gpu.PTWError):
        G16.tune = gpu.Tune(ilp=3)
    with pytest.raises(gpu.PTWError):
        G16.tune = gpu.Tune(gather_slots=4)
    with pytest.raises(gpu.PTWError):
        G16.tune = gpu.Tune(block=512, warp_agg=1, min_blocks=2)
    with pytest.raises(gpu.PTWError):
        G16.tune = gpu.Tune(block=512, gather_slots=8)
    saved = G16.tune
    try:
        # 16 slots x 256 threads x 36 B + 40000 hot counters x 4 B > 227 KB of shared memory
        G16.tune = gpu.Tune(block=256, hot_k=40000, gather_slots=16)
        with pytest.raises(gpu.PTWError):
            gpu.pagerank(G16, 1000, 0.15, 1)
    finally:
        G16.tune = saved


@pytest.mark.parametrize("start,W,qid", [("per_vertex", None, 0), ("uniform", 10001, 3)])
def test_rwr_pairs_bit_exact(gpu, G16, s16_canon, start, W, qid):
    W = G16.n if W is None else W
    got, st = gpu.rwr(G16, W, 0.5, 7, start, first_walker=qid << 32, stats=True)
    w0 = qid << 32
    want, moves = oracle.replay_pairs(s16_canon, w0, w0 + W, 0.5, 7, MODES[start])
    assert np.array_equal(got, want)
    assert st.moves == int(moves.sum())


@pytest.mark.parametrize("W_mult,extra,start,sp,seed,max_moves,first", [
    (1, 0, "per_vertex", 0.15, 1, 0, 0),
    (3, 17, "per_vertex", 0.15, 2, 0, 12345),
    (0, 4099, "uniform", 0.2, 0xDEADBEEFCAFEF00D, 0, 1 << 33),
    (1, 0, "per_vertex", 1.0, 4, 0, 0),
    (1, 0, "per_vertex", 0.001, 5, 7, 0),
    (0, 20000, "sources", 0.15, 6, 0, 0),
])
def test_counts_by_name_on_extended_columns(gpu, G16, s16_canon, W_mult, extra, start, sp, seed, max_moves, first):
    """The count walk on extended columns counts straight into the output
    by name; every start mode, offset and termination equals the replay."""
    saved = G16.tune
    try:
        G16.tune = gpu.Tune(block=768, ilp=2, chunk=64, hot_k=8192, cache_hints=1, ext_columns=3)
        W = W_mult * G16.n + extra
        sources = [5, 900, 4242] if start == "sources" else None
        got, st = gpu.pagerank(G16, W, sp, seed, start, sources, max_moves, first_walker=first, stats=True)
    finally:
        G16.tune = saved
    want, moves = oracle.replay_counts(s16_canon, first, first + W, sp, seed, MODES[start], sources, max_moves)
    assert np.array_equal(got, want) and st.moves == moves


@pytest.mark.parametrize("L,W,start", [(80, None, "per_vertex"), (1, 100, "per_vertex"),
                                       (33, 1000, "uniform"), (64, 4097, "per_vertex"),
                                       (5, 31, "uniform")])
def test_deepwalk_paths_bit_exact(gpu, G16, s16_canon, L, W, start):
    W = G16.n if W is None else W
    got = gpu.deepwalk(G16, W, L, 13, start)
    want = oracle.replay_paths(s16_canon, 0, W, L, 13, MODES[start])
    assert np.array_equal(got, want)


@pytest.mark.parametrize("ext", [0, 2])
def test_deepwalk_host_delivery_in_chunks(gpu, G16, s16_canon, ext):
    """More than 2^20 walkers: the host call walks them in chunks whose
    copies overlap the next chunks' walks; the paths equal the replay."""
    saved = G16.tune
    try:
        t = G16.tune
        t.ext_columns = ext
        G16.tune = t
        W, L, w0 = 2_500_000, 6, 1_000_003
        got, st = gpu.deepwalk(G16, W, L, 19, "uniform", first_walker=w0, stats=True)
        want = oracle.replay_paths(s16_canon, w0, w0 + W, L, 19, START_UNIFORM, threads=8)
        assert np.array_equal(got, want)
        assert st.total_ms >= st.kernel_ms > 0
    finally:
        G16.tune = saved


@pytest.mark.parametrize("paths_ilp,hints,named,ext", [(1, 0, 0, 0), (2, 0, 0, 0), (4, 0, 1, 0), (2, 1, 1, 0),
                                                       (4, 1, 0, 0), (1, 1, 1, 0), (1, 1, 0, 2), (2, 1, 1, 3),
                                                       (4, 0, 0, 2), (2, 0, 1, 1)])
def test_deepwalk_groups_per_warp(gpu, G16, s16_canon, paths_ilp, hints, named, ext):
    saved = G16.tune
    try:
        t = G16.tune
        t.paths_ilp = paths_ilp
        t.cache_hints = hints
        t.paths_named = named
        t.ext_columns = ext
        G16.tune = t
        for W, L in ((G16.n, 40), (4096 + 33, 7), (65, 33)):
            got = gpu.deepwalk(G16, W, L, 17)
            assert np.array_equal(got, oracle.replay_paths(s16_canon, 0, W, L, 17, START_PER_VERTEX))
    finally:
        G16.tune = saved


def test_rwr_with_register_capped_kernel(gpu, G16, s16_canon):
    saved = G16.tune
    try:
        G16.tune = gpu.Tune(block=512, ilp=4, chunk=128, hot_k=0, min_blocks=2)
        got = gpu.rwr(G16, 3 * G16.n, 0.3, 23, "uniform")
    finally:
        G16.tune = saved
    want, _ = oracle.replay_pairs(s16_canon, 0, 3 * G16.n, 0.3, 23, START_UNIFORM)
    assert np.array_equal(got, want)


def test_autotune_keeps_results(gpu, G16, s16_canon):
    saved = G16.tune
    try:
        t = G16.autotune(0.15)
        assert t.ilp in (1, 2, 4) and t.paths_ilp in (1, 2, 4) and t.min_blocks in (0, 2)
        got = gpu.pagerank(G16, G16.n, 0.15, 99)
    finally:
        G16.tune = saved
    want, _ = oracle.replay_counts(s16_canon, 0, G16.n, 0.15, 99, START_PER_VERTEX)
    assert np.array_equal(got, want)


def test_deepwalk_sources(gpu, G16, s16_canon):
    got = gpu.deepwalk(G16, 3000, 20, 2, "sources", sources=[5, 6, 7])
    want = oracle.replay_paths(s16_canon, 0, 3000, 20, 2, START_SOURCES, [5, 6, 7])
    assert np.array_equal(got, want)


@pytest.mark.parametrize("tune", [None, dict(block=256, ilp=2, chunk=64, hot_k=64, gather_slots=16),
                                  dict(block=128, ilp=2, chunk=5, hot_k=0, gather_slots=8, ext_columns=3),
                                  dict(block=128, ilp=2, chunk=5, hot_k=64, ext_columns=3)])
def test_dead_ends_and_sparse_names(gpu, tune):
    rng = np.random.default_rng(1)
    names = np.sort(rng.choice(1 << 20, size=500, replace=False)).astype(np.uint32)
    src = names[rng.integers(0, 400, 4000)]  # the last 100 names have no out-edge
    dst = names[rng.integers(0, 500, 4000)]
    canon = oracle.canonical_from_edges(src, dst)
    with gpu.Graph.from_edges(src, dst) as G:
        if tune:
            G.tune = gpu.Tune(**tune)
        W = 3 * G.n + 1
        got, st = gpu.pagerank(G, W, 0.1, 5, "per_vertex", stats=True)
        want, moves = oracle.replay_counts(canon, 0, W, 0.1, 5, START_PER_VERTEX)
        assert np.array_equal(got, by_name(canon, want, G.id_bound)) and st.moves == moves
        got = gpu.rwr(G, W, 0.1, 5)
        want, _ = oracle.replay_pairs(canon, 0, W, 0.1, 5)
        assert np.array_equal(got, canon.names[want])
        got = gpu.deepwalk(G, W, 9, 5)
        want = oracle.replay_paths(canon, 0, W, 9, 5)
        want_names = np.where(want < 0, -1, canon.names[np.maximum(want, 0)].astype(np.int64))
        assert np.array_equal(got, want_names.astype(np.int32))
        got = gpu.ppr(G, int(names[3]), 999, 0.1, 5, query_id=2)
        want, _ = oracle.replay_counts(canon, 2 << 32, (2 << 32) + 999, 0.1, 5, START_SOURCES,
                                       [int(names[3])])
        assert np.array_equal(got, by_name(canon, want, G.id_bound))
        with pytest.raises(gpu.PTWError):
            gpu.ppr(G, 1 << 21, 10, 0.1, 5)  # names are < 2^20: not a vertex


def test_device_outputs_equal_host_outputs(gpu, G16):
    import torch
    W = G16.n
    host = gpu.pagerank(G16, W, 0.15, 8)
    dev = torch.empty(G16.id_bound, dtype=torch.int32, device="cuda")
    gpu.pagerank(G16, W, 0.15, 8, out=dev)
    assert np.array_equal(dev.cpu().numpy().view(np.uint32), host)
    pairs = torch.empty((W, 2), dtype=torch.int32, device="cuda")
    gpu.rwr(G16, W, 0.3, 8, out=pairs)
    assert np.array_equal(pairs.cpu().numpy().view(np.uint32), gpu.rwr(G16, W, 0.3, 8))
    paths = torch.empty((1000, 40), dtype=torch.int32, device="cuda")
    gpu.deepwalk(G16, 1000, 40, 8, out=paths)
    assert np.array_equal(paths.cpu().numpy(), gpu.deepwalk(G16, 1000, 40, 8))


def test_pipelined_pagerank_equals_synchronous_calls(gpu, G16):
    """ptw_pagerank_submit / ptw_pagerank_wait with two calls in flight: every
    call's counts and moves equal ptw_pagerank's for the same configuration,
    whatever overlaps it; a third call in flight and unknown tickets are
    refused."""
    import torch
    W = G16.n
    bufs = [torch.empty(G16.id_bound, dtype=torch.int32, pin_memory=True) for _ in range(2)]
    want = {}
    for seed in range(5):
        want[seed] = gpu.pagerank(G16, W, 0.15, 100 + seed, stats=True)
    pend = []
    for seed in range(5):
        if len(pend) == 2:
            s0, t0 = pend.pop(0)
            st = gpu.pagerank_wait(G16, t0)
            assert np.array_equal(bufs[s0 % 2].numpy().view(np.uint32), want[s0][0])
            assert st.moves == want[s0][1].moves and st.walkers == W
        pend.append((seed, gpu.pagerank_submit(G16, bufs[seed % 2], W, 0.15, 100 + seed)))
    extra = np.empty(G16.id_bound, dtype=np.uint32)
    with pytest.raises(gpu.PTWError, match="PTW_EBUSY"):
        gpu.pagerank_submit(G16, extra, W, 0.15, 7)
    for s0, t0 in pend:
        st = gpu.pagerank_wait(G16, t0)
        assert np.array_equal(bufs[s0 % 2].numpy().view(np.uint32), want[s0][0])
        assert st.moves == want[s0][1].moves
    with pytest.raises(gpu.PTWError, match="PTW_EINVAL"):
        gpu.pagerank_wait(G16, pend[0][1])  # already waited for
    # a synchronous call between pipelined ones does not disturb them
    t = gpu.pagerank_submit(G16, extra, W, 0.15, 100)
    mid = gpu.pagerank(G16, W, 0.15, 101)
    gpu.pagerank_wait(G16, t)
    assert np.array_equal(extra, want[0][0]) and np.array_equal(mid, want[1][0])


def test_zero_walkers_and_bad_args(gpu, G16):
    z = gpu.pagerank(G16, 0, 0.15, 1)
    assert z.sum() == 0
    with pytest.raises(gpu.PTWError):
        gpu.pagerank(G16, 10, 0.0, 1)          # never terminates
    with pytest.raises(gpu.PTWError):
        gpu.pagerank(G16, 10, 1.5, 1)
    with pytest.raises(gpu.PTWError):
        gpu.pagerank(G16, 10, 0.15, 1, "sources", [10 ** 9])


def test_app_template_mirror(gpu, G16, s16_canon):
    """walk(solver, W, len, mem, app) fills the app's result member like the
    reference apps do (rooted_value / walker_pair / paths)."""
    solver = gpu.Solver(G16)
    app = gpu.PageRankApp(0.15, G16, start="uniform", seed=4)
    gpu.walk(solver, 5000, 7, 0, app)
    want, _ = oracle.replay_counts(s16_canon, 0, 5000, 0.15, 4, START_UNIFORM)
    assert np.array_equal(app.rooted_value, want)
    app = gpu.PPRApp(0.15, G16, source=77, seed=4)
    gpu.walk(solver, 5000, 7, 0, app)
    want, _ = oracle.replay_counts(s16_canon, 0, 5000, 0.15, 4, START_SOURCES, [77])
    assert np.array_equal(app.rooted_value, want)
    app = gpu.RWRApp(0.5, G16, seed=4)
    gpu.walk(solver, 5000, 3, 0, app)
    want, _ = oracle.replay_pairs(s16_canon, 0, 5000, 0.5, 4, START_UNIFORM)
    assert np.array_equal(app.walker_pair, want)
    app = gpu.DeepWalkApp(10, G16, seed=4)
    gpu.walk(solver, 5000, 10, 0, app)
    assert np.array_equal(app.paths, oracle.replay_paths(s16_canon, 0, 5000, 10, 4, START_UNIFORM))


def test_pagerank_vs_fp64_oracle(gpu, G16, s16_canon):
    """Estimates agree with the FP64 power-iteration expectation: per-vertex
    z-scores of the counts and the L1 of normalised counts (tolerance: the
    L1 must be below 1.5x the 99th percentile of replay-vs-replay L1)."""
    W = 10 * G16.n
    got = gpu.pagerank(G16, W, 0.15, 77, "per_vertex").astype(np.float64)
    exp = oracle.expected_visits_per_vertex_start(s16_canon, 0.15, n_walkers=W)
    l1 = np.abs(got / got.sum() - exp / exp.sum()).sum()
    reps = [oracle.replay_counts(s16_canon, 0, W, 0.15, 500 + k, START_PER_VERTEX, threads=4)[0]
            .astype(np.float64) for k in range(6)]
    ref_l1 = [np.abs(r / r.sum() - exp / exp.sum()).sum() for r in reps]
    assert l1 <= 1.5 * max(ref_l1), (l1, ref_l1)
    zz = (got - exp) / np.sqrt(exp)
    assert abs(zz.mean()) < 0.05 and zz.std() < 1.5


@pytest.mark.parametrize("tune", [dict(block=256, ilp=4, chunk=64, hot_k=0, ext_columns=3),
                                  dict(block=256, ilp=2, chunk=64, hot_k=0, ext_columns=3, gather_slots=16),
                                  dict(block=128, ilp=2, chunk=33, hot_k=512, ext_columns=3, gather_slots=8)])
def test_rwr_and_ppr_with_extended_columns(gpu, G16, s16_canon, tune):
    saved = G16.tune
    try:
        G16.tune = gpu.Tune(**tune)
        got = gpu.rwr(G16, 3 * G16.n, 0.3, 29, "uniform")
        want, _ = oracle.replay_pairs(s16_canon, 0, 3 * G16.n, 0.3, 29, START_UNIFORM)
        assert np.array_equal(got, want)
        got = gpu.ppr(G16, 77, 50000, 0.2, 5, query_id=9)
        want, _ = oracle.replay_counts(s16_canon, 9 << 32, (9 << 32) + 50000, 0.2, 5, START_SOURCES, [77])
        assert np.array_equal(got, want)
        with_ext = G16.device_bytes
    finally:
        G16.tune = saved
    # turning the copy off releases its 16 bytes per CSR entry and per vertex
    assert with_ext - G16.device_bytes == 16 * (G16.m + G16.n)


@pytest.mark.parametrize("slots", [8, 16])
def test_async_walkers_with_max_moves_and_offsets(gpu, G16, s16_canon, slots):
    saved = G16.tune
    try:
        G16.tune = gpu.Tune(block=256, ilp=2, chunk=64, hot_k=2048, gather_slots=slots)
        W = 3 * G16.n + 1
        got, st = gpu.pagerank(G16, W, 0.001, 3, "uniform", max_moves=7, stats=True)
        want, moves = oracle.replay_counts(s16_canon, 0, W, 0.001, 3, START_UNIFORM, max_moves=7)
        assert np.array_equal(got, want) and st.moves == moves
        got = gpu.rwr(G16, 5000, 0.3, 4, "per_vertex", max_moves=3, first_walker=(5 << 32) + 11)
        want, _ = oracle.replay_pairs(s16_canon, (5 << 32) + 11, (5 << 32) + 5011, 0.3, 4, START_PER_VERTEX,
                                      max_moves=3)
        assert np.array_equal(got, want)
    finally:
        G16.tune = saved
