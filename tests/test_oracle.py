"""CPU tests of the oracle: Philox known answers, R-MAT clean-up, replay
invariants, the FP64 expectation, and the statistical pin against the
reference binary's own output (tests/golden/ref_pagerank_*.npz)."""
import os

import numpy as np
import pytest

import oracle

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


# Published known-answer vectors for Philox4x32-10 (Salmon et al., SC'11).
KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,want", KAT)
def test_philox_known_answers(ctr, key, want):
    assert tuple(int(x) for x in oracle.philox4x32_10(ctr, key)) == want


def test_rmat_s16_clean(s16_edges, s16_canon):
    s, d = s16_edges
    g = s16_canon
    assert np.all(s != d)                       # no self-loops
    keys = (s.astype(np.uint64) << np.uint64(32)) | d
    assert np.all(np.diff(keys.astype(np.int64)) > 0)  # sorted, no duplicates
    rev = np.sort((d.astype(np.uint64) << np.uint64(32)) | s)
    assert np.array_equal(rev, keys)            # symmetric
    assert g.n == int(s.max()) + 1              # names compacted 0..n-1
    assert np.all(g.degree > 0)                 # isolated vertices removed
    assert g.n == 46879 and g.m == 1819276      # seed-1 R-MAT scale 16


def test_rmat_deterministic():
    a = oracle.rmat_raw_edges(10, 4, seed=7)
    b = oracle.rmat_raw_edges(10, 4, seed=7)
    c = oracle.rmat_raw_edges(10, 4, seed=8)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert not np.array_equal(a[0], c[0])


def test_canonical_keeps_duplicates_and_loops():
    src = [5, 5, 5, 9, 9, 2]
    dst = [9, 9, 5, 2, 5, 5]
    g = oracle.canonical_from_edges(src, dst)
    assert list(g.names) == [2, 5, 9]
    assert list(g.row_ptr) == [0, 1, 4, 6]
    assert list(g.col) == [1, 1, 2, 2, 0, 1]  # 5 -> 5, 9, 9 ; 9 -> 2, 5


def test_replay_conservation(s16_canon):
    g = s16_canon
    counts, moves = oracle.replay_counts(g, 0, g.n, 0.15, seed=3)
    assert int(counts.sum()) == g.n + moves
    pairs, mv = oracle.replay_pairs(g, 0, g.n, 0.15, seed=3)
    assert int(mv.sum()) == moves
    assert np.array_equal(pairs[:, 0], np.arange(g.n, dtype=np.uint32))
    # mean walk length 1/sp
    assert abs(moves / g.n - 1 / 0.15) < 0.1


def test_replay_threads_equal_serial(s16_canon):
    g = s16_canon
    a, ma = oracle.replay_counts(g, 0, 2 * g.n, 0.2, seed=11, start_mode=1)
    b, mb = oracle.replay_counts(g, 0, 2 * g.n, 0.2, seed=11, start_mode=1, threads=4)
    assert ma == mb and np.array_equal(a, b)


def test_paths_are_walks_and_prefix_of_counts(s16_canon):
    g = s16_canon
    L = 12
    paths = oracle.replay_paths(g, 0, 500, L, seed=5)
    assert np.array_equal(paths[:, 0], np.arange(500))
    for row in paths:
        for a, b in zip(row[:-1], row[1:]):
            nb = g.col[g.row_ptr[a]:g.row_ptr[a + 1]]
            assert b in nb
    # DeepWalk and count walks share the draw stream: a count walk that made
    # k moves follows the first k+1 path positions.
    pairs, moves = oracle.replay_pairs(g, 0, 500, 0.15, seed=5)
    for j in range(500):
        if moves[j] < L:
            assert paths[j, moves[j]] == pairs[j, 1]


@pytest.mark.parametrize("part_bytes", [1 << 12, 1 << 16, 1 << 20, 1 << 40])
def test_partitioned_port_equals_replay(s16_canon, part_bytes):
    """The timed CPU baseline (partition sweeps with per-(thread, partition)
    walker pools, partitioned.c) counts exactly what the replay counts, for
    every start mode, with move caps, across partition sizes and thread
    counts (from thousands of partitions down to one)."""
    g = s16_canon
    from oracle.replay import START_PER_VERTEX, START_SOURCES, START_UNIFORM
    cases = [(0, g.n, 0.15, 31, START_PER_VERTEX, None, 0),
             (1 << 33, (1 << 33) + 60000, 0.3, 9, START_UNIFORM, None, 4),
             (5 << 32, (5 << 32) + 40000, 0.2, 3, START_SOURCES, [int(g.names[5]), int(g.names[17]), int(g.names[99])], 0)]
    for w0, w1, sp, seed, mode, src, mm in cases:
        want, mv = oracle.replay_counts(g, w0, w1, sp, seed, mode, src, max_moves=mm, threads=4)
        for th in (1, 3):
            got, m2, info = oracle.partitioned_counts(g, w0, w1, sp, seed, mode, src, max_moves=mm, threads=th,
                                                      part_bytes=part_bytes)
            assert m2 == mv and np.array_equal(got, want), (part_bytes, th, mode)
            assert info["partitions"] >= 1 and info["sweeps"] >= 1


def test_dead_end_semantics():
    # 0 -> 1 -> 2, vertex 2 has no out-edge
    g = oracle.canonical_from_edges([0, 1], [1, 2])
    counts, moves = oracle.replay_counts(g, 0, 3, 0.01, seed=1)
    assert list(counts) == [1, 2, 3] and moves == 3
    paths = oracle.replay_paths(g, 0, 3, 4, seed=1)
    assert paths.tolist() == [[0, 1, 2, -1], [1, 2, -1, -1], [2, -1, -1, -1]]


def test_max_moves_and_sp_one(s16_canon):
    g = s16_canon
    _, mv = oracle.replay_pairs(g, 0, 1000, 0.0001, seed=2, max_moves=3)
    assert mv.max() == 3
    _, mv = oracle.replay_pairs(g, 0, 1000, 1.0, seed=2)
    assert np.all(mv == 1)


def test_fp64_expectation_matches_replay_tiny():
    z = np.load(os.path.join(GOLDEN, "ref_pagerank_tiny.npz"))
    e = z["edges"]
    g = oracle.canonical_from_edges(e[:, 0], e[:, 1])
    sp = float(z["sp"])
    W = 200000
    counts, _ = oracle.replay_counts(g, 0, W, sp, seed=9, start_mode=1, threads=4)
    exp = oracle.expected_visits_per_vertex_start(g, sp) * (W / g.n)
    zsc = (counts - exp) / np.sqrt(exp)
    assert np.abs(zsc).max() < 5.0
    # single source: E[c|s] and the endpoint law
    src = 3
    W = 100000
    counts, _ = oracle.replay_counts(g, 0, W, sp, seed=4, start_mode=2, sources=[src])
    exp = oracle.expected_visits_from_source(g, sp, g.name_to_index([src])[0]) * W
    assert np.abs((counts - exp) / np.sqrt(exp)).max() < 5.0
    pairs, _ = oracle.replay_pairs(g, 0, W, sp, seed=4, start_mode=2, sources=[src])
    end = np.bincount(pairs[:, 1], minlength=g.n)
    exp = oracle.expected_endpoint_from_source(g, sp, g.name_to_index([src])[0]) * W
    assert abs(exp.sum() - W) < 1e-6 * W
    assert np.abs((end - exp) / np.sqrt(exp + 1e-9)).max() < 5.0


def test_reference_binary_tiny_matches_fp64():
    """The reference's own pagerank output (duplicate edge and self-loop
    included) agrees with the FP64 expectation of the restated semantics."""
    z = np.load(os.path.join(GOLDEN, "ref_pagerank_tiny.npz"))
    e = z["edges"]
    g = oracle.canonical_from_edges(e[:, 0], e[:, 1])
    W, sp = int(z["W"]), float(z["sp"])
    c = z["counts"].astype(np.float64)
    assert int(c.sum()) == int(z["visits"])
    exp = oracle.expected_visits_per_vertex_start(g, sp) * (W / g.n)
    assert np.abs((c - exp) / np.sqrt(exp)).max() < 5.0
    # mean walk length: steps / W = 1/sp within sampling error
    assert abs(int(z["steps"]) / W - 1 / sp) < 0.02


def test_reference_binary_s16_calibrated(s16_canon):
    """Reference counts vs the oracle replay, with the tolerance calibrated
    from the replay's own seed-to-seed spread: L1 of normalised counts and
    max |z| must fall within 1.5x the 99th percentile of replay-vs-replay."""
    g = s16_canon
    z = np.load(os.path.join(GOLDEN, "ref_pagerank_s16.npz"))
    W, sp = int(z["W"]), float(z["sp"])
    ref = z["counts"].astype(np.float64)
    assert ref.shape[0] == g.n
    assert abs(int(z["steps"]) / W - 1 / sp) < 0.05
    runs = [oracle.replay_counts(g, 0, W, sp, seed=100 + k, start_mode=1, threads=4)[0]
            .astype(np.float64) for k in range(8)]

    def l1(a, b):
        return np.abs(a / a.sum() - b / b.sum()).sum()

    def maxz(a, b):
        return np.max(np.abs(a - b) / np.sqrt(a + b + 1.0))

    pair_l1 = [l1(runs[i], runs[j]) for i in range(8) for j in range(i + 1, 8)]
    pair_z = [maxz(runs[i], runs[j]) for i in range(8) for j in range(i + 1, 8)]
    ref_l1 = np.mean([l1(ref, r) for r in runs])
    ref_z = np.max([maxz(ref, r) for r in runs])
    assert ref_l1 <= 1.5 * np.percentile(pair_l1, 99), (ref_l1, np.percentile(pair_l1, 99))
    assert ref_z <= 1.5 * np.percentile(pair_z, 99), (ref_z, np.percentile(pair_z, 99))


def test_mlp_oracle_gradient_finite_differences():
    from oracle import mlp as omlp
    rng = np.random.default_rng(0)
    p = rng.normal(0, 0.3, omlp.NPARAMS)
    norm = np.concatenate([rng.normal(0, 1, 8), rng.uniform(0.5, 2, 8), [0.2, 1.5]])
    x = rng.normal(0, 1, (50, 8))
    t = rng.normal(0, 1, 50)
    loss, g, _ = omlp.forward_backward(p, norm, x, t)
    for k in rng.choice(omlp.NPARAMS, 40, replace=False):
        h = 1e-6
        pp = p.copy()
        pp[k] += h
        pm = p.copy()
        pm[k] -= h
        fd = (omlp.forward_backward(pp, norm, x, t)[0] - omlp.forward_backward(pm, norm, x, t)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 + 1e-4 * abs(g[k])
