"""GPU graph construction vs the oracle's canonical layout (bit-exact)."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def assert_same_graph(G, canon):
    names, row_ptr, col = G.export_csr()
    assert G.n == canon.n and G.m == canon.m
    assert np.array_equal(names, canon.names)
    assert np.array_equal(row_ptr, canon.row_ptr)
    assert np.array_equal(col, canon.col)


def test_rmat_s16_device_equals_oracle(gpu, s16_edges, s16_canon):
    with gpu.Graph.rmat(16, 16, 0.57, 0.19, 0.19, seed=1, clean=True) as G:
        assert_same_graph(G, s16_canon)
        assert G.id_bound == s16_canon.n
        assert G.max_degree == int(s16_canon.degree.max())
        s, d = G.export_edges()
        assert np.array_equal(s, s16_edges[0]) and np.array_equal(d, s16_edges[1])


def test_rmat_raw_multigraph(gpu):
    # clean=False keeps duplicates and self-loops of the raw R-MAT stream
    s, d = oracle.rmat_raw_edges(12, 8, seed=3)
    canon = oracle.canonical_from_edges(s, d)
    with gpu.Graph.rmat(12, 8, seed=3, clean=False) as G:
        assert_same_graph(G, canon)
        assert G.id_bound == int(max(s.max(), d.max())) + 1


def test_from_edges_sparse_names_dups_loops(gpu):
    rng = np.random.default_rng(0)
    names = rng.choice(1 << 24, size=300, replace=False).astype(np.uint32)
    src = names[rng.integers(0, 300, 5000)]
    dst = names[rng.integers(0, 300, 5000)]
    src = np.concatenate([src, src[:50], names[:10]])   # duplicates
    dst = np.concatenate([dst, dst[:50], names[:10]])   # self-loops
    for undirected in (False, True):
        canon = oracle.canonical_from_edges(src, dst, as_undirected=undirected)
        with gpu.Graph.from_edges(src, dst, as_undirected=undirected) as G:
            assert_same_graph(G, canon)
            assert G.id_bound == int(names.max()) + 1


def test_load_text_and_binary(gpu, tmp_path, s16_edges, s16_canon):
    s, d = s16_edges
    tp = tmp_path / "g.txt"
    bp = tmp_path / "g.bin"
    oracle.write_text_edges(str(tp), s, d)
    oracle.write_binary_edges(str(bp), s, d)
    with open(tp, "r+") as f:  # comment lines are skipped
        body = f.read()
        f.seek(0)
        f.write("# R-MAT scale 16\n" + body)
    for path, fmt in ((tp, "text"), (bp, "binary")):
        with gpu.Graph.load(path, fmt) as G:
            assert_same_graph(G, s16_canon)


def test_single_edge_and_errors(gpu):
    with gpu.Graph.from_edges([7], [9]) as G:
        names, row_ptr, col = G.export_csr()
        assert list(names) == [7, 9] and list(row_ptr) == [0, 1, 1] and list(col) == [1]
    with pytest.raises(gpu.PTWError):
        gpu.Graph.from_edges([], [])


def test_from_csr_round_trip_and_unsorted_rows(gpu, s16_canon):
    c = s16_canon
    with gpu.Graph.from_csr(c.row_ptr, c.col, c.names) as G:
        assert_same_graph(G, c)
    # rows in any order, duplicates and self-loops kept, names default to row indices
    rng = np.random.default_rng(5)
    n = 200
    deg = rng.integers(0, 12, n)
    deg[-1] = 0                                        # a row no one points to and with no entries
    row_ptr = np.concatenate([[0], np.cumsum(deg)]).astype(np.uint64)
    col = rng.integers(0, n - 1, int(row_ptr[-1])).astype(np.uint32)
    col[:5] = 3                                        # duplicates
    src = np.repeat(np.arange(n, dtype=np.uint32), deg)
    col[src == 7] = 7                                  # self-loops
    with gpu.Graph.from_csr(row_ptr, col) as G:
        assert_same_graph(G, oracle.canonical_from_edges(src, col))
        assert n - 1 not in G.export_csr()[0]
    names = rng.choice(1 << 30, size=n, replace=False).astype(np.uint32)
    with gpu.Graph.from_csr(row_ptr, col, names) as G:
        assert_same_graph(G, oracle.canonical_from_edges(names[src], names[col]))


def test_from_csr_errors(gpu):
    ok_row = np.array([0, 2, 3], np.uint64)
    ok_col = np.array([1, 0, 0], np.uint32)
    with gpu.Graph.from_csr(ok_row, ok_col) as G:
        assert G.n == 2 and G.m == 3
    bad = [
        (np.array([1, 2, 3], np.uint64), ok_col, None),                    # row_ptr[0] != 0
        (np.array([0, 2, 1, 3], np.uint64), ok_col, None),                 # decreasing
        (ok_row, np.array([1, 2, 0], np.uint32), None),                    # column index >= n
        (ok_row, ok_col, np.array([5, 5], np.uint32)),                     # repeated names
        (np.array([0, 0, 0], np.uint64), np.zeros(0, np.uint32), None),    # no entries
    ]
    for r, c, nm in bad:
        with pytest.raises(gpu.PTWError) as e:
            gpu.Graph.from_csr(r, c, nm)
        assert e.value.code == -1
    # the library stays usable after each refusal
    with gpu.Graph.from_csr(ok_row, ok_col, np.array([10, 4], np.uint32)) as G:
        names, row_ptr, col = G.export_csr()
        assert list(names) == [4, 10] and list(row_ptr) == [0, 1, 3] and list(col) == [1, 0, 1]


def test_gather_probe_reports_a_rate(gpu):
    small = gpu.probe_gather(1 << 20, 4)        # L2-resident
    large = gpu.probe_gather(1 << 30, 4)        # far above L2
    assert small > large > 1e9


def test_save_round_trip_and_text_bytes(gpu, tmp_path, s16_edges, s16_canon):
    s, d = s16_edges
    want_txt = tmp_path / "oracle.txt"
    oracle.write_text_edges(str(want_txt), s, d)
    with gpu.Graph.rmat(16, 16, 0.57, 0.19, 0.19, seed=1, clean=True) as G:
        for fmt in ("text", "binary"):
            p = tmp_path / ("g." + fmt)
            G.save(p, fmt)
            with gpu.Graph.load(p, fmt) as H:
                assert_same_graph(H, s16_canon)
        assert (tmp_path / "g.text").read_bytes() == want_txt.read_bytes()
        raw = np.fromfile(tmp_path / "g.binary", dtype=np.uint32).reshape(-1, 2)
        assert np.array_equal(raw[:, 0], s) and np.array_equal(raw[:, 1], d)
        with pytest.raises(gpu.PTWError):
            G.save(tmp_path / "no_such_dir" / "g.txt", "text")
