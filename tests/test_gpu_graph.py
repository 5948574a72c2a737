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
