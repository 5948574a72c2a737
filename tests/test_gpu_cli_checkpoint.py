"""C++ CLI apps end to end, checkpoint / resume, and admission refusal."""
import os
import subprocess

import numpy as np
import pytest

import oracle
from oracle.replay import START_PER_VERTEX, START_SOURCES

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G16(gpu):
    G = gpu.Graph.rmat(16, 16, 0.57, 0.19, 0.19, seed=1, clean=True)
    yield G
    G.close()


def bin_path(app):
    from ptwalker_gb300 import _build
    return os.path.join(_build.BIN_DIR, app)


def test_cli_apps_match_replay(gpu, tmp_path, s16_edges, s16_canon):
    g = tmp_path / "g.txt"
    oracle.write_text_edges(str(g), *s16_edges)
    out = tmp_path / "c.u32"
    r = subprocess.run([bin_path("pagerank"), "-f", "text", "-g", str(g), "-w", "46879", "--sp", "0.15",
                        "--seed", "3", "-t", "20", "-s", "1", "--out", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    want, _ = oracle.replay_counts(s16_canon, 0, 46879, 0.15, 3, START_PER_VERTEX)
    assert np.array_equal(np.fromfile(out, dtype=np.uint32), want)
    assert r.stdout.startswith("ppr value %d" % want[0])
    r = subprocess.run([bin_path("ppr"), "-f", "text", "-g", str(g), "-e", "1", "--sp", "0.2", "--seed", "5",
                        "--source", "77", "--out", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    want, _ = oracle.replay_counts(s16_canon, 0, 46879, 0.2, 5, START_SOURCES, [77])
    assert np.array_equal(np.fromfile(out, dtype=np.uint32), want)
    paths = tmp_path / "p.i32"
    r = subprocess.run([bin_path("deepwalk"), "-f", "text", "-g", str(g), "-w", "1000", "-l", "10",
                        "--seed", "7", "--paths-out", str(paths)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    want = oracle.replay_paths(s16_canon, 0, 1000, 10, 7)
    assert np.array_equal(np.fromfile(paths, dtype=np.int32).reshape(1000, 10), want)
    r = subprocess.run([bin_path("node2vec"), "-f", "text", "-g", str(g), "-w", "1000", "-l", "12",
                        "-p", "0.5", "-q", "2", "--seed", "9", "--paths-out", str(paths)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    want, _ = oracle.replay_node2vec(s16_canon, 0, 1000, 12, 9, 0.5, 2.0)
    assert np.array_equal(np.fromfile(paths, dtype=np.int32).reshape(1000, 12), want)
    r = subprocess.run([bin_path("node2vec"), "-f", "text", "-g", str(g), "-w", "10", "-l", "5"],
                       capture_output=True, text=True)
    assert r.returncode != 0 and "-p and -q" in r.stderr


def _read_batch_out(path):
    raw = np.fromfile(path, dtype=np.uint8)
    nq = int(raw[:8].view(np.uint64)[0])
    off = raw[8:8 + 8 * (nq + 1)].view(np.uint64)
    ne = int(off[-1])
    rest = raw[8 + 8 * (nq + 1):]
    return off, rest[:4 * ne].view(np.uint32), rest[4 * ne:8 * ne].view(np.uint32)


def test_cli_ppr_sources_fixed_and_learned_budgets(gpu, tmp_path, s16_edges):
    """ppr --sources runs one batched launch; its lists equal ppr_batch's
    with the same budgets (fixed -w, or learned from a saved model), and
    --tune changes no result."""
    from ptwalker_gb300 import learned
    g = tmp_path / "g.txt"
    oracle.write_text_edges(str(g), *s16_edges)
    G = gpu.Graph.load(str(g), "text")
    try:
        rng = np.random.default_rng(5)
        src = rng.integers(0, G.n, 40).astype(np.uint32)
        srcf = tmp_path / "src.txt"
        srcf.write_text("\n".join(str(int(x)) for x in src) + "\n")
        out, bout = tmp_path / "b.bin", tmp_path / "budgets.u64"
        r = subprocess.run([bin_path("ppr"), "-f", "text", "-g", str(g), "-w", "3000", "--sp", "0.2", "--seed", "4",
                            "--sources", str(srcf), "--tune", "512,4,64,8192", "--out", str(out),
                            "--budgets-out", str(bout)], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        off, names, counts = _read_batch_out(out)
        assert np.array_equal(np.fromfile(bout, dtype=np.uint64), np.full(40, 3000, np.uint64))
        want = gpu.ppr_batch(G, src, 3000, sp=0.2, seed=4)
        for i in range(40):
            wn, wc = want.query(i)
            assert np.array_equal(names[off[i]:off[i + 1]], wn) and np.array_equal(counts[off[i]:off[i + 1]], wc)
        want.close()
        assert r.stdout.startswith("ppr queries 40 entries %d" % int(off[-1]))
        # learned budgets from a saved model (trained briefly on made-up labels)
        feats = learned.source_features(G, src)
        m = learned.BudgetModel(seed=3)
        m.fit(G, src, np.log(2000 + 50 * feats[:, 0]), epochs=30)
        model = tmp_path / "model.bin"
        m.save(str(model), b_min=500, b_max=20000, fallback=7000)
        m2, lim = learned.BudgetModel.load(str(model))
        assert lim == (500, 20000, 7000) and m2.kappa == m.kappa
        r = subprocess.run([bin_path("ppr"), "-f", "text", "-g", str(g), "-w", "1", "--sp", "0.2", "--seed", "6",
                            "--sources", ",".join(str(int(x)) for x in src), "--budget", "learned",
                            "--model", str(model), "--tune", "auto", "--out", str(out), "--budgets-out", str(bout)],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        used = np.fromfile(bout, dtype=np.uint64).astype(np.int64)
        expect = m2.budgets(G, src, b_min=500, b_max=20000, fallback=7000)
        assert np.all(np.abs(used - expect) <= 1) and len(set(used.tolist())) > 1
        off, names, counts = _read_batch_out(out)
        want = gpu.ppr_batch(G, src, used, sp=0.2, seed=6)
        for i in range(40):
            wn, wc = want.query(i)
            assert np.array_equal(names[off[i]:off[i + 1]], wn) and np.array_equal(counts[off[i]:off[i + 1]], wc)
        want.close()
    finally:
        G.close()


def test_resume_equals_uninterrupted(gpu, G16, tmp_path):
    from ptwalker_gb300.checkpoint import resumable_pagerank
    W = 5 * G16.n + 3
    full, done = resumable_pagerank(G16, str(tmp_path / "a.npz"), W, 0.15, 9, chunk=20000)
    assert done
    assert np.array_equal(full, gpu.pagerank(G16, W, 0.15, 9).astype(np.uint64))
    part, done = resumable_pagerank(G16, str(tmp_path / "b.npz"), W, 0.15, 9, chunk=20000, stop_after=3)
    assert not done and part.sum() < full.sum()
    resumed, done = resumable_pagerank(G16, str(tmp_path / "b.npz"), W, 0.15, 9, chunk=20000)
    assert done and np.array_equal(resumed, full)
    with pytest.raises(ValueError):
        resumable_pagerank(G16, str(tmp_path / "b.npz"), W, 0.2, 9, chunk=20000)


def test_admission_refused_when_a_table_exceeds_the_arena(gpu, G16):
    with gpu.Server(G16, sp=0.2, table_bytes=8 * 1024) as srv:  # 1024-slot arena
        srv.submit(3, 100000, 0)                                 # needs a far larger table
        with pytest.raises(gpu.PTWError) as e:
            srv.step()
        assert "arena" in str(e.value)
