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
