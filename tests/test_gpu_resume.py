"""Checkpoint / resume of batched queries and of the serving loop.

Draws depend on (seed, query id, walker rank) only, so a batch run wave by
wave across calls (and processes) through its checkpoint file, or a server
saved mid-run and restored, must finish with the same counts as one
uninterrupted run: compared bit for bit here, and with the replay of single
queries."""
import os

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


def _same(a, b):
    oa, na, ca = a.export()
    ob, nb, cb = b.export()
    return np.array_equal(oa, ob) and np.array_equal(na, nb) and np.array_equal(ca, cb)


@pytest.mark.parametrize("top_k", [0, 30])
def test_resumable_batch_equals_one_call(gpu, G16, s16_canon, tmp_path, top_k):
    rng = np.random.default_rng(21)
    nq = 36
    src = rng.integers(0, G16.n, nq)
    bud = np.exp(rng.uniform(np.log(10), np.log(2e5), nq)).astype(np.int64)
    qids = rng.permutation(9000)[:nq]
    # small tables: several waves, and hash tables that fill (dense reruns)
    kw = dict(sp=0.2, seed=7, query_ids=qids, table_bytes=512 << 10, table_factor=0.05, top_k=top_k)
    ref = gpu.ppr_batch(G16, src, bud, **kw)
    ck = tmp_path / ("batch%d.ckpt" % top_k)
    calls, res = 0, None
    while res is None:
        calls += 1
        assert calls < 200
        res = gpu.ppr_batch_resumable(G16, src, bud, ck, max_waves=2, **kw)
        if res is None and calls == 2:
            # a record cut short, as by a process that ended while writing it
            with open(ck, "r+b") as f:
                f.truncate(os.path.getsize(ck) - 7)
    assert calls > 3
    assert _same(ref, res)
    assert res.moves == ref.moves and res.walkers == ref.walkers
    # the file now holds everything: a call runs no wave and returns the same
    again = gpu.ppr_batch_resumable(G16, src, bud, ck, max_waves=1, **kw)
    assert again is not None and _same(ref, again) and again.phases()["waves"] == 0
    if not top_k:
        for i in (0, nq - 1):
            w0 = int(qids[i]) << 32
            want, _ = oracle.replay_counts(s16_canon, w0, w0 + int(bud[i]), 0.2, 7, START_SOURCES, [int(src[i])])
            nz = np.nonzero(want)[0]
            names, counts = res.query(i)
            assert np.array_equal(names, nz.astype(np.uint32)) and np.array_equal(counts, want[nz])
    # another batch's checkpoint is refused
    with pytest.raises(gpu.PTWError):
        gpu.ppr_batch_resumable(G16, src, bud + 1, ck, **kw)
    for r in (ref, res, again):
        r.close()


def _drain(srv):
    out = {}
    while srv.n_active or srv.n_pending:
        for r in srv.step():
            out[r["query_id"]] = r
    for r in srv.results():
        out[r["query_id"]] = r
    return out


def test_server_save_and_restore(gpu, G16, tmp_path):
    rng = np.random.default_rng(22)
    nq = 40
    src = rng.integers(0, G16.n, nq)
    bud = np.exp(rng.uniform(np.log(1e3), np.log(3e5), nq)).astype(np.int64)
    kw = dict(sp=0.2, seed=4, tick_walkers=1 << 14, max_active=8, table_bytes=64 << 20, top_k=0)
    # uninterrupted
    with gpu.Server(G16, **kw) as a:
        for i in range(nq):
            a.submit(int(src[i]), int(bud[i]), 100 + i)
        a.n_pending = nq
        want = _drain(a)
    # interrupted: a few ticks, keep some results untaken, save, restore
    b = gpu.Server(G16, **kw)
    for i in range(nq):
        b.submit(int(src[i]), int(bud[i]), 100 + i)
    got = {}
    for _ in range(6):
        b.step(take=False)
    st = b.stats()
    assert st["active"] > 0 and st["pending"] > 0 and st["completed"] > 0
    ck = tmp_path / "server.ckpt"
    b.save(ck)
    b.close()
    c = gpu.Server.restore(G16, ck)
    got.update(_drain(c))
    assert c.stats()["completed"] == nq
    c.close()
    assert sorted(got) == sorted(want)
    for q in want:
        assert np.array_equal(got[q]["names"], want[q]["names"]) and np.array_equal(got[q]["counts"], want[q]["counts"])
    # the state of another graph is refused
    with gpu.Graph.rmat(12, 8, seed=3, clean=True) as other:
        with pytest.raises(gpu.PTWError):
            gpu.Server.restore(other, ck)
