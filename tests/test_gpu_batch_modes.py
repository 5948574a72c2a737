"""Batched PPR: device-resident results, per-phase timing and launch tunes.

Draws depend on (query id, walker rank) only, so the results of a batch must
not depend on where its lists end up (host or device memory), on the
launch parameters of the walker kernel (descriptor size, descriptor groups,
blocks per SM, column layout) or on which queries count into dense arrays
instead of hash tables: every variant is compared bit for bit with the
default host-result run, and that run with the oracle replay."""
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


def _batch(rng, G, nq=40):
    sources = rng.integers(0, G.n, nq)
    budgets = np.exp(rng.uniform(np.log(10), np.log(3e5), nq)).astype(np.int64)
    qids = rng.permutation(5000)[:nq]
    return sources, budgets, qids


def _same(a, b):
    oa, na, ca = a.export()
    ob, nb, cb = b.export()
    return np.array_equal(oa, ob) and np.array_equal(na, nb) and np.array_equal(ca, cb)


@pytest.mark.parametrize("top_k", [0, 50])
def test_device_results_equal_host_results(gpu, G16, s16_canon, top_k):
    rng = np.random.default_rng(11)
    sources, budgets, qids = _batch(rng, G16)
    host = gpu.ppr_batch(G16, sources, budgets, sp=0.2, seed=3, query_ids=qids, top_k=top_k)
    dev = gpu.ppr_batch(G16, sources, budgets, sp=0.2, seed=3, query_ids=qids, top_k=top_k,
                        device_results=True)
    assert dev.names is None and dev.d_offsets is not None
    assert np.array_equal(dev.d_offsets.cpu().numpy().view(np.uint64), host.offsets)
    assert _same(host, dev)
    for i in (0, 7, len(sources) - 1):
        hn, hc = host.query(i)
        dn, dc = dev.query(i)
        assert np.array_equal(hn, dn) and np.array_equal(hc, dc)
    if not top_k:  # and the host run equals the replay of each query alone
        for i in (0, 13):
            w0 = int(qids[i]) << 32
            want, _ = oracle.replay_counts(s16_canon, w0, w0 + int(budgets[i]), 0.2, 3, START_SOURCES,
                                           [int(sources[i])])
            nz = np.nonzero(want)[0]
            names, counts = host.query(i)
            assert np.array_equal(names, nz.astype(np.uint32)) and np.array_equal(counts, want[nz])
        # FP64 L1 reads device-resident lists too
        assert np.allclose(host.l1(tol=1e-8), dev.l1(tol=1e-8), rtol=0, atol=1e-12)
    ph_h, ph_d = host.phases(), dev.phases()
    assert ph_d["copy_bytes"] == 0 and ph_d["copy_ms"] == 0
    assert ph_h["copy_bytes"] == 8 * host.entries
    for ph in (ph_h, ph_d):
        assert ph["walk_ms"] > 0 and ph["count_ms"] > 0 and ph["place_ms"] > 0 and ph["upload_ms"] > 0
        assert ph["device_ms"] >= ph["walk_ms"] + ph["count_ms"] * 0.99
        assert ph["call_ms"] >= ph["plan_ms"] and ph["waves"] >= 1
    host.close()
    dev.close()


def test_device_results_across_waves_and_reruns(gpu, G16):
    """A small table budget splits the batch into several waves, and a tiny
    table factor makes hash tables fill (their queries rerun with dense
    arrays): the device lists are then concatenated on the device."""
    rng = np.random.default_rng(12)
    sources, budgets, qids = _batch(rng, G16, nq=30)
    kw = dict(sp=0.2, seed=5, query_ids=qids, table_bytes=256 << 10, table_factor=0.05)
    host = gpu.ppr_batch(G16, sources, budgets, **kw)
    dev = gpu.ppr_batch(G16, sources, budgets, device_results=True, **kw)
    ph = dev.phases()
    assert ph["waves"] > 2 and ph["reruns"] >= 1
    assert _same(host, dev)
    ref = gpu.ppr_batch(G16, sources, budgets, sp=0.2, seed=5, query_ids=qids)
    assert _same(host, ref)
    for r in (host, dev, ref):
        r.close()


def test_batch_tunes_give_the_same_results(gpu, G16):
    rng = np.random.default_rng(13)
    sources, budgets, qids = _batch(rng, G16, nq=48)
    saved = gpu.get_batch_tune(G16)
    ref = gpu.ppr_batch(G16, sources, budgets, sp=0.15, seed=8, query_ids=qids)
    try:
        for t in (gpu.BatchTune(desc_walkers=32, group_bytes=1 << 20, blocks_per_sm=1, ext_columns=2),
                  gpu.BatchTune(desc_walkers=4096, group_bytes=(1 << 64) - 1, dense_ratio=8, ext_columns=1),
                  gpu.BatchTune(desc_walkers=100, blocks_per_sm=3, dense_ratio=64)):
            gpu.set_batch_tune(G16, t)
            got = gpu.get_batch_tune(G16)
            assert got.as_dict() == t.as_dict()
            res = gpu.ppr_batch(G16, sources, budgets, sp=0.15, seed=8, query_ids=qids)
            assert _same(ref, res), t
            res.close()
        with pytest.raises(gpu.PTWError):
            gpu.set_batch_tune(G16, gpu.BatchTune(desc_walkers=8))
    finally:
        gpu.set_batch_tune(G16, saved)
        ref.close()


def test_autotune_batch(gpu, G16):
    rng = np.random.default_rng(14)
    sources, budgets, qids = _batch(rng, G16, nq=64)
    saved = gpu.get_batch_tune(G16)
    try:
        tune, ms = gpu.autotune_batch(G16, sources, budgets, sp=0.2, seed=1, query_ids=qids)
        assert ms > 0 and tune.desc_walkers in (128, 256, 512, 1024)
        assert gpu.get_batch_tune(G16).as_dict() == tune.as_dict()
        a = gpu.ppr_batch(G16, sources, budgets, sp=0.2, seed=2, query_ids=qids)
        gpu.set_batch_tune(G16, saved)
        b = gpu.ppr_batch(G16, sources, budgets, sp=0.2, seed=2, query_ids=qids)
        assert _same(a, b)
        a.close()
        b.close()
    finally:
        gpu.set_batch_tune(G16, saved)


def test_shared_fp64_l1_and_pair_l1(gpu, G16):
    """ptw_batch_l1_many scores several batches over the same sources with
    one power iteration: each row equals that batch scored alone.
    ptw_batch_l1_pair (summed on the device) equals the L1 of the exported
    lists computed on the host."""
    from ptwalker_gb300 import learned
    from ptwalker_gb300.batch import l1_many
    rng = np.random.default_rng(15)
    sources, budgets, qids = _batch(rng, G16, nq=40)
    a = gpu.ppr_batch(G16, sources, budgets, sp=0.2, seed=4, query_ids=qids)
    b = gpu.ppr_batch(G16, sources, budgets // 3 + 1, sp=0.2, seed=4, query_ids=qids, device_results=True)
    ref = gpu.ppr_batch(G16, sources, 4 * budgets, sp=0.2, seed=4, query_ids=qids, device_results=True)
    both = l1_many(G16, [a, b], tol=1e-9)
    assert np.allclose(both[0], a.l1(tol=1e-9), rtol=0, atol=1e-12)
    assert np.allclose(both[1], b.l1(tol=1e-9), rtol=0, atol=1e-12)
    for x in (a, b):
        got = x.l1_vs(ref)
        o1, n1, c1 = x.export()
        o2, n2, c2 = ref.export()
        want = np.array([learned.sparse_l1(n1[o1[i]:o1[i + 1]], c1[o1[i]:o1[i + 1]],
                                           n2[o2[i]:o2[i + 1]], c2[o2[i]:o2[i + 1]]) for i in range(len(sources))])
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-9)
    assert np.allclose(ref.l1_vs(ref), 0.0, atol=1e-12)
    other = gpu.ppr_batch(G16, sources[::-1].copy(), budgets, sp=0.2, seed=4)
    with pytest.raises(gpu.PTWError):
        a.l1_vs(other)
    for x in (a, b, ref, other):
        x.close()
