"""Multi-process walker sharding on CPU (gloo, world size 2): the per-rank
shards of the global walker stream, summed by one all-reduce, equal the
single-process run bit for bit, and so do node2vec path shards gathered in
rank order; query shards cover every query once; a
rank that fails before the exchange is detected by the other rank through a
short collective timeout, on the host."""
import os
import socket
import tempfile

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import oracle
from ptwalker_gb300 import shard


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, mode, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import datetime
    timeout = datetime.timedelta(seconds=5 if mode == "fail" else 60)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=timeout)
    try:
        canon = oracle.canonical_from_edges(*oracle.rmat_clean_edges(11, 8, seed=4))
        if mode == "paths":
            # second-order walks: each rank walks its range of the global
            # walker ids; the shards, gathered in rank order, are the whole run
            first, count = shard.strong_range(rank, world, canon.n + 3)
            paths, _ = oracle.replay_node2vec(canon, first, first + count, 9, 13, 0.5, 2.0)
            parts = [None] * world
            dist.all_gather_object(parts, paths)
            if rank == 0:
                np.save(os.path.join(out_dir, "paths.npy"), np.concatenate(parts))
            return
        if mode == "weak":
            first, count = shard.weak_range(rank, world, canon.n)
        else:
            first, count = shard.strong_range(rank, world, 3 * canon.n + 5)
        c, _ = oracle.replay_counts(canon, first, first + count, 0.15, 77, 0)
        t = torch.from_numpy(c.astype(np.int64))
        if mode == "fail" and rank == 1:
            raise RuntimeError("rank 1 fails before the exchange")
        try:
            shard.sum_counts(t)
        except Exception as e:  # the surviving rank learns of the failure here
            np.save(os.path.join(out_dir, "error_%d.npy" % rank), np.array(str(e)))
            return
        if rank == 0:
            np.save(os.path.join(out_dir, "sum.npy"), t.numpy())
    finally:
        try:
            dist.destroy_process_group()
        except Exception:
            pass


def _run(mode):
    world = 2
    port = free_port()
    with tempfile.TemporaryDirectory() as td:
        ctx = mp.get_context("spawn")
        procs = [ctx.Process(target=_worker, args=(r, world, port, mode, td)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
        files = {f: np.load(os.path.join(td, f)) for f in os.listdir(td)}
        return files, [p.exitcode for p in procs]


@pytest.mark.parametrize("mode", ["weak", "strong"])
def test_sharded_counts_equal_single_process(mode):
    files, codes = _run(mode)
    assert codes == [0, 0]
    canon = oracle.canonical_from_edges(*oracle.rmat_clean_edges(11, 8, seed=4))
    total = 2 * canon.n if mode == "weak" else 3 * canon.n + 5
    want, _ = oracle.replay_counts(canon, 0, total, 0.15, 77, 0)
    assert np.array_equal(files["sum.npy"], want.astype(np.int64))


def test_sharded_node2vec_paths_equal_single_process():
    files, codes = _run("paths")
    assert codes == [0, 0]
    canon = oracle.canonical_from_edges(*oracle.rmat_clean_edges(11, 8, seed=4))
    want, _ = oracle.replay_node2vec(canon, 0, canon.n + 3, 9, 13, 0.5, 2.0)
    assert np.array_equal(files["paths.npy"], want)


def test_failed_rank_is_detected_by_the_survivor():
    files, codes = _run("fail")
    assert codes[1] != 0                      # the failing rank exited with an error
    assert "error_0.npy" in files             # rank 0's collective ended with an error
    assert "sum.npy" not in files


def test_ranges_and_query_shards():
    for world in (1, 2, 3, 8):
        spans = [shard.strong_range(r, world, 1001) for r in range(world)]
        assert spans[0][0] == 0 and sum(c for _, c in spans) == 1001
        assert all(spans[i][0] + spans[i][1] == spans[i + 1][0] for i in range(world - 1))
        q = np.concatenate([shard.query_shard(50, r, world) for r in range(world)])
        assert sorted(q.tolist()) == list(range(50))
    assert shard.weak_range(3, 4, 10) == (30, 10)
    with pytest.raises(ValueError):
        shard.weak_range(4, 4, 10)
