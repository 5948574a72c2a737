"""Small, self-contained workloads for profiling one kernel family at a time.

    python -m ptwalker_gb300.profile_workloads pagerank --scale 22
    python -m ptwalker_gb300.profile_workloads deepwalk --scale 22 --walk-len 80
    python -m ptwalker_gb300.profile_workloads node2vec --scale 22 --walk-len 80 --p 2 --q 0.5
    python -m ptwalker_gb300.profile_workloads batch --scale 20 --queries 512
    python -m ptwalker_gb300.profile_workloads exact --scale 18
    python -m ptwalker_gb300.profile_workloads learned --scale 18 --queries 256
    python -m ptwalker_gb300.profile_workloads mlp
    python -m ptwalker_gb300.profile_workloads build --scale 22
    python -m ptwalker_gb300.profile_workloads serve --n 8400000 --queries 600 --top-k 1000

Each runs a warm-up call and `--reps` measured calls and prints one JSON line
with CUDA-event timings.  Sizes default to cases that fit a full ncu capture
(inputs larger than L2, a few GB of device memory).
"""
import argparse
import json
import time

import numpy as np


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("what", choices=["pagerank", "deepwalk", "node2vec", "batch", "exact", "learned", "mlp", "build",
                                    "serve"])
    p.add_argument("--scale", type=int, default=22)
    p.add_argument("--walk-len", type=int, default=80)
    p.add_argument("--queries", type=int, default=512)
    p.add_argument("--reps", type=int, default=3)
    p.add_argument("--sp", type=float, default=0.15)
    p.add_argument("--p", type=float, default=2.0, help="node2vec return parameter")
    p.add_argument("--q", type=float, default=0.5, help="node2vec in-out parameter")
    p.add_argument("--n", type=int, default=8_400_000, help="Chung-Lu vertices (serve)")
    p.add_argument("--top-k", type=int, default=1000)
    p.add_argument("--budget-max", type=float, default=1e5, help="batch: budgets log-uniform in [1e3, this]")
    p.add_argument("--tune", default=None,
                   help="launch parameters as name=value pairs, e.g. block=1024,ilp=2,hot_k=8192")
    p.add_argument("--batch-tune", default=None,
                   help="batch: launch parameters of the batched kernel as name=value pairs, e.g. "
                        "desc_walkers=256,blocks_per_sm=6,group_bytes=402653184,dense_ratio=2,ext_columns=1")
    a = p.parse_args(argv)

    import torch
    import ptwalker_gb300 as ptw

    out = {"what": a.what}
    t0 = time.perf_counter()
    if a.what == "build":
        for _ in range(a.reps):
            G = ptw.Graph.rmat(a.scale, 16, seed=1, clean=True)
            out.update(vertices=G.n, edges=G.m)
            G.close()
        out["seconds_per_build"] = (time.perf_counter() - t0) / a.reps
        print(json.dumps(out))
        return
    if a.what == "mlp":
        from ptwalker_gb300 import learned
        rng = np.random.default_rng(0)
        x = rng.normal(0, 1, (20000, 8)).astype(np.float32)
        t = (x[:, 0] + np.sin(x[:, 1])).astype(np.float32)
        m = learned.MLP(seed=1)
        curve = m.train(x, t, epochs=a.reps, batch=4096, lr=1e-3)
        out.update(loss=[float(curve[0]), float(curve[-1])])
        print(json.dumps(out))
        return
    if a.what == "serve":
        # closed loop: every query queued at once, served to completion
        G = ptw.Graph.chung_lu(a.n, 2.1, 32.0, seed=1)
        rng = np.random.default_rng(4)
        src = rng.integers(0, G.n, a.queries)
        bud = np.exp(rng.uniform(np.log(1e3), np.log(1e6), a.queries)).astype(np.int64)
        with ptw.Server(G, sp=0.2, seed=3, tick_walkers=1 << 23, top_k=a.top_k) as srv:
            srv.submit(int(src[0]), 1000, 1 << 30)
            srv.drain()
            t1 = time.perf_counter()
            for q in range(a.queries):
                srv.submit(int(src[q]), int(bud[q]), q)
            res = srv.drain()
            wall = time.perf_counter() - t1
            out.update(vertices=G.n, edges=G.m, queries=len(res), seconds=wall, qps=len(res) / wall,
                       stats=srv.stats())
        G.close()
        print(json.dumps(out))
        return
    G = ptw.Graph.rmat(a.scale, 16, seed=1, clean=True)
    out.update(vertices=G.n, edges=G.m)
    if a.tune:
        G.tune = ptw.Tune(**{k: int(v) for k, v in (kv.split("=") for kv in a.tune.split(","))})
        out["tune"] = G.tune.as_dict()
    if a.batch_tune:
        ptw.set_batch_tune(G, ptw.BatchTune(**{k: int(v) for k, v in (kv.split("=") for kv in a.batch_tune.split(","))}))
        out["batch_tune"] = a.batch_tune
    if a.what == "pagerank":
        dev = torch.empty(G.id_bound, dtype=torch.int32, device="cuda")
        ptw.pagerank(G, G.n, a.sp, 1, out=dev)
        ms = []
        for k in range(a.reps):
            _, st = ptw.pagerank(G, G.n, a.sp, 2 + k, out=dev, stats=True)
            ms.append(st.kernel_ms)
        out.update(kernel_ms=ms, moves=st.moves)
    elif a.what == "deepwalk":
        paths = torch.empty((G.n, a.walk_len), dtype=torch.int32, device="cuda")
        ptw.deepwalk(G, G.n, a.walk_len, 1, out=paths)
        ms = []
        for k in range(a.reps):
            _, st = ptw.deepwalk(G, G.n, a.walk_len, 2 + k, out=paths, stats=True)
            ms.append(st.kernel_ms)
        out.update(kernel_ms=ms, steps=G.n * (a.walk_len - 1))
    elif a.what == "node2vec":
        paths = torch.empty((G.n, a.walk_len), dtype=torch.int32, device="cuda")
        ptw.node2vec(G, G.n, a.walk_len, a.p, a.q, 1, out=paths)
        ms = []
        for k in range(a.reps):
            _, st = ptw.node2vec(G, G.n, a.walk_len, a.p, a.q, 2 + k, out=paths, stats=True)
            ms.append(st.kernel_ms)
        out.update(kernel_ms=ms, moves=st.moves, trials=st.trials, checks=st.checks, probes=st.probes)
    elif a.what == "batch":
        names, row_ptr, col = G.export_csr()
        rng = np.random.default_rng(2)
        src = names[col[rng.integers(0, G.m, a.queries)]]
        bud = np.exp(rng.uniform(np.log(1e3), np.log(a.budget_max), a.queries)).astype(np.int64)
        ptw.ppr_batch(G, src, bud, sp=0.2, seed=1).close()
        res = [ptw.ppr_batch(G, src, bud, sp=0.2, seed=2 + k) for k in range(a.reps)]
        out.update(kernel_ms=[r.kernel_ms for r in res], total_ms=[r.ms for r in res], moves=res[-1].moves)
    elif a.what == "exact":
        src = np.arange(32, dtype=np.uint32)
        res = ptw.ppr_batch(G, src, 1000, sp=0.2, seed=1)
        l1 = res.l1(tol=1e-9)
        out.update(l1_p50=float(np.median(l1)))
    elif a.what == "learned":
        # the learned-budget evaluation at a small size: labels by pairwise
        # L1 of device-resident batches, training, three held-out runs scored
        # by one shared FP64 pass
        from ptwalker_gb300 import learned
        names, row_ptr, col = G.export_csr()
        rng = np.random.default_rng(3)
        tr = names[col[rng.integers(0, G.m, a.queries)]]
        te = names[col[rng.integers(0, G.m, a.queries)]]
        r = learned.evaluate(G, tr, te, b_fix=int(a.budget_max), sp=0.2, seed=5, epochs=100)
        out.update(gain=r["gain"], ceiling=r["label_ceiling"], stage_seconds=r["stage_seconds"])
    out["seconds"] = time.perf_counter() - t0
    G.close()
    print(json.dumps(out))


if __name__ == "__main__":
    main()
