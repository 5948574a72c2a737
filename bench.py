#!/usr/bin/env python
"""Walker-update benchmark: PageRank walks on an R-MAT scale-24 graph.

Workload (one "step"): W = |V| walkers, one per non-isolated vertex, stop
probability 0.15 after every move, every position counted into uint32 visit
counts; graph = R-MAT scale 24, edge factor 16, a/b/c/d = .57/.19/.19/.05,
seed 1, symmetrised with self-loops, duplicates and isolated vertices
removed (synthetic, built on the device).  Each step uses a new seed.

  value     walker steps/s with the graph resident in HBM (device output)
  e2e       the same walks through the host-facing C ABI calls for walk
            after walk, ptw_pagerank_submit / ptw_pagerank_wait (two calls
            in flight), host wall clock: every step's counts are read back
            into pinned host memory inside the timed region, the copy of
            one step overlapping the next step's walk.  A step's only input
            is its walk configuration (passed by value, no copy): the graph
            stays resident, as in the reference, whose walk timer excludes
            the graph load.  e2e.synchronous: the same through ptw_pagerank,
            which returns with the counts on the host (CUDA events)
  roofline  random-gather bound: 64 B per move (row record + column
            sector) + 32 B per counted visit, against the measured HBM peak;
            traffic = the ncu DRAM bytes per move of the scale-24 capture of
            the same column layout times this run's moves per launch; gather_peak = random
            4-byte loads/s this GPU serves from a 2 GB array, measured here
  cpu_baseline  the oracle port (C, all host threads) on a bounded sample of
            the same workload
  graph_replay  the same timed steps captured in one CUDA graph and
            replayed once (no host launch gaps)

--impl reference times the reference's walker semantics on the host CPU
(the oracle port; the reference's own sources do not exist on the GPU host)
for the same metric and config.  Under torchrun, rank r runs walkers
[r|V|, (r+1)|V|) (weak scaling; every rank replicates the graph) and the
count vectors are summed with one NCCL all_reduce per step.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "walker steps/s (PageRank walks on R-MAT)"
UNIT = "steps/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=200)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--scale", type=int, default=24)
    p.add_argument("--edge-factor", type=int, default=16)
    p.add_argument("--sp", type=float, default=0.15)
    p.add_argument("--seed", type=int, default=1)
    p.add_argument("--walk-len", type=int, default=80, help="DeepWalk length for the side line")
    p.add_argument("--no-deepwalk", action="store_true")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-autotune", action="store_true")
    p.add_argument("--tune", default=None,
                   help="block,ilp,chunk,hot_k[,min_blocks[,paths_ilp[,cache_hints[,paths_named[,ext_columns"
                        "[,gather_slots[,warp_agg]]]]]]]: "
                        "fixed launch parameters "
                        "(skips the autotuner)")
    p.add_argument("--no-batch", action="store_true", help="skip the batched-PPR side line")
    p.add_argument("--no-serve", action="store_true", help="skip the serving side line")
    p.add_argument("--no-ingest", action="store_true", help="skip the edge-list ingest side line")
    p.add_argument("--no-learned", action="store_true", help="skip the learned-budget side line")
    p.add_argument("--learned-train", type=int, default=4096, help="training queries of the learned line")
    p.add_argument("--learned-test", type=int, default=4096, help="held-out queries of the learned line")
    p.add_argument("--batch-scale", type=int, default=22)
    p.add_argument("--batch-queries", type=int, default=4096)
    p.add_argument("--serve-n", type=int, default=8_400_000)
    p.add_argument("--serve-rates", default="1000,10000,50000")
    p.add_argument("--serve-queries", type=int, default=3000)
    p.add_argument("--serve-budget-max", type=float, default=1e6)
    p.add_argument("--serve-tick", type=int, default=1 << 23, help="walkers per serving tick")
    p.add_argument("--serve-top-k", type=int, default=1000,
                   help="entries returned per query (largest counts); 0 = full vectors.  With k > 0 one "
                        "extra run at the second rate returns full vectors")
    return p.parse_args()


def config(args, world):
    return {"workload": "pagerank walks, R-MAT scale %d (edge factor %d, a/b/c .57/.19/.19, seed %d, "
                        "cleaned), W=|V| one walker per vertex, sp=%g"
                        % (args.scale, args.edge_factor, args.seed, args.sp),
            "graph": "rmat-s%d-ef%d" % (args.scale, args.edge_factor),
            "walkers_per_gpu": "|V|", "sp": args.sp, "parallelism": "walker-shard x%d" % world,
            "l2": l2_note(args)}


def l2_note(args):
    """R-MAT with edge factor ef keeps about 1.9 * ef * 2^scale CSR entries after
    symmetrising and de-duplication at these quadrant probabilities."""
    col_bytes = 4 * 1.9 * args.edge_factor * (1 << args.scale)
    if col_bytes > 2 * 129e6:
        return "inputs exceed L2 (CSR column array about %.1f GB, L2 129 MB); no flush" % (col_bytes / 1e9)
    return "small graph: CSR column array about %.0f MB may sit in the 129 MB L2; no flush" % (col_bytes / 1e6)


# ---- clocks ---------------------------------------------------------------

class Clocks:
    """nvidia-smi samples during the timed region (read-only queries)."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if self.proc is None:
            return out
        time.sleep(0.3)
        self.proc.terminate()
        try:
            self.proc.wait(5)
        except Exception:
            self.proc.kill()
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return out
        sm = sorted(float(r[1]) for r in rows if r[1].replace(".", "").isdigit())
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for k, nm in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        out.update(sm_mhz=sm[len(sm) // 2] if sm else None, sm_max_mhz=max(mx) if mx else None,
                   reasons=sorted(reasons), samples=len(rows))
        return out


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ---- CPU baseline ---------------------------------------------------------------

# Partition size of the partitioned port: a core's L2 (1 MB on Grace).
PORT_PART_BYTES = 1 << 20
PORT_KIND = ("partitioned port: the reference's partition sweeps with per-(thread, partition) walker pools "
             "(src/core/solver.hpp:222-493) restated in C with OpenMP (oracle/partitioned.c), Philox draws, "
             "counts equal to the oracle's")


# The reference's own binary cannot run on the GPU host (its sources are not
# there; no cross compiler here).  oracle/ref/calibrate.py timed it beside the
# ports on one 8-core x86 host (R-MAT, W = |V|, sp 0.15, uniform starts, median
# of 3): reference binary / partitioned port = 1.26 at scale 16 (54.9 vs
# 43.6 M steps/s) and 2.10 at scale 20 (100.1 vs 47.7 M steps/s); at scale 22
# the binary aborts with glibc heap corruption, so no larger figure exists.
PORT_CALIBRATION = {"host": "x86_64, 8 cores (the build container)", "script": "oracle/ref/calibrate.py",
                    "reference_over_partitioned_port": {"rmat-s16": 1.26, "rmat-s20": 2.10,
                                                        "rmat-s22": "reference binary aborts (heap corruption)"},
                    "reference_over_atomic_port": {"rmat-s16": 1.38, "rmat-s20": 3.18}}


def cpu_port_run(canon, sp, seed, n_walkers, threads):
    import oracle
    t0 = time.perf_counter()
    _, moves, _ = oracle.partitioned_counts(canon, 0, n_walkers, sp, seed, 0, threads=threads,
                                            part_bytes=PORT_PART_BYTES)
    dt = time.perf_counter() - t0
    return moves, dt


def cpu_port_sample(canon, sp, seed, threads, target_s=2.0):
    """Times the port on the first S walkers of the workload, S sized so a run
    takes about target_s seconds of wall time (at least one calibration)."""
    n = canon.n
    # a probe of a million walkers: the partitioned port's sweeps cost about
    # the same whatever the number of walkers, so a small probe undersells it
    probe = min(n, 1 << 20)
    moves, dt = cpu_port_run(canon, sp, seed, probe, threads)
    S = probe
    if dt > 0:
        S = int(min(n, max(probe, probe * target_s / dt)))
    if S > probe:
        moves, dt = cpu_port_run(canon, sp, seed, S, threads)
    return S, moves, dt


# ---- reference arm ------------------------------------------------------------

def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return 0
    import oracle
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    canon = oracle.rmat_clean_csr(args.scale, args.edge_factor, 0.57, 0.19, 0.19, args.seed, threads)
    oracle.replay.degree_relabelled(canon, threads)  # graph-load work, as in the reference
    build_s = time.perf_counter() - t0
    # each step a bounded sample, sized so that warm-up + timed steps take
    # about 150 s of walking whatever K and W are (at most 3 s per step; the
    # whole W = |V| workload once a step has the time)
    S, _, _ = cpu_port_sample(canon, args.sp, args.seed, threads,
                              target_s=min(3.0, 150.0 / max(1, args.steps + args.warmup)))
    for k in range(args.warmup):
        cpu_port_run(canon, args.sp, 1000 + k, S, threads)
    tot_moves, tot_s = 0, 0.0
    for k in range(args.steps):
        mv, dt = cpu_port_run(canon, args.sp, 2000 + k, S, threads)
        tot_moves += mv
        tot_s += dt
    value = tot_moves / tot_s
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000 * tot_s / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": config(args, world), "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "port": PORT_KIND, "calibration": PORT_CALIBRATION,
                         "sample": "first %d of %d walkers per step (per-vertex starts) of the same "
                                   "workload; graph built on the host in %.1f s"
                                   % (S, canon.n, build_s)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# ---- side lines: batched PPR, serving, learned budgets -------------------------------

def degree_sources(G, n, seed):
    """Sources drawn degree-proportionally: the endpoint of a uniform edge."""
    import numpy as np
    names, row_ptr, col = G.export_csr()
    rng = np.random.default_rng(seed)
    e = rng.integers(0, G.m, n)
    return names[col[e]]


# DRAM bytes per move of the count walk on R-MAT scale 24, W = |V|, sp 0.15:
# ncu dram__bytes_read.sum + dram__bytes_write.sum over two launches of each
# launch configuration, divided by the moves of a launch (one-pass capture
# of the full-size bench command; profiles/k_walk_dram_bytes_rmat-s24.md).
TRAFFIC_PER_MOVE_S24 = {True: 127.0, False: 130.1}  # extended columns (counting by name) / plain columns
TRAFFIC_SOURCE = ("ncu dram__bytes_read.sum + dram__bytes_write.sum per move of k_walk at R-MAT scale 24 "
                  "(two launches of the %s-column configuration, profiles/k_walk_dram_bytes_rmat-s24.md), "
                  "times this run's moves per launch")


def traffic_per_move(scale, ext):
    """DRAM bytes per move of the walk kernel at the bench workload, for the
    column layout the launch reads; None at other scales."""
    if scale != 24:
        return None
    return TRAFFIC_PER_MOVE_S24[bool(ext)]


def loguniform_budgets(n, lo, hi, seed):
    import numpy as np
    rng = np.random.default_rng(seed)
    return np.exp(rng.uniform(np.log(lo), np.log(hi), n)).astype(np.int64)


PHASE_KEYS = ("call_ms", "plan_ms", "device_ms", "upload_ms", "walk_ms", "count_ms", "place_ms", "copy_ms",
              "copy_tail_ms", "host_pages_ms", "copy_bytes", "waves", "reruns")


def phase_line(ph):
    """One call's phases (ms, bytes) rounded; gap_ms = device time outside
    the timed phases (the device waiting on host steps between them)."""
    out = {k: (round(ph[k], 2) if k.endswith("_ms") else ph[k]) for k in PHASE_KEYS}
    busy = ph["upload_ms"] + ph["walk_ms"] + ph["count_ms"] + ph["place_ms"] + ph["copy_tail_ms"]
    out["gap_ms"] = round(ph["device_ms"] - busy, 2)
    return out


def get_batch_tune(G, ptw, args, src, bud):
    """The batched kernel's launch parameters: from the tune cache (keyed by
    device, graph and batch), else ptw_autotune_batch on this batch."""
    import torch
    key = "%s|batch|s%d|n%d|m%d|nq%d|sp0.2" % (torch.cuda.get_device_name(), args.batch_scale, G.n, G.m,
                                               len(src))
    path = tune_cache_path()
    cache = {}
    if os.path.exists(path):
        try:
            cache = json.load(open(path))
        except Exception:
            cache = {}
    if key in cache:
        t = ptw.BatchTune(**{k: v for k, v in cache[key].items() if k in ptw.BatchTune.FIELDS})
        ptw.set_batch_tune(G, t)
        return t, "cache", cache[key].get("ms")
    t0 = time.perf_counter()
    t, ms = ptw.autotune_batch(G, src, bud, sp=0.2, seed=99)
    cache[key] = dict(t.as_dict(), ms=ms, seconds=time.perf_counter() - t0)
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as f:
            json.dump(cache, f, indent=1)
    except Exception:
        pass
    return t, "autotune", ms


def bench_batch(args, ptw):
    """Config: R-MAT scale 22, 4096 degree-proportional sources (seed 2),
    budgets log-uniform in [1e3, 1e6] (seed 3), sp 0.2.  Launch parameters
    from the batch autotuner.  Five timed batch calls with the lists copied
    to host memory (seeds 7-11; the median is the figure, all five are
    listed with their phases), then five with the lists left in device
    memory (PTW_BATCH_DEVICE_RESULTS: a GPU consumer's view), each after one
    untimed call of the same kind (cold_seconds: it maps the count tables'
    device memory and faults in the host result pages)."""
    import numpy as np
    G = ptw.Graph.rmat(args.batch_scale, 16, 0.57, 0.19, 0.19, seed=1, clean=True)
    src = degree_sources(G, args.batch_queries, 2)
    bud = loguniform_budgets(args.batch_queries, 1e3, 1e6, 3)
    tune, tune_src, tune_ms = get_batch_tune(G, ptw, args, src, bud)

    def timed(device_results):
        t0 = time.perf_counter()
        ptw.ppr_batch(G, src, bud, sp=0.2, seed=6, device_results=device_results).close()
        cold = time.perf_counter() - t0
        walls, phases, res = [], [], None
        for k in range(5):
            if res is not None:
                res.close()
            t0 = time.perf_counter()
            res = ptw.ppr_batch(G, src, bud, sp=0.2, seed=7 + k, device_results=device_results)
            walls.append(time.perf_counter() - t0)
            phases.append(phase_line(res.phases()))
        return cold, walls, phases, res

    cold, walls, phases, res = timed(False)
    wall = float(np.median(walls))
    out = {"graph": "rmat-s%d" % args.batch_scale, "vertices": G.n, "edges": G.m,
           "queries": int(args.batch_queries), "walkers": int(res.walkers), "moves": int(res.moves),
           "entries": int(res.entries), "seconds": wall, "queries_per_s": args.batch_queries / wall,
           "cold_seconds": cold, "seconds_each": walls, "phases_each": phases,
           "steps_per_s": res.moves / wall, "device_ms": res.ms, "walk_kernel_ms": res.kernel_ms,
           "walk_kernel_steps_per_s": res.moves / (res.kernel_ms / 1000.0),
           "walk_kernel_gbs": (64 * res.moves + 32 * res.visits) / (res.kernel_ms / 1000.0) / 1e9,
           "tune": dict(tune.as_dict(), source=tune_src, autotune_ms=tune_ms)}
    res.close()
    cold_d, walls_d, phases_d, res_d = timed(True)
    wall_d = float(np.median(walls_d))
    out["device_results"] = {"seconds": wall_d, "queries_per_s": args.batch_queries / wall_d,
                             "steps_per_s": res_d.moves / wall_d, "cold_seconds": cold_d,
                             "seconds_each": walls_d, "phases_each": phases_d,
                             "same_entries_as_host_call": int(res_d.entries) == out["entries"]}
    res_d.close()
    sub = np.arange(0, args.batch_queries, max(1, args.batch_queries // 64))[:64]
    one = ptw.ppr_batch(G, src[sub], bud[sub], sp=0.2, seed=7, query_ids=sub.astype(np.uint32))
    l1 = one.l1(tol=1e-6)
    out["fp64_l1_sample"] = {"queries": int(len(sub)), "p50": float(np.median(l1)),
                             "p90": float(np.quantile(l1, 0.9)), "max": float(l1.max()), "tol": 1e-6}
    one.close()
    G.close()
    return out


def bench_ingest(args, ptw):
    """Edge-list ingest (the reference's Graph::load, graph.hpp:277-785, whose
    text reader is one thread of sscanf, io.hpp:76-90): the R-MAT scale-22
    graph written by ptw_graph_save as text and as binary Edge[], then timed
    through ptw_graph_load: parse on all host threads, upload, device CSR
    build with the degree-sorted relabelling."""
    import shutil
    G = ptw.Graph.rmat(args.batch_scale, 16, 0.57, 0.19, 0.19, seed=1, clean=True)
    tmp = tempfile.mkdtemp(prefix="ptw_ingest_")
    out = {"graph": "rmat-s%d" % args.batch_scale, "vertices": G.n, "edges": G.m}
    try:
        for fmt in ("text", "binary"):
            path = os.path.join(tmp, "g." + fmt)
            t0 = time.perf_counter()
            G.save(path, fmt)
            save_s = time.perf_counter() - t0
            size = os.path.getsize(path)
            ptw.Graph.load(path, fmt).close()  # warm: page cache, CUDA context
            t0 = time.perf_counter()
            H = ptw.Graph.load(path, fmt)
            load_s = time.perf_counter() - t0
            ok = H.n == G.n and H.m == G.m
            H.close()
            out[fmt] = {"file_bytes": size, "save_s": save_s, "load_s": load_s,
                        "edges_per_s": G.m / load_s, "gb_per_s": size / load_s / 1e9, "same_graph": ok,
                        "threads": os.cpu_count()}
    finally:
        G.close()
        shutil.rmtree(tmp, ignore_errors=True)
    return out


def bench_serve(args, ptw):
    """Config: Chung-Lu power-law graph (8.4M vertices, exponent 2.1, mean
    degree 32), Poisson arrivals at each rate, random sources, fixed budgets
    log-uniform in [1e3, serve_budget_max], sp 0.2.  Each rate line carries
    the server's own counters: ticks, walk moves, and where the host time of
    the steps went (device time of the ticks, result collection)."""
    import numpy as np
    G = ptw.Graph.chung_lu(args.serve_n, 2.1, 32.0, seed=1)
    rng = np.random.default_rng(4)
    out = {"graph": "chung-lu n=%d gamma=2.1 mean_degree=32" % args.serve_n, "vertices": G.n, "edges": G.m,
           "budgets": "log-uniform [1e3, %.0e]" % args.serve_budget_max, "sp": 0.2,
           "tick_walkers": args.serve_tick, "rates": []}
    out["top_k"] = args.serve_top_k
    runs = [(float(r), args.serve_top_k) for r in args.serve_rates.split(",")]
    if args.serve_top_k:
        runs.append((float(args.serve_rates.split(",")[1 if "," in args.serve_rates else 0]), 0))
    for k, (rate, top_k) in enumerate(runs):
        src = rng.integers(0, G.n, args.serve_queries)
        bud = loguniform_budgets(args.serve_queries, 1e3, args.serve_budget_max, 10 + k)
        # full vectors: reserve the page-locked result staging the largest ticks need
        with ptw.Server(G, sp=0.2, seed=3, tick_walkers=args.serve_tick, use_graph=True, top_k=top_k,
                        staging_mb=0 if top_k else 1024) as srv:
            r = ptw.open_loop(srv, src, bud, rate=rate, seed=k, query_id0=k << 20)
            st = srv.stats()
        line = {kk: r[kk] for kk in ("rate", "n", "qps", "p50_ms", "p99_ms", "mean_ms")}
        line["top_k"] = top_k
        line["steps_per_s"] = st["moves"] / r["span_s"]
        line["server"] = {kk: st[kk] for kk in ("ticks", "moves", "walkers", "entries", "retries", "step_ms",
                                                 "device_ms", "collect_ms")}
        out["rates"].append(line)
    G.close()
    return out


def bench_learned(args, ptw):
    """Learned walker budgets against the fixed plain budget of 1e6 walkers
    per query (sp 0.2), scored by the FP64 oracle on held-out queries, on
    three workloads: R-MAT scale 22 with degree-proportional sources (the
    configuration's own: args.learned_train training and args.learned_test
    held-out queries), R-MAT scale 22 with uniform sources and the Chung-Lu
    serving graph (half the training and half the held-out queries).  Each
    line gives the gain at equal 90th-percentile L1 and at equal mean L1,
    and the ceiling the needed budgets themselves allow for each."""
    import numpy as np
    from ptwalker_gb300 import learned
    out = {"fixed_budget": 1_000_000, "sp": 0.2, "workloads": []}
    nt, ne = args.learned_train, args.learned_test

    def one(name, G, train, test):
        t0 = time.perf_counter()
        r = learned.evaluate(G, train, test, b_fix=1_000_000, sp=0.2, seed=5, epochs=300)
        r.pop("train_loss", None)
        r.update(workload=name, vertices=G.n, edges=G.m, seconds=time.perf_counter() - t0)
        out["workloads"].append(r)

    G = ptw.Graph.rmat(args.batch_scale, 16, 0.57, 0.19, 0.19, seed=1, clean=True)
    one("rmat-s%d degree-proportional sources" % args.batch_scale, G, degree_sources(G, nt, 21),
        degree_sources(G, ne, 22))
    names = G.export_csr()[0]
    rng = np.random.default_rng(23)
    one("rmat-s%d uniform sources" % args.batch_scale, G, names[rng.integers(0, G.n, nt // 2)],
        names[rng.integers(0, G.n, ne // 2)])
    G.close()
    G = ptw.Graph.chung_lu(args.serve_n, 2.1, 32.0, seed=1)
    names = G.export_csr()[0]
    one("chung-lu n=%d uniform sources" % args.serve_n, G, names[rng.integers(0, G.n, nt // 2)],
        names[rng.integers(0, G.n, ne // 2)])
    G.close()
    return out


# ---- our arm ----------------------------------------------------------------------

def tune_cache_path():
    return os.path.join(ROOT, "ptwalker_gb300", "_lib", "tune_cache.json")


def get_tune(G, ptw, args, dev_name):
    key = "%s|s%d|ef%d|seed%d|n%d|m%d|sp%g" % (dev_name, args.scale, args.edge_factor, args.seed,
                                               G.n, G.m, args.sp)
    if args.tune:
        v = [int(x) for x in args.tune.split(",")]
        names = ["block", "ilp", "chunk", "hot_k", "min_blocks", "paths_ilp", "cache_hints", "paths_named",
                 "ext_columns", "gather_slots", "warp_agg"]
        G.tune = ptw.Tune(**dict(zip(names, v)))
        return G.tune, "fixed"
    path = tune_cache_path()
    cache = {}
    if os.path.exists(path):
        try:
            cache = json.load(open(path))
        except Exception:
            cache = {}
    if key in cache:
        G.tune = ptw.Tune(**cache[key])
        return G.tune, "cache"
    if args.no_autotune:
        return G.tune, "default"
    t = G.autotune(args.sp, 0)
    cache[key] = t.as_dict()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as f:
            json.dump(cache, f, indent=1)
    except Exception:
        pass
    return t, "autotune"


def graph_replay(G, ptw, torch, stream, args, seeds, d_counts, first, total_moves):
    """The timed steps again, captured into one CUDA graph and replayed once
    (same seeds, so the same moves): the step loop without host launch gaps."""
    try:
        cg = torch.cuda.CUDAGraph()
        torch.cuda.synchronize()
        with torch.cuda.graph(cg, stream=stream):
            for k in range(args.steps):
                ptw.pagerank(G, G.n, args.sp, seeds[k], "per_vertex", out=d_counts, first_walker=first)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):  # replay where the events are recorded
            cg.replay()  # warm-up replay
            torch.cuda.synchronize()
            e0.record(stream)
            cg.replay()
            e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        del cg
        # the replay's last step left its counts in d_counts: check them
        # against the same step run directly
        direct = torch.empty_like(d_counts)
        ptw.pagerank(G, G.n, args.sp, seeds[-1], "per_vertex", out=direct, first_walker=first)
        torch.cuda.synchronize()
        return {"steps": args.steps, "ms_per_step": ms / args.steps, "value": total_moves / (ms / 1000.0),
                "unit": UNIT, "last_step_equals_direct_call": bool(torch.equal(direct, d_counts))}
    except Exception as e:  # report, do not fail the headline
        torch.cuda.synchronize()
        return {"error": "%s: %s" % (type(e).__name__, e)}


def run_ours(args):
    import numpy as np
    import torch
    import torch.distributed as dist

    import ptwalker_gb300 as ptw

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev_name = torch.cuda.get_device_name(local)

    t0 = time.perf_counter()
    G = ptw.Graph.rmat(args.scale, args.edge_factor, 0.57, 0.19, 0.19, seed=args.seed, clean=True)
    build_s = time.perf_counter() - t0
    tune, tune_src = get_tune(G, ptw, args, dev_name)
    stream = torch.cuda.Stream()
    G.set_stream(stream)
    n = G.n
    first = rank * n
    d_counts = torch.empty(G.id_bound, dtype=torch.int32, device="cuda")
    seeds = [args.seed * 7919 + 100 + k for k in range(args.steps)]

    def step(seed, out):
        ptw.pagerank(G, n, args.sp, seed, "per_vertex", out=out, first_walker=first)
        if world > 1:
            with torch.cuda.stream(stream):
                dist.all_reduce(d_counts)

    for k in range(args.warmup):
        step(10 + k, d_counts)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()

    clocks = Clocks(local)
    clocks.start()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    evs[0].record(stream)
    for k in range(args.steps):
        step(seeds[k], d_counts)
        evs[k + 1].record(stream)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clk = clocks.stop()
    per_step = [evs[k].elapsed_time(evs[k + 1]) for k in range(args.steps)]
    t_ms = evs[0].elapsed_time(evs[-1])
    if world > 1:
        tt = torch.tensor([t_ms], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_ms = float(tt.item())

    # moves of each timed step (a pure function of the seed: re-run with stats)
    moves, kern_ms = [], []
    for k in range(args.steps):
        _, st = ptw.pagerank(G, n, args.sp, seeds[k], "per_vertex", out=d_counts,
                             first_walker=first, stats=True)
        moves.append(st.moves)
        kern_ms.append(st.kernel_ms)
    total_moves = sum(moves) * world
    value = total_moves / (t_ms / 1000.0)

    # roofline of the walk kernel: 64 B per move + 32 B per counted visit
    bytes_per_launch = [64 * mv + 32 * (n + mv) for mv in moves]
    launch_ms = sum(per_step) / len(per_step)
    achieved = (sum(bytes_per_launch) / len(bytes_per_launch)) / (launch_ms / 1000.0) / 1e9
    peak, peak_kind = measured_peaks()

    # e2e through the host-facing call: counts copied into pinned host memory
    e2e = None
    if world == 1:
        host = torch.empty(G.id_bound, dtype=torch.int32, pin_memory=True)
        for k in range(2):
            ptw.pagerank(G, n, args.sp, 10 + k, "per_vertex", out=host)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        e0.record(stream)
        for k in range(args.steps):
            ptw.pagerank(G, n, args.sp, seeds[k], "per_vertex", out=host)
        e1.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - w0
        e_ms = e0.elapsed_time(e1)
        sync_e2e = {"value": sum(moves) / (e_ms / 1000.0), "unit": UNIT, "host_wall_value": sum(moves) / wall,
                    "api": "ptw_pagerank (synchronous: each call returns with its counts on the host)"}
        # The same walks through the pipelined pair (ptw_pagerank_submit /
        # ptw_pagerank_wait, two calls in flight): each step's counts still
        # reach pinned host memory inside the timed region, while the next
        # step walks.  Host wall clock from the first submit to the last wait.
        hosts = [host, torch.empty(G.id_bound, dtype=torch.int32, pin_memory=True)]
        for k in range(2):
            ptw.pagerank_wait(G, ptw.pagerank_submit(G, hosts[k], n, args.sp, 10 + k, "per_vertex"))
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        pend, p_moves = [], 0
        for k in range(args.steps):
            if len(pend) == 2:
                p_moves += ptw.pagerank_wait(G, pend.pop(0)).moves
            pend.append(ptw.pagerank_submit(G, hosts[k % 2], n, args.sp, seeds[k], "per_vertex"))
        for t in pend:
            p_moves += ptw.pagerank_wait(G, t).moves
        p_wall = time.perf_counter() - w0
        # e2e: the walks through the library's call for walk after walk, host
        # wall clock from the first submit to the last wait; every step's
        # counts reach pinned host memory inside that time
        e2e = {"value": p_moves / p_wall, "unit": UNIT, "h2d_bytes_per_step": 0,
               "d2h_bytes_per_step": 4 * G.id_bound,
               "api": "ptw_pagerank_submit / ptw_pagerank_wait, two calls in flight (host wall clock)",
               "same_moves_as_device_loop": p_moves == sum(moves), "synchronous": sync_e2e}

    # DeepWalk side line: one walker per vertex, L = walk_len, paths in HBM
    deepwalk = None
    if not args.no_deepwalk and world == 1:
        L = args.walk_len
        paths = torch.empty((n, L), dtype=torch.int32, device="cuda")
        ptw.deepwalk(G, n, L, 5, out=paths)
        d0 = torch.cuda.Event(enable_timing=True)
        d1 = torch.cuda.Event(enable_timing=True)
        reps = max(2, min(args.steps, 5))
        torch.cuda.synchronize()
        d0.record(stream)
        for k in range(reps):
            ptw.deepwalk(G, n, L, 50 + k, out=paths)
        d1.record(stream)
        torch.cuda.synchronize()
        dms = d0.elapsed_time(d1) / reps
        dsteps = n * (L - 1)
        dbytes = 64 * dsteps + 4 * n * L
        deepwalk = {"walk_len": L, "walkers": n, "steps_per_s": dsteps / (dms / 1000.0),
                    "ms_per_step": dms, "achieved_gbs": dbytes / (dms / 1000.0) / 1e9,
                    "frac": dbytes / (dms / 1000.0) / 1e9 / peak,
                    "path_bytes": 4 * n * L,
                    "kernel": "k_lane_paths" if tune.ext_columns & 2 else "k_paths"}
        # paths delivered to page-locked host memory through ptw_deepwalk
        # (walker chunks whose copies overlap the next chunks' walks); host
        # wall clock per call
        try:
            hpaths = torch.empty((n, L), dtype=torch.int32, pin_memory=True)
            ptw.deepwalk(G, n, L, 6, out=hpaths)
            w0 = time.perf_counter()
            for k in range(reps):
                ptw.deepwalk(G, n, L, 70 + k, out=hpaths)
            hs = (time.perf_counter() - w0) / reps
            deepwalk["e2e_host"] = {"steps_per_s": dsteps / hs, "ms_per_call": 1e3 * hs,
                                    "d2h_bytes_per_call": 4 * n * L,
                                    "api": "ptw_deepwalk into page-locked host memory (host wall clock)"}
            del hpaths
        except Exception as e:  # a side measurement must not cost the line
            deepwalk["e2e_host"] = {"error": "%s: %s" % (type(e).__name__, e)}
        # node2vec side line (second-order walks, same walkers and length):
        # algorithmic bytes = 64 B per candidate draw (row record + column
        # sector, as a DeepWalk move) + 32 B per neighbour test (one filter
        # sector) + 32 B per probe of the previous vertex's row + 4 B per
        # path entry
        node2vec = []
        for p_, q_ in ((2.0, 0.5), (0.5, 2.0)):
            _, st = ptw.node2vec(G, n, L, p_, q_, 5, out=paths, stats=True)
            torch.cuda.synchronize()
            d0.record(stream)
            for k in range(reps):
                ptw.node2vec(G, n, L, p_, q_, 60 + k, out=paths)
            d1.record(stream)
            torch.cuda.synchronize()
            nms = d0.elapsed_time(d1) / reps
            nbytes = 64 * st.trials + 32 * st.checks + 32 * st.probes + 4 * n * L
            node2vec.append({"p": p_, "q": q_, "walk_len": L, "walkers": n, "ms_per_step": nms,
                             "steps_per_s": st.moves / (nms / 1000.0),
                             "trials_per_move": st.trials / st.moves, "checks_per_move": st.checks / st.moves,
                             "probes_per_move": st.probes / st.moves,
                             "achieved_gbs": nbytes / (nms / 1000.0) / 1e9,
                             "frac": nbytes / (nms / 1000.0) / 1e9 / peak, "kernel": "k_lane_paths"})
        deepwalk["node2vec"] = node2vec
        del paths

    # DRAM bytes per walk launch: the ncu capture's bytes per move at this
    # workload (committed summary) times this run's moves per launch.
    traffic, traffic_src = None, None
    ext_walk = bool(tune.ext_columns & 1)
    per_move = traffic_per_move(args.scale, ext_walk)
    if per_move:
        traffic = per_move * sum(moves) / len(moves)
        traffic_src = TRAFFIC_SOURCE % ("extended" if ext_walk else "plain")
    # Random-gather ceiling measured on this GPU: a move is one dependent
    # random gather into the column array (2 GB > L2), so moves/s over this
    # rate is the kernel's share of what random access can deliver.
    gather = None
    if rank == 0:
        g_rate = ptw.probe_gather(2 << 30, 8)
        gather = {"loads_per_s": g_rate, "array_bytes": 2 << 30,
                  "moves_per_s_over_loads_per_s": value / world / g_rate}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        names, row_ptr, col = G.export_csr()
        import oracle
        canon = oracle.CanonicalGraph(names=names, row_ptr=row_ptr, col=col)
        threads = os.cpu_count() or 1
        oracle.replay.degree_relabelled(canon, threads)  # graph-load work, as in the reference
        S, mv, dt = cpu_port_sample(canon, args.sp, 4242, threads, target_s=3.0)
        cpu = {"value": mv / dt, "unit": UNIT, "cores": threads, "kind": "port", "port": PORT_KIND,
               "calibration": PORT_CALIBRATION,
               "sample": "first %d of %d walkers (per-vertex starts) of the same workload, %d moves "
                         "in %.2f s" % (S, n, mv, dt)}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": config(args, world),
        "e2e": e2e,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "traffic_source": traffic_src,
                     "peak_kind": peak_kind,
                     "gather_peak": gather,
                     "bytes_per_launch": sum(bytes_per_launch) / len(bytes_per_launch),
                     "launch_ms": launch_ms, "walk_kernel_ms": sum(kern_ms) / len(kern_ms)},
        "cpu_baseline": cpu,
        "gpu_launches": args.steps * 2,  # k_walk + k_counts_by_name per step
        "clocks": clk,
        "graph": {"vertices": n, "edges": G.m, "max_degree": G.max_degree, "build_s": build_s,
                  "device_bytes": G.device_bytes},
        "tune": dict(tune.as_dict(), source=tune_src),
        "moves_per_step": sum(moves) / len(moves),
        "deepwalk": deepwalk,
    }
    if world == 1:
        line["graph_replay"] = graph_replay(G, ptw, torch, stream, args, seeds, d_counts, first,
                                            sum(moves))
    G.set_stream(None)
    G.close()
    if rank == 0 and world == 1:
        for key, flag, fn in (("batched_ppr", args.no_batch, bench_batch), ("serving", args.no_serve, bench_serve),
                              ("ingest", args.no_ingest, bench_ingest),
                              ("learned_budgets", args.no_learned, bench_learned)):
            if flag:
                continue
            try:
                line[key] = fn(args, ptw)
            except Exception as e:  # a side line must not cost the headline
                line[key] = {"error": "%s: %s" % (type(e).__name__, e)}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
