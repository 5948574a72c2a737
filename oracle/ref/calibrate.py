"""Times the reference's own pagerank binary beside the CPU ports.

TEST / MEASUREMENT INFRASTRUCTURE.  The GPU host has no copy of the
reference tree and this image has no aarch64 cross compiler, so the CPU
baseline there is a port: the partitioned port (oracle/partitioned.c: the
reference's partition sweeps and walker pools) and, for comparison, the
oracle's replay (oracle/oracle.c: OpenMP over walkers, atomic counters).
This script measures, on one host, how the ports' rates compare with the
reference binary's (built by oracle/ref/build_ref.py) on the same graph,
walker count, stop probability and thread count, so that a port's rate on
the GPU host can be read against the reference's.

Workload: R-MAT scale S (edge factor 16, a/b/c = .57/.19/.19, seed 1,
cleaned), W = |V| walkers, sp 0.15.  The reference starts its walkers
uniformly at random (src/core/pagerank.cpp:70-80) and the ports are run
with uniform starts too.  Reference time = its own walk timer (walker init plus
walk, graph load excluded: src/core/solver.hpp:1055-1073), the median of
`reps` epochs; port time = wall time of one call, the median of `reps`.
Steps = visits - W for both.

Usage: PTW_REFERENCE_DIR=/path/to/reference python oracle/ref/calibrate.py [--scales 16,20,22] [--reps 5]
Prints one JSON object.
"""
import json
import os
import platform
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from oracle.ref import build_ref  # noqa: E402
from oracle.replay import START_UNIFORM  # noqa: E402


def main():
    scales = [16, 20, 22]
    reps = 5
    if "--scales" in sys.argv:
        scales = [int(x) for x in sys.argv[sys.argv.index("--scales") + 1].split(",")]
    if "--reps" in sys.argv:
        reps = int(sys.argv[sys.argv.index("--reps") + 1])
    binary = build_ref.build()
    if binary is None:
        raise SystemExit("no reference tree: set PTW_REFERENCE_DIR")
    threads = os.cpu_count() or 1
    out = {"host": platform.machine(), "cores": threads, "sp": 0.15, "reps": reps, "graphs": []}
    for scale in scales:
        s, d = oracle.rmat_clean_edges(scale, 16, 0.57, 0.19, 0.19, 1)
        canon = oracle.canonical_from_edges(s, d)
        W = canon.n
        with tempfile.TemporaryDirectory() as td:
            path = os.path.join(td, "g.txt")
            oracle.write_text_edges(path, s, d)
            js = os.path.join(td, "r.json")
            cmd = [binary, "-f", "text", "-g", path, "-w", str(W), "--sp", "0.15", "-t", str(threads),
                   "--reps", str(reps), "--json", js]
            r = subprocess.run(cmd, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE, text=True)
            meta = json.load(open(js)) if r.returncode == 0 and os.path.exists(js) else None
        ref_rate = None
        if meta is not None:
            ref_s = sorted(meta["walk_s"])[len(meta["walk_s"]) // 2]
            ref_rate = meta["steps"] / ref_s
        def median_rate(fn):
            rates = []
            for k in range(reps):
                t0 = time.perf_counter()
                moves = fn(100 + k)
                rates.append(moves / (time.perf_counter() - t0))
            return sorted(rates)[len(rates) // 2]

        atomic = median_rate(lambda sd: oracle.replay_counts(canon, 0, W, 0.15, sd, START_UNIFORM,
                                                             threads=threads)[1])
        part = median_rate(lambda sd: oracle.partitioned_counts(canon, 0, W, 0.15, sd, START_UNIFORM,
                                                                threads=threads)[1])
        line = {"scale": scale, "vertices": canon.n, "edges": canon.m, "walkers": W,
                "reference_steps_per_s": ref_rate, "partitioned_port_steps_per_s": part,
                "atomic_port_steps_per_s": atomic}
        if ref_rate is None:
            line["reference_failed"] = "exit %d: %s" % (r.returncode, " | ".join(r.stderr.strip().splitlines()[-3:]))
        else:
            line.update(reference_over_partitioned_port=ref_rate / part, reference_over_atomic_port=ref_rate / atomic)
        out["graphs"].append(line)
        print(json.dumps(line), file=sys.stderr, flush=True)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
