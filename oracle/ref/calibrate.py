"""Times the reference's own pagerank binary beside the oracle port.

TEST / MEASUREMENT INFRASTRUCTURE.  The GPU host has no copy of the
reference tree and this image has no aarch64 cross compiler, so the CPU
baseline there is the oracle port (oracle/oracle.c: the same walker
semantics, OpenMP over walkers).  This script measures, on one host, how
the port's rate compares with the reference binary's (built by
oracle/ref/build_ref.py) on the same graph, walker count, stop probability
and thread count, so that the port's rate on the GPU host can be read
against the reference's.

Workload: R-MAT scale S (edge factor 16, a/b/c = .57/.19/.19, seed 1,
cleaned), W = |V| walkers, sp 0.15.  The reference starts its walkers
uniformly at random (src/core/pagerank.cpp:70-80) and the port is run with
uniform starts too.  Reference time = its own walk timer (walker init plus
walk, graph load excluded: src/core/solver.hpp:1055-1073), the median of
`reps` epochs; port time = replay_counts wall time, the median of `reps`.
Steps = visits - W for both.

Usage: PTW_REFERENCE_DIR=/path/to/reference python oracle/ref/calibrate.py [--scales 16,20] [--reps 5]
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
    scales = [16, 20]
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
            subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            meta = json.load(open(js))
        ref_s = sorted(meta["walk_s"])[len(meta["walk_s"]) // 2]
        ref_rate = meta["steps"] / ref_s
        rates = []
        for k in range(reps):
            t0 = time.perf_counter()
            _, moves = oracle.replay_counts(canon, 0, W, 0.15, 100 + k, START_UNIFORM, threads=threads)
            rates.append(moves / (time.perf_counter() - t0))
        port_rate = sorted(rates)[len(rates) // 2]
        out["graphs"].append({"scale": scale, "vertices": canon.n, "edges": canon.m, "walkers": W,
                              "reference_steps_per_s": ref_rate, "port_steps_per_s": port_rate,
                              "reference_over_port": ref_rate / port_rate})
    print(json.dumps(out))


if __name__ == "__main__":
    main()
