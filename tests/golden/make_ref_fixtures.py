"""Generates the reference-binary fixtures in tests/golden/.

Runs the reference's own pagerank app (built from its sources by
oracle/ref/build_ref.py) and stores its visit counts by vertex name:

  ref_pagerank_s16.npz   R-MAT scale 16, edge factor 16, a/b/c = .57/.19/.19,
                         seed 1, cleaned; W = 10 * |V| uniform-start walkers,
                         --sp 0.15
  ref_pagerank_tiny.npz  a 7-vertex directed graph with a duplicate edge and
                         a self-loop; W = 400000, --sp 0.3

The reference's RNG is seeded from std::random_device, so these are one
draw of its output; the tests compare them statistically (z-scores against
the FP64 expectation).  Re-running this script gives different counts.

Usage (from the repo root; the reference tree is named as for
oracle/ref/build_ref.py):
    PTW_REFERENCE_DIR=/path/to/reference python tests/golden/make_ref_fixtures.py
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from oracle.ref import build_ref  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

TINY_EDGES = [(0, 1), (0, 2), (0, 2), (1, 2), (2, 0), (2, 3), (3, 3), (3, 4), (4, 0),
              (4, 5), (5, 6), (6, 4), (6, 1)]


def run_ref(binary, path, W, sp, threads=8):
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "counts.u32")
        js = os.path.join(td, "r.json")
        cmd = [binary, "-f", "text", "-g", path, "-w", str(W), "--sp", str(sp), "-t", str(threads),
               "--out", out, "--json", js]
        subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        counts = np.fromfile(out, dtype=np.uint32)
        meta = json.load(open(js))
    return counts, meta, cmd


def main():
    binary = build_ref.build()
    if binary is None:
        raise SystemExit("no reference tree: set PTW_REFERENCE_DIR (or build with oracle/ref/build_ref.py --ref)")
    with tempfile.TemporaryDirectory() as td:
        # scale-16 R-MAT
        s, d = oracle.rmat_clean_edges(16, 16, 0.57, 0.19, 0.19, 1)
        path = os.path.join(td, "s16.txt")
        oracle.write_text_edges(path, s, d)
        n = int(max(s.max(), d.max())) + 1
        W, sp = 10 * n, 0.15
        counts, meta, cmd = run_ref(binary, path, W, sp)
        np.savez_compressed(os.path.join(OUT, "ref_pagerank_s16.npz"), counts=counts, W=W, sp=sp,
                            scale=16, edge_factor=16, abc=np.array([0.57, 0.19, 0.19]), seed=1,
                            visits=meta["visits"], steps=meta["steps"],
                            cmd=" ".join(os.path.basename(c) if c.startswith(td) else c for c in cmd))
        # tiny graph with a duplicate edge and a self-loop
        path = os.path.join(td, "tiny.txt")
        with open(path, "w") as f:
            f.write("# tiny directed graph\n")
            for a, b in TINY_EDGES:
                f.write("%d %d\n" % (a, b))
        # One thread: with several threads the reference overflows its
        # per-partition pool lists once W is far above |V| and crashes.
        W, sp = 400000, 0.3
        counts, meta, cmd = run_ref(binary, path, W, sp, threads=1)
        np.savez_compressed(os.path.join(OUT, "ref_pagerank_tiny.npz"), counts=counts, W=W, sp=sp,
                            edges=np.array(TINY_EDGES, dtype=np.uint32), visits=meta["visits"],
                            steps=meta["steps"],
                            cmd=" ".join(os.path.basename(c) if c.startswith(td) else c for c in cmd))
    print("fixtures written to", OUT)


if __name__ == "__main__":
    main()
