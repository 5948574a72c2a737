"""The index-checked build of the library (-DPTW_CHECKED) on the GPU.

Every index the kernels derive from data (vertex ids, CSR entries, count
table slots, query entries, path positions, edge-filter blocks) is checked
against its bound; a failure is recorded on the device, the access is kept
in bounds, and the entry point returns PTW_ECUDA.  The same workloads run
under the checked and the normal build in child processes: none may trip a
check, and both must give the same results.  The workloads cover every
walk kernel and launch variant, batches with dense and hash tables, served
queries, and the batched workload whose extended-column kernel an ncu
capture once failed on (R-MAT scale 22, 256 queries, budgets up to 1e6).
"""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKLOAD = r"""
import hashlib, json, sys
import numpy as np
import ptwalker_gb300 as ptw
from ptwalker_gb300 import _capi

out = {"lib": _capi.lib_path()}
def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()[:16]

G = ptw.Graph.rmat(16, 16, 0.57, 0.19, 0.19, seed=1, clean=True)
tunes = {"default": ptw.Tune(),
         "ext_512x4": ptw.Tune(block=512, ilp=4, chunk=64, hot_k=8192, ext_columns=3, paths_ilp=1),
         "plain_1024x2": ptw.Tune(block=1024, ilp=2, chunk=256, hot_k=8192, ext_columns=0, paths_named=0),
         "agg": ptw.Tune(block=256, ilp=2, chunk=64, hot_k=2048, warp_agg=1, ext_columns=1),
         "slots": ptw.Tune(block=256, ilp=2, chunk=64, hot_k=0, gather_slots=8)}
for name, t in tunes.items():
    G.tune = t
    out["pagerank_" + name] = digest(ptw.pagerank(G, 3 * G.n, 0.15, 5, "uniform"))
    out["rwr_" + name] = digest(ptw.rwr(G, G.n, 0.3, 6))
    out["deepwalk_" + name] = digest(ptw.deepwalk(G, 20000, 30, 7, "uniform"))
G.tune = ptw.Tune()
for p, q in ((2.0, 0.5), (0.5, 2.0), (0.25, 4.0)):
    out["node2vec_%g_%g" % (p, q)] = digest(ptw.node2vec(G, 20000, 25, p, q, 8, "uniform"))
rng = np.random.default_rng(3)
src = rng.integers(0, G.n, 64)
bud = np.exp(rng.uniform(np.log(1e2), np.log(3e5), 64)).astype(np.int64)
for ext in (0, 1):
    ptw.set_batch_tune(G, ptw.BatchTune(ext_columns=ext, dense_ratio=2))
    for top_k in (0, 50):
        r = ptw.ppr_batch(G, src, bud, sp=0.2, seed=9, top_k=top_k)
        out["batch_ext%d_top%d" % (ext, top_k)] = digest(*[np.concatenate(r.query(i)) for i in range(64)])
        r.close()
with ptw.Server(G, sp=0.2, seed=3, tick_walkers=1 << 14, top_k=0) as srv:
    for i in range(24):
        srv.submit(int(src[i]), int(bud[i]), i)
    res = sorted(srv.drain(), key=lambda r: r["query_id"])
    out["serve"] = digest(*[np.concatenate([r["names"], r["counts"]]) for r in res])
G.close()

# the batched workload an ncu capture of the extended-column kernel failed on
G = ptw.Graph.rmat(22, 16, seed=1, clean=True)
names, row_ptr, col = G.export_csr()
rng = np.random.default_rng(2)
src = names[col[rng.integers(0, G.m, 256)]]
bud = np.exp(rng.uniform(np.log(1e3), np.log(1e6), 256)).astype(np.int64)
ptw.set_batch_tune(G, ptw.BatchTune(desc_walkers=256, blocks_per_sm=6, group_bytes=402653184, dense_ratio=2,
                                    ext_columns=1))
for seed in (1, 2):
    r = ptw.ppr_batch(G, src, bud, sp=0.2, seed=seed)
    out["batch_s22_ext_seed%d" % seed] = digest(*[np.concatenate(r.query(i)) for i in range(0, 256, 5)])
    r.close()
G.close()
print(json.dumps(out))
"""


def run(checked):
    env = dict(os.environ)
    env.pop("PTW_CHECKED", None)
    if checked:
        env["PTW_CHECKED"] = "1"
    r = subprocess.run([sys.executable, "-c", WORKLOAD], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_checked_build_trips_no_check_and_matches(gpu):
    from ptwalker_gb300 import _build

    _build.build_checked()
    checked = run(True)
    normal = run(False)
    assert checked.pop("lib").endswith(os.path.join("checked", "libptw.so"))
    assert not normal.pop("lib").endswith(os.path.join("checked", "libptw.so"))
    assert checked == normal
