"""Checkpoint / resume of long count walks.

Draws depend on (seed, global walker id, step) only, so a walk of W walkers
run as consecutive chunks [k, k + c) and summed equals the one-shot run bit
for bit.  A checkpoint is therefore just the counts accumulated so far, the
next walker id and the configuration they belong to.
"""
import json
import os

import numpy as np

from .api import pagerank


def _key(graph, n_walkers, sp, seed, start, sources, max_moves):
    return json.dumps(dict(n=graph.n, m=graph.m, id_bound=graph.id_bound, W=int(n_walkers), sp=float(sp),
                           seed=int(seed), start=start, max_moves=int(max_moves),
                           sources=None if sources is None else [int(x) for x in np.atleast_1d(sources)]),
                      sort_keys=True)


def resumable_pagerank(graph, path, n_walkers=None, sp=0.15, seed=0, start="per_vertex", sources=None,
                       max_moves=0, chunk=1 << 22, stop_after=None):
    """Count walk of n_walkers walkers in chunks, saving (counts, next walker)
    to `path` after every chunk and resuming from it when present.
    stop_after = number of chunks to run in this call (None = finish).
    Returns (counts, done)."""
    n_walkers = graph.n if n_walkers is None else int(n_walkers)
    key = _key(graph, n_walkers, sp, seed, start, sources, max_moves)
    counts = np.zeros(graph.id_bound, dtype=np.uint64)
    nxt = 0
    if os.path.exists(path):
        with np.load(path, allow_pickle=False) as z:
            if str(z["key"]) != key:
                raise ValueError("checkpoint %s belongs to another walk" % path)
            counts = z["counts"].astype(np.uint64)
            nxt = int(z["next"])
    runs = 0
    while nxt < n_walkers and (stop_after is None or runs < stop_after):
        c = min(chunk, n_walkers - nxt)
        part = pagerank(graph, c, sp, seed, start, sources, max_moves, first_walker=nxt)
        counts += part
        nxt += c
        runs += 1
        tmp = path + ".tmp.npz"
        np.savez(tmp, counts=counts, next=np.int64(nxt), key=np.array(key))
        os.replace(tmp, path)
    return counts, nxt >= n_walkers
