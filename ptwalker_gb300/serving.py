"""Serving loop with continuous batching (ptw_serve_*), and an open-loop
load generator that replays Poisson arrivals in real time and reports
p50/p99 latency beside throughput.

Queries are submitted as they arrive; every `step()` admits waiting queries
whose count tables fit the device arena, runs one tick in which all active
queries share the GPU, and hands back the queries that completed.
"""
import ctypes
import time

import numpy as np

from . import _capi as C
from .batch import APPS


class Server:
    def __init__(self, graph, sp=0.2, seed=0, app="visits", max_moves=0, table_bytes=0,
                 tick_walkers=0, max_active=0, use_graph=True, table_factor=0.0, top_k=0, staging_mb=0):
        self._lib = C.load()
        self.graph = graph
        cfg = C.ServeCfg(float(sp), int(seed) & 0xFFFFFFFFFFFFFFFF, APPS[app], int(max_moves),
                         int(table_bytes), int(tick_walkers), int(max_active), int(bool(use_graph)),
                         float(table_factor), int(top_k), int(staging_mb))
        h = ctypes.c_void_p()
        C.check(self._lib.ptw_serve_open(graph.handle, ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self.n_active = 0
        self.n_pending = 0

    def save(self, path):
        """Writes the server's state between steps (ptw_serve_save)."""
        C.check(self._lib.ptw_serve_save(self._h, str(path).encode()))

    @classmethod
    def restore(cls, graph, path):
        """A server on `graph` in the state saved at `path` (ptw_serve_restore)."""
        obj = cls.__new__(cls)
        obj._lib = C.load()
        obj.graph = graph
        h = ctypes.c_void_p()
        C.check(obj._lib.ptw_serve_restore(graph.handle, str(path).encode(), ctypes.byref(h)))
        obj._h = h
        st = obj.stats()
        obj.n_active, obj.n_pending = st["active"], st["pending"]
        return obj

    def clock(self):
        return float(self._lib.ptw_serve_clock(self._h))

    def submit(self, source, budget, query_id):
        q = C.Query(int(source), int(query_id), int(budget))
        C.check(self._lib.ptw_serve_submit(self._h, ctypes.byref(q)))

    def step(self, take=True, copy=True):
        """One admission + tick; returns the list of completed results as
        dicts with keys query_id, source, budget, names, counts, submit_s,
        admit_s, done_s.  take=False leaves them on the server for a later
        results() call; copy=False as in results()."""
        nd, na, npd = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        C.check(self._lib.ptw_serve_step(self._h, ctypes.byref(nd), ctypes.byref(na), ctypes.byref(npd)))
        self.n_active, self.n_pending = int(na.value), int(npd.value)
        return self.results(copy) if take else []

    def results(self, copy=True):
        """Takes every completed result the server holds.  copy=False gives
        names and counts as read-only views of the server's page-locked
        staging (no copy), valid until the next step()."""
        out = []
        r = C.ServeResult()
        pn, pc = ctypes.POINTER(ctypes.c_uint32)(), ctypes.POINTER(ctypes.c_uint32)()
        while self._lib.ptw_serve_poll(self._h, ctypes.byref(r)) == 1:
            ne = int(r.n_entries)
            if ne:
                # the entries sit in the page-locked block the device wrote them to
                C.check(self._lib.ptw_serve_view(self._h, ctypes.byref(pn), ctypes.byref(pc)))
                names = np.ctypeslib.as_array(pn, shape=(ne,))
                counts = np.ctypeslib.as_array(pc, shape=(ne,))
                if copy:
                    names, counts = names.copy(), counts.copy()
                else:
                    names.flags.writeable = False
                    counts.flags.writeable = False
            else:
                names = np.empty(0, dtype=np.uint32)
                counts = np.empty(0, dtype=np.uint32)
            C.check(self._lib.ptw_serve_take(self._h, None, None))
            out.append(dict(query_id=int(r.query_id), source=int(r.source), budget=int(r.budget),
                            names=names, counts=counts, submit_s=float(r.submit_s),
                            admit_s=float(r.admit_s), done_s=float(r.done_s)))
        return out

    def stats(self):
        """Counters since open (ptw_serve_stats) as a dict."""
        st = C.ServeStats()
        C.check(self._lib.ptw_serve_get_stats(self._h, ctypes.byref(st)))
        return {f: getattr(st, f) for f, _ in st._fields_}

    def drain(self):
        out = []
        while True:
            out.extend(self.step())
            if self.n_active == 0 and self.n_pending == 0:
                return out

    def close(self):
        if self._h:
            self._lib.ptw_serve_close(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def open_loop(server, sources, budgets, rate, seed=0, query_id0=0, keep_results=False):
    """Replays Poisson arrivals at `rate` queries/s in real time: a query is
    submitted once the server clock passes its arrival time, and its latency
    is completion time minus arrival time (queueing included)."""
    rng = np.random.default_rng(seed)
    n = len(sources)
    gaps = rng.exponential(1.0 / rate, n)
    arrive = np.cumsum(gaps)
    t0 = server.clock() + 0.01
    arrive = arrive + t0
    lat = np.zeros(n)
    done_at = np.zeros(n)
    results = {}
    nxt = 0
    n_done = 0
    while n_done < n:
        now = server.clock()
        while nxt < n and arrive[nxt] <= now:
            server.submit(sources[nxt], budgets[nxt], query_id0 + nxt)
            nxt += 1
        if server.n_active == 0 and server.n_pending == 0 and nxt < n and arrive[nxt] > now:
            # idle: no work until the next arrival
            time.sleep(min(arrive[nxt] - now, 0.002))
            if nxt < n and arrive[nxt] > server.clock():
                continue
        for r in server.step(copy=keep_results):
            i = r["query_id"] - query_id0
            lat[i] = r["done_s"] - arrive[i]
            done_at[i] = r["done_s"]
            n_done += 1
            if keep_results:
                results[i] = r
    span = done_at.max() - arrive.min()
    out = dict(n=n, rate=rate, qps=n / span, p50_ms=1000 * float(np.percentile(lat, 50)),
               p99_ms=1000 * float(np.percentile(lat, 99)), mean_ms=1000 * float(lat.mean()),
               span_s=float(span))
    if keep_results:
        out["results"] = results
    return out
