"""Host-side logic on the CPU: the open-loop load generator of the serving
layer, driven by a fake server that completes every submitted query one
tick after it was submitted."""
import time

import numpy as np

from ptwalker_gb300.serving import open_loop


class FakeServer:
    """Clock, submit and step as ptwalker_gb300.serving.Server has them; a
    step finishes every query submitted before it, tick_s later."""

    def __init__(self, tick_s=0.001):
        self.tick_s = tick_s
        self.queue = []
        self.n_active = 0
        self.n_pending = 0
        self.copy_flags = []

    def clock(self):
        return time.perf_counter()

    def submit(self, source, budget, query_id):
        self.queue.append(dict(query_id=query_id, source=source, budget=budget, submit_s=self.clock()))
        self.n_pending = len(self.queue)

    def step(self, take=True, copy=True):
        self.copy_flags.append(copy)
        time.sleep(self.tick_s)
        done, self.queue = self.queue, []
        self.n_pending = 0
        now = self.clock()
        out = []
        for q in done:
            names = np.arange(3, dtype=np.uint32)
            out.append(dict(q, names=names, counts=names + 1, admit_s=q["submit_s"], done_s=now))
        return out


def test_open_loop_latencies_and_rate():
    srv = FakeServer(tick_s=0.001)
    n, rate = 60, 2000.0
    r = open_loop(srv, np.arange(n), np.full(n, 100), rate=rate, seed=1, query_id0=500)
    assert r["n"] == n
    assert 0 < r["p50_ms"] <= r["p99_ms"] < 1000
    assert r["mean_ms"] > 0
    assert 0 < r["qps"] <= 10 * rate
    assert "results" not in r
    assert srv.copy_flags and not any(srv.copy_flags)   # nothing kept: no copies asked for


def test_open_loop_keeps_results_with_copies():
    srv = FakeServer(tick_s=0.0005)
    n = 20
    r = open_loop(srv, np.arange(n) + 7, np.full(n, 50), rate=5000.0, seed=2, keep_results=True)
    assert sorted(r["results"]) == list(range(n))
    assert all(r["results"][i]["source"] == i + 7 for i in range(n))
    assert all(srv.copy_flags)
