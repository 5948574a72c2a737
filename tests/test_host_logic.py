"""Host-side logic on the CPU: the open-loop load generator of the serving
layer, driven by a fake server that completes every submitted query one
tick after it was submitted; the learned-budget labels (log-log
interpolation of the error curve) and the sparse L1 between two results."""
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


def test_budget_labels_interpolate_the_grid():
    from ptwalker_gb300 import learned
    grid = np.array([1000, 2000, 4000, 8000])
    errs = np.array([[0.4, 0.28, 0.2, 0.14], [0.1, 0.07, 0.05, 0.035], [1.0, 0.9, 0.8, 0.7]])
    lb = learned.needed_budget(errs, grid, 0.2)
    assert abs(np.exp(lb[0]) - 4000) < 1e-6
    assert np.exp(lb[1]) < 1000          # below the grid: extrapolated down
    assert np.exp(lb[2]) > 8000          # above the grid: extrapolated up


def test_sparse_l1_equals_dense_l1():
    from ptwalker_gb300 import learned
    rng = np.random.default_rng(5)
    for _ in range(50):
        n = int(rng.integers(1, 200))
        a = rng.integers(0, 4, n) * (rng.random(n) < 0.5)
        b = rng.integers(0, 4, n) * (rng.random(n) < 0.5)
        na, nb = np.nonzero(a)[0].astype(np.uint32), np.nonzero(b)[0].astype(np.uint32)
        got = learned.sparse_l1(na, a[na].astype(np.uint32), nb, b[nb].astype(np.uint32))
        pa = a / max(a.sum(), 1)
        pb = b / max(b.sum(), 1)
        assert abs(got - np.abs(pa - pb).sum()) < 1e-12
