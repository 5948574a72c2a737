"""Learned walker budgets for PPR queries.

The Monte Carlo PPR estimate of a source s with b walkers has an L1 error
close to C_s / sqrt(b), where C_s depends on how widely s's PPR mass spreads.
The engine measures C_s on its own runs, learns it from cheap source
features, and sizes each query's budget for a target error:

  labels   C_s = L1(est_b0, est_B) / sqrt(1/b0 - 1/B): a budget-b0 run is the
           first b0 walkers of the budget-B run of the same query id (the
           draws depend on (query id, walker rank) only), so both come from
           one nested pair of runs of the method itself;
  model    the 8 -> 64 -> 64 -> 1 MLP of libptw (ptw_mlp_*), trained on the
           GPU on log C_s from the features of ptw_source_features;
  budget   b_s = clamp(kappa * (C_s_predicted / eps)^2, b_min, b_max), with
           kappa calibrated on the training queries so that a chosen share
           of them gets at least the budget they need; a fixed plain budget
           is the fallback when no model is given or a prediction is not
           finite.
"""
import ctypes

import numpy as np

from . import _capi as C
from .batch import ppr_batch


def _f32p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def source_features(graph, sources):
    src = np.ascontiguousarray(np.atleast_1d(sources), dtype=np.uint32)
    out = np.empty((src.shape[0], C.PTW_MLP_IN), dtype=np.float32)
    C.check(C.load().ptw_source_features(graph.handle, src.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                                         src.shape[0], _f32p(out)))
    return out


class MLP:
    """Handle on the device MLP (ptw_mlp_*)."""

    def __init__(self, seed=0):
        self._lib = C.load()
        h = ctypes.c_void_p()
        C.check(self._lib.ptw_mlp_create(int(seed), ctypes.byref(h)))
        self._h = h

    def params(self):
        p = np.empty(C.PTW_MLP_NPARAMS, dtype=np.float32)
        n = np.empty(C.PTW_MLP_NNORM, dtype=np.float32)
        C.check(self._lib.ptw_mlp_get_params(self._h, _f32p(p), _f32p(n)))
        return p, n

    def set_params(self, params=None, norm=None):
        p = None if params is None else np.ascontiguousarray(params, dtype=np.float32)
        n = None if norm is None else np.ascontiguousarray(norm, dtype=np.float32)
        C.check(self._lib.ptw_mlp_set_params(self._h, None if p is None else _f32p(p),
                                             None if n is None else _f32p(n)))

    def forward(self, x):
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.empty(x.shape[0], dtype=np.float32)
        C.check(self._lib.ptw_mlp_forward(self._h, _f32p(x), x.shape[0], _f32p(y)))
        return y

    def grad(self, x, t):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        g = np.empty(C.PTW_MLP_NPARAMS, dtype=np.float32)
        loss = ctypes.c_double()
        C.check(self._lib.ptw_mlp_grad(self._h, _f32p(x), _f32p(t), x.shape[0], ctypes.byref(loss), _f32p(g)))
        return float(loss.value), g

    def train(self, x, t, epochs=200, batch=256, lr=3e-3, seed=0):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        curve = np.empty(epochs, dtype=np.float32)
        C.check(self._lib.ptw_mlp_train(self._h, _f32p(x), _f32p(t), x.shape[0], batch, epochs, lr, int(seed),
                                        _f32p(curve)))
        return curve

    def close(self):
        if self._h:
            self._lib.ptw_mlp_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def sparse_l1(names_a, counts_a, names_b, counts_b):
    """L1 between two sparse count vectors (sorted names), each normalised."""
    ca = counts_a.astype(np.float64) / max(counts_a.sum(), 1)
    cb = counts_b.astype(np.float64) / max(counts_b.sum(), 1)
    pos = np.searchsorted(names_b, names_a)
    pos_c = np.minimum(pos, max(len(names_b) - 1, 0))
    hit = (pos < len(names_b)) & (names_b[pos_c] == names_a) if len(names_b) else np.zeros(len(names_a), bool)
    l1 = np.abs(ca - np.where(hit, cb[pos_c] if len(names_b) else 0.0, 0.0)).sum()
    only_b = np.ones(len(names_b), bool)
    only_b[pos_c[hit]] = False
    return float(l1 + cb[only_b].sum())


def error_constants(graph, sources, b0=2000, mult=16, sp=0.2, seed=0, query_id0=0, table_bytes=0):
    """Measured C_s per source from one nested pair of runs (see module doc)."""
    sources = np.atleast_1d(np.asarray(sources, dtype=np.uint32))
    qids = np.arange(query_id0, query_id0 + len(sources), dtype=np.uint32)
    lo = ppr_batch(graph, sources, b0, sp=sp, seed=seed, query_ids=qids, table_bytes=table_bytes)
    hi = ppr_batch(graph, sources, b0 * mult, sp=sp, seed=seed, query_ids=qids, table_bytes=table_bytes)
    scale = 1.0 / np.sqrt(1.0 / b0 - 1.0 / (b0 * mult))
    out = np.empty(len(sources))
    for i in range(len(sources)):
        na, ca = lo.query(i)
        nb, cb = hi.query(i)
        out[i] = sparse_l1(na, ca, nb, cb) * scale
    return out, lo.moves + hi.moves


class BudgetModel:
    """Features -> predicted log C_s -> walker budget for a target L1."""

    def __init__(self, seed=0):
        self.mlp = MLP(seed)
        self.kappa = 1.0

    def fit(self, graph, sources, log_c, epochs=300, batch=256, lr=3e-3, seed=0, coverage=0.9):
        x = source_features(graph, sources)
        curve = self.mlp.train(x, np.asarray(log_c, np.float32), epochs, batch, lr, seed)
        pred = self.mlp.forward(x).astype(np.float64)
        # kappa: the share `coverage` of training queries gets >= its need
        ratio2 = np.exp(2.0 * (np.asarray(log_c, np.float64) - pred))
        self.kappa = float(np.quantile(ratio2, coverage))
        return curve

    def predict_log_c(self, graph, sources):
        return self.mlp.forward(source_features(graph, sources)).astype(np.float64)

    def budgets(self, graph, sources, eps, b_min=1000, b_max=1_000_000, fallback=1_000_000):
        pred = self.predict_log_c(graph, sources)
        b = self.kappa * np.exp(2.0 * pred) / (eps * eps)
        b = np.where(np.isfinite(b), np.clip(b, b_min, b_max), fallback)
        return b.astype(np.int64)


def plain_budgets(n, fixed=1_000_000):
    """The fallback / baseline: the same budget for every query."""
    return np.full(n, int(fixed), dtype=np.int64)
