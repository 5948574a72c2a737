"""Learned walker budgets for PPR queries.

Each query needs a different number of walkers to reach a target L1 error:
a source whose PPR mass spreads widely needs more than one whose mass stays
near it.  The engine measures that need on its own runs, learns it from
cheap source features, and sizes each query's budget from the prediction.

  labels   for a training query, the budget-b estimates on a log grid of b
           are prefixes of one high-budget run of the same query id (draws
           depend on (query id, walker rank) only); the label is the budget
           b* at which L1(est_b, est_high) falls to the target eps, log-log
           interpolated on the grid (extrapolated with the 1/sqrt(b) law
           outside it);
  model    the 8 -> 64 -> 64 -> 1 MLP of libptw (ptw_mlp_*), trained on the
           GPU on log b* from the features of ptw_source_features;
  budget   b = clamp(kappa * exp(prediction), b_min, b_max), kappa set on the
           training queries so that a chosen share of them gets at least its
           b*; a fixed plain budget is the fallback when no model is given or
           a prediction is not finite.
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
    ca = counts_a.astype(np.float64) / max(int(counts_a.sum()), 1)
    cb = counts_b.astype(np.float64) / max(int(counts_b.sum()), 1)
    if len(names_b) == 0:
        return float(ca.sum())
    pos = np.searchsorted(names_b, names_a)
    pos_c = np.minimum(pos, len(names_b) - 1)
    hit = (pos < len(names_b)) & (names_b[pos_c] == names_a)
    l1 = np.abs(ca - np.where(hit, cb[pos_c], 0.0)).sum()
    only_b = np.ones(len(names_b), bool)
    only_b[pos_c[hit]] = False
    return float(l1 + cb[only_b].sum())


def grid_errors(graph, sources, grid, ref_budget, sp=0.2, seed=0, query_id0=0, chunk=512):
    """L1(est_b, est_ref) for every source and grid budget b; returns [ns, len(grid)]
    and the total moves spent.  The budget-b run of a query id is the first b
    walkers of its ref run.  Results stay in device memory and the L1 is
    summed on the device (ptw_batch_l1_pair)."""
    sources = np.atleast_1d(np.asarray(sources, dtype=np.uint32))
    out = np.empty((len(sources), len(grid)))
    moves = 0
    for c0 in range(0, len(sources), chunk):
        src = sources[c0:c0 + chunk]
        qids = np.arange(query_id0 + c0, query_id0 + c0 + len(src), dtype=np.uint32)
        ref = ppr_batch(graph, src, ref_budget, sp=sp, seed=seed, query_ids=qids, device_results=True)
        moves += ref.moves
        for k, b in enumerate(grid):
            run = ppr_batch(graph, src, int(b), sp=sp, seed=seed, query_ids=qids, device_results=True)
            moves += run.moves
            out[c0:c0 + len(src), k] = run.l1_vs(ref)
            run.close()
        ref.close()
    return out, moves


def needed_budget(errors, grid, eps):
    """Budget at which each row of errors (over the log grid) reaches eps."""
    grid = np.asarray(grid, dtype=np.float64)
    lg = np.log(grid)
    out = np.empty(errors.shape[0])
    for i, e in enumerate(errors):
        le = np.log(np.maximum(e, 1e-12))
        below = np.nonzero(e <= eps)[0]
        if len(below) == 0:  # beyond the grid: 1/sqrt(b) from the last point
            out[i] = lg[-1] + 2.0 * (le[-1] - np.log(eps))
        elif below[0] == 0:  # already below at the smallest budget
            out[i] = lg[0] - 2.0 * (np.log(eps) - le[0])
        else:
            k = below[0]
            t = (np.log(eps) - le[k - 1]) / (le[k] - le[k - 1]) if le[k] != le[k - 1] else 1.0
            out[i] = lg[k - 1] + t * (lg[k] - lg[k - 1])
    return out  # log budgets


class BudgetModel:
    """Features -> predicted log b* -> walker budget."""

    def __init__(self, seed=0):
        self.mlp = MLP(seed)
        self.kappa = 1.0

    def fit(self, graph, sources, log_budget, epochs=300, batch=256, lr=3e-3, seed=0, coverage=0.9):
        x = source_features(graph, sources)
        curve = self.mlp.train(x, np.asarray(log_budget, np.float32), epochs, batch, lr, seed)
        pred = self.mlp.forward(x).astype(np.float64)
        # kappa: the share `coverage` of training queries gets >= its b*
        self.kappa = float(np.quantile(np.exp(np.asarray(log_budget, np.float64) - pred), coverage))
        return curve

    def predict_log_budget(self, graph, sources):
        return self.mlp.forward(source_features(graph, sources)).astype(np.float64)

    def budgets(self, graph, sources, b_min=1000, b_max=1_000_000, fallback=1_000_000):
        b = self.kappa * np.exp(self.predict_log_budget(graph, sources))
        b = np.where(np.isfinite(b), np.clip(b, b_min, b_max), fallback)
        return b.astype(np.int64)

    # Model file read by the command-line apps (ppr --budget learned --model FILE):
    #   magic "PTWBUD1\0", f64 kappa, u64 b_min, b_max, fallback,
    #   f32 params[4801] (ptw_mlp_get_params order), f32 norm[18].
    MAGIC = b"PTWBUD1\0"

    def save(self, path, b_min=1000, b_max=1_000_000, fallback=1_000_000):
        params, norm = self.mlp.params()
        with open(path, "wb") as f:
            f.write(self.MAGIC)
            f.write(np.array([self.kappa], np.float64).tobytes())
            f.write(np.array([b_min, b_max, fallback], np.uint64).tobytes())
            f.write(np.ascontiguousarray(params, np.float32).tobytes())
            f.write(np.ascontiguousarray(norm, np.float32).tobytes())

    @classmethod
    def load(cls, path):
        """(model, (b_min, b_max, fallback)) from a file written by save()."""
        with open(path, "rb") as f:
            raw = f.read()
        if raw[:8] != cls.MAGIC:
            raise ValueError("%s is not a budget model" % path)
        kappa = float(np.frombuffer(raw, np.float64, 1, 8)[0])
        lim = np.frombuffer(raw, np.uint64, 3, 16)
        params = np.frombuffer(raw, np.float32, C.PTW_MLP_NPARAMS, 40).copy()
        norm = np.frombuffer(raw, np.float32, C.PTW_MLP_NNORM, 40 + 4 * C.PTW_MLP_NPARAMS).copy()
        m = cls()
        m.mlp.set_params(params, norm)
        m.kappa = kappa
        return m, tuple(int(x) for x in lim)


def plain_budgets(n, fixed=1_000_000):
    """The fallback / baseline: the same budget for every query."""
    return np.full(n, int(fixed), dtype=np.int64)


def label_ceilings(b_star):
    """What exact per-query budgets could save over one fixed budget, from
    the needed budgets b* of a set of queries.  Equal 90th-percentile error:
    the fixed budget must be p90(b*), exact budgets spend mean(b*).  Equal
    mean error (error of a query ~ c_q / sqrt(b), c_q ~ sqrt(b*_q)): the
    least total budget at a given mean error puts b_q ~ b*_q^(1/3), which
    saves mean(sqrt b*)^2 / mean(b*^(1/3))^3."""
    b = np.asarray(b_star, np.float64)
    return {"equal_p90": float(np.quantile(b, 0.9) / b.mean()),
            "equal_mean": float(np.mean(np.sqrt(b)) ** 2 / np.mean(np.cbrt(b)) ** 3)}


def evaluate(graph, train_src, test_src, b_fix, sp=0.2, seed=0, grid_points=7, ref_mult=8, coverage=0.9,
             epochs=300, b_min=None, l1_tol=1e-4, label_chunk=512):
    """Learned budgets vs the fixed budget b_fix on held-out queries, scored
    by the FP64 oracle (one power iteration shared by the three runs; the
    truncated series is within about 2 * l1_tol of exact in L1).

    eps is the fixed budget's 90th-percentile error on the training queries
    (measured against their high-budget runs); b* of a training query is
    the budget at which its error reaches eps.  Two budget rules from the
    same model:
      p90   b = kappa * exp(pred), kappa such that 90% of the training
            queries get at least their b* (equal 90th-percentile error);
      mean  b = lam * exp(pred)^(1/3), lam such that the predicted mean
            training error equals the fixed budget's (equal mean error).
    Returns a dict of the measured figures."""
    import time
    clock = [time.perf_counter()]
    stages = {}

    def stage(name):
        now = time.perf_counter()
        stages[name] = round(now - clock[0], 2)
        clock[0] = now

    grid = np.unique(np.geomspace(b_fix / 2 ** (grid_points - 1), b_fix * 2, grid_points + 1).astype(np.int64))
    ref_budget = int(b_fix * ref_mult)
    errs, label_moves = grid_errors(graph, train_src, grid, ref_budget, sp, seed, query_id0=1 << 20,
                                    chunk=label_chunk)
    stage("labels")
    k_fix = int(np.argmin(np.abs(grid - b_fix)))
    eps = float(np.quantile(errs[:, k_fix], 0.9))
    log_b = needed_budget(errs, grid, eps)
    model = BudgetModel(seed=seed)
    curve = model.fit(graph, train_src, log_b, epochs=epochs, coverage=coverage)
    stage("fit")
    b_min = b_min or int(grid[0])
    b_star = np.exp(np.asarray(log_b, np.float64))
    # equal-mean rule: error_q ~ eps * sqrt(b*_q / b_q); lam from the training labels
    pred_tr = np.exp(model.predict_log_budget(graph, train_src))
    lam = b_fix * (np.mean(np.sqrt(b_star / np.cbrt(pred_tr))) / np.mean(np.sqrt(b_star))) ** 2
    qids = np.arange(len(test_src), dtype=np.uint32) + (1 << 24)
    kw = dict(sp=sp, seed=seed + 1, query_ids=qids, device_results=True)
    fixed = ppr_batch(graph, test_src, b_fix, **kw)
    budgets = model.budgets(graph, test_src, b_min=b_min, b_max=4 * b_fix, fallback=b_fix)
    learned = ppr_batch(graph, test_src, budgets, **kw)
    pred_te = np.exp(model.predict_log_budget(graph, test_src))
    b_mean = np.where(np.isfinite(pred_te), np.clip(lam * np.cbrt(pred_te), b_min, 4 * b_fix),
                      b_fix).astype(np.int64)
    learned_mean = ppr_batch(graph, test_src, b_mean, **kw)
    stage("held_out_runs")
    from .batch import l1_many
    l1_f, l1_l, l1_m = l1_many(graph, [fixed, learned, learned_mean], tol=l1_tol)
    stage("fp64_scoring")
    out = dict(eps_train=eps, fixed_budget=int(b_fix), ref_budget=ref_budget, grid=[int(x) for x in grid],
               fixed_moves=int(fixed.moves),
               label_ceiling=label_ceilings(b_star),
               label_ceiling_first_half=label_ceilings(b_star[: len(b_star) // 2]),
               label_budget_quantiles=[float(np.quantile(b_star, q) / b_fix) for q in (0.1, 0.5, 0.9)],
               equal_p90={"learned_moves": int(learned.moves), "gain": fixed.moves / max(learned.moves, 1),
                          "fixed_l1_p90": float(np.quantile(l1_f, 0.9)),
                          "learned_l1_p90": float(np.quantile(l1_l, 0.9)),
                          "fixed_l1_p50": float(np.median(l1_f)), "learned_l1_p50": float(np.median(l1_l)),
                          "budget_min": int(budgets.min()), "budget_max": int(budgets.max()),
                          "budget_mean": float(budgets.mean()), "kappa": model.kappa},
               equal_mean={"learned_moves": int(learned_mean.moves),
                           "gain": fixed.moves / max(learned_mean.moves, 1),
                           "fixed_l1_mean": float(l1_f.mean()), "learned_l1_mean": float(l1_m.mean()),
                           "budget_min": int(b_mean.min()), "budget_max": int(b_mean.max()),
                           "budget_mean": float(b_mean.mean()), "lambda": float(lam)},
               label_moves=int(label_moves), train_loss=[float(curve[0]), float(curve[-1])],
               n_train=int(len(train_src)), n_test=int(len(test_src)), l1_tol=l1_tol, stage_seconds=stages)
    # the flat keys of the equal 90th-percentile rule
    out.update(gain=out["equal_p90"]["gain"], learned_moves=out["equal_p90"]["learned_moves"],
               fixed_l1_p90=out["equal_p90"]["fixed_l1_p90"], learned_l1_p90=out["equal_p90"]["learned_l1_p90"],
               ideal_gain_from_labels=out["label_ceiling"]["equal_p90"])
    for r in (fixed, learned, learned_mean):
        r.close()
    return out
