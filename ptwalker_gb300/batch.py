"""Batched single-source PPR / RWR (ptw_ppr_batch) and its FP64 error oracle.

A batch is a table of queries (source name, query id, walker budget).  The
reference answers one source per process (src/core/ppr.cpp:121-138); here
all queries of a batch share persistent walker launches, and each query's
counts stay sparse: (vertex name, count) pairs sorted by name.
"""
import ctypes

import numpy as np

from . import _capi as C

APPS = {"visits": C.PTW_APP_VISITS, "endpoint": C.PTW_APP_ENDPOINT}

PHASE_FIELDS = [f for f, _ in C.BatchPhases._fields_]


class _DeviceArray:
    """A device array the library owns, exposed through the CUDA array
    interface so torch.as_tensor wraps it without a copy."""

    def __init__(self, ptr, n, typestr):
        self.__cuda_array_interface__ = {"shape": (int(n),), "typestr": typestr, "data": (int(ptr), False),
                                         "version": 2}


class BatchTune:
    """Launch parameters of the batched walker kernel (ptw_batch_tune)."""

    FIELDS = [f for f, _ in C.BatchTune._fields_]

    def __init__(self, desc_walkers=0, blocks_per_sm=0, group_bytes=0, dense_ratio=0, ext_columns=0):
        self.desc_walkers, self.blocks_per_sm, self.group_bytes = desc_walkers, blocks_per_sm, group_bytes
        self.dense_ratio, self.ext_columns = dense_ratio, ext_columns

    def to_c(self):
        return C.BatchTune(int(self.desc_walkers), int(self.blocks_per_sm), int(self.group_bytes),
                           int(self.dense_ratio), int(self.ext_columns))

    @classmethod
    def from_c(cls, t):
        return cls(t.desc_walkers, t.blocks_per_sm, t.group_bytes, t.dense_ratio, t.ext_columns)

    def as_dict(self):
        return {f: int(getattr(self, f)) for f in self.FIELDS}

    def __repr__(self):
        return "BatchTune(%s)" % ", ".join("%s=%s" % kv for kv in self.as_dict().items())


def get_batch_tune(graph):
    t = C.BatchTune()
    C.check(graph._lib.ptw_graph_get_batch_tune(graph.handle, ctypes.byref(t)))
    return BatchTune.from_c(t)


def set_batch_tune(graph, tune):
    t = tune.to_c()
    C.check(graph._lib.ptw_graph_set_batch_tune(graph.handle, ctypes.byref(t)))


class BatchResult:
    """Sparse per-query results, held in host memory by the library (or, for
    a batch run with device_results=True, in device memory: d_offsets,
    d_names and d_counts are then zero-copy torch views of it and names /
    counts are None)."""

    def __init__(self, graph, handle, sources, budgets, query_ids, sp, app, device_results=False):
        self._lib = C.load()
        self._h = handle
        self.graph = graph
        self.sources = np.asarray(sources, dtype=np.uint32)
        self.budgets = np.asarray(budgets, dtype=np.uint64)
        self.query_ids = np.asarray(query_ids, dtype=np.uint32)
        self.sp, self.app = sp, app
        nq = ctypes.c_uint32()
        ne = ctypes.c_uint64()
        st = C.WalkStats()
        C.check(self._lib.ptw_batch_info(self._h, ctypes.byref(nq), ctypes.byref(ne), ctypes.byref(st)))
        self.nq, self.entries = int(nq.value), int(ne.value)
        self.walkers, self.moves, self.visits = int(st.walkers), int(st.moves), int(st.visits)
        self.ms = float(st.total_ms)
        self.kernel_ms = float(st.kernel_ms)
        # zero-copy views of the batch's host arrays (valid until close())
        po = ctypes.POINTER(ctypes.c_uint64)()
        pn = ctypes.POINTER(ctypes.c_uint32)()
        pc = ctypes.POINTER(ctypes.c_uint32)()
        C.check(self._lib.ptw_batch_view(self._h, ctypes.byref(po), ctypes.byref(pn), ctypes.byref(pc)))
        self.offsets = np.ctypeslib.as_array(po, shape=(self.nq + 1,))
        self.device_results = device_results
        self.d_offsets = self.d_names = self.d_counts = None
        if device_results:
            import torch
            C.check(self._lib.ptw_batch_view_device(self._h, ctypes.byref(po), ctypes.byref(pn),
                                                    ctypes.byref(pc)))
            self.d_offsets = torch.as_tensor(_DeviceArray(ctypes.addressof(po.contents), self.nq + 1, "<u8"),
                                             device="cuda")
            if self.entries:
                self.d_names = torch.as_tensor(_DeviceArray(ctypes.addressof(pn.contents), self.entries, "<u4"),
                                               device="cuda")
                self.d_counts = torch.as_tensor(_DeviceArray(ctypes.addressof(pc.contents), self.entries, "<u4"),
                                                device="cuda")
            self.names = self.counts = None
        elif self.entries:
            self.names = np.ctypeslib.as_array(pn, shape=(self.entries,))
            self.counts = np.ctypeslib.as_array(pc, shape=(self.entries,))
        else:
            self.names = np.empty(0, dtype=np.uint32)
            self.counts = np.empty(0, dtype=np.uint32)

    def query(self, i):
        a, b = int(self.offsets[i]), int(self.offsets[i + 1])
        if self.device_results:
            if b == a:
                return np.empty(0, dtype=np.uint32), np.empty(0, dtype=np.uint32)
            return (self.d_names[a:b].cpu().numpy().view(np.uint32),
                    self.d_counts[a:b].cpu().numpy().view(np.uint32))
        return self.names[a:b], self.counts[a:b]

    def export(self):
        """(offsets, names, counts) copied into new host arrays (ptw_batch_export)."""
        off = np.empty(self.nq + 1, dtype=np.uint64)
        names = np.empty(self.entries, dtype=np.uint32)
        counts = np.empty(self.entries, dtype=np.uint32)
        C.check(self._lib.ptw_batch_export(self._h, off.ctypes.data_as(C._u64p), names.ctypes.data_as(C._u32p),
                                           counts.ctypes.data_as(C._u32p)))
        return off, names, counts

    def phases(self):
        """Where the call's time went (ptw_batch_get_phases): device phases
        from CUDA events, host phases from the wall clock; milliseconds."""
        p = C.BatchPhases()
        C.check(self._lib.ptw_batch_get_phases(self._h, ctypes.byref(p)))
        return {f: (float(getattr(p, f)) if f.endswith("_ms") else int(getattr(p, f))) for f in PHASE_FIELDS}

    def dense(self, i, size=None):
        names, counts = self.query(i)
        out = np.zeros(self.graph.id_bound if size is None else size, dtype=np.uint32)
        out[names] = counts
        return out

    def l1(self, tol=1e-6):
        """Per-query L1 between the normalised counts and the FP64 expected
        counts (device power iteration to residual tol, ptw_batch_l1)."""
        out = np.empty(self.nq, dtype=np.float64)
        C.check(self._lib.ptw_batch_l1(self.graph.handle, self._h, self.sp, APPS[self.app], tol,
                                       out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return out

    def l1_vs(self, ref):
        """Per-query L1 between this batch's normalised counts and those of
        ref, a batch over the same sources (ptw_batch_l1_pair)."""
        out = np.empty(self.nq, dtype=np.float64)
        C.check(self._lib.ptw_batch_l1_pair(self.graph.handle, self._h, ref._h,
                                            out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return out

    def close(self):
        """Frees the results; the arrays of this object are no longer valid."""
        if self._h:
            self.offsets = self.names = self.counts = None
            self.d_offsets = self.d_names = self.d_counts = None
            self._lib.ptw_batch_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def l1_many(graph, results, tol=1e-6):
    """FP64-oracle L1 of several batches over the same sources, one power
    iteration shared by all (ptw_batch_l1_many); returns [len(results), nq]."""
    r0 = results[0]
    hs = (ctypes.c_void_p * len(results))(*[r._h.value if hasattr(r._h, "value") else r._h for r in results])
    out = np.empty((len(results), r0.nq), dtype=np.float64)
    C.check(graph._lib.ptw_batch_l1_many(graph.handle, hs, len(results), r0.sp, APPS[r0.app], tol,
                                         out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
    return out


def _queries(sources, budgets, query_ids):
    sources = np.atleast_1d(np.asarray(sources, dtype=np.uint32))
    budgets = np.broadcast_to(np.asarray(budgets, dtype=np.uint64), sources.shape).copy()
    if query_ids is None:
        query_ids = np.arange(sources.shape[0], dtype=np.uint32)
    query_ids = np.asarray(query_ids, dtype=np.uint32)
    nq = sources.shape[0]
    qs = (C.Query * max(nq, 1))()
    for i in range(nq):
        qs[i].source = int(sources[i])
        qs[i].query_id = int(query_ids[i])
        qs[i].budget = int(budgets[i])
    return sources, budgets, query_ids, qs


def autotune_batch(graph, sources, budgets, sp=0.2, seed=0, app="visits", query_ids=None, max_moves=0,
                   top_k=0):
    """Times this batch under candidate BatchTune values (ptw_autotune_batch),
    keeps the fastest in the graph; returns (tune, median device ms)."""
    sources, budgets, query_ids, qs = _queries(sources, budgets, query_ids)
    cfg = C.BatchCfg(float(sp), int(seed) & 0xFFFFFFFFFFFFFFFF, APPS[app], int(max_moves), 0, 0.0, int(top_k), 0)
    t = C.BatchTune()
    ms = ctypes.c_double()
    C.check(graph._lib.ptw_autotune_batch(graph.handle, qs, sources.shape[0], ctypes.byref(cfg), ctypes.byref(t),
                                          ctypes.byref(ms)))
    return BatchTune.from_c(t), float(ms.value)


def ppr_batch_resumable(graph, sources, budgets, checkpoint, sp=0.2, seed=0, app="visits", query_ids=None,
                        max_moves=0, table_bytes=0, table_factor=0.0, top_k=0, max_waves=0):
    """ppr_batch with its completed waves kept in the file `checkpoint`
    (ptw_ppr_batch_resumable): runs at most max_waves waves (0 = all) and
    returns None while queries remain, the BatchResult once all are done.
    A later call, in this process or another, continues from the file."""
    sources, budgets, query_ids, qs = _queries(sources, budgets, query_ids)
    cfg = C.BatchCfg(float(sp), int(seed) & 0xFFFFFFFFFFFFFFFF, APPS[app], int(max_moves),
                     int(table_bytes), float(table_factor), int(top_k), 0)
    h = ctypes.c_void_p()
    C.check(graph._lib.ptw_ppr_batch_resumable(graph.handle, qs, sources.shape[0], ctypes.byref(cfg),
                                               str(checkpoint).encode(), int(max_waves), ctypes.byref(h)))
    if not h.value:
        return None
    return BatchResult(graph, h, sources, budgets, query_ids, sp, app)


def ppr_batch(graph, sources, budgets, sp=0.2, seed=0, app="visits", query_ids=None, max_moves=0,
              table_bytes=0, table_factor=0.0, top_k=0, device_results=False):
    sources = np.atleast_1d(np.asarray(sources, dtype=np.uint32))
    budgets = np.broadcast_to(np.asarray(budgets, dtype=np.uint64), sources.shape).copy()
    if query_ids is None:
        query_ids = np.arange(sources.shape[0], dtype=np.uint32)
    query_ids = np.asarray(query_ids, dtype=np.uint32)
    nq = sources.shape[0]
    qs = (C.Query * max(nq, 1))()
    for i in range(nq):
        qs[i].source = int(sources[i])
        qs[i].query_id = int(query_ids[i])
        qs[i].budget = int(budgets[i])
    cfg = C.BatchCfg(float(sp), int(seed) & 0xFFFFFFFFFFFFFFFF, APPS[app], int(max_moves),
                     int(table_bytes), float(table_factor), int(top_k),
                     C.PTW_BATCH_DEVICE_RESULTS if device_results else 0)
    h = ctypes.c_void_p()
    C.check(graph._lib.ptw_ppr_batch(graph.handle, qs, nq, ctypes.byref(cfg), ctypes.byref(h)))
    return BatchResult(graph, h, sources, budgets, query_ids, sp, app, device_results=device_results)
