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


class BatchResult:
    """Sparse per-query results, held in host memory by the library."""

    def __init__(self, graph, handle, sources, budgets, query_ids, sp, app):
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
        if self.entries:
            self.names = np.ctypeslib.as_array(pn, shape=(self.entries,))
            self.counts = np.ctypeslib.as_array(pc, shape=(self.entries,))
        else:
            self.names = np.empty(0, dtype=np.uint32)
            self.counts = np.empty(0, dtype=np.uint32)

    def query(self, i):
        a, b = int(self.offsets[i]), int(self.offsets[i + 1])
        return self.names[a:b], self.counts[a:b]

    def dense(self, i, size=None):
        names, counts = self.query(i)
        out = np.zeros(self.graph.id_bound if size is None else size, dtype=np.uint32)
        out[names] = counts
        return out

    def l1(self, tol=1e-10):
        """Per-query L1 between the normalised counts and the FP64 expected
        counts (device power iteration, ptw_batch_l1)."""
        out = np.empty(self.nq, dtype=np.float64)
        C.check(self._lib.ptw_batch_l1(self.graph.handle, self._h, self.sp, APPS[self.app], tol,
                                       out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return out

    def close(self):
        """Frees the results; the arrays of this object are no longer valid."""
        if self._h:
            self.offsets = self.names = self.counts = None
            self._lib.ptw_batch_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def ppr_batch(graph, sources, budgets, sp=0.2, seed=0, app="visits", query_ids=None, max_moves=0,
              table_bytes=0, table_factor=0.0, top_k=0):
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
                     int(table_bytes), float(table_factor), int(top_k))
    h = ctypes.c_void_p()
    C.check(graph._lib.ptw_ppr_batch(graph.handle, qs, nq, ctypes.byref(cfg), ctypes.byref(h)))
    return BatchResult(graph, h, sources, budgets, query_ids, sp, app)
