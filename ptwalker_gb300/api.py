"""Host-side mirror of the reference's graph / app / walk interface.

The reference (PTWalker) drives a walk as

    Graph graph(mtcfg); graph.load(path, fmt, as_undirected, db);   src/core/graph.hpp:277
    PPR myapp(sp, &graph);                                           src/core/pagerank.cpp:22
    FMobSolver solver(&graph, mtcfg);                                src/core/solver.hpp:120
    walk(&solver, walker_num, walk_len, mem_quota, myapp, ws);       src/core/solver.hpp:1049
    myapp.rooted_value[v]                                            src/core/pagerank.cpp:13

Here the same steps are ``Graph.load`` / ``PageRankApp`` / ``Solver`` /
``walk``; the app object receives its results the way the reference's app
structs do (``rooted_value`` for the counting apps, ``walker_pair`` for RWR,
``paths`` for DeepWalk).  Results are indexed by vertex name (the ids of the
edge list), not by the reference's random internal relabelling.  Every call
runs on the GPU through libptw.so; there is no CPU fallback.
"""
import ctypes

import numpy as np

from . import _capi as C

START_MODES = {"per_vertex": C.PTW_START_PER_VERTEX, "uniform": C.PTW_START_UNIFORM,
               "sources": C.PTW_START_SOURCES}


def _ptr(arr, ctype=ctypes.c_uint32):
    return arr.ctypes.data_as(ctypes.POINTER(ctype))


def _dev_ptr(t):
    """Device pointer of a torch CUDA tensor."""
    if not getattr(t, "is_cuda", False):
        raise ValueError("expected a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError("expected a contiguous tensor")
    return ctypes.c_void_p(t.data_ptr())


def _host_ptr(arr):
    """Host pointer of a numpy array or a (pinned) CPU torch tensor."""
    if isinstance(arr, np.ndarray):
        if not arr.flags["C_CONTIGUOUS"] or not arr.flags["WRITEABLE"]:
            raise ValueError("output array must be writable and C-contiguous")
        return ctypes.c_void_p(arr.ctypes.data)
    if hasattr(arr, "data_ptr") and not getattr(arr, "is_cuda", False):
        if not arr.is_contiguous():
            raise ValueError("output tensor must be contiguous")
        return ctypes.c_void_p(arr.data_ptr())
    raise TypeError("output must be a numpy array or a CPU torch tensor")


class Tune:
    """Launch parameters of the walk kernels (see ptw_tune in include/ptw.h)."""

    def __init__(self, block=256, ilp=2, chunk=256, hot_k=0, blocks_per_sm=0, min_blocks=0,
                 paths_ilp=2, cache_hints=1, paths_named=1, ext_columns=0, gather_slots=0, warp_agg=0):
        self.block, self.ilp, self.chunk = block, ilp, chunk
        self.hot_k, self.blocks_per_sm, self.min_blocks = hot_k, blocks_per_sm, min_blocks
        self.paths_ilp, self.cache_hints, self.paths_named = paths_ilp, cache_hints, paths_named
        self.ext_columns, self.gather_slots, self.warp_agg = ext_columns, gather_slots, warp_agg

    def to_c(self):
        return C.Tune(self.block, self.ilp, self.chunk, self.hot_k, self.blocks_per_sm,
                      self.min_blocks, self.paths_ilp, self.cache_hints, self.paths_named,
                      self.ext_columns, self.gather_slots, self.warp_agg)

    @classmethod
    def from_c(cls, t):
        return cls(t.block, t.ilp, t.chunk, t.hot_k, t.blocks_per_sm, t.min_blocks, t.paths_ilp,
                   t.cache_hints, t.paths_named, t.ext_columns, t.gather_slots, t.warp_agg)

    def as_dict(self):
        return dict(block=self.block, ilp=self.ilp, chunk=self.chunk, hot_k=self.hot_k,
                    blocks_per_sm=self.blocks_per_sm, min_blocks=self.min_blocks,
                    paths_ilp=self.paths_ilp, cache_hints=self.cache_hints,
                    paths_named=self.paths_named, ext_columns=self.ext_columns,
                    gather_slots=self.gather_slots, warp_agg=self.warp_agg)

    def __repr__(self):
        return "Tune(%s)" % ", ".join("%s=%s" % kv for kv in self.as_dict().items())


class WalkStats:
    def __init__(self, s):
        self.walkers, self.moves, self.visits = int(s.walkers), int(s.moves), int(s.visits)
        self.kernel_ms, self.total_ms = float(s.kernel_ms), float(s.total_ms)

    def __repr__(self):
        return ("WalkStats(walkers=%d, moves=%d, visits=%d, kernel_ms=%.3f, total_ms=%.3f)"
                % (self.walkers, self.moves, self.visits, self.kernel_ms, self.total_ms))


class Graph:
    """Device-resident graph (replaces Graph, src/core/graph.hpp:95-829)."""

    def __init__(self, handle):
        self._lib = C.load()
        self._h = handle
        info = C.GraphInfo()
        C.check(self._lib.ptw_graph_get_info(self._h, ctypes.byref(info)))
        self.n = int(info.n_vertices)
        self.m = int(info.n_edges)
        self.id_bound = int(info.id_bound)
        self.max_degree = int(info.max_degree)
        self._inflight = {}  # ticket -> host buffer of a pipelined pagerank call

    @property
    def device_bytes(self):
        """Device memory the graph holds now (the column copies built on
        demand by DeepWalk or tune.ext_columns included)."""
        info = C.GraphInfo()
        C.check(self._lib.ptw_graph_get_info(self._h, ctypes.byref(info)))
        return int(info.device_bytes)

    # -- construction ------------------------------------------------------
    @classmethod
    def load(cls, path, fmt="text", as_undirected=False):
        """Reads a text (``%u %u`` lines, ``#`` comments) or binary Edge[] file."""
        lib = C.load()
        f = {"text": C.PTW_FMT_TEXT, "binary": C.PTW_FMT_BINARY}[fmt]
        h = ctypes.c_void_p()
        C.check(lib.ptw_graph_load(str(path).encode(), f, int(bool(as_undirected)), ctypes.byref(h)))
        return cls(h)

    @classmethod
    def from_edges(cls, src, dst, as_undirected=False):
        lib = C.load()
        s = np.ascontiguousarray(src, dtype=np.uint32)
        d = np.ascontiguousarray(dst, dtype=np.uint32)
        if s.shape != d.shape:
            raise ValueError("src and dst differ in length")
        h = ctypes.c_void_p()
        C.check(lib.ptw_graph_from_edges(_ptr(s), _ptr(d), s.shape[0], int(bool(as_undirected)),
                                         ctypes.byref(h)))
        return cls(h)

    @classmethod
    def from_csr(cls, row_ptr, col, names=None):
        """Graph from a CSR (row_ptr[n+1], col[row_ptr[n]] row indices, optional names[n]):
        the inverse of export_csr."""
        lib = C.load()
        r = np.ascontiguousarray(row_ptr, dtype=np.uint64)
        c = np.ascontiguousarray(col, dtype=np.uint32)
        if r.ndim != 1 or r.shape[0] < 2:
            raise ValueError("row_ptr needs n + 1 >= 2 entries")
        n = r.shape[0] - 1
        if c.shape[0] != int(r[-1]):
            raise ValueError("col has %d entries, row_ptr[n] = %d" % (c.shape[0], int(r[-1])))
        nm = None
        if names is not None:
            nm = np.ascontiguousarray(names, dtype=np.uint32)
            if nm.shape[0] != n:
                raise ValueError("names has %d entries for %d rows" % (nm.shape[0], n))
        h = ctypes.c_void_p()
        C.check(lib.ptw_graph_from_csr(_ptr(r, ctypes.c_uint64), _ptr(c), n,
                                       _ptr(nm) if nm is not None else None, ctypes.byref(h)))
        return cls(h)

    @classmethod
    def rmat(cls, scale, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=1, clean=True):
        lib = C.load()
        h = ctypes.c_void_p()
        C.check(lib.ptw_graph_rmat(scale, edge_factor, a, b, c, seed, int(bool(clean)), ctypes.byref(h)))
        return cls(h)

    @classmethod
    def chung_lu(cls, n, gamma=2.1, mean_degree=32.0, seed=1):
        """Chung-Lu power-law graph (symmetrised, cleaned, names 0..n'-1)."""
        lib = C.load()
        h = ctypes.c_void_p()
        C.check(lib.ptw_graph_chung_lu(int(n), float(gamma), float(mean_degree), int(seed), ctypes.byref(h)))
        return cls(h)

    def save(self, path, fmt="text"):
        """Writes the directed edge list (sorted by source, then destination
        name) as text (``%u %u`` lines) or binary Edge[] (include/io.hpp)."""
        f = {"text": C.PTW_FMT_TEXT, "binary": C.PTW_FMT_BINARY}[fmt]
        C.check(self._lib.ptw_graph_save(self.handle, str(path).encode(), f))

    # -- lifetime ----------------------------------------------------------
    def close(self):
        if self._h:
            self._lib.ptw_graph_free(self._h)  # waits for the graph's streams
            self._h = None
        self._inflight.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        if not self._h:
            raise ValueError("graph is closed")
        return self._h

    # -- inspection --------------------------------------------------------
    def export_csr(self):
        """(names[n], row_ptr[n+1] u64, col[m]) in canonical index order."""
        names = np.empty(self.n, dtype=np.uint32)
        row_ptr = np.empty(self.n + 1, dtype=np.uint64)
        col = np.empty(self.m, dtype=np.uint32)
        C.check(self._lib.ptw_graph_export_csr(self.handle, _ptr(names),
                                               _ptr(row_ptr, ctypes.c_uint64), _ptr(col)))
        return names, row_ptr, col

    def export_edges(self):
        src = np.empty(self.m, dtype=np.uint32)
        dst = np.empty(self.m, dtype=np.uint32)
        C.check(self._lib.ptw_graph_export_edges(self.handle, _ptr(src), _ptr(dst)))
        return src, dst

    @property
    def tune(self):
        t = C.Tune()
        C.check(self._lib.ptw_graph_get_tune(self.handle, ctypes.byref(t)))
        return Tune.from_c(t)

    @tune.setter
    def tune(self, t):
        ct = t.to_c()
        C.check(self._lib.ptw_graph_set_tune(self.handle, ctypes.byref(ct)))

    def autotune(self, sp=0.15, n_walkers=0):
        t = C.Tune()
        C.check(self._lib.ptw_autotune(self.handle, sp, n_walkers, ctypes.byref(t)))
        return Tune.from_c(t)

    def sync(self):
        C.check(self._lib.ptw_graph_sync(self.handle))

    def set_stream(self, stream=None):
        """Issue work on a torch.cuda.Stream (or a raw cudaStream_t int);
        None returns to the graph's own stream.  With a caller stream set,
        device-output calls are asynchronous on that stream; without one
        they are ordered after the current torch stream and complete before
        returning."""
        ptr = None
        if stream is not None:
            ptr = stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)
        C.check(self._lib.ptw_graph_set_stream(self.handle, ctypes.c_void_p(ptr) if ptr else None))
        self._user_stream = ptr is not None

    def _before_device_call(self):
        if not getattr(self, "_user_stream", False):
            import torch
            torch.cuda.current_stream().synchronize()

    def _after_device_call(self):
        if not getattr(self, "_user_stream", False):
            self.sync()


def _cfg(n_walkers, sp, seed, start, sources, max_moves, first_walker=0):
    if isinstance(start, str):
        start = START_MODES[start]
    cfg = C.WalkCfg()
    cfg.n_walkers = int(n_walkers)
    cfg.sp = float(sp)
    cfg.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    cfg.start_mode = int(start)
    cfg.max_moves = int(max_moves)
    keep = None
    if sources is not None:
        keep = np.ascontiguousarray(np.atleast_1d(sources), dtype=np.uint32)
        cfg.h_sources = _ptr(keep)
        cfg.n_sources = keep.shape[0]
        if start != C.PTW_START_SOURCES:
            raise ValueError("sources given but start mode is not 'sources'")
    cfg.first_walker = int(first_walker)
    return cfg, keep


def probe_gather(array_bytes=2 << 30, chains=8):
    """Random 4-byte gathers per second the current GPU serves from an array
    of array_bytes (ptw_probe_gather): the ceiling of a walk move's dependent
    gather once the array exceeds L2."""
    out = ctypes.c_double()
    C.check(C.load().ptw_probe_gather(int(array_bytes), int(chains), ctypes.byref(out)))
    return float(out.value)


def trim_memory():
    """Hands the device memory the engine keeps cached between batched and
    served calls back to the CUDA driver (ptw_trim_memory)."""
    C.check(C.load().ptw_trim_memory())


def pagerank(graph, n_walkers=None, sp=0.15, seed=0, start="per_vertex", sources=None,
             max_moves=0, out=None, first_walker=0, stats=False):
    """Visit counts by name (uint32[id_bound]); every position is counted.

    ``out`` may be a numpy array, a (pinned) CPU tensor, or a CUDA tensor; a
    CUDA tensor keeps the result on the device (ptw_pagerank_dev)."""
    n_walkers = graph.n if n_walkers is None else n_walkers
    cfg, _keep = _cfg(n_walkers, sp, seed, start, sources, max_moves, first_walker)
    if out is None:
        out = np.empty(graph.id_bound, dtype=np.uint32)
    return _run(graph, "ptw_pagerank", (ctypes.byref(cfg),), out, graph.id_bound, stats)


def pagerank_submit(graph, out, n_walkers=None, sp=0.15, seed=0, start="per_vertex", sources=None,
                    max_moves=0, first_walker=0):
    """Pipelined pagerank (ptw_pagerank_submit): launches the walk and the
    copy of its counts into ``out`` (uint32[id_bound], best page-locked, e.g.
    a pinned CPU tensor) and returns a ticket at once.  Two calls may be in
    flight per graph; ``pagerank_wait(graph, ticket)`` returns the call's
    WalkStats once ``out`` holds its counts."""
    n_walkers = graph.n if n_walkers is None else n_walkers
    if getattr(out, "is_cuda", False):
        raise ValueError("pagerank_submit copies to host memory; use pagerank(out=<CUDA tensor>) on the device")
    itemsize = out.itemsize if isinstance(out, np.ndarray) else out.element_size()
    if itemsize != 4 or _nelem(out) < graph.id_bound:
        raise ValueError("output needs at least %d 4-byte elements" % graph.id_bound)
    cfg, _keep = _cfg(n_walkers, sp, seed, start, sources, max_moves, first_walker)
    t = ctypes.c_uint64()
    C.check(graph._lib.ptw_pagerank_submit(graph.handle, ctypes.byref(cfg), _host_ptr(out), ctypes.byref(t)))
    graph._inflight[int(t.value)] = out  # the buffer stays referenced until the wait
    return int(t.value)


def pagerank_wait(graph, ticket):
    """Waits for a pagerank_submit call; returns its WalkStats."""
    st = C.WalkStats()
    try:
        C.check(graph._lib.ptw_pagerank_wait(graph.handle, int(ticket), ctypes.byref(st)))
    finally:
        graph._inflight.pop(int(ticket), None)
    return WalkStats(st)


def _nelem(out):
    return int(out.size) if isinstance(out, np.ndarray) else int(out.numel())


def _run(graph, fn, args, out, need, stats):
    """Calls fn (host output) or fn_dev (CUDA tensor output) after checking
    that out holds at least `need` 4-byte elements: the C ABI cannot check
    the size of a caller's buffer."""
    itemsize = out.itemsize if isinstance(out, np.ndarray) else out.element_size()
    if itemsize != 4 or _nelem(out) < need:
        raise ValueError("output needs at least %d 4-byte elements" % need)
    st = C.WalkStats()
    stp = ctypes.byref(st) if stats else None
    if getattr(out, "is_cuda", False):
        graph._before_device_call()
        C.check(getattr(graph._lib, fn + "_dev")(graph.handle, *args, _dev_ptr(out), stp))
        graph._after_device_call()
    else:
        C.check(getattr(graph._lib, fn)(graph.handle, *args, _host_ptr(out), stp))
    return (out, WalkStats(st)) if stats else out


def ppr(graph, source, n_walkers, sp=0.15, seed=0, query_id=0, max_moves=0, out=None, stats=False):
    """Single-source PPR visit counts (src/core/ppr.cpp); walker ids are
    (query_id << 32) + j, so a query's result does not depend on what runs
    beside it."""
    return pagerank(graph, n_walkers, sp, seed, "sources", [source], max_moves, out,
                    first_walker=int(query_id) << 32, stats=stats)


def rwr(graph, n_walkers=None, sp=0.5, seed=0, start="per_vertex", sources=None, max_moves=0,
        out=None, first_walker=0, stats=False):
    """(start, end) name pairs per walker, uint32[n_walkers, 2] (src/core/RWR.cpp)."""
    n_walkers = graph.n if n_walkers is None else n_walkers
    cfg, _keep = _cfg(n_walkers, sp, seed, start, sources, max_moves, first_walker)
    if out is None:
        out = np.empty((n_walkers, 2), dtype=np.uint32)
    return _run(graph, "ptw_rwr", (ctypes.byref(cfg),), out, 2 * int(n_walkers), stats)


def deepwalk(graph, n_walkers=None, walk_len=80, seed=0, start="per_vertex", sources=None,
             out=None, first_walker=0, stats=False):
    """int32[n_walkers, walk_len] paths of names, -1 after a dead end (src/core/deepwalk.cpp)."""
    n_walkers = graph.n if n_walkers is None else n_walkers
    cfg, _keep = _cfg(n_walkers, 0.0, seed, start, sources, 0, first_walker)
    if out is None:
        out = np.empty((n_walkers, walk_len), dtype=np.int32)
    return _run(graph, "ptw_deepwalk", (ctypes.byref(cfg), int(walk_len)), out,
                int(n_walkers) * int(walk_len), stats)


class Node2vecStats:
    def __init__(self, s):
        self.walkers, self.moves = int(s.walkers), int(s.moves)
        self.trials, self.checks, self.probes = int(s.trials), int(s.checks), int(s.probes)
        self.kernel_ms, self.total_ms = float(s.kernel_ms), float(s.total_ms)

    def __repr__(self):
        return ("Node2vecStats(walkers=%d, moves=%d, trials=%d, checks=%d, probes=%d, kernel_ms=%.3f, "
                "total_ms=%.3f)" % (self.walkers, self.moves, self.trials, self.checks, self.probes,
                                    self.kernel_ms, self.total_ms))


def node2vec(graph, n_walkers=None, walk_len=80, p=1.0, q=1.0, seed=0, start="per_vertex", sources=None,
             out=None, first_walker=0, stats=False):
    """int32[n_walkers, walk_len] second-order paths of names, -1 after a dead
    end (src/core/node2vec.cpp with -p / -q, include/option.hpp:447-469): from
    v, reached from t, the next vertex x has weight 1/p if x == t, 1 if x is a
    neighbour of t, 1/q otherwise."""
    n_walkers = graph.n if n_walkers is None else n_walkers
    cfg, _keep = _cfg(n_walkers, 0.0, seed, start, sources, 0, first_walker)
    if out is None:
        out = np.empty((n_walkers, walk_len), dtype=np.int32)
    itemsize = out.itemsize if isinstance(out, np.ndarray) else out.element_size()
    if itemsize != 4 or _nelem(out) < int(n_walkers) * int(walk_len):
        raise ValueError("output needs at least %d 4-byte elements" % (int(n_walkers) * int(walk_len)))
    st = C.Node2vecStats()
    stp = ctypes.byref(st) if stats else None
    args = (graph.handle, ctypes.byref(cfg), int(walk_len), float(p), float(q))
    if getattr(out, "is_cuda", False):
        graph._before_device_call()
        C.check(graph._lib.ptw_node2vec_dev(*args, _dev_ptr(out), stp))
        graph._after_device_call()
    else:
        C.check(graph._lib.ptw_node2vec(*args, _host_ptr(out), stp))
    return (out, Node2vecStats(st)) if stats else out


# ---- app-template mirror (src/core/pagerank.cpp, ppr.cpp, RWR.cpp, deepwalk.cpp) ----

class PageRankApp:
    """pagerank.cpp ``PPR``: type 0 (count before move), counts every position."""
    type = 0

    def __init__(self, sp, graph, start="uniform", seed=0):
        self.tp_ = sp
        self.graph_ = graph
        self.start = start
        self.seed = seed
        self.start_vertices = []
        self.rooted_value = None


class PPRApp(PageRankApp):
    """ppr.cpp ``PPR``: every walker starts at the single source."""

    def __init__(self, sp, graph, source, seed=0):
        super().__init__(sp, graph, "sources", seed)
        self.start_vertices = [source]


class RWRApp:
    """RWR.cpp ``PPR``: type 1 (move then update), records (start, end)."""
    type = 1

    def __init__(self, sp, graph, start="uniform", seed=0, sources=None):
        self.tp_ = sp
        self.graph_ = graph
        self.start = start
        self.seed = seed
        self.start_vertices = list(sources) if sources is not None else []
        self.walker_pair = None


class DeepWalkApp:
    """deepwalk.cpp ``deepwalk``: fixed walk length, records the path."""
    type = 0

    def __init__(self, walk_len, graph, start="uniform", seed=0):
        self.tp_ = walk_len
        self.graph_ = graph
        self.start = start
        self.seed = seed
        self.paths = None


class Solver:
    """Stands in for FMobSolver(Graph*, MultiThreadConfig) (solver.hpp:120);
    the GPU needs no thread configuration."""

    def __init__(self, graph, mtcfg=None):
        self.graph = graph
        self.is_node2vec = False
        self.p = self.q = 1.0

    def set_node2vec(self, p, q):
        """FMobSolver::set_node2vec (solver.hpp:156-159): fixed-length walks
        of this solver become second-order (node2vec) walks."""
        self.is_node2vec = True
        self.p, self.q = float(p), float(q)


def walk(solver, walker_num, walk_len, mem_quota, app, walker_size=4196):
    """Mirror of walk() (src/core/solver.hpp:1049-1074).  ``walk_len`` only
    matters for DeepWalk; ``mem_quota`` and ``walker_size`` size CPU pools in
    the reference and are accepted and ignored."""
    del mem_quota, walker_size
    g = solver.graph if isinstance(solver, Solver) else solver
    if isinstance(app, DeepWalkApp):
        start = "sources" if getattr(app, "start_vertices", None) else app.start
        if getattr(solver, "is_node2vec", False):
            app.paths = node2vec(g, walker_num, app.tp_, solver.p, solver.q, app.seed, start)
        else:
            app.paths = deepwalk(g, walker_num, app.tp_, app.seed, start)
        return app
    sources = app.start_vertices if app.start_vertices else None
    start = "sources" if sources else app.start
    if isinstance(app, RWRApp):
        app.walker_pair = rwr(g, walker_num, app.tp_, app.seed, start, sources)
    else:
        app.rooted_value = pagerank(g, walker_num, app.tp_, app.seed, start, sources)
    return app
