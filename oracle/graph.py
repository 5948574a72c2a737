"""Canonical graph layout and R-MAT pipeline (test infrastructure).

Restates the reference loader's semantics (src/core/graph.hpp:277-366 and
include/io.hpp:39-90):
  * an edge list of (src, dst) u32 names, read as text ``"%u %u"`` lines with
    ``#`` comment lines, or as a raw array of ``Edge{u32 src; u32 dst}``;
  * the vertex set is every name that appears; edges are kept as given
    (directed, duplicates and self-loops kept; ``as_undirected`` adds the
    reverse of every edge, graph.hpp:286-318);
  * the sampler picks uniformly among a vertex's out-edges, so a duplicate
    edge counts twice (sampler.hpp:214-217).
The reference stores rows in a nondeterministic order and relabels vertices
randomly (graph.hpp:515-781).  The canonical layout used for bit-exact
replay fixes both: vertex index i is the i-th smallest name and each row
lists neighbour indices in ascending order.
"""
import os
from dataclasses import dataclass

import numpy as np

from .lib import load_lib


@dataclass
class CanonicalGraph:
    names: np.ndarray    # uint32 [n], ascending
    row_ptr: np.ndarray  # uint64 [n+1]
    col: np.ndarray      # uint32 [m], neighbour indices, rows ascending

    @property
    def n(self):
        return int(self.names.shape[0])

    @property
    def m(self):
        return int(self.col.shape[0])

    @property
    def degree(self):
        return np.diff(self.row_ptr).astype(np.int64)

    def name_to_index(self, names):
        names = np.asarray(names, dtype=np.uint32)
        idx = np.searchsorted(self.names, names)
        if np.any(idx >= self.n) or np.any(self.names[np.minimum(idx, self.n - 1)] != names):
            raise KeyError("name not in graph")
        return idx.astype(np.uint32)


def canonical_from_edges(src, dst, as_undirected=False):
    src = np.asarray(src, dtype=np.uint32)
    dst = np.asarray(dst, dtype=np.uint32)
    if as_undirected:
        src, dst = np.concatenate([src, dst]), np.concatenate([dst, src])
    names = np.unique(np.concatenate([src, dst]))
    si = np.searchsorted(names, src).astype(np.uint64)
    di = np.searchsorted(names, dst).astype(np.uint64)
    keys = np.sort((si << np.uint64(32)) | di)
    s_sorted = (keys >> np.uint64(32)).astype(np.int64)
    col = (keys & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    deg = np.bincount(s_sorted, minlength=names.shape[0]).astype(np.uint64)
    row_ptr = np.zeros(names.shape[0] + 1, dtype=np.uint64)
    np.cumsum(deg, out=row_ptr[1:])
    return CanonicalGraph(names=names.astype(np.uint32), row_ptr=row_ptr, col=col)


def rmat_thresholds(a, b, c):
    """Integer quadrant thresholds: floor(p * 2^32) of the cumulative a, a+b, a+b+c."""
    def t(p):
        return min(int(p * 4294967296.0), 0xFFFFFFFF)
    return t(a), t(a + b), t(a + b + c)


def rmat_raw_edges(scale, edge_factor, a=0.57, b=0.19, c=0.19, seed=1):
    lib = load_lib()
    m = int(edge_factor) << int(scale)
    src = np.empty(m, dtype=np.uint32)
    dst = np.empty(m, dtype=np.uint32)
    ta, tab, tabc = rmat_thresholds(a, b, c)
    u32p = lib.ora_rmat_edges.argtypes[7]
    lib.ora_rmat_edges(scale, 0, m, ta, tab, tabc, seed,
                       src.ctypes.data_as(u32p), dst.ctypes.data_as(u32p))
    return src, dst


def rmat_clean_edges(scale, edge_factor, a=0.57, b=0.19, c=0.19, seed=1):
    """R-MAT benchmark graph: symmetrised, self-loops and duplicates removed,
    isolated vertices dropped and the remaining names compacted to 0..V-1 in
    ascending order.  Returns (src, dst) sorted by (src, dst)."""
    src, dst = rmat_raw_edges(scale, edge_factor, a, b, c, seed)
    keep = src != dst
    src, dst = src[keep], dst[keep]
    s2 = np.concatenate([src, dst]).astype(np.uint64)
    d2 = np.concatenate([dst, src]).astype(np.uint64)
    keys = np.unique((s2 << np.uint64(32)) | d2)
    s = (keys >> np.uint64(32)).astype(np.uint32)
    d = (keys & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    present = np.unique(s)  # symmetric: every endpoint is also a source
    s = np.searchsorted(present, s).astype(np.uint32)
    d = np.searchsorted(present, d).astype(np.uint32)
    return s, d


def rmat_clean_csr(scale, edge_factor, a=0.57, b=0.19, c=0.19, seed=1, threads=None):
    """Same graph as ``canonical_from_edges(*rmat_clean_edges(...))``, built
    in C with a parallel radix sort (practical at scale 24)."""
    import ctypes
    lib = load_lib()
    threads = threads or os.cpu_count() or 1
    ta, tab, tabc = rmat_thresholds(a, b, c)
    n = ctypes.c_uint32()
    m = ctypes.c_uint64()
    rp = ctypes.POINTER(ctypes.c_uint64)()
    cp = ctypes.POINTER(ctypes.c_uint32)()
    rc = lib.ora_rmat_clean_csr(scale, edge_factor, ta, tab, tabc, seed, threads,
                                ctypes.byref(n), ctypes.byref(m), ctypes.byref(rp), ctypes.byref(cp))
    if rc != 0:
        raise MemoryError("oracle R-MAT clean-up could not allocate")
    try:
        row_ptr = np.ctypeslib.as_array(rp, shape=(n.value + 1,)).copy()
        col = np.ctypeslib.as_array(cp, shape=(max(m.value, 1),))[: m.value].copy()
    finally:
        lib.ora_free(ctypes.cast(rp, ctypes.c_void_p))
        lib.ora_free(ctypes.cast(cp, ctypes.c_void_p))
    return CanonicalGraph(names=np.arange(n.value, dtype=np.uint32), row_ptr=row_ptr, col=col)


def read_edge_file(path, fmt):
    """fmt: 'text' (``%u %u`` per line, ``#`` comments) or 'binary' (Edge[])."""
    if fmt == "binary":
        raw = np.fromfile(path, dtype=np.uint32)
        raw = raw[: (raw.shape[0] // 2) * 2].reshape(-1, 2)
        return raw[:, 0].copy(), raw[:, 1].copy()
    src, dst = [], []
    with open(path, "r") as f:
        for line in f:
            if line.startswith("#"):
                continue
            parts = line.split()
            if len(parts) < 2:
                continue
            src.append(int(parts[0]))
            dst.append(int(parts[1]))
    return np.array(src, dtype=np.uint32), np.array(dst, dtype=np.uint32)


def write_text_edges(path, src, dst):
    tmp = path + ".tmp%d" % os.getpid()
    with open(tmp, "w") as f:
        pairs = np.stack([np.asarray(src, np.uint32), np.asarray(dst, np.uint32)], axis=1)
        chunk = 1 << 20
        for i in range(0, pairs.shape[0], chunk):
            f.write("\n".join("%d %d" % (int(a), int(b)) for a, b in pairs[i:i + chunk]))
            f.write("\n")
    os.replace(tmp, path)


def write_binary_edges(path, src, dst):
    pairs = np.stack([np.asarray(src, np.uint32), np.asarray(dst, np.uint32)], axis=1)
    pairs.tofile(path)
