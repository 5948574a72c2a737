"""FP64 oracle for expected visit counts (test infrastructure).

With P = D^-1 A (row-stochastic over out-edges, multi-edges weighted) and
stop probability sp after every move, a walker from s that counts its start
and every position after a move (src/core/solver.hpp:242-263 with
src/core/pagerank.cpp:41-68 and :86-89) has expected visits

    E[c | s] = e_s + sum_{n>=1} (1-sp)^(n-1) e_s^T P^n
             = pi_s / (sp (1-sp)) - sp/(1-sp) e_s,

where pi_s = sp sum_{n>=0} (1-sp)^n e_s^T P^n is textbook personalised
PageRank.  The endpoint after the last move (src/core/RWR.cpp:99-105) has law
(pi_s - sp e_s) / (1-sp).  pi is computed by power iteration
x <- sp e + (1-sp) P^T x until the L1 change is below ``tol``.
Vertices without out-edges end the walk (mass leaks), matching the replay.
"""
import numpy as np
import scipy.sparse as sp_sparse


def _transition_T(g):
    n = g.n
    deg = np.diff(g.row_ptr).astype(np.float64)
    rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(g.row_ptr).astype(np.int64))
    inv = np.zeros(n)
    nz = deg > 0
    inv[nz] = 1.0 / deg[nz]
    data = inv[rows]
    # P[u, v] = multiplicity / deg(u); duplicates are summed by coo->csr.
    P = sp_sparse.coo_matrix((data, (rows, g.col.astype(np.int64))), shape=(n, n)).tocsr()
    return P.T.tocsr()


def ppr_vector(g, sp, teleport, tol=1e-12, max_iter=10000, PT=None):
    """Personalised PageRank pi = sp * sum_n (1-sp)^n teleport^T P^n (FP64)."""
    PT = _transition_T(g) if PT is None else PT
    e = np.asarray(teleport, dtype=np.float64)
    x = sp * e.copy()
    term = x.copy()
    for _ in range(max_iter):
        term = (1.0 - sp) * (PT @ term)
        x += term
        if np.abs(term).sum() < tol:
            break
    return x


def expected_visits_from_source(g, sp, s_index, tol=1e-12, PT=None):
    e = np.zeros(g.n)
    e[s_index] = 1.0
    pi = ppr_vector(g, sp, e, tol=tol, PT=PT)
    out = pi / (sp * (1.0 - sp))
    out[s_index] -= sp / (1.0 - sp)
    return out


def expected_visits_per_vertex_start(g, sp, n_walkers=None, tol=1e-12, PT=None):
    """Expected counts when walker w starts at vertex w mod n (n_walkers = n)."""
    n = g.n
    n_walkers = n if n_walkers is None else n_walkers
    starts = np.full(n, n_walkers // n, dtype=np.float64)
    starts[: n_walkers % n] += 1.0
    pi = ppr_vector(g, sp, starts, tol=tol, PT=PT)
    return pi / (sp * (1.0 - sp)) - (sp / (1.0 - sp)) * starts


def expected_endpoint_from_source(g, sp, s_index, tol=1e-12, PT=None):
    e = np.zeros(g.n)
    e[s_index] = 1.0
    pi = ppr_vector(g, sp, e, tol=tol, PT=PT)
    out = pi.copy()
    out[s_index] -= sp
    return out / (1.0 - sp)
