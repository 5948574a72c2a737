"""DeepWalk transition statistics, restating the reference's real-graph
validator (src/test/release/test_dataset.cpp:55-196).

Paths of length 80 are accumulated epoch by epoch into per-edge counters.
After each epoch every vertex's empirical neighbour distribution is compared
with the exact one (uniform over its out-edges: the graph has no duplicate
edges): Bhattacharyya distance -log(sum sqrt(p q)) and the largest absolute
difference between the two distributions (the reference's "total variation
distance", test_dataset.cpp:161-171); a vertex never left scores 10 and 1.
Over all vertices the test stops once, as in the reference (:173-181),
  mean < 0.005, median < 0.005, 99th percentile < 0.015   (Bhattacharyya)
  mean < 0.01,  median < 0.01,  99th percentile < 0.03    (largest difference)
and fails if that does not happen within the epoch limit.  Every consecutive
pair of a path must be an edge (test_dataset.cpp:109-120).  The counting
runs on the GPU with torch (sorted edge keys, searchsorted, bincount).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def metric(x):
    """avg, median and 99th percentile as cal_prob_dist_metric computes them
    (test_dataset.cpp:40-51)."""
    s, _ = x.sort()
    n = s.numel()
    return float(s.mean()), float(s[n // 2]), float(s[int(n * 0.99)])


def test_deepwalk_neighbour_distributions_converge(gpu):
    import torch
    dev = "cuda"
    with gpu.Graph.rmat(16, 16, 0.57, 0.19, 0.19, seed=1, clean=True) as G:
        names, row_ptr, col = G.export_csr()
        n = G.n
        assert G.id_bound == n                     # names 0..n-1: name == row index
        rp = torch.as_tensor(row_ptr.astype(np.int64), device=dev)
        cl = torch.as_tensor(col.astype(np.int64), device=dev)
        deg = rp[1:] - rp[:-1]
        assert int(deg.min()) >= 1
        src = torch.repeat_interleave(torch.arange(n, device=dev), deg)
        keys = src * n + cl                        # rows in order, neighbours ascending: sorted
        assert bool((keys[1:] > keys[:-1]).all())
        a0 = 1.0 / deg[src].double()
        cnt = torch.zeros(keys.numel(), dtype=torch.int64, device=dev)
        W, L = 32 * n, 80
        paths = torch.empty((W, L), dtype=torch.int32, device=dev)
        converged, transitions, last = False, 0, None
        for epoch in range(60):
            gpu.deepwalk(G, W, L, 7, out=paths, first_walker=epoch * W)
            for part in paths.split(W // 4):
                u = part[:, :-1].reshape(-1).long()
                v = part[:, 1:].reshape(-1).long()
                k = u * n + v
                pos = torch.searchsorted(keys, k).clamp_(max=keys.numel() - 1)
                assert bool((keys[pos] == k).all()), "a path step that is not an edge"
                cnt += torch.bincount(pos, minlength=keys.numel())
                transitions += k.numel()
            c = cnt.double()
            tot = torch.zeros(n, dtype=torch.float64, device=dev).index_add_(0, src, c)
            seen = tot > 0
            a1 = c / tot[src].clamp(min=1.0)
            bc = torch.zeros(n, dtype=torch.float64, device=dev).index_add_(0, src, torch.sqrt(a0 * a1))
            bd = torch.where(seen, -torch.log(bc.clamp(min=1e-300)), torch.full_like(bc, 10.0))
            dmax = torch.zeros(n, dtype=torch.float64, device=dev).scatter_reduce_(
                0, src, (a0 - a1).abs(), reduce="amax", include_self=True)
            dmax = torch.where(seen, dmax, torch.ones_like(dmax))
            last = (epoch + 1, transitions, metric(bd), metric(dmax))
            b, t = last[2], last[3]
            if b[0] < 0.005 and b[1] < 0.005 and b[2] < 0.015 and t[0] < 0.01 and t[1] < 0.01 and t[2] < 0.03:
                converged = True
                break
        assert converged, "not converged: epochs, transitions, (avg, median, p99) BD, diff = %r" % (last,)
