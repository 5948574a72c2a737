"""FP64 CPU oracle for the learned-budget kernels (test infrastructure).

Restates, in float64 numpy, the math of the device kernels in
ptwalker_gb300/csrc/mlp.cu: the eight source features and the
8 -> 64 -> 64 -> 1 ReLU MLP with standardised inputs / target, its MSE loss
and its gradient.  Parameter order W1[8][64], b1[64], W2[64][64], b2[64],
w3[64], b3.
"""
import numpy as np

IN, H = 8, 64
OW1, OB1 = 0, IN * H
OW2 = OB1 + H
OB2 = OW2 + H * H
OW3 = OB2 + H
OB3 = OW3 + H
NPARAMS = OB3 + 1


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[OW1:OB1].reshape(IN, H), p[OB1:OW2], p[OW2:OB2].reshape(H, H), p[OB2:OW3],
            p[OW3:OB3], p[OB3])


def forward_backward(params, norm, x, t):
    """Returns (loss, grad[NPARAMS], y_normalised[B])."""
    W1, b1, W2, b2, w3, b3 = unpack(params)
    norm = np.asarray(norm, dtype=np.float64)
    mu, sd = norm[:IN], np.where(norm[IN:2 * IN] > 0, norm[IN:2 * IN], 1.0)
    tmu, tsd = norm[2 * IN], (norm[2 * IN + 1] if norm[2 * IN + 1] > 0 else 1.0)
    x = (np.asarray(x, dtype=np.float64) - mu) / sd
    tn = (np.asarray(t, dtype=np.float64) - tmu) / tsd
    B = x.shape[0]
    z1 = x @ W1 + b1
    a1 = np.maximum(z1, 0)
    z2 = a1 @ W2 + b2
    a2 = np.maximum(z2, 0)
    y = a2 @ w3 + b3
    d = y - tn
    loss = float(np.mean(d * d))
    e = 2.0 * d / B
    dz2 = np.outer(e, w3) * (z2 > 0)
    dz1 = (dz2 @ W2.T) * (z1 > 0)
    g = np.zeros(NPARAMS)
    g[OW1:OB1] = (x.T @ dz1).ravel()
    g[OB1:OW2] = dz1.sum(0)
    g[OW2:OB2] = (a1.T @ dz2).ravel()
    g[OB2:OW3] = dz2.sum(0)
    g[OW3:OB3] = a2.T @ e
    g[OB3] = e.sum()
    return loss, g, y


def source_features(canon, sources):
    """Eight features per source name from the canonical CSR (see ptw.h)."""
    idx = canon.name_to_index(sources)
    deg = np.diff(canon.row_ptr).astype(np.float64)
    out = np.zeros((len(idx), IN))
    for k, s in enumerate(idx):
        nb = canon.col[canon.row_ptr[s]:canon.row_ptr[s + 1]]
        d = float(len(nb))
        du = deg[nb]
        l = np.log1p(du)
        out[k, 0] = np.log1p(d)
        if len(nb):
            out[k, 1] = l.mean()
            out[k, 2] = l.max()
            out[k, 3] = l.min()
            out[k, 5] = np.sqrt(max((l * l).mean() - l.mean() ** 2, 0.0))
            out[k, 6] = np.mean(du == 1)
        out[k, 4] = np.log1p(du.sum())
        out[k, 7] = np.log1p(du.sum() / (d if d else 1.0))
    return out
