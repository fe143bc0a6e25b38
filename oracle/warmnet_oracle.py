"""warmnet_oracle.py -- TEST INFRASTRUCTURE ONLY.

numpy restatement of the learned warm-start correction of the library
(k_warmnet.cu): forward pass, mean squared error against the target
eigenvectors and its analytic gradient, the checker of the CUDA training
kernels.  The net: 3 x 3 conv (10 -> 16, zero padding), ReLU, 1 x 1 conv
(16 -> 9), added to the first 9 normalised start columns."""
import numpy as np

NIN, NHID, NOUT = 10, 16, 9
NPARAM = NHID * NIN * 9 + NHID + NOUT * NHID + NOUT


def unpack(w):
    w = np.asarray(w, np.float64)
    i = 0
    W1 = w[i:i + NHID * NIN * 9].reshape(NHID, NIN, 9); i += NHID * NIN * 9
    b1 = w[i:i + NHID]; i += NHID
    W2 = w[i:i + NOUT * NHID].reshape(NOUT, NHID); i += NOUT * NHID
    b2 = w[i:i + NOUT]
    return W1, b1, W2, b2


def taps(xt, mpb, H, W):
    """(N, 10, 9): the 10 input channels at the 9 taps of each pixel"""
    inp = np.concatenate([xt.reshape(H, W, NOUT), mpb.reshape(H, W, 1)], axis=2)
    pad = np.pad(inp, ((1, 1), (1, 1), (0, 0)))
    out = np.zeros((H, W, NIN, 9))
    for t in range(9):
        dy, dx = t // 3 - 1, t % 3 - 1
        out[:, :, :, t] = pad[1 + dy:1 + dy + H, 1 + dx:1 + dx + W, :]
    return out.reshape(H * W, NIN, 9)


def forward(w, xt, mpb, H, W):
    W1, b1, W2, b2 = unpack(w)
    T = taps(xt, mpb, H, W)
    a = np.einsum("kct,nct->nk", W1, T) + b1
    h = np.maximum(a, 0.0)
    y = xt.reshape(-1, NOUT) + h @ W2.T + b2
    return y, h, T


def loss_grad(w, patches):
    """patches: list of (xt (N,9), mpb (N,), vt (N,9), H, W); mean over all
    pixels and the 9 columns"""
    W1, b1, W2, b2 = unpack(w)
    ntot = sum(p[3] * p[4] for p in patches) * NOUT
    L = 0.0
    g = [np.zeros_like(W1), np.zeros_like(b1), np.zeros_like(W2), np.zeros_like(b2)]
    for xt, mpb, vt, H, W in patches:
        y, h, T = forward(w, xt, mpb, H, W)
        r = y - vt.reshape(-1, NOUT)
        L += (r * r).sum() / ntot
        gy = 2.0 * r / ntot
        g[3] += gy.sum(0)
        g[2] += gy.T @ h
        dh = (gy @ W2) * (h > 0)
        g[1] += dh.sum(0)
        g[0] += np.einsum("nk,nct->kct", dh, T)
    return L, np.concatenate([x.ravel() for x in g])


def init_weights(seed=0, scale=0.02):
    rng = np.random.default_rng(seed)
    w = np.zeros(NPARAM)
    W1, b1, W2, b2 = unpack(w)
    w[:NHID * NIN * 9] = rng.normal(0, scale, NHID * NIN * 9)
    i = NHID * NIN * 9 + NHID
    w[i:i + NOUT * NHID] = rng.normal(0, scale, NOUT * NHID)
    return w
