"""FP64 numpy restatement of the learned warm-start network (test
infrastructure only: tests/ use it to check the library's CUDA forward and
backward kernels; the product never imports it).

The network maps per-pixel features of a patch -- its mPb and its affinity
degree / 81, zero-padded to 16 channels -- to 32 fields that start the block
eigensolver.  A 4-level encoder-decoder of 3 x 3 convolutions:

    enc0: 16->16, 16->16            skip0          (full resolution)
    pool, enc1: 16->32, 32->32      skip1          (1/2)
    pool, enc2: 32->64, 64->64      skip2          (1/4)
    pool, enc3: 64->64, 64->64                     (1/8)
    up + [skip2] (128): 128->64, 64->64
    up + [skip1] (96):  96->32,  32->32
    up + [skip0] (48):  48->16,  16->16
    head: 16->32 (no ReLU)

ReLU after every convolution but the head; zero padding at the patch border;
pooling is the 2 x 2 mean over the pixels that exist (ceil sizes); up-sampling
is nearest-neighbour to the skip's size; concatenation puts the up-sampled
channels first.  Parameters: per convolution W[cout][3][3][cin] then
b[cout], in the order above.

Loss (per patch, summed): 9 - tr(V^T P_Y V), the energy of the solver's 9
orthonormal eigenvectors V outside span(Y), P_Y = Y (Y^T Y + eps)^-1 Y^T with
eps = 1e-4 tr(Y^T Y) / 32 I.  It depends on span(V) only, so clustered
eigenvalues do not make the target ambiguous.

With bf=True the values are rounded to bfloat16 (nearest-even) where the
CUDA kernels store or feed them to the tensor cores: weights, every stored
activation, and every gradient a backward convolution consumes.
"""
import numpy as np

CONVS = [  # (name, cin, cout, relu)
    ("e0a", 16, 16, True), ("e0b", 16, 16, True),
    ("e1a", 16, 32, True), ("e1b", 32, 32, True),
    ("e2a", 32, 64, True), ("e2b", 64, 64, True),
    ("e3a", 64, 64, True), ("e3b", 64, 64, True),
    ("d2a", 128, 64, True), ("d2b", 64, 64, True),
    ("d1a", 96, 32, True), ("d1b", 32, 32, True),
    ("d0a", 48, 16, True), ("d0b", 16, 16, True),
    ("head", 16, 32, False),
]
NOUT = 32
NIN = 16


def param_layout():
    """(name, w_offset, b_offset, cin, cout) per convolution, and the total."""
    out, o = [], 0
    for name, ci, co, _ in CONVS:
        out.append((name, o, o + co * 9 * ci, ci, co))
        o += co * 9 * ci + co
    return out, o


def nparams():
    return param_layout()[1]


def init_params(seed=0):
    """He-normal weights, zero biases."""
    rng = np.random.default_rng(seed)
    lay, n = param_layout()
    p = np.zeros(n, np.float64)
    for name, wo, bo, ci, co in lay:
        std = np.sqrt(2.0 / (9 * ci)) if name != "head" else np.sqrt(1.0 / (9 * ci))
        p[wo:wo + co * 9 * ci] = rng.normal(0.0, std, co * 9 * ci)
    return p.astype(np.float32)


def bf16(x):
    """Round float64 values to bfloat16 (via float32, nearest-even), as float64."""
    f = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((f + 0x7FFF + ((f >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def _rnd(x, on):
    return bf16(x) if on else x


def features(mpb, deg):
    """H x W x 16 input: mPb, degree / 81, zeros."""
    H, W = mpb.shape
    f = np.zeros((H, W, NIN))
    f[..., 0] = mpb
    f[..., 1] = deg / 81.0
    return f


def conv3(x, w, b):
    """'same' 3 x 3 correlation, zero padding: x H x W x ci, w co x 3 x 3 x ci."""
    H, W, _ = x.shape
    xp = np.pad(x, ((1, 1), (1, 1), (0, 0)))
    out = np.zeros((H, W, w.shape[0]))
    for dy in range(3):
        for dx in range(3):
            out += xp[dy:dy + H, dx:dx + W, :] @ w[:, dy, dx, :].T
    return out + b


def conv3_bwd(x, w, dz):
    """gradients of conv3 w.r.t. x, w and b for output gradient dz."""
    H, W, ci = x.shape
    xp = np.pad(x, ((1, 1), (1, 1), (0, 0)))
    dxp = np.zeros_like(xp)
    dw = np.zeros_like(w)
    for dy in range(3):
        for dx in range(3):
            dw[:, dy, dx, :] = dz.reshape(-1, dz.shape[-1]).T @ xp[dy:dy + H, dx:dx + W, :].reshape(-1, ci)
            dxp[dy:dy + H, dx:dx + W, :] += dz @ w[:, dy, dx, :]
    return dxp[1:-1, 1:-1, :], dw, dz.sum((0, 1))


def pool(x):
    H, W, C = x.shape
    h, w = (H + 1) // 2, (W + 1) // 2
    s = np.zeros((h, w, C))
    n = np.zeros((h, w, 1))
    for a in range(2):
        for c in range(2):
            blk = x[a::2, c::2, :]
            s[:blk.shape[0], :blk.shape[1]] += blk
            n[:blk.shape[0], :blk.shape[1]] += 1
    return s / n, n


def pool_bwd(dy, n, shape):
    dx = np.zeros(shape)
    g = dy / n
    for a in range(2):
        for c in range(2):
            hh, ww = dx[a::2, c::2, :].shape[:2]
            dx[a::2, c::2, :] = g[:hh, :ww]
    return dx


def up(x, shape):
    H, W = shape[:2]
    return x[np.arange(H) // 2][:, np.arange(W) // 2]


def up_bwd(dy, small_shape):
    dx = np.zeros(small_shape)
    H, W = dy.shape[:2]
    np.add.at(dx, (np.arange(H)[:, None] // 2, np.arange(W)[None, :] // 2), dy)
    return dx


def _wb(p, name):
    lay, _ = param_layout()
    for nm, wo, bo, ci, co in lay:
        if nm == name:
            return (p[wo:wo + co * 9 * ci].astype(np.float64).reshape(co, 3, 3, ci),
                    p[bo:bo + co].astype(np.float64))
    raise KeyError(name)


def forward(p, feat, bf=False, keep=False):
    """The 32 output fields (H x W x 32) of one patch; with keep, also the
    tensors the backward pass needs."""
    st = {}
    pw = {nm: _wb(p, nm) for nm, *_ in CONVS}
    if bf:
        pw = {k: (bf16(w), b) for k, (w, b) in pw.items()}

    def cv(name, x, relu=True):
        w, b = pw[name]
        z = conv3(x, w, b)
        a = np.maximum(z, 0) if relu else z
        a = _rnd(a, bf and relu)
        st[name] = (x, a)
        return a

    x = _rnd(feat, bf)
    s0 = cv("e0b", cv("e0a", x))
    p0, n0 = pool(s0)
    p0 = _rnd(p0, bf)
    s1 = cv("e1b", cv("e1a", p0))
    p1, n1 = pool(s1)
    p1 = _rnd(p1, bf)
    s2 = cv("e2b", cv("e2a", p1))
    p2, n2 = pool(s2)
    p2 = _rnd(p2, bf)
    b3 = cv("e3b", cv("e3a", p2))
    c2 = np.concatenate([up(b3, s2.shape), s2], -1)
    d2 = cv("d2b", cv("d2a", c2))
    c1 = np.concatenate([up(d2, s1.shape), s1], -1)
    d1 = cv("d1b", cv("d1a", c1))
    c0 = np.concatenate([up(d1, s0.shape), s0], -1)
    d0 = cv("d0b", cv("d0a", c0))
    y = cv("head", d0, relu=False)
    if keep:
        st.update(s0=s0, s1=s1, s2=s2, b3=b3, d2=d2, d1=d1, p0=p0, p1=p1, p2=p2, n0=n0, n1=n1, n2=n2, pw=pw)
        return y, st
    return y


def subspace_loss(y, v, grad=False):
    """9 - tr(V^T P_Y V) for Y = y (N x 32) and orthonormal V (N x 9); with
    grad, also dL/dY."""
    Y = y.reshape(-1, y.shape[-1])
    V = v.reshape(-1, v.shape[-1])
    G = Y.T @ Y
    G = G + 1e-4 * np.trace(G) / G.shape[0] * np.eye(G.shape[0])
    B = V.T @ Y
    Gi = np.linalg.inv(G)
    loss = V.shape[1] - np.trace(B @ Gi @ B.T)
    if not grad:
        return loss
    C1 = B @ Gi
    C2 = Gi @ B.T @ B @ Gi
    dY = -2.0 * (V @ C1 - Y @ C2)
    return loss, dY.reshape(y.shape)


def backward(p, feat, dy, bf=False):
    """Gradient of <dy, forward(p, feat)> w.r.t. the parameters (float64)."""
    y, st = forward(p, feat, bf=bf, keep=True)
    pw = st["pw"]
    lay, n = param_layout()
    g = np.zeros(n)
    off = {nm: (wo, bo, ci, co) for nm, wo, bo, ci, co in lay}

    def cvb(name, da, relu=True):
        x, a = st[name]
        dz = da * (a > 0) if relu else da
        dz = _rnd(dz, bf)
        dx, dw, db = conv3_bwd(x, pw[name][0], dz)
        wo, bo, ci, co = off[name]
        g[wo:wo + co * 9 * ci] += dw.ravel()
        g[bo:bo + co] += db
        return dx

    dd0 = cvb("head", dy, relu=False)
    dc0 = cvb("d0a", cvb("d0b", dd0))
    c_up = dc0.shape[-1] - st["s0"].shape[-1]
    dd1 = up_bwd(dc0[..., :c_up], st["d1"].shape)
    ds0 = dc0[..., c_up:]
    dc1 = cvb("d1a", cvb("d1b", dd1))
    c_up = dc1.shape[-1] - st["s1"].shape[-1]
    dd2 = up_bwd(dc1[..., :c_up], st["d2"].shape)
    ds1 = dc1[..., c_up:]
    dc2 = cvb("d2a", cvb("d2b", dd2))
    c_up = dc2.shape[-1] - st["s2"].shape[-1]
    db3 = up_bwd(dc2[..., :c_up], st["b3"].shape)
    ds2 = dc2[..., c_up:]
    dp2 = cvb("e3a", cvb("e3b", db3))
    ds2 = ds2 + pool_bwd(dp2, st["n2"], st["s2"].shape)
    dp1 = cvb("e2a", cvb("e2b", ds2))
    ds1 = ds1 + pool_bwd(dp1, st["n1"], st["s1"].shape)
    dp0 = cvb("e1a", cvb("e1b", ds1))
    ds0 = ds0 + pool_bwd(dp0, st["n0"], st["s0"].shape)
    cvb("e0a", cvb("e0b", ds0))
    return g
