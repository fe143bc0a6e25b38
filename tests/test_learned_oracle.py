"""The FP64 oracle of the learned warm-start network: its backward pass and
its subspace loss gradient against central finite differences."""
import numpy as np


def _lo():
    import learned_oracle
    return learned_oracle


def test_parameter_count():
    lo = _lo()
    assert 300_000 <= lo.nparams() <= 320_000


def test_subspace_loss_gradient():
    lo = _lo()
    rng = np.random.default_rng(1)
    y = rng.normal(size=(7, 9, 32))
    v, _ = np.linalg.qr(rng.normal(size=(63, 9)))
    v = v.reshape(7, 9, 9)
    L, g = lo.subspace_loss(y, v, grad=True)
    assert 0 <= L <= 9
    for idx in [(0, 0, 0), (3, 4, 17), (6, 8, 31), (2, 5, 9)]:
        e = np.zeros_like(y)
        e[idx] = 1e-6
        fd = (lo.subspace_loss(y + e, v) - lo.subspace_loss(y - e, v)) / 2e-6
        assert abs(fd - g[idx]) < 1e-5 * max(1.0, abs(fd)), (idx, fd, g[idx])
    # a block that contains the eigenvectors (at the other columns' scale:
    # the regulariser is relative to the mean column norm) captures them
    yy = np.concatenate([8 * v, rng.normal(size=(7, 9, 23))], -1)
    assert lo.subspace_loss(yy, v) < 1e-3


def test_backward_matches_finite_differences():
    lo = _lo()
    rng = np.random.default_rng(2)
    H, W = 13, 11
    feat = lo.features(rng.uniform(0, 1, (H, W)), rng.uniform(1, 81, (H, W)))
    p = lo.init_params(3).astype(np.float64)
    lay, n = lo.param_layout()
    p[[bo + k for _, _, bo, _, co in lay for k in range(co)]] = rng.normal(0, 0.05, sum(co for *_, co in lay))
    dy = rng.normal(size=(H, W, lo.NOUT))
    g = lo.backward(p, feat, dy)
    f = lambda q: float((lo.forward(q, feat) * dy).sum())
    picks = []
    for name, wo, bo, ci, co in lay:
        picks += [wo + int(rng.integers(co * 9 * ci)), bo + int(rng.integers(co))]
    for i in picks:
        e = np.zeros(n)
        e[i] = 1e-5
        fd = (f(p + e) - f(p - e)) / 2e-5
        assert abs(fd - g[i]) <= 1e-4 * max(1.0, abs(fd)), (i, fd, g[i])
