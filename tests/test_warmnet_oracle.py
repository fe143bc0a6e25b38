"""The numpy oracle of the warm-start correction (oracle/warmnet_oracle.py),
the checker of the CUDA training kernels: its analytic gradient against
central finite differences, and the identity of a zero-weight net."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import warmnet_oracle as wo  # noqa: E402


def _data(seed):
    rng = np.random.default_rng(seed)
    return [(rng.normal(size=(H * W, 9)), rng.random(H * W), rng.normal(size=(H * W, 9)), H, W)
            for (H, W) in [(5, 7), (4, 4), (3, 9)]]


def test_gradient_matches_finite_differences():
    pats = _data(1)
    w = wo.init_weights(3, 0.3)
    _, g = wo.loss_grad(w, pats)
    rng = np.random.default_rng(2)
    for i in list(rng.choice(wo.NPARAM, 40, replace=False)) + [0, 1439, 1440, 1455, 1456, 1599, 1600, 1608]:
        e = np.zeros_like(w)
        e[i] = 1e-6
        fd = (wo.loss_grad(w + e, pats)[0] - wo.loss_grad(w - e, pats)[0]) / 2e-6
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(g[i])


def test_zero_net_is_identity():
    xt, mpb, _, H, W = _data(4)[0]
    y, h, _ = wo.forward(np.zeros(wo.NPARAM), xt, mpb, H, W)
    assert np.array_equal(y, xt) and not h.any()
