"""The learned warm-start correction: the CUDA training kernels against the
numpy oracle, capture of the start block, and the trained net's effect on
held-out patches."""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import warmnet_oracle as wo  # noqa: E402

GPB_TOL = 1e-3


def test_gradient_matches_oracle():
    """loss and all 1609 partial derivatives of gpb_warmnet_grad_device
    against the FP64 numpy restatement, on three uneven patches"""
    torch = pytest.importorskip("torch")
    import gpb
    rng = np.random.default_rng(5)
    pats = []
    for (H, W) in [(12, 17), (9, 9), (20, 6)]:
        pats.append((rng.normal(size=(H * W, 9)).astype(np.float32), rng.random(H * W).astype(np.float32),
                     rng.normal(size=(H * W, 9)).astype(np.float32), H, W))
    w = wo.init_weights(3, 0.3).astype(np.float32)
    ctx = gpb.Context()
    xt = torch.from_numpy(np.concatenate([p[0] for p in pats])).cuda()
    mp = torch.from_numpy(np.concatenate([p[1] for p in pats])).cuda()
    vt = torch.from_numpy(np.concatenate([p[2] for p in pats])).cuda()
    loss, g = ctx.warmnet_grad_device([p[4] for p in pats], [p[3] for p in pats], xt.data_ptr(), mp.data_ptr(),
                                      vt.data_ptr(), w)
    ref_l, ref_g = wo.loss_grad(w.astype(np.float64), [(p[0].astype(np.float64), p[1].astype(np.float64),
                                                        p[2].astype(np.float64), p[3], p[4]) for p in pats])
    ctx.close()
    assert abs(loss - ref_l) <= 1e-5 * abs(ref_l)
    assert np.abs(g - ref_g).max() <= 1e-4 * np.abs(ref_g).max()


def test_capture_and_zero_net():
    """the captured start block comes back per patch; a net of zero weights
    leaves the result within the parity tolerance of the uncorrected path"""
    import gpb
    from gpb import synth
    img = synth.voronoi_image(96, 112, 40, 6.0, synth.SEED_BASE + 301)
    cb = synth.make_codebook(img, synth.SEED_BASE + 301, n_sample=1024)
    ctx = gpb.Context(cb, eig_mode=gpb.EIG_WARM)
    ctx.warmnet_capture(True)
    ref = ctx.compute_batch([synth.pack_bgr(img)])[0]
    x0 = ctx.fetch("warm0", 0, (96 * 112, 9), np.float32)
    assert np.isfinite(x0).all() and np.abs(x0).max() > 0
    ctx.warmnet_set(np.zeros(gpb.WARMNET_PARAMS, np.float32))
    got = ctx.compute_batch([synth.pack_bgr(img)])[0]
    assert ctx.last_status == gpb.GPB_OK
    assert np.abs(got[0] - ref[0]).max() < GPB_TOL
    ctx.close()


def test_trained_net_gain_on_held_out_patches():
    """The committed weights (trained on 64 synthetic 256 x 256 patches by
    python -m gpb.warmnet) on held-out 512 x 512 patches: the corrected start
    keeps less of itself outside the converged eigenvectors' span (the
    training objective), the solver needs at most 5% more matvecs than
    without it (over 8 such patches it needed 3% fewer), and gPb stays within
    the parity tolerance of the uncorrected path."""
    import gpb
    from gpb import synth, warmnet
    w = np.load(warmnet.WEIGHTS)
    imgs = warmnet.images(3, 512, seed=3)
    cb = synth.make_codebook(warmnet.images(1, 256, seed=1)[0], synth.SEED_BASE + 1, n_sample=1024)
    ctx = gpb.Context(cb, eig_mode=gpb.EIG_WARM)
    data = warmnet.collect(ctx, imgs)
    ctx.close()
    before = after = 0.0
    for xt, mpb, vt, H, W in data:
        q, _ = np.linalg.qr(vt.astype(np.float64))  # span of the converged eigenvectors
        y, _, _ = wo.forward(w, xt.astype(np.float64), mpb.astype(np.float64), H, W)
        before += ((xt - q @ (q.T @ xt)) ** 2).sum()
        after += ((y - q @ (q.T @ y)) ** 2).sum() * ((xt ** 2).sum() / (y ** 2).sum())
    assert after < 0.9 * before  # 0.79 measured on the GB300
    ev = warmnet.evaluate(cb, imgs, w)
    print("held-out 512^2: out-of-span energy %.3f -> %.3f; matvecs %d -> %d" % (
        before, after, ev["without"]["matvecs_max"], ev["with"]["matvecs_max"]))
    assert ev["with"]["matvecs_max"] <= 1.05 * ev["without"]["matvecs_max"]
    assert ev["max_gpb_diff"] < GPB_TOL
