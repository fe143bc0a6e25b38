"""The learned warm start's network on the GPU (BF16 tensor cores, FP32
accumulation) against its FP64 oracle, which rounds to bfloat16 where the
kernels store or feed values to the tensor cores: the forward fields, the
subspace loss and every parameter's gradient.  Then training lowers the
loss, and the trained network, as the start of the block eigensolver, is
measured against a random start on held-out patches."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _lo():
    import learned_oracle
    return learned_oracle


def _inputs(seed, shapes):
    """smooth-ish mPb in [0, 1], degree in [1, 81] and 9 orthonormal targets"""
    rng = np.random.default_rng(seed)
    out = []
    for (H, W) in shapes:
        mpb = np.clip(rng.normal(0.2, 0.2, (H, W)), 0, 1)
        deg = rng.uniform(5, 81, (H, W))
        v, _ = np.linalg.qr(rng.normal(size=(H * W, 9)))
        out.append((mpb, deg, v))
    return out


def _dev(torch, arrs):
    return torch.from_numpy(np.concatenate([np.ascontiguousarray(a, np.float32).ravel() for a in arrs])).cuda()


def _params(seed):
    lo = _lo()
    p = lo.init_params(seed)
    lay, _ = lo.param_layout()
    rng = np.random.default_rng(seed + 1)
    for _, _, bo, _, co in lay:
        p[bo:bo + co] = rng.normal(0, 0.02, co)
    return p


SHAPES = [(37, 29), (24, 40), (16, 16)]


def test_forward_matches_oracle():
    torch = pytest.importorskip("torch")
    import gpb
    lo = _lo()
    data = _inputs(3, SHAPES)
    p = _params(5)
    ctx = gpb.Context()
    ctx.learned_set(p)
    assert np.array_equal(ctx.learned_get(), p)
    d_m, d_d = _dev(torch, [d[0] for d in data]), _dev(torch, [d[1] for d in data])
    total = sum(H * W for H, W in SHAPES)
    d_y = torch.zeros(total * lo.NOUT, dtype=torch.float32, device="cuda")
    ctx.learned_forward_device(SHAPES, d_m.data_ptr(), d_d.data_ptr(), d_y.data_ptr())
    y = d_y.cpu().numpy().astype(np.float64)
    at = 0
    for (H, W), (mpb, deg, _) in zip(SHAPES, data):
        want = lo.forward(p, lo.features(mpb, deg), bf=True)
        got = y[at * lo.NOUT:(at + H * W) * lo.NOUT].reshape(H, W, lo.NOUT)
        rel = np.linalg.norm(got - want) / np.linalg.norm(want)
        assert rel < 1e-2, rel
        at += H * W
    ctx.close()


def _cos(a, b):
    return float(a @ b / (np.linalg.norm(a) * np.linalg.norm(b)))


def test_loss_and_gradient_match_oracle():
    """The CUDA kernels' loss and gradient of every parameter against the
    oracle's backward pass (bfloat16 at the same places).  The two differ by
    bfloat16 roundings that land differently (the GPU's output gradient comes
    from its FP32 fields, the oracle's from FP64) and compound over 15
    layers: the whole gradient within 5% and at cosine > 0.999, each
    convolution's at cosine > 0.99 -- a wrong index or transpose gives
    cosines far below."""
    torch = pytest.importorskip("torch")
    import gpb
    lo = _lo()
    data = _inputs(7, SHAPES)
    p = _params(9)
    ctx = gpb.Context()
    ctx.learned_set(p)
    d_m, d_d = _dev(torch, [d[0] for d in data]), _dev(torch, [d[1] for d in data])
    d_v = _dev(torch, [d[2] for d in data])
    loss, g = ctx.learned_grad_device(SHAPES, d_m.data_ptr(), d_d.data_ptr(), d_v.data_ptr())
    ctx.close()
    want_loss, want_g = 0.0, np.zeros(lo.nparams())
    for (H, W), (mpb, deg, v) in zip(SHAPES, data):
        f = lo.features(mpb, deg)
        y = lo.forward(p, f, bf=True)
        L, dy = lo.subspace_loss(y, v.reshape(H, W, 9), grad=True)
        want_loss += L
        want_g += lo.backward(p, f, dy, bf=True)
    assert abs(loss - want_loss) < 1e-3 * max(1.0, want_loss), (loss, want_loss)
    g = g.astype(np.float64)
    assert np.linalg.norm(g - want_g) / np.linalg.norm(want_g) < 5e-2
    assert _cos(g, want_g) > 0.999
    lay, _ = lo.param_layout()
    for name, wo, bo, ci, co in lay:
        gw, ww = g[wo:bo + co], want_g[wo:bo + co]
        assert _cos(gw, ww) > 0.99, (name, _cos(gw, ww))


def test_training_lowers_the_loss():
    """A few epochs of the library's own Adam on the GPU on eigenvectors the
    plain solver finds for small synthetic patches."""
    torch = pytest.importorskip("torch")
    import gpb
    from gpb import learned
    lo = _lo()
    shapes, mpb, deg, v = learned.make_dataset(12, 64, seed=11)
    ctx = gpb.Context()
    ctx.learned_set(lo.init_params(0))
    hist = ctx.learned_train_device(shapes, mpb.data_ptr(), deg.data_ptr(), v.data_ptr(), batch=4, epochs=6,
                                    lr=2e-3, seed=1)
    assert np.all(np.isfinite(hist))
    assert hist[-1] < 0.8 * hist[0], hist
    ctx.close()


def _held_out(n):
    from gpb import learned, synth
    imgs = learned.images(n, 512, 1077)  # the evaluation set; training used seed 0
    cb = synth.make_codebook(imgs[0], synth.SEED_BASE + 77, n_sample=4096)
    return cb, [synth.pack_bgr(im) for im in imgs]


def _solve(cb, packed, mode, w=None, **kw):
    import gpb
    ctx = gpb.Context(cb, eig_mode=mode, **kw)
    if w is not None:
        ctx.learned_set(w)
    ctx.compute_batch(packed[:2])  # layout, autotuning, graphs
    outs = ctx.compute_batch(packed)
    st = ctx.stats()
    ctx.close()
    return outs, st


def test_trained_start_on_held_out_patches(orc):
    """The shipped weights (gpb/learned_weights.npy: 2,000 training patches
    of 256^2 labelled by the plain solver, 60 epochs) on 8 held-out 512^2
    patches.  At the workload's evaluation residual (1e-4, gap rule off) the
    block solver started from the network needs fewer matvecs than from a
    random block (measured over 200 such patches: 6,816 vs 7,084 per patch,
    11.2 vs 11.5 ms).  At the library's tolerance (1e-6, which gPb within
    1e-3 needs) it converges to the same residual bound and gPb within 1e-3
    of the oracle; there the start's advantage is gone (54.7 vs 54.8 ms)."""
    import gpb
    from gpb import learned
    w = np.load(learned.WEIGHTS)
    assert w.size == gpb.learned_nparams()
    cb, packed = _held_out(8)
    _, st_l = _solve(cb, packed, gpb.EIG_LEARNED, w, eig_tol=1e-4, eig_gap_frac=0.0)
    _, st_c = _solve(cb, packed, gpb.EIG_BLOCK, eig_tol=1e-4, eig_gap_frac=0.0)
    assert st_l["max_residual"] <= 1e-4 and st_c["max_residual"] <= 1e-4
    assert st_l["matvecs_total"] < st_c["matvecs_total"], (st_l["matvecs_total"], st_c["matvecs_total"])
    outs, st = _solve(cb, packed[:2], gpb.EIG_LEARNED, w)
    assert st["eig_fallback"] == 0 and st["max_residual"] <= 3 * 1e-6
    imgs = learned.images(1, 512, 1077)
    ref = orc.globalpb(imgs[0], cb)
    assert np.abs(outs[0][1].reshape(8, 512, 512) - ref["gpb_o"]).max() < 1e-3
