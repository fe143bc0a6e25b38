"""Edge cases of the batch path on the GPU, through the C ABI: the smallest
patch the library accepts (32 x 32) in every eigensolver mode, a codebook of
fewer than 32 codewords, a batch of many tiny uneven patches, and one large
single patch."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GPB_TOL = 1e-3


def _img(H, W, cells, seed, lines=0):
    from gpb import synth
    img = synth.voronoi_image(H, W, cells, 8.0, synth.SEED_BASE + seed, lines=lines)
    cb = synth.make_codebook(img, synth.SEED_BASE + seed, n_sample=1024)
    return img, cb


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_minimum_patch_all_solvers(orc, mode):
    import gpb
    from gpb import synth
    img, cb = _img(32, 32, 3, 91)
    ref = orc.globalpb(img, cb)
    ctx = gpb.Context(cb, eig_mode=mode)
    nm, orr = ctx.compute_batch([synth.pack_bgr(img)])[0]
    assert ctx.last_status == gpb.GPB_OK
    assert np.abs(nm - ref["nmax"]).max() < GPB_TOL
    assert np.abs(orr.reshape(8, 32, 32) - ref["gpb_o"]).max() < GPB_TOL
    ctx.close()


def test_small_codebook(orc):
    """K = 8 codewords: texton labels stay bit-exact and below K."""
    import gpb
    from gpb import synth
    img = synth.voronoi_image(60, 76, 6, 8.0, synth.SEED_BASE + 92)
    cb = synth.make_codebook(img, synth.SEED_BASE + 92, k=8, n_sample=1024)
    ref = orc.globalpb(img, cb)
    ctx = gpb.Context(cb, eig_mode=gpb.EIG_WARM, keep_intermediates=1)
    nm, orr = ctx.compute_batch([synth.pack_bgr(img)])[0]
    tex = ctx.fetch("texton", 0, (60, 76), np.uint8)
    assert np.array_equal(tex, ref["texton"]) and tex.max() < 8
    assert np.abs(nm - ref["nmax"]).max() < GPB_TOL
    ctx.close()


def test_many_tiny_uneven_patches(orc):
    """100 patches with sides in [32, 48] in one warm-started batch."""
    import gpb
    from gpb import synth
    img, cb = _img(400, 400, 60, 93)
    rng = np.random.default_rng(7)
    boxes = []
    for _ in range(100):
        h, w = (int(v) for v in rng.integers(32, 49, 2))
        y0, x0 = int(rng.integers(0, 400 - h)), int(rng.integers(0, 400 - w))
        boxes.append((y0, x0, h, w))
    crops = [np.ascontiguousarray(img[y0:y0 + h, x0:x0 + w]) for (y0, x0, h, w) in boxes]
    ctx = gpb.Context(cb, eig_mode=gpb.EIG_WARM)
    outs = ctx.compute_batch([synth.pack_bgr(c) for c in crops])
    assert ctx.last_status == gpb.GPB_OK
    assert 0 < ctx.stats()["max_residual"] <= 3 * ctx.params.eig_tol
    for i in (0, 57, 99):
        ref = orc.globalpb(crops[i], cb)
        assert np.abs(outs[i][0] - ref["nmax"]).max() < GPB_TOL
    ctx.close()


def test_large_single_patch():
    """One 1536 x 1024 patch (1.6 Mpix, 96 cells: a spectrum clustered near
    zero): converges to within the FP32 residual floor (4x eig_tol), finite,
    non-negative."""
    import gpb
    from gpb import synth
    img, cb = _img(1024, 1536, 96, 94, lines=6)
    ctx = gpb.Context(cb, eig_mode=gpb.EIG_WARM)
    nm, orr = ctx.compute_batch([synth.pack_bgr(img)])[0]
    assert ctx.last_status == gpb.GPB_OK
    assert np.isfinite(nm).all() and np.isfinite(orr).all() and nm.min() >= 0 and nm.max() > 0
    assert 0 < ctx.stats()["max_residual"] <= 4 * ctx.params.eig_tol
    ctx.close()


def test_lanczos_fallback(orc):
    """A block solver that misses its target (here: a matvec cap too small
    for 32-vector filtering, ample for single-vector Lanczos) hands the batch
    to plain Lanczos, and the result still matches the oracle."""
    import gpb
    from gpb import synth
    img, cb = _img(64, 80, 6, 95)
    ref = orc.globalpb(img, cb)
    plain = gpb.Context(cb, eig_mode=gpb.EIG_LANCZOS)
    plain.compute_batch([synth.pack_bgr(img)])
    need = plain.stats()["matvecs_max"]
    plain.close()
    # enough for Lanczos, one fine outer iteration (32 + 43 x 32 matvecs) for the block solver
    cap = max(1500, need + 50)
    assert cap < 32 + 2 * 43 * 32
    ctx = gpb.Context(cb, eig_mode=gpb.EIG_WARM, eig_max_matvecs=cap)
    nm, orr = ctx.compute_batch([synth.pack_bgr(img)])[0]
    st = ctx.stats()
    assert st["eig_fallback"] == 1 and ctx.last_status == gpb.GPB_OK
    assert np.abs(nm - ref["nmax"]).max() < GPB_TOL
    assert np.abs(orr.reshape(8, 64, 80) - ref["gpb_o"]).max() < GPB_TOL
    ctx.close()
