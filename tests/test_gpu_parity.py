"""Parity of the CUDA library (through its C ABI) with the oracle.

Tolerances: texton labels, Lab bins and raw half-disc histogram counts
bit-exact; cue maps 1e-5 and mPb / W 1e-6 absolute (FP32 vs FP64); gPb
1e-3 absolute (the target of the gPb stage); eigenvectors checked by their
FP64 residual on the oracle's matrix.
"""
import ctypes
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GPB_TOL = 1e-3


def _img(H, W, cells, seed, lines=0):
    from gpb import synth
    img = synth.voronoi_image(H, W, cells, 8.0, synth.SEED_BASE + seed, lines=lines)
    cb = synth.make_codebook(img, synth.SEED_BASE + seed, n_sample=2048)
    return img, cb


@pytest.fixture(scope="module")
def small(orc):
    img, cb = _img(56, 72, 7, 11)
    return img, cb, orc.globalpb(img, cb, intermediates=True)


@pytest.fixture(scope="module")
def ctx_small(small):
    import gpb
    img, cb, _ = small
    ctx = gpb.Context(cb, keep_intermediates=2)
    orient, nmax = gpb.GlobalPbCuda(ctx, img)
    yield ctx, orient, nmax
    ctx.close()


def test_texton_labels_bit_exact(small, ctx_small):
    img, cb, ref = small
    ctx, _, _ = ctx_small
    H, W, _ = img.shape
    assert np.array_equal(ctx.fetch("texton", 0, (H, W), np.uint8), ref["texton"])


def test_lab_bins_bit_exact(small, ctx_small, orc):
    img, _, _ = small
    ctx, _, _ = ctx_small
    H, W, _ = img.shape
    assert np.array_equal(ctx.fetch("labbins", 0, (3, H, W), np.uint8), orc.lab_bins(img))


def test_histogram_counts_bit_exact(small, ctx_small, orc):
    """Raw slice counts of every pixel, cue and radius against
    compute_hist_gradient_2D's integer counts (lib_image.cc:3160-3186)."""
    img, _, ref = small
    ctx, _, _ = ctx_small
    H, W, _ = img.shape
    cnt = ctx.fetch("counts", 0, (H, W, 4, 4, 32, 32), np.uint8).astype(np.int32)
    per_slice = cnt[..., :16, :] + cnt[..., 16:, :]          # two halves of each slice
    q = orc.lab_bins(img)
    labels = [q[0], q[1], q[2], ref["texton"]]
    for ann, r in enumerate((3, 5, 10, 20)):
        for c in range(4):
            if (ann == 0 and c != 0) or (ann == 3 and c == 0):
                continue  # radii the cue does not use
            lp = orc.mirror(labels[c], 30)
            _, oc = orc.hist_gradient(lp, 30, r, None, counts=True)
            nb = oc.shape[-1]
            assert np.array_equal(per_slice[:, :, ann, c, :, :nb], oc), (r, c)


def test_cues_and_mpb(small, ctx_small):
    img, _, ref = small
    ctx, _, _ = ctx_small
    H, W, _ = img.shape
    cues = ctx.fetch("cues", 0, (12, 8, H, W), np.float32)
    assert np.abs(cues - ref["cues"]).max() < 1e-5
    mpb = ctx.fetch("mpb", 0, (H, W), np.float32)
    assert np.abs(mpb - ref["mpb"]).max() < 1e-6


def test_buildw_on_gpu_mpb(small, ctx_small, orc):
    img, _, _ = small
    ctx, _, _ = ctx_small
    H, W, _ = img.shape
    mpb = ctx.fetch("mpb", 0, (H, W), np.float32).astype(np.float64)
    Wg = ctx.fetch("W", 0, (H, W, 81), np.float32)
    assert np.abs(Wg - orc.buildW(mpb)).max() < 1e-6


def _residuals(orc, Wd, evals, evecs):
    """FP64 |A y - lambda y| of unit y on A = I - D^-1/2 W D^-1/2."""
    import scipy.sparse as sp
    H, W, _ = Wd.shape
    N = H * W
    dy, dx = orc.stencil()
    yy, xx = np.divmod(np.arange(N), W)
    r, c, v = [], [], []
    for k in range(81):
        y2, x2 = yy + dy[k], xx + dx[k]
        m = (y2 >= 0) & (y2 < H) & (x2 >= 0) & (x2 < W)
        r.append(np.arange(N)[m]); c.append((y2 * W + x2)[m]); v.append(Wd.reshape(N, 81)[m, k])
    Wm = sp.csr_matrix((np.concatenate(v), (np.concatenate(r), np.concatenate(c))), shape=(N, N))
    dis = 1 / np.sqrt(np.asarray(Wm.sum(1)).ravel())
    A = sp.identity(N) - sp.diags(dis) @ Wm @ sp.diags(dis)
    out = []
    for lam, y in zip(evals, evecs):
        y = y / np.linalg.norm(y)
        out.append(np.linalg.norm(A @ y - lam * y))
    return np.array(out)


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_eigenvectors_residual(small, orc, mode):
    import gpb
    img, cb, _ = small
    ctx = gpb.Context(cb, keep_intermediates=1, eig_mode=mode)
    gpb.GlobalPbCuda(ctx, img)
    H, W, _ = img.shape
    Wg = ctx.fetch("W", 0, (H, W, 81), np.float32).astype(np.float64)
    ev = ctx.fetch("evals", 0, (9,), np.float32).astype(np.float64)
    X = ctx.fetch("evecs", 0, (9, H * W), np.float32).astype(np.float64)
    res = _residuals(orc, Wg, ev, X)
    assert res.max() <= 1e-4          # the stated criterion
    assert res.max() <= 3 * ctx.params.eig_tol
    np.testing.assert_allclose(X @ X.T / np.outer(np.linalg.norm(X, axis=1), np.linalg.norm(X, axis=1)),
                               np.eye(9), atol=1e-4)
    ctx.close()


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_gpb_small_both_solvers(small, mode):
    import gpb
    img, cb, ref = small
    ctx = gpb.Context(cb, eig_mode=mode)
    orient, nmax = gpb.GlobalPbCuda(ctx, img)
    assert np.abs(np.stack(orient) - ref["gpb_o"]).max() < GPB_TOL
    assert np.abs(nmax - ref["nmax"]).max() < GPB_TOL
    ctx.close()


@pytest.mark.parametrize("mode", [0, 1])
def test_gpb_single_patch_321x481(orc, mode):
    """321 x 481, 24 cells: the reference's single-patch case."""
    import gpb
    from gpb import synth
    img, cb = synth.image_321x481()
    ref = orc.globalpb(img, cb)
    ctx = gpb.Context(cb, eig_mode=mode, keep_intermediates=1)
    orient, nmax = gpb.GlobalPbCuda(ctx, img)
    assert np.array_equal(ctx.fetch("texton", 0, img.shape[:2], np.uint8), ref["texton"])
    err = np.abs(np.stack(orient) - ref["gpb_o"])
    assert err.max() < GPB_TOL, err.max()
    assert np.abs(nmax - ref["nmax"]).max() < GPB_TOL
    ctx.close()


def test_damascene_layout(small):
    """GPB_COMPAT_DAMASCENE: GPU weight sets, nmax masked by mPb > 0.05, orient
    planes sigmoid-rescaled, oriMap-permuted and column-major."""
    import gpb
    img, cb, _ = small
    H, W, _ = img.shape
    ctx = gpb.Context(cb, compat=gpb.COMPAT_DAMASCENE, keep_intermediates=1)
    nm, orr = gpb.compute_gpb(ctx, gpb.synth.pack_bgr(img))
    g = ctx.fetch("gpb_o", 0, (8, H, W), np.float32).astype(np.float64)
    mpb = ctx.fetch("mpb", 0, (H, W), np.float32)
    want_nm = np.where(mpb > 0.05, g.max(0), 0.0)
    assert np.abs(nm.reshape(H, W) - want_nm).max() < 1e-6
    ori_map = [4, 5, 6, 7, 0, 1, 2, 3]
    v = np.clip(g * 1.2, None, 1.0)
    v = np.where(g * 1.2 > 1, 1.0, g * 1.2)
    v[v < 0] = 0
    v = (1 / (1 + np.exp(2.6433 - 10.7998 * v)) - 0.0667) / 0.9333
    planes = orr.reshape(8, W, H)
    for i in range(8):
        assert np.abs(planes[i].T - v[ori_map[i]]).max() < 1e-5
    # GlobalPbCuda's reading of the same buffers (src/globalPb.cpp:293-301)
    orient, nmax = gpb.GlobalPbCuda(ctx, img)
    assert np.abs(orient[0] - v[4]).max() < 1e-5
    ctx.close()


def test_batch_matches_single():
    """Uneven patches in one batch give the same result as one at a time."""
    import gpb
    from gpb import synth
    img, cb = _img(200, 260, 20, 21)
    boxes = [(0, 0, 64, 100), (20, 30, 97, 33), (100, 120, 100, 140), (5, 200, 40, 60)]
    patches = [synth.pack_bgr(img[y:y + h, x:x + w]) for (y, x, h, w) in boxes]
    ctx = gpb.Context(cb)
    batch = ctx.compute_batch(patches)
    for p, (nm_b, or_b) in zip(patches, batch):
        nm_s, or_s = ctx.compute_batch([p])[0]
        assert np.abs(or_b - or_s).max() < 1e-6
        assert np.abs(nm_b - nm_s).max() < 1e-6
    ctx.close()


@pytest.mark.parametrize("mode", [1, 2])
def test_batch_of_different_images_per_patch_parity(orc, mode):
    """Two unlike images in one batch converge after different numbers of
    block iterations; each patch still matches its own oracle run."""
    import gpb
    from gpb import synth
    imgs = [synth.voronoi_image(96, 128, 10, 8.0, synth.SEED_BASE + 5),
            synth.voronoi_image(120, 100, 25, 8.0, synth.SEED_BASE + 9, lines=3)]
    cb = synth.make_codebook(imgs[0], synth.SEED_BASE + 5, n_sample=2048)
    ctx = gpb.Context(cb, eig_mode=mode)
    outs = ctx.compute_batch([synth.pack_bgr(im) for im in imgs])
    assert ctx.last_status == gpb.GPB_OK
    for im, (nm, orr) in zip(imgs, outs):
        ref = orc.globalpb(im, cb)
        H, W, _ = im.shape
        assert np.abs(nm - ref["nmax"]).max() < GPB_TOL
        assert np.abs(orr.reshape(8, H, W) - ref["gpb_o"]).max() < GPB_TOL
    ctx.close()


def test_contexts_interleaved():
    """Contexts with different codebooks and compat modes share the device's
    constant tables; using them in turn gives each its own results."""
    import gpb
    from gpb import synth
    img_a, cb_a = _img(64, 80, 6, 31)
    img_b, cb_b = _img(72, 64, 9, 32)
    a = gpb.Context(cb_a)
    first = a.compute_batch([synth.pack_bgr(img_a)])[0]
    b = gpb.Context(cb_b, compat=gpb.COMPAT_DAMASCENE)
    only_b = b.compute_batch([synth.pack_bgr(img_b)])[0]
    again = a.compute_batch([synth.pack_bgr(img_a)])[0]
    b_again = b.compute_batch([synth.pack_bgr(img_b)])[0]
    for x, y in zip(first + only_b, again + b_again):
        assert np.array_equal(x, y)
    a.close()
    b.close()


def test_errors_are_reported():
    import gpb
    from gpb import synth
    img, cb = _img(64, 64, 4, 3)
    ctx = gpb.Context()
    with pytest.raises(gpb.GpbError) as e:  # no codebook yet
        ctx.compute_batch([synth.pack_bgr(img)])
    assert e.value.status == gpb.GPB_ERR_ARG
    ctx.set_codebook(cb)
    with pytest.raises(gpb.GpbError) as e:  # below the 32-pixel minimum side
        ctx.compute_batch([synth.pack_bgr(img[:16, :40])])
    assert e.value.status == gpb.GPB_ERR_ARG
    with pytest.raises(gpb.GpbError):
        gpb.Context(nvec=1)
    ctx.close()


def test_computeGPb_shim(small):
    """computeGPb / getCudaDeviceCount through their C++ symbols, as
    GlobalPbCuda calls them (src/globalPb.cpp:282)."""
    import gpb
    img, cb, _ = small
    H, W, _ = img.shape
    L = ctypes.CDLL(gpb.LIBPATH)
    cnt = getattr(L, "_Z18getCudaDeviceCountv")
    assert cnt() >= 1
    setcb = getattr(L, "_Z20gpbSetTextonCodebookPKfi")
    cbc = np.ascontiguousarray(cb, np.float32)
    assert setcb(cbc.ctypes.data_as(ctypes.c_void_p), ctypes.c_int(cb.shape[1])) == 0
    comp = getattr(L, "_Z10computeGPbjjjPjPPfS1_")
    packed = np.ascontiguousarray(gpb.synth.pack_bgr(img))
    p_nm, p_or = ctypes.c_void_p(), ctypes.c_void_p()
    comp(ctypes.c_uint(0), ctypes.c_uint(W), ctypes.c_uint(H), packed.ctypes.data_as(ctypes.c_void_p),
         ctypes.byref(p_nm), ctypes.byref(p_or))
    nm = np.ctypeslib.as_array((ctypes.c_float * (H * W)).from_address(p_nm.value)).copy()
    orr = np.ctypeslib.as_array((ctypes.c_float * (8 * H * W)).from_address(p_or.value)).copy()
    L.gpb_free(p_nm)
    L.gpb_free(p_or)
    ctx = gpb.Context(cb, compat=gpb.COMPAT_DAMASCENE)
    nm2, or2 = gpb.compute_gpb(ctx, packed)
    assert np.abs(nm - nm2).max() < 1e-6 and np.abs(orr - or2).max() < 1e-6
    ctx.close()


def test_batch_1024_sixteen_patches(orc):
    """The benchmark workload (16 halo'd patches of a 1024^2 image, one batch):
    every patch converges, eigen-residuals hold in FP64, and two patches match
    the full oracle within the gPb tolerance."""
    import gpb
    from gpb import synth
    img, cb = synth.image_1024()
    boxes = synth.grid_patches(1024, 1024, 4, 4, 5)
    patches = [synth.pack_bgr(img[y0:y0 + h, x0:x0 + w]) for (y0, x0, h, w, *_r) in boxes]
    ctx = gpb.Context(cb, keep_intermediates=1, eig_mode=gpb.EIG_WARM)
    outs = ctx.compute_batch(patches)
    assert ctx.last_status == gpb.GPB_OK
    for i in (0, 5):
        y0, x0, h, w = boxes[i][:4]
        ref = orc.globalpb(np.ascontiguousarray(img[y0:y0 + h, x0:x0 + w]), cb)
        assert np.abs(outs[i][1].reshape(8, h, w) - ref["gpb_o"]).max() < GPB_TOL
        Wg = ctx.fetch("W", i, (h, w, 81), np.float32).astype(np.float64)
        ev = ctx.fetch("evals", i, (9,), np.float32).astype(np.float64)
        X = ctx.fetch("evecs", i, (9, h * w), np.float32).astype(np.float64)
        assert _residuals(orc, Wg, ev, X).max() <= 1e-4
    ctx.close()


def test_batch_4096_uneven_patches(orc):
    """64 rectangles with sides in [200, 700] of a 4096^2 image (4096 cells,
    sigma 6, 40 lines), one warm-started batch: every patch converges, the
    outputs are finite gPb maps, and the two smallest patches match their own
    oracle runs within the gPb tolerance."""
    import gpb
    from gpb import synth
    img, cb, boxes = synth.image_4096_uneven()
    crops = [np.ascontiguousarray(img[y0:y0 + h, x0:x0 + w]) for (y0, x0, h, w) in boxes]
    ctx = gpb.Context(cb, eig_mode=gpb.EIG_WARM)
    outs = ctx.compute_batch([synth.pack_bgr(c) for c in crops])
    assert ctx.last_status == gpb.GPB_OK
    st = ctx.stats()
    assert 0 < st["max_residual"] <= 3 * ctx.params.eig_tol
    for (nm, orr), (_, _, h, w) in zip(outs, boxes):
        assert nm.shape == (h, w) and orr.size == 8 * h * w
        assert np.isfinite(nm).all() and np.isfinite(orr).all() and nm.min() >= 0
    smallest = sorted(range(len(boxes)), key=lambda i: boxes[i][2] * boxes[i][3])[:2]
    for i in smallest:
        ref = orc.globalpb(crops[i], cb)
        h, w = boxes[i][2], boxes[i][3]
        assert np.abs(outs[i][0] - ref["nmax"]).max() < GPB_TOL
        assert np.abs(outs[i][1].reshape(8, h, w) - ref["gpb_o"]).max() < GPB_TOL
    ctx.close()


def test_codebook_yml_round_trip(tmp_path):
    """A codebook written with gpb_write_yml and read with
    gpb_load_codebook_yml gives the same textons as gpb_set_codebook."""
    import gpb
    from gpb import synth
    img, cb = _img(48, 64, 5, 81)
    p = str(tmp_path / "texton_codebook.yml")
    c = np.ascontiguousarray(cb, np.float32)
    assert gpb._lib().gpb_write_yml(p.encode(), b"texton_codebook", c.ctypes.data, c.shape[0], c.shape[1]) == 0
    a = gpb.Context(cb, keep_intermediates=1)
    b = gpb.Context(keep_intermediates=1)
    b.load_codebook_yml(p)
    a.compute_batch([synth.pack_bgr(img)])
    b.compute_batch([synth.pack_bgr(img)])
    assert np.array_equal(a.fetch("texton", 0, (48, 64), np.uint8), b.fetch("texton", 0, (48, 64), np.uint8))
    a.close()
    b.close()
