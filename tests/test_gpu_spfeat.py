"""gpb_superpixel_features (the GLSVM superpixel descriptors of SPFeatures,
src/SPFeatures.cpp:101-114, 260-275, 380-391) against the restatement in the
oracle, on the texton map and grey image of a computed patch: integer counts
and the reference's FP64 normalisation, so the rows are bit-exact."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("bin_step,with_textons", [(8, True), (16, False), (1, True)])
def test_superpixel_features_match_oracle(orc, bin_step, with_textons):
    torch = pytest.importorskip("torch")
    import gpb
    from gpb import synth
    H, W = 96, 128
    img = synth.voronoi_image(H, W, 12, 8.0, synth.SEED_BASE + 71)
    cb = synth.make_codebook(img, synth.SEED_BASE + 71, n_sample=2048)
    ctx = gpb.Context(cb, eig_mode=gpb.EIG_WARM, keep_intermediates=1)
    ctx.compute_batch([synth.pack_bgr(img)])
    texton = ctx.fetch("texton", 0, (H, W), np.uint8)
    # superpixels: a coarse Voronoi partition of its own, some pixels unlabelled
    rng = np.random.default_rng(3)
    sites = rng.uniform([0, 0], [H, W], (40, 2))
    yy, xx = np.mgrid[0:H, 0:W]
    labels = np.argmin((yy[..., None] - sites[:, 0]) ** 2 + (xx[..., None] - sites[:, 1]) ** 2, axis=2).astype(np.int32)
    labels[:5, :7] = -1
    labels[50, 60] = 1000          # out of range: skipped
    n = 45                          # labels 40..44 are empty: zero rows
    d_lab = torch.from_numpy(labels.ravel()).cuda()
    K = cb.shape[1] if with_textons else 0
    ncol = K + 255 // bin_step + 1 + 4
    d_out = torch.full((n * ncol,), -1.0, dtype=torch.float64, device="cuda")
    ctx.superpixel_features(0, d_lab.data_ptr(), n, d_out.data_ptr(), bin_step=bin_step, with_textons=with_textons)
    got = d_out.cpu().numpy().reshape(n, ncol)
    want = orc.superpixel_features(img, texton, labels, n, bin_step, K=K)
    assert np.array_equal(got, want)
    assert not got[40:].any()
    ctx.close()
