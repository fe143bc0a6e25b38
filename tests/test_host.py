"""Host-side logic without a GPU: synthetic inputs, tiling, packing, the
oracle's own invariants."""
import numpy as np
import pytest

from gpb import synth


def test_voronoi_deterministic():
    a = synth.voronoi_image(40, 50, 6, 8.0, 123)
    b = synth.voronoi_image(40, 50, 6, 8.0, 123)
    assert a.dtype == np.uint8 and a.shape == (40, 50, 3)
    assert np.array_equal(a, b)
    assert not np.array_equal(a, synth.voronoi_image(40, 50, 6, 8.0, 124))


def test_lines_drawn():
    a = synth.voronoi_image(64, 64, 1, 0.0, 7, lines=3, ramp=0.0)
    assert len(np.unique(a.reshape(-1, 3), axis=0)) > 1


def test_pack_bgr_matches_reference_packing():
    img = np.zeros((2, 3, 3), np.uint8)
    img[0, 1] = (10, 20, 30)  # B, G, R
    p = synth.pack_bgr(img)
    assert p[0, 1] == (10 << 16) | (20 << 8) | 30


def test_grey_matches_oracle(orc):
    img = synth.voronoi_image(30, 40, 5, 8.0, 5)
    assert np.array_equal(synth.grey_u8(img), orc.grey_bgr(img))


def test_schmid_bank_matches_oracle(orc):
    assert np.allclose(synth.schmid_bank(), orc.schmid_bank(), rtol=0, atol=1e-15)


def test_codebook_shape():
    img = synth.voronoi_image(48, 48, 4, 8.0, 9)
    cb = synth.make_codebook(img, 9, n_sample=512, iters=3)
    assert cb.shape == (13, 32) and cb.dtype == np.float32 and np.isfinite(cb).all()


@pytest.mark.parametrize("H,W,r,c,h", [(1024, 1024, 4, 4, 5), (300, 451, 3, 2, 5), (64, 64, 1, 1, 0)])
def test_grid_patches_cover_exactly_once(H, W, r, c, h):
    owner = np.zeros((H, W), np.int32)
    for (y0, x0, ph, pw, iy, ix, ih, iw) in synth.grid_patches(H, W, r, c, h):
        assert 0 <= y0 and y0 + ph <= H and 0 <= x0 and x0 + pw <= W
        assert 0 <= iy and iy + ih <= ph and 0 <= ix and ix + iw <= pw
        owner[y0 + iy:y0 + iy + ih, x0 + ix:x0 + ix + iw] += 1
    assert (owner == 1).all()


def test_texton_argmin_fix(orc):
    img = synth.voronoi_image(40, 40, 5, 8.0, 3)
    cb = synth.make_codebook(img, 3, n_sample=512, iters=2)
    g = synth.grey_u8(img)
    lab, R = orc.texton_map(g, cb, responses=True)
    # fixed: true nearest codeword; as shipped (D4): constant K-1
    d = ((R.reshape(13, -1).T[:, :, None] - cb[None].astype(np.float64)) ** 2).sum(1)
    assert np.array_equal(lab.ravel(), d.argmin(1))
    assert (orc.texton_map(g, cb, fix_argmin=0) == 31).all()


def test_eigs_residual_and_orthonormality(orc):
    rng = np.random.default_rng(0)
    m = np.clip(rng.random((24, 30)) ** 3, 0, 1)
    Wd = orc.buildW(m)
    ev, vec, it, res = orc.eigs(Wd, 9, tol=1e-10)
    assert it > 0 and res.max() <= 1e-10
    assert np.all(np.diff(ev) >= -1e-14) and abs(ev[0]) < 1e-10
    np.testing.assert_allclose(vec @ vec.T, np.eye(9), atol=1e-8)


def test_oefilter_is_an_oriented_derivative(orc):
    for o in range(8):
        f = orc.oefilter(o * 3.1415926535 / 8)
        assert abs(f.sum()) < 1e-12 and abs(np.abs(f).sum() - 1) < 1e-12
        assert np.allclose(f, -f[::-1, ::-1], atol=1e-12)  # odd symmetry


def test_spb_orientation_follows_local_cues(orc):
    """A straight vertical step edge: the orientation of maximal sPb and of
    maximal texture gradient must agree (the ch_per slot mapping)."""
    H, W = 48, 48
    lab = np.zeros((H, W), np.uint8)
    lab[:, W // 2:] = 5
    cues = orc.hist_gradient(orc.mirror(lab, 30), 30, 5, None)
    v = np.tile(np.linspace(0, 1, W), (H, 1))
    v[:, W // 2:] += 1.0
    spb = orc.spb(np.array([0.0, 0.5]), np.stack([np.ones(H * W), v.ravel()]), np.ones(H * W), H, W, 2)
    y, x = H // 2, W // 2
    assert int(np.argmax(cues[:, y, x])) == int(np.argmax(spb[:, y, x]))


def test_superpixel_features_oracle_known_answer(orc):
    """The SPFeatures restatement on a hand-checked 2 x 3 case: two
    superpixels, one skipped pixel (label -1), bin_step 128 (2 grey bins)."""
    bgr = np.array([[[0, 0, 0], [255, 255, 255], [10, 20, 30]],
                    [[255, 255, 255], [0, 0, 0], [1, 2, 3]]], np.uint8)
    texton = np.array([[0, 1, 1], [2, 0, 0]], np.uint8)
    labels = np.array([[0, 0, 1], [1, 0, -1]], np.int32)
    out = orc.superpixel_features(bgr, texton, labels, 2, 128, K=3)
    grey = orc.grey_bgr(bgr)
    assert out.shape == (2, 3 + 2 + 4)
    # superpixel 0: pixels (0,0) black, (0,1) white, (1,1) black; textons 0, 1, 0
    np.testing.assert_array_equal(out[0, :3], np.array([2, 1, 0]) / 3 * 10)
    np.testing.assert_array_equal(out[0, 3:5], np.array([2, 1]) / 3 * 10)
    assert out[0, 5] == 0
    np.testing.assert_allclose(out[0, 6:], np.array([255, 255, 255]) / 3 * (10 / 255))
    # superpixel 1: (0,2) and (1,0); textons 1 and 2
    np.testing.assert_array_equal(out[1, :3], np.array([0, 1, 1]) / 2 * 10)
    assert grey[0, 2] < 128 <= grey[1, 0]
    np.testing.assert_array_equal(out[1, 3:5], np.array([1, 1]) / 2 * 10)
    np.testing.assert_allclose(out[1, 6:], np.array([10 + 255, 20 + 255, 30 + 255]) / 2 * (10 / 255))
