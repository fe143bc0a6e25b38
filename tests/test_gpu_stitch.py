"""gpb_stitch_device (whole-image planes from the halo'd patches of one batch,
the device twin of Pieces2Gpb, src/utilities.cpp:180-213) against the same
stitching done on the host from the per-patch outputs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _weights(h, w, y0, x0, H, W, ramp):
    yy, xx = np.meshgrid(np.arange(h) + 0.5, np.arange(w) + 0.5, indexing="ij")
    wt = np.ones((h, w), np.float64)
    if y0 > 0:
        wt = np.minimum(wt, yy / ramp)
    if x0 > 0:
        wt = np.minimum(wt, xx / ramp)
    if y0 + h < H:
        wt = np.minimum(wt, (h - yy) / ramp)
    if x0 + w < W:
        wt = np.minimum(wt, (w - xx) / ramp)
    return wt


@pytest.fixture(scope="module")
def batch():
    import gpb
    from gpb import synth
    H, W = 300, 420
    img = synth.voronoi_image(H, W, 30, 8.0, synth.SEED_BASE + 61)
    cb = synth.make_codebook(img, synth.SEED_BASE + 61, n_sample=2048)
    boxes = synth.grid_patches(H, W, 2, 3, 5)
    outs = {}
    for compat in (gpb.COMPAT_CPU, gpb.COMPAT_DAMASCENE):
        ctx = gpb.Context(cb, eig_mode=gpb.EIG_WARM, compat=compat)
        res = ctx.compute_batch([synth.pack_bgr(img[y0:y0 + h, x0:x0 + w]) for (y0, x0, h, w, *_r) in boxes])
        outs[compat] = (ctx, res)
    yield H, W, boxes, outs
    for ctx, _ in outs.values():
        ctx.close()


def _planes(res, boxes, compat):
    """Per-patch (nmax H x W, orient 8 x H x W) in row-major image orientation."""
    import gpb
    out = []
    for (nm, orr), (_, _, h, w, *_r) in zip(res, boxes):
        o = orr.reshape(8, w, h).transpose(0, 2, 1) if compat == gpb.COMPAT_DAMASCENE else orr.reshape(8, h, w)
        out.append((nm.reshape(h, w), o))
    return out


@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("compat", [0, 1])
def test_stitch_matches_host(batch, mode, compat):
    torch = pytest.importorskip("torch")
    H, W, boxes, outs = batch
    ctx, res = outs[compat]
    places = [(x0, y0, ix, iy, iw, ih) for (y0, x0, h, w, iy, ix, ih, iw) in boxes]
    d_nm = torch.full((H * W,), -7.0, dtype=torch.float32, device="cuda")
    d_or = torch.full((8 * H * W,), -7.0, dtype=torch.float32, device="cuda")
    ctx.stitch_device(mode, W, H, places, d_nm.data_ptr(), d_or.data_ptr(), ramp=10)
    got_nm = d_nm.cpu().numpy().reshape(H, W)
    got_or = d_or.cpu().numpy().reshape(8, H, W)
    per = _planes(res, boxes, compat)
    want_nm = np.full((H, W), -7.0)
    want_or = np.full((8, H, W), -7.0)
    if mode == 2:
        acc = np.zeros((10, H, W))
        for (nm, o), (y0, x0, h, w, *_r) in zip(per, boxes):
            wt = _weights(h, w, y0, x0, H, W, 10.0)
            acc[0, y0:y0 + h, x0:x0 + w] += wt
            acc[1, y0:y0 + h, x0:x0 + w] += wt * nm
            acc[2:, y0:y0 + h, x0:x0 + w] += wt * o
        want_nm = acc[1] / acc[0]
        want_or = acc[2:] / acc[0]
        assert np.abs(got_nm - want_nm).max() < 1e-5 and np.abs(got_or - want_or).max() < 1e-5
        return
    for (nm, o), (y0, x0, h, w, iy, ix, ih, iw) in zip(per, boxes):
        if mode == 0:   # the reference's order: later patches overwrite
            want_nm[y0:y0 + h, x0:x0 + w] = nm
            want_or[:, y0:y0 + h, x0:x0 + w] = o
        else:
            want_nm[y0 + iy:y0 + iy + ih, x0 + ix:x0 + ix + iw] = nm[iy:iy + ih, ix:ix + iw]
            want_or[:, y0 + iy:y0 + iy + ih, x0 + ix:x0 + ix + iw] = o[:, iy:iy + ih, ix:ix + iw]
    assert np.array_equal(got_nm, want_nm.astype(np.float32))
    assert np.array_equal(got_or, want_or.astype(np.float32))


def test_stitch_rejects_mismatched_places(batch):
    import gpb
    H, W, boxes, outs = batch
    ctx, _ = outs[0]
    with pytest.raises(gpb.GpbError):
        ctx.stitch_device(1, W, H, [(0, 0, 0, 0, 1, 1)], 16, 16)
