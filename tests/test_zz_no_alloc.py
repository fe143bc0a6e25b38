"""gpb_texton_labels_static, the allocation-free texton entry point, against
the batch entry point (gpb_compute_batch + gpb_fetch) on the same images.

The file sorts last so that it also runs after every other GPU test has
used (and reloaded) the device's constant tables and the library's kernels.
Device buffers come from torch; only the entry point must not allocate.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _images():
    from gpb import synth
    a = synth.voronoi_image(96, 128, 10, 8.0, synth.SEED_BASE + 41)
    b = synth.voronoi_image(120, 100, 25, 8.0, synth.SEED_BASE + 42, lines=3)
    cb = synth.make_codebook(a, synth.SEED_BASE + 41, n_sample=2048)
    return a, b, cb


def _batch_labels(ctx, img):
    """L | a<<8 | b<<16 | texton<<24 through the existing entry point."""
    from gpb import synth
    H, W, _ = img.shape
    ctx.compute_batch([synth.pack_bgr(img)])
    tex = ctx.fetch("texton", 0, (H, W), np.uint8).astype(np.uint32)
    bins = ctx.fetch("labbins", 0, (3, H, W), np.uint8).astype(np.uint32)
    return (bins[0] | (bins[1] << 8) | (bins[2] << 16) | (tex << 24)).ravel()


def _dev(torch, arr_u32):
    return torch.from_numpy(np.ascontiguousarray(arr_u32).view(np.int32).ravel()).cuda()


def test_static_labels_match_batch_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    import gpb
    from gpb import synth
    a, b, cb = _images()
    ctx = gpb.Context(cb, keep_intermediates=1)
    want = [_batch_labels(ctx, a), _batch_labels(ctx, b)]
    pa, pb = _dev(torch, synth.pack_bgr(a)), _dev(torch, synth.pack_bgr(b))
    oa = torch.full((a.shape[0] * a.shape[1],), -1, dtype=torch.int32, device="cuda")
    ob = torch.full((b.shape[0] * b.shape[1],), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    # two calls in a row on one stream, different sizes: the second must not
    # see the first one's tile list, counter or repair list
    ctx.texton_labels_static(a.shape[1], a.shape[0], pa.data_ptr(), oa.data_ptr(), stream)
    ctx.texton_labels_static(b.shape[1], b.shape[0], pb.data_ptr(), ob.data_ptr(), stream)
    torch.cuda.synchronize()
    assert np.array_equal(oa.cpu().numpy().view(np.uint32), want[0])
    assert np.array_equal(ob.cpu().numpy().view(np.uint32), want[1])
    ctx.close()


def test_static_labels_allocate_nothing():
    """After the first call (the per-device set-up), further calls leave the
    device's free memory unchanged."""
    torch = pytest.importorskip("torch")
    import gpb
    from gpb import synth
    a, b, cb = _images()
    ctx = gpb.Context(cb)
    pa, pb = _dev(torch, synth.pack_bgr(a)), _dev(torch, synth.pack_bgr(b))
    oa = torch.empty(a.shape[0] * a.shape[1], dtype=torch.int32, device="cuda")
    ob = torch.empty(b.shape[0] * b.shape[1], dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    ctx.texton_labels_static(a.shape[1], a.shape[0], pa.data_ptr(), oa.data_ptr(), stream)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        ctx.texton_labels_static(a.shape[1], a.shape[0], pa.data_ptr(), oa.data_ptr(), stream)
        ctx.texton_labels_static(b.shape[1], b.shape[0], pb.data_ptr(), ob.data_ptr(), stream)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    ctx.close()


def test_static_labels_reject_oversize_and_bad_arguments():
    torch = pytest.importorskip("torch")
    import gpb
    _, _, cb = _images()
    ctx = gpb.Context(cb)
    buf = torch.zeros(64, dtype=torch.int32, device="cuda")
    p = buf.data_ptr()
    # 2048 x 1024 = 2^21 pixels: beyond the fixed scratch, nothing launched
    with pytest.raises(gpb.GpbError) as e:
        ctx.texton_labels_static(2048, 1024, p, p)
    assert e.value.status == gpb.GPB_ERR_TOO_LARGE
    with pytest.raises(gpb.GpbError) as e:  # a side below 32
        ctx.texton_labels_static(16, 64, p, p)
    assert e.value.status == gpb.GPB_ERR_ARG
    with pytest.raises(gpb.GpbError) as e:  # misaligned output
        ctx.texton_labels_static(32, 32, p, p + 2)
    assert e.value.status == gpb.GPB_ERR_ARG
    ctx.close()
    no_cb = gpb.Context()
    with pytest.raises(gpb.GpbError) as e:
        no_cb.texton_labels_static(32, 32, p, p)
    assert e.value.status == gpb.GPB_ERR_ARG
    no_cb.close()


def test_static_labels_then_other_codebook_on_another_stream():
    """A context with another codebook reloads the device's constant tables
    right after a static call queued behind other work on a side stream: the
    reload waits for the static call's kernels, which keep their own
    codebook."""
    torch = pytest.importorskip("torch")
    import gpb
    from gpb import synth
    a, b, cb_a = _images()
    cb_b = synth.make_codebook(b, synth.SEED_BASE + 42, n_sample=2048)
    ca = gpb.Context(cb_a, keep_intermediates=1)
    cbb = gpb.Context(cb_b)
    want = _batch_labels(ca, a)
    pa = _dev(torch, synth.pack_bgr(a))
    oa = torch.full((a.shape[0] * a.shape[1],), -1, dtype=torch.int32, device="cuda")
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())  # the input copy and the output fill first
    with torch.cuda.stream(side):
        torch.cuda._sleep(40_000_000)  # about 20 ms of GPU time ahead of the static kernels
    ca.texton_labels_static(a.shape[1], a.shape[0], pa.data_ptr(), oa.data_ptr(), side.cuda_stream)
    cbb.compute_batch([synth.pack_bgr(b)])  # reloads the tables with cb_b
    torch.cuda.synchronize()
    assert np.array_equal(oa.cpu().numpy().view(np.uint32), want)
    ca.close()
    cbb.close()
