"""OWT-UCM stage on the GPU through the C ABI (gpb_ucm): the golden
fixtures written by the reference's own UCM sources, the oracle restatement
stage by stage on larger seeded inputs, device-resident input, and the
gPb -> UCM chain on a synthetic image."""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import ucm_oracle as uo  # noqa: E402

GOLD = os.path.join(ROOT, "tests", "golden", "ucm_cases.npz")
CASES = ["rand40x50", "rand80x64", "gpb48x64", "tiny5x7", "flat32", "noise2x3", "noise4x9"]
UCM_TOL = 1e-12  # calibration uses exp(); libm builds may differ in the last bit


@pytest.fixture(scope="module")
def gold():
    z = np.load(GOLD)
    return {c: {k.split("/", 1)[1]: z[k] for k in z.files if k.startswith(c + "/")} for c in CASES}


@pytest.fixture(scope="module")
def ctx():
    import gpb
    c = gpb.Context()
    yield c
    c.close()


@pytest.mark.parametrize("case", CASES)
def test_ucm_matches_reference_fixtures(ctx, gold, case):
    import gpb
    g = gold[case]
    u2, info = ctx.ucm(g["planes"], double_size=True)
    assert np.array_equal(ctx.ucm_fetch(gpb.UCM_QUANT), g["quant"])
    assert np.array_equal(ctx.ucm_fetch(gpb.UCM_ARCS), g["arcs"])
    assert np.array_equal(ctx.ucm_fetch(gpb.UCM_WSWT).astype(np.float64), g["wswt"])
    assert np.array_equal(ctx.ucm_fetch(gpb.UCM_WSWT2).astype(np.float64), g["wswt2"])
    assert np.array_equal(ctx.ucm_fetch(gpb.UCM_REGIONS), g["labels"])
    assert np.abs(u2 - g["ucm2"]).max() <= UCM_TOL
    assert info["fit_ok"] == 1 and info["n_edges"] == len(g["edges"])
    u, _ = ctx.ucm(g["planes"], double_size=False)
    assert u.shape == g["ucm"].shape and np.abs(u - g["ucm"]).max() <= UCM_TOL


def _planes(H, W, seed, sigma):
    from scipy.ndimage import gaussian_filter
    rng = np.random.default_rng(seed)
    g = np.stack([gaussian_filter(rng.random((H, W)), sigma) for _ in range(8)])
    g = (g - g.min()) / (g.max() - g.min())
    return (g ** 2).astype(np.float32)


@pytest.mark.parametrize("H,W,seed,sigma", [(150, 120, 21, 1.4), (266, 266, 22, 2.0), (97, 301, 23, 0.9)])
def test_ucm_stages_against_oracle(ctx, H, W, seed, sigma):
    """Every device stage against the oracle on inputs with no fixture; the
    contours are the library's host fitting (pinned to the reference on
    the CPU)."""
    import gpb
    p = _planes(H, W, seed, sigma)
    g = p.astype(np.float64)
    u2, info = ctx.ucm(p)
    q = ctx.ucm_fetch(gpb.UCM_QUANT)
    assert np.array_equal(q, uo.quantize(g))
    arcs = ctx.ucm_fetch(gpb.UCM_ARCS)
    assert np.array_equal(arcs, (uo.watershed(q) == 0).astype(np.uint8))
    vert, edges, off, px = gpb.ucm_fit_contours(arcs)
    w = ctx.ucm_fetch(gpb.UCM_WSWT).astype(np.float64)
    assert np.array_equal(w, uo.paint(g, vert, edges, off, px))
    w2, lab, nart, nreg = uo.super_clean(w)
    assert np.array_equal(ctx.ucm_fetch(gpb.UCM_WSWT2).astype(np.float64), w2)
    assert np.array_equal(ctx.ucm_fetch(gpb.UCM_REGIONS), lab)
    assert info["n_artefacts"] == nart and info["n_regions"] == nreg
    assert np.abs(u2 - uo.normalize(gpb.ucm_mean_pb(w2, lab))).max() == 0.0
    assert np.abs(u2 - uo.normalize(uo.mean_pb(w2, lab))).max() <= UCM_TOL


def test_ucm_device_input_and_reuse(ctx):
    """Planes already on the device give the same map as host planes; a
    context serves images of different sizes one after another."""
    import torch
    for (H, W, s) in [(64, 80, 31), (120, 40, 32), (64, 80, 31)]:
        p = _planes(H, W, s, 1.3)
        host, _ = ctx.ucm(p)
        d = torch.from_numpy(p).cuda()
        dev, _ = ctx.ucm(None, d_orient=d.data_ptr(), shape=(H, W))
        torch.cuda.synchronize()
        assert np.array_equal(host, dev)


def test_ucm_of_constant_planes(ctx):
    u2, info = ctx.ucm(np.full((8, 33, 47), 0.3, np.float32))
    assert info["n_edges"] == 0 and info["n_regions"] == 1 and not u2.any()


def test_gpb_to_ucm_chain(orc):
    """gPb of a synthetic image through GlobalPbCuda's planes, then UCM: the
    map equals the oracle chain on the same planes, and region boundaries
    at a middle scale follow strong gPb."""
    import gpb
    from gpb import synth
    img = synth.voronoi_image(96, 128, 12, 8.0, synth.SEED_BASE + 41, lines=1)
    cb = synth.make_codebook(img, synth.SEED_BASE + 41, n_sample=1024)
    c = gpb.Context(cb, compat=gpb.COMPAT_DAMASCENE)
    orient, nmax = gpb.GlobalPbCuda(c, img)
    planes = np.stack(orient).astype(np.float32)
    u2, info = c.ucm(planes)
    c.close()
    g = planes.astype(np.float64)
    q = uo.quantize(g)
    arcs = (uo.watershed(q) == 0).astype(np.uint8)
    vert, edges, off, px = gpb.ucm_fit_contours(arcs)
    w2, lab, _, _ = uo.super_clean(uo.paint(g, vert, edges, off, px))
    assert np.abs(u2 - uo.normalize(uo.mean_pb(w2, lab))).max() <= UCM_TOL
    assert info["n_regions"] > 1 and u2.max() > 0


def test_ucm_is_ultrametric_at_scale(ctx):
    """Size-independent properties on a 640 x 512 image: values in [0, 1],
    even-even points the max of their 4 neighbours, and the regions at a
    higher threshold are unions of the regions at a lower one."""
    import gpb
    u2, info = ctx.ucm(_planes(640, 512, 51, 1.6))
    assert info["fit_ok"] == 1 and 0.0 <= u2.min() and u2.max() <= 1.0
    e = u2[2:-2:2, 2:-2:2]
    nbr = np.maximum.reduce([u2[1:-3:2, 2:-2:2], u2[3:-1:2, 2:-2:2], u2[2:-2:2, 1:-3:2], u2[2:-2:2, 3:-1:2]])
    assert np.array_equal(e, nbr)
    prev = None
    for k in (0.05, 0.15, 0.3, 0.6):
        lab, n = gpb.ucm_labels_at_scale(u2, k)
        if prev is not None:
            pl, pn = prev
            assert n <= pn
            # every finer region maps into exactly one coarser region
            pairs = np.unique(np.stack([pl.ravel(), lab.ravel()]), axis=1)
            assert len(np.unique(pairs[0])) == pairs.shape[1]
        prev = (lab, n)


def test_ucm_batch_equals_single_calls(ctx):
    """A batch of uneven images (flooded together, fitted and merged on
    the host threads) gives each image the map and intermediates of its
    own single call."""
    import gpb
    shapes = [(64, 80, 61), (33, 47, 62), (150, 120, 63), (40, 40, 64), (97, 30, 65)]
    planes = [_planes(h, w, s, 1.3) for (h, w, s) in shapes]
    got = ctx.ucm_batch(planes)
    arcs_b = [ctx.ucm_fetch(gpb.UCM_ARCS, i) for i in range(len(planes))]
    regs_b = [ctx.ucm_fetch(gpb.UCM_REGIONS, i) for i in range(len(planes))]
    for i, p in enumerate(planes):
        u, info = ctx.ucm(p)
        assert np.array_equal(got[i][0], u)
        assert got[i][1]["n_regions"] == info["n_regions"] and got[i][1]["n_edges"] == info["n_edges"]
        assert np.array_equal(arcs_b[i], ctx.ucm_fetch(gpb.UCM_ARCS))
        assert np.array_equal(regs_b[i], ctx.ucm_fetch(gpb.UCM_REGIONS))
    small = ctx.ucm_batch(planes[:2], double_size=False)
    for i in range(2):
        assert np.array_equal(small[i][0], ctx.ucm(planes[i], double_size=False)[0])


def test_ucm_rejects_bad_arguments(ctx):
    """sizes below 2, an empty batch, a NULL plane and an image index past
    the last call's batch return GPB_ERR_ARG and launch nothing"""
    import ctypes
    import gpb
    L = gpb._lib()
    out = np.zeros(64, np.float64)
    planes = np.zeros((8, 4, 4), np.float32)
    assert L.gpb_ucm(ctx._h, 1, 4, planes.ctypes.data, 0, 1, out.ctypes.data, None) == gpb.GPB_ERR_ARG
    assert L.gpb_ucm(ctx._h, 4, 4, None, 0, 1, out.ctypes.data, None) == gpb.GPB_ERR_ARG
    w = np.array([4], np.uint32)
    ptrs = (ctypes.c_void_p * 1)(planes.ctypes.data)
    outs = (ctypes.c_void_p * 1)(out.ctypes.data)
    assert L.gpb_ucm_batch(ctx._h, 0, w.ctypes.data, w.ctypes.data, ptrs, 0, 1, outs, None) == gpb.GPB_ERR_ARG
    ctx.ucm(_planes(9, 11, 71, 1.0))
    buf = np.zeros(99, np.uint8)
    assert L.gpb_ucm_fetch(ctx._h, 1, gpb.UCM_QUANT, buf.ctypes.data, buf.nbytes) == gpb.GPB_ERR_ARG
    assert L.gpb_ucm_fetch(ctx._h, 0, gpb.UCM_QUANT, buf.ctypes.data, 10) == gpb.GPB_ERR_ARG
    assert L.gpb_ucm_fetch(ctx._h, 0, gpb.UCM_QUANT, buf.ctypes.data, buf.nbytes) == gpb.GPB_OK
