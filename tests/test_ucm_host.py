"""OWT-UCM stage on the CPU: the oracle restatement against the golden
fixtures written by the reference's own UCM sources, the library's host
stages (contour fitting, mean-boundary merge, labels at a scale) against
the same fixtures, and -- where the reference is built on this machine --
both against the reference on further seeded inputs."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import ucm_oracle as uo  # noqa: E402

GOLD = os.path.join(ROOT, "tests", "golden", "ucm_cases.npz")
CASES = ["rand40x50", "rand80x64", "gpb48x64", "tiny5x7", "flat32", "noise2x3", "noise4x9"]
UCM_TOL = 1e-12  # calibration goes through exp(); numpy's and libm's may differ in the last bit


@pytest.fixture(scope="module")
def gold():
    z = np.load(GOLD)
    return {c: {k.split("/", 1)[1]: z[k] for k in z.files if k.startswith(c + "/")} for c in CASES}


@pytest.mark.parametrize("case", CASES)
def test_oracle_chain_matches_reference_fixtures(gold, case):
    g = gold[case]
    planes = g["planes"].astype(np.float64)
    q = uo.quantize(planes)
    assert np.array_equal(q, g["quant"])
    assert np.array_equal((uo.watershed(q) == 0).astype(np.uint8), g["arcs"])
    w = uo.paint(planes, g["vertices"], g["edges"], g["off"], g["pixels"])
    assert np.array_equal(w, g["wswt"])
    w2, lab, _, _ = uo.super_clean(w)
    assert np.array_equal(w2, g["wswt2"]) and np.array_equal(lab, g["labels"])
    u2 = uo.normalize(uo.mean_pb(w2, lab))
    assert np.abs(u2 - g["ucm2"]).max() <= UCM_TOL
    assert np.abs(uo.downsample(u2) - g["ucm"]).max() <= UCM_TOL


@pytest.mark.parametrize("case", CASES)
def test_library_host_fit_matches_reference(gold, case):
    import gpb
    g = gold[case]
    fit = gpb.ucm_fit_contours(g["arcs"])
    assert fit is not None
    vert, edges, off, px = fit
    assert np.array_equal(vert, g["vertices"])
    assert np.array_equal(edges, g["edges"])
    assert np.array_equal(off, g["off"]) and np.array_equal(px, g["pixels"])


@pytest.mark.parametrize("case", CASES)
def test_library_host_merge_matches_reference(gold, case):
    import gpb
    g = gold[case]
    u = gpb.ucm_mean_pb(g["wswt2"], g["labels"])
    assert np.array_equal(u, uo.mean_pb(g["wswt2"], g["labels"].astype(np.int64)))
    assert np.abs(uo.normalize(u) - g["ucm2"]).max() <= UCM_TOL


@pytest.mark.parametrize("k", [-1.0, 0.0, 0.05, 0.2, 0.5, 1.0, 2.0])
def test_labels_at_scale(gold, k):
    import gpb
    u2 = gold["rand80x64"]["ucm2"]
    lab, n = gpb.ucm_labels_at_scale(u2, k)
    ref_lab, ref_n = uo.labels_at_scale(u2, k)
    assert n == ref_n and np.array_equal(lab, ref_lab)


def test_fit_of_empty_map():
    import gpb
    vert, edges, off, px = gpb.ucm_fit_contours(np.zeros((9, 11), np.uint8))
    assert len(vert) == 0 and len(edges) == 0 and list(off) == [0] and len(px) == 0


# ---------------------------------------------------------------- against the reference itself

def _planes(H, W, seed, sigma):
    from scipy.ndimage import gaussian_filter
    rng = np.random.default_rng(seed)
    g = np.stack([gaussian_filter(rng.random((H, W)), sigma) for _ in range(8)])
    g = (g - g.min()) / (g.max() - g.min())
    return np.ascontiguousarray((g ** 2).astype(np.float32).astype(np.float64))


def _P(a):
    import ctypes
    return a.ctypes.data_as(ctypes.c_void_p)


def _ref_fit(L, bw):
    H, W = bw.shape
    cv, ce, cp = H * W, 4 * H * W, 4 * H * W
    nv = np.zeros(1, np.int32)
    vert, ed = np.zeros(2 * cv, np.int32), np.zeros(2 * ce, np.int32)
    cm, off, xy = np.zeros(ce, np.int32), np.zeros(ce + 1, np.int32), np.zeros(2 * cp, np.int32)
    ne = L.ref_ucm_fit_contour(_P(np.ascontiguousarray(bw, np.float64)), H, W, cv, ce, cp, _P(nv), _P(vert),
                               _P(ed), _P(cm), _P(off), _P(xy))
    nc = int((cm[:ne] == 0).sum())
    return vert[:2 * nv[0]].reshape(-1, 2), ed[:2 * nc].reshape(-1, 2), off[:nc + 1], xy[:2 * off[nc]].reshape(-1, 2)


@pytest.mark.parametrize("H,W,seed,sigma", [(64, 64, 2, 2.0), (128, 160, 4, 2.5), (200, 200, 5, 1.8),
                                            (266, 266, 6, 2.0), (150, 90, 8, 1.0)])
def test_host_stages_against_reference(ref, H, W, seed, sigma):
    import gpb
    L = ref.ref()
    g = _planes(H, W, seed, sigma)
    q = uo.quantize(g)
    ws = np.zeros((H, W), np.int32)
    L.ref_ucm_watershed(_P(q), H, W, _P(ws))
    bw = (ws == 0).astype(np.uint8)
    mine, theirs = gpb.ucm_fit_contours(bw), _ref_fit(L, bw)
    for a, b in zip(mine, theirs):
        assert np.array_equal(a, b)
    w = np.zeros((H, W))
    L.ref_ucm_finest_partition(_P(g), H, W, _P(w))
    w2, lab = np.zeros((2 * H + 1, 2 * W + 1)), np.zeros((H, W), np.int32)
    L.ref_ucm_super_clean(_P(w), H, W, _P(w2), _P(lab))
    u = np.zeros_like(w2)
    L.ref_ucm_mean_pb(_P(w2), _P(lab), H, W, _P(u))
    assert np.array_equal(gpb.ucm_mean_pb(w2, lab), u)


@pytest.mark.parametrize("H,W,seed,sigma", [(40, 50, 1, 1.5), (64, 64, 2, 2.0), (90, 70, 9, 1.1)])
def test_oracle_pins_against_reference(ref, H, W, seed, sigma):
    L = ref.ref()
    g = _planes(H, W, seed, sigma)
    q = uo.quantize(g)
    ws = np.zeros((H, W), np.int32)
    L.ref_ucm_watershed(_P(q), H, W, _P(ws))
    assert np.array_equal(uo.watershed(q) == 0, ws == 0)
    vert, edges, off, px = _ref_fit(L, (ws == 0).astype(np.uint8))
    w = np.zeros((H, W))
    L.ref_ucm_finest_partition(_P(g), H, W, _P(w))
    assert np.array_equal(uo.paint(g, vert, edges, off, px), w)
    w2, lab = np.zeros((2 * H + 1, 2 * W + 1)), np.zeros((H, W), np.int32)
    L.ref_ucm_super_clean(_P(w), H, W, _P(w2), _P(lab))
    ow2, olab, _, _ = uo.super_clean(w)
    assert np.array_equal(ow2, w2) and np.array_equal(olab, lab)
    u = np.zeros_like(w2)
    L.ref_ucm_mean_pb(_P(w2), _P(lab), H, W, _P(u))
    assert np.array_equal(uo.mean_pb(w2, lab.astype(np.int64)), u)
    full = np.zeros_like(w2)
    L.ref_ucm_contours2ucm(_P(g), H, W, 1, _P(full))
    assert np.abs(uo.normalize(u) - full).max() <= UCM_TOL
    bwl = (w2[:-1, :-1] == 0).astype(np.int32)
    rl = np.zeros_like(bwl)
    L.ref_ucm_bwlabel(_P(np.ascontiguousarray(bwl)), bwl.shape[0], bwl.shape[1], _P(rl))
    assert np.array_equal(uo.bwlabel(bwl == 1)[0], rl)


def _voronoi(H, W, k, rng):
    ys, xs = rng.integers(0, H, k), rng.integers(0, W, k)
    yy, xx = np.mgrid[0:H, 0:W]
    lab, best = np.zeros((H, W), np.int32), np.full((H, W), np.inf)
    for i in range(k):
        d = (yy - ys[i]) ** 2 + (xx - xs[i]) ** 2
        m = d < best
        best[m], lab[m] = d[m], i
    return lab


def _islands(H, W, step, rng):
    """square islands of two regions each (left and right half) on a
    background whose id is the largest: the background's neighbour list is
    far longer than any island region's, and a half that merges into it
    still has the other half for a neighbour"""
    ny, nx = H // step, W // step
    lab = np.full((H, W), 2 * ny * nx, np.int32)
    ids = rng.permutation(2 * ny * nx)
    for i in range(ny):
        for j in range(nx):
            s, y0, x0 = int(rng.integers(2, step)), i * step, j * step
            lab[y0:y0 + s, x0:x0 + s // 2] = ids[2 * (i * nx + j)]
            lab[y0:y0 + s, x0 + s // 2:x0 + s] = ids[2 * (i * nx + j) + 1]
    return lab


@pytest.mark.parametrize("layout", ["voronoi", "islands"])
@pytest.mark.parametrize("strength", ["random", "quarters", "flat"])
def test_merge_layouts_against_reference(ref, layout, strength):
    """the library's merge on region layouts of many regions (queue entries
    of merged-away regions dropped in bulk; the father's pairs found through
    the pair table) and on strengths with many equal energies (ties broken
    by region ids), against the reference's UcmMeanPb"""
    import gpb
    rng = np.random.default_rng(17)
    H, W = (160, 150) if layout == "voronoi" else (120, 128)
    lab = _voronoi(H, W, 1500, rng) if layout == "voronoi" else _islands(H, W, 4, rng)
    G = (2 * H + 1, 2 * W + 1)
    w2 = {"random": rng.random(G), "quarters": rng.integers(0, 4, G) / 4.0, "flat": np.full(G, 0.5)}[strength]
    w2 = np.ascontiguousarray(w2)
    u = np.zeros(G)
    ref.ref().ref_ucm_mean_pb(_P(w2), _P(lab), H, W, _P(u))
    assert np.array_equal(gpb.ucm_mean_pb(w2, lab), u)


def test_host_stages_reject_sizes_beyond_32_bit_indices():
    """the checks come before any input is read, so one-element arrays stand in"""
    import gpb
    L = gpb._lib()
    one = np.zeros(1)
    lab = np.zeros(1, np.int32)
    assert L.gpb_ucm_mean_pb(one.ctypes.data, lab.ctypes.data, 40000, 40000, one.ctypes.data) == gpb.GPB_ERR_ARG
    assert L.gpb_ucm_labels_at_scale(one.ctypes.data, 40000, 40000, 0.5, lab.ctypes.data) == -1
    bw, i32 = np.zeros(1, np.uint8), np.zeros(4, np.int32)
    assert L.gpb_ucm_fit_contours(bw.ctypes.data, 50000, 50000, 1, 1, 1, i32.ctypes.data, i32.ctypes.data,
                                  i32.ctypes.data, i32.ctypes.data, i32.ctypes.data) == -1


def _edge_label_maps():
    rng = np.random.default_rng(29)
    yield "1x1", np.zeros((1, 1), np.int32)
    yield "1x9", np.array([[0, 0, 1, 1, 2, 0, 3, 3, 1]], np.int32)
    yield "9x1", np.array([[0], [1], [1], [2], [0], [0], [3], [2], [2]], np.int32)
    yield "one region", np.zeros((6, 7), np.int32)
    yield "two halves", np.repeat(np.array([[0, 0, 0, 1, 1, 1, 1]], np.int32), 5, axis=0)
    yield "ids with gaps", (_voronoi(20, 17, 12, rng) * 5).astype(np.int32)
    yield "checkerboard", (np.indices((8, 8)).sum(0) % 2).astype(np.int32)
    yield "stripes", np.tile(np.arange(9, dtype=np.int32), (4, 1))


@pytest.mark.parametrize("case", [c for c, _ in _edge_label_maps()])
def test_merge_edge_layouts_against_reference(ref, case):
    """degenerate shapes and layouts: single pixels, single rows and
    columns, no boundary at all, unused ids, every pixel its own neighbour's
    opposite"""
    import gpb
    lab = dict(_edge_label_maps())[case]
    H, W = lab.shape
    rng = np.random.default_rng(H * 100 + W)
    for w2 in (rng.random((2 * H + 1, 2 * W + 1)), np.full((2 * H + 1, 2 * W + 1), 0.25)):
        w2 = np.ascontiguousarray(w2)
        u = np.zeros_like(w2)
        ref.ref().ref_ucm_mean_pb(_P(w2), _P(np.ascontiguousarray(lab)), H, W, _P(u))
        assert np.array_equal(gpb.ucm_mean_pb(w2, lab), u)


def test_merge_negative_labels_are_skipped():
    """pixels with a negative id (the reference indexes region -1 there)
    take part in no boundary; the library skips them as the oracle does"""
    import gpb
    rng = np.random.default_rng(31)
    lab = _voronoi(24, 30, 40, rng)
    lab[rng.random(lab.shape) < 0.1] = -1
    w2 = np.ascontiguousarray(rng.random((49, 61)))
    u = gpb.ucm_mean_pb(w2, lab)
    assert np.array_equal(u, uo.mean_pb(w2, lab.astype(np.int64)))


def _edge_arc_maps():
    z = lambda h, w: np.zeros((h, w), np.uint8)  # noqa: E731
    m = z(1, 1); m[0, 0] = 1; yield "pixel", m
    m = z(1, 12); m[0, 2:10] = 1; yield "row", m
    m = z(12, 1); m[1:11, 0] = 1; yield "column", m
    m = z(6, 6); m[2:4, 2:4] = 1; yield "2x2 block", m
    m = z(7, 7); m[1:6, 1:6] = 1; yield "5x5 block", m
    m = z(9, 9); m[1, 1:8] = m[7, 1:8] = m[1:8, 1] = m[1:8, 7] = 1; yield "square loop", m
    m = z(9, 9); m[4, :] = m[:, 4] = 1; yield "plus", m
    m = z(11, 11); np.fill_diagonal(m, 1); m[np.arange(11), 10 - np.arange(11)] = 1; yield "x", m
    m = z(10, 14); m[2, 1:13] = m[7, 1:13] = 1; m[2:8, 3] = m[2:8, 10] = 1; m[4, 3:11] = 1; yield "ladder", m
    yield "all arcs", np.ones((5, 6), np.uint8)


@pytest.mark.parametrize("case", [c for c, _ in _edge_arc_maps()])
def test_fit_edge_maps_against_reference(ref, case):
    import gpb
    bw = np.ascontiguousarray(dict(_edge_arc_maps())[case])
    mine, theirs = gpb.ucm_fit_contours(bw), _ref_fit(ref.ref(), bw)
    assert mine is not None
    for a, b in zip(mine, theirs):
        assert np.array_equal(a, b)
