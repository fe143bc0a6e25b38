"""Seeded synthetic inputs: Voronoi images and the Schmid texton codebook.

They stand in for the reference's satellite imagery (``labeledData/rio1.jpg``
and the unpublished tiles split by ``src/main.cpp:110-226``) and for its
``*_texton_codebook.yml`` (13 x 32 FP32, ``src/SPFeatures.cpp:300-313``).

Image model: piecewise-constant RGB over Voronoi cells with sites and colours
uniform in the image and in [0, 255], a linear intensity ramp of +0..40
across x, optional straight lines (uniform endpoints, width 2-4 px, uniform
colour) and Gaussian noise of the given sigma, rounded and clipped to uint8.
Images are returned as H x W x 3 in OpenCV's BGR channel order.
"""
import numpy as np

SEED_BASE = 20261203

SCHMID_ST = [(2, 1), (4, 1), (4, 2), (6, 1), (6, 2), (6, 3), (8, 1), (8, 2), (8, 3),
             (10, 1), (10, 2), (10, 3), (10, 4)]
REF_PI = 3.1415926535


def _query(tree, pts):
    """Nearest site of every point, on all host threads where SciPy allows."""
    try:
        return tree.query(pts, workers=-1)
    except TypeError:
        return tree.query(pts)


def _nearest_site(H, W, sites):
    from scipy.spatial import cKDTree
    tree = cKDTree(sites)
    lab = np.empty((H, W), np.int32)
    xs = np.arange(W, dtype=np.float64)
    step = max(1, (1 << 22) // max(W, 1))
    for y0 in range(0, H, step):
        y1 = min(H, y0 + step)
        yy, xx = np.meshgrid(np.arange(y0, y1, dtype=np.float64), xs, indexing="ij")
        _, idx = _query(tree, np.stack([yy.ravel(), xx.ravel()], 1))
        lab[y0:y1] = idx.reshape(y1 - y0, W)
    return lab


def _draw_lines(img, rng, n_lines):
    """Paint n_lines straight lines: every pixel centre within width / 2 of a
    segment takes its colour.  Each row is tested only over a span that
    contains the segment's capsule with a 2-px margin; the test itself is the
    same elementwise formula as over the line's whole bounding box."""
    H, W, _ = img.shape
    for _ in range(n_lines):
        p0 = rng.uniform([0, 0], [H, W])
        p1 = rng.uniform([0, 0], [H, W])
        width = int(rng.integers(2, 5))
        col = rng.uniform(0, 255, 3)
        y0, y1 = int(max(0, min(p0[0], p1[0]) - width)), int(min(H, max(p0[0], p1[0]) + width + 1))
        x0, x1 = int(max(0, min(p0[1], p1[1]) - width)), int(min(W, max(p0[1], p1[1]) + width + 1))
        if y1 <= y0 or x1 <= x0:
            continue
        d = p1 - p0
        L2 = max(float(d @ d), 1e-12)
        rows = np.arange(y0, y1)
        yc = rows + 0.5
        r = width / 2.0 + 2.0
        if abs(d[0]) > 1e-9:
            ta = np.clip((yc - r - p0[0]) / d[0], 0.0, 1.0)
            tb = np.clip((yc + r - p0[0]) / d[0], 0.0, 1.0)
            hit = np.ones(len(rows), bool)
        else:
            ta = np.zeros(len(rows))
            tb = np.ones(len(rows))
            hit = np.abs(yc - p0[0]) <= r
        xa, xb = p0[1] + ta * d[1], p0[1] + tb * d[1]
        lo = np.maximum(np.floor(np.minimum(xa, xb) - r - 0.5), x0).astype(np.int64)
        hi = np.minimum(np.ceil(np.maximum(xa, xb) + r + 0.5) + 1, x1).astype(np.int64)
        n = np.where(hit, np.maximum(hi - lo, 0), 0)
        if n.sum() == 0:
            continue
        ys = np.repeat(rows, n)
        xs = np.repeat(lo - np.cumsum(n) + n, n) + np.arange(n.sum())
        yy, xx = ys + 0.5, xs + 0.5
        t = np.clip(((yy - p0[0]) * d[0] + (xx - p0[1]) * d[1]) / L2, 0, 1)
        dist = np.hypot(yy - (p0[0] + t * d[0]), xx - (p0[1] + t * d[1]))
        m = dist <= width / 2.0
        img[ys[m], xs[m]] = col


def voronoi_image(H, W, cells, sigma, seed, lines=0, ramp=40.0):
    """H x W x 3 uint8 BGR image (see module docstring)."""
    rng = np.random.default_rng(seed)
    sites = rng.uniform([0, 0], [H, W], size=(cells, 2))
    colours = rng.uniform(0, 255, size=(cells, 3))
    lab = _nearest_site(H, W, sites)
    img = colours[lab]
    if lines:
        _draw_lines(img, rng, lines)
    img = img + (ramp * np.arange(W, dtype=np.float64) / max(W - 1, 1))[None, :, None]
    img = img + rng.normal(0.0, sigma, size=img.shape)
    return np.clip(np.rint(img), 0, 255).astype(np.uint8)


def grey_u8(bgr):
    """8-bit Rec.601 luma as OpenCV's CV_BGR2GRAY computes it (Q14 fixed point)."""
    b = bgr[..., 0].astype(np.int32)
    g = bgr[..., 1].astype(np.int32)
    r = bgr[..., 2].astype(np.int32)
    return ((r * 4899 + g * 9617 + b * 1868 + (1 << 13)) >> 14).astype(np.uint8)


def schmid_bank():
    """The 13 S filters (49 x 49, FP64) of src/SPFeatures.cpp:117-183."""
    F = np.zeros((13, 49, 49))
    x = np.arange(49, dtype=np.float64) - 24
    r = np.sqrt(x[None, :] ** 2 + x[:, None] ** 2)
    for f, (s, t) in enumerate(SCHMID_ST):
        v = np.cos(r * (REF_PI * t / s)) * np.exp(-r * r / (2 * s * s))
        F[f] = (v - v.sum() / (49 * 49)) * (1.0 / np.abs(v).sum())
    return F


def schmid_responses_at(grey, ys, xs):
    """FP64 responses of the FP32-rounded S filters at the given pixels
    (correlation with BORDER_REFLECT padding of 24)."""
    H, W = grey.shape
    K = schmid_bank().astype(np.float32).astype(np.float64).reshape(13, -1)
    g = np.pad(grey.astype(np.float64), 24, mode="symmetric")
    out = np.empty((len(ys), 13))
    for i0 in range(0, len(ys), 1024):
        yy, xx = ys[i0:i0 + 1024], xs[i0:i0 + 1024]
        win = np.stack([g[y:y + 49, x:x + 49].ravel() for y, x in zip(yy, xx)])
        out[i0:i0 + len(yy)] = win @ K.T
    return out


def make_codebook(bgr, seed, k=32, n_sample=8192, iters=10):
    """13 x k FP32 codebook: Schmid responses at k seeded pixels refined by
    `iters` Lloyd iterations over a seeded sample of `n_sample` pixels."""
    rng = np.random.default_rng(seed + 7)
    grey = grey_u8(bgr)
    H, W = grey.shape
    n = min(n_sample, H * W)
    idx = rng.choice(H * W, size=n, replace=False)
    R = schmid_responses_at(grey, idx // W, idx % W)
    C = R[rng.choice(n, size=k, replace=False)].copy()
    for _ in range(iters):
        d = ((R[:, None, :] - C[None, :, :]) ** 2).sum(-1)
        a = d.argmin(1)
        for j in range(k):
            m = a == j
            if m.any():
                C[j] = R[m].mean(0)
    return np.ascontiguousarray(C.T.astype(np.float32))


def pack_bgr(bgr):
    """uint32 per pixel, B<<16 | G<<8 | R (src/globalPb.cpp:264-276)."""
    b = bgr[..., 0].astype(np.uint32)
    g = bgr[..., 1].astype(np.uint32)
    r = bgr[..., 2].astype(np.uint32)
    return np.ascontiguousarray((b << 16) | (g << 8) | r)


# ------------------------------------------------------------ named workloads
def image_321x481():
    """321 x 481, 24 cells, sigma 8: one patch."""
    img = voronoi_image(321, 481, 24, 8.0, SEED_BASE + 1)
    return img, make_codebook(img, SEED_BASE + 1)


def image_1024():
    """1024 x 1024, 256 cells, sigma 8: 16 x 256^2 patches with a 5-px halo."""
    img = voronoi_image(1024, 1024, 256, 8.0, SEED_BASE + 2)
    return img, make_codebook(img, SEED_BASE + 2)


def grid_patches(H, W, rows, cols, halo):
    """Equal grid split with a halo clipped at the image border.  Returns a list
    of (y0, x0, h, w, iy0, ix0, ih, iw): the patch box and, inside it, the
    interior box that the patch owns in the stitched output."""
    out = []
    ys = [H * i // rows for i in range(rows + 1)]
    xs = [W * j // cols for j in range(cols + 1)]
    for i in range(rows):
        for j in range(cols):
            a0, a1, b0, b1 = ys[i], ys[i + 1], xs[j], xs[j + 1]
            y0, y1 = max(0, a0 - halo), min(H, a1 + halo)
            x0, x1 = max(0, b0 - halo), min(W, b1 + halo)
            out.append((y0, x0, y1 - y0, x1 - x0, a0 - y0, b0 - x0, a1 - a0, b1 - b0))
    return out


def image_4096_uneven():
    """4096 x 4096, 4096 cells, sigma 6, 40 lines: the uneven-batching image.
    Returns (image, codebook, boxes) with 64 rectangles whose sides are uniform
    in [200, 700] px at uniform positions, as (y0, x0, h, w)."""
    img = voronoi_image(4096, 4096, 4096, 6.0, SEED_BASE + 3, lines=40)
    rng = np.random.default_rng(SEED_BASE + 33)
    boxes = []
    for _ in range(64):
        h, w = (int(v) for v in rng.integers(200, 701, 2))
        y0, x0 = int(rng.integers(0, 4096 - h + 1)), int(rng.integers(0, 4096 - w + 1))
        boxes.append((y0, x0, h, w))
    return img, make_codebook(img, SEED_BASE + 3), boxes


def image_8192():
    """8192 x 8192, 16384 cells, sigma 8, 200 lines: 256 patches of 512^2 with
    a 5-px halo (grid_patches(8192, 8192, 16, 16, 5))."""
    img = voronoi_image(8192, 8192, 16384, 8.0, SEED_BASE + 5, lines=200)
    return img, make_codebook(img, SEED_BASE + 5)
