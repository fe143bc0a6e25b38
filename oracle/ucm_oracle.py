"""ucm_oracle.py -- TEST INFRASTRUCTURE ONLY.

Plain numpy / Python restatement of the reference's OWT-UCM glue, the
checker of the library's gpb_ucm stage.  Each function follows the
reference file and lines named in its docstring.  Contour fitting
(lib_image's contour_set) is not restated here: the tests take it from the
reference itself (oracle/_ref, where it is built) or from the golden
fixtures, and compare the library's own fitting with those.  Pure-Python
loops: meant for images of a few thousand pixels.
"""
import heapq
from collections import deque

import numpy as np


def quantize(planes):
    """max over orientations, then convertTo(CV_8UC1, alpha, beta) with
    round-half-even saturation (src/contours2ucm.cpp:255-278)."""
    pb = np.asarray(planes, np.float64).max(0)
    lo, hi = pb.min(), pb.max()
    with np.errstate(divide="ignore", invalid="ignore"):
        alpha = 255.0 / (hi - lo)
        beta = (-255.0 * lo) / (hi - lo)
        v = pb * alpha + beta
    v = np.where(np.isnan(v), 0.0, np.rint(v))
    return np.clip(v, 0, 255).astype(np.uint8)


def watershed(q):
    """watershed_yupeng (src/watershed.cpp:28-108), 8-connected: levels in
    increasing order, pixels of a level in raster order; a pixel joins the
    one region among its labelled neighbours, becomes a watershed pixel (0)
    between two, or starts a new region."""
    H, W = q.shape
    L = -np.ones((H, W), np.int64)
    order = np.argsort(q.ravel(), kind="stable")
    col = 1
    for p in order:
        x, y = divmod(int(p), W)
        state = -1
        for i in (-1, 0, 1):
            for j in (-1, 0, 1):
                if (i or j) and 0 <= x + i < H and 0 <= y + j < W:
                    v = L[x + i, y + j]
                    if v > 0:
                        state = v if state == -1 else (0 if v != state else state)
        if state >= 0:
            L[x, y] = state
        else:
            L[x, y] = col
            col += 1
    return L


def orientation(v1, v2):
    """Orientation bin of an edge from its end points, float arithmetic
    (src/contours2ucm.cpp:336-372)."""
    ang = np.float32(np.pi / 2)
    if v1[1] != v2[1]:
        ang = np.float32(np.arctan((v1[0] - v2[0]) * 1.0 / (v1[1] - v2[1])))
    deg = float(np.float32(float(np.float32(ang * np.float32(180))) / np.pi))
    if deg < -78.75 or deg >= 78.75:
        o = 1
    elif 56.25 <= deg < 78.75:
        o = 2
    elif 33.75 <= deg < 56.25:
        o = 3
    elif 11.25 <= deg < 33.75:
        o = 4
    elif -11.25 <= deg < 11.25:
        o = 5
    elif -33.75 <= deg < -11.25:
        o = 6
    elif -56.25 <= deg < -33.75:
        o = 7
    else:
        o = 8
    return o - 1


def paint(planes, vertices, edges, off, pixels):
    """ws_wt of CreateFinestPartition (src/contours2ucm.cpp:374-399): along
    every non-completion edge, its interior pixels and both end points take
    the max of their current value and the edge's orientation plane."""
    planes = np.asarray(planes, np.float64)
    H, W = planes.shape[1:]
    w = np.zeros((H, W))
    for e in range(len(edges)):
        a, b = vertices[edges[e][0]], vertices[edges[e][1]]
        o = orientation(a, b)
        pts = [tuple(p) for p in pixels[off[e]:off[e + 1]]] + [tuple(a), tuple(b)]
        for (r, c) in pts:
            v = planes[o, r, c]
            w[r, c] = w[r, c] if not (w[r, c] < v) else v
    return w


def super_contour(w):
    """SuperContour4C (src/contours2ucm.cpp:24-78)."""
    tx, ty = w.shape
    V = np.minimum(w[:-1, :], w[1:, :])
    Hh = np.minimum(w[:, :-1], w[:, 1:])
    pb2 = np.zeros((2 * tx, 2 * ty))
    pb2[0::2, 0::2] = w
    pb2[0::2, 1:-1:2] = Hh
    pb2[1:-1:2, 0::2] = V
    pb2[-1, :] = pb2[-2, :]
    last, prev = pb2[:, -1].copy(), pb2[:, -2]
    pb2[:, -1] = np.where(last < prev, prev, last)
    return pb2


def _at(g, r, c):
    """an element of a continuous row-major matrix by (row, column), with
    columns wrapping into the neighbouring row; 0 outside the buffer"""
    k = r * g.shape[1] + c
    return g.flat[k] if 0 <= k < g.size else 0.0


def clean(pb2):
    """CleanWatersheds (src/contours2ucm.cpp:80-189) with bwmorph 'clean'
    and regionprops (src/MATLAB_functions.cpp:8-90): every isolated zero,
    in row-major order, is closed towards its weakest diagonal pair."""
    g = pb2.copy()
    R, C = g.shape
    z = g == 0
    pad = np.pad(z, 1)
    nb = sum(pad[1 + i:1 + i + R, 1 + j:1 + j + C] for i in (-1, 0, 1) for j in (-1, 0, 1) if i or j)
    arts = np.argwhere(z & (nb == 0))
    for xc, yc in arts:
        xc, yc = int(xc), int(yc)
        vec = [max(_at(g, xc - 2, yc - 1), _at(g, xc - 1, yc - 2)), max(_at(g, xc + 2, yc - 1), _at(g, xc + 1, yc - 2)),
               max(_at(g, xc + 2, yc + 1), _at(g, xc + 1, yc + 2)), max(_at(g, xc - 2, yc + 1), _at(g, xc - 1, yc + 2))]
        i = int(np.argmin(vec))
        sx = 1 if i in (1, 2) else -1
        sy = 1 if i >= 2 else -1

        def put(r, c, v):
            k = r * C + c
            if 0 <= k < g.size:
                g.flat[k] = v
        if _at(g, xc + 2 * sx, yc + sy) < _at(g, xc + sx, yc + 2 * sy):
            put(xc, yc + sy, 0.0)
            put(xc + sx, yc, vec[i])
        else:
            put(xc, yc + sy, vec[i])
            put(xc + sx, yc, 0.0)
        put(xc + sx, yc + sy, vec[i])
    return g, len(arts)


def bwlabel(mask):
    """bwlabelManu (src/MATLAB_functions.cpp:164-217): 8-connected
    components numbered from 1 in row-major order of their first pixel."""
    R, C = mask.shape
    lab = np.zeros((R, C), np.int64)
    n = 0
    for r in range(R):
        for c in range(C):
            if mask[r, c] and not lab[r, c]:
                n += 1
                lab[r, c] = n
                q = deque([(r, c)])
                while q:
                    a, b = q.popleft()
                    for i in (-1, 0, 1):
                        for j in (-1, 0, 1):
                            u, v = a + i, b + j
                            if 0 <= u < R and 0 <= v < C and mask[u, v] and not lab[u, v]:
                                lab[u, v] = n
                                q.append((u, v))
    return lab, n


def super_clean(w):
    """ws_wt2 and the pixels' region ids (src/contours2ucm.cpp:418-458)."""
    g, nart = clean(super_contour(w))
    l2, n = bwlabel(g == 0)
    labels = l2[1::2, 1::2] - 1
    w2 = np.pad(g, ((0, 1), (0, 1)), mode="edge")
    return w2, labels, nart, n


def mean_pb(w2, labels):
    """ComputeUcm + CompleteContourMap (src/ucm_mean_pb.cpp:230-398): greedy
    merging of the pair of regions with the smallest mean boundary strength,
    ties in (energy, region1, region2) order; pixels with negative ids are
    skipped."""
    H, W = labels.shape
    GH, GW = 2 * H + 1, 2 * W + 1
    n = int(labels.max()) + 1
    ucm = np.zeros((GH, GW))
    if n <= 0:
        return ucm
    lab = list(range(n))
    bnd = [[] for _ in range(n)]
    for y in range(W):
        for x in range(H):
            a = int(labels[x, y])
            if a < 0:
                continue
            for dx, dy in ((1, 0), (0, 1), (-1, 0), (0, -1)):
                u, v = x + dx, y + dy
                if 0 <= u < H and 0 <= v < W:
                    b = int(labels[u, v])
                    if b >= 0 and a != b:
                        bnd[a].append(((x + u + 1) * GW + (y + v + 1), b))
    elements = [[c] for c in range(n)]
    nbr = [dict() for _ in range(n)]
    q = []
    for c in range(n):
        items = sorted(bnd[c], key=lambda e: (e[1], (e[0] % GW) * GH + e[0] // GW))
        groups = {}
        for coord, b in items:
            t = groups.setdefault(b, [0.0, 0.0])
            t[0] += w2.flat[coord]
            t[1] += 1.0
        for b, (tot, ln) in groups.items():
            nbr[c][b] = [tot / ln, tot, ln]
            if b > c:
                heapq.heappush(q, (tot / ln, c, b))
    while q:
        e, r1, r2 = heapq.heappop(q)
        if lab[r1] != r1 or lab[r2] != r2:
            continue
        cur = nbr[r1].setdefault(r2, [0.0, 0.0, 0.0])
        if e != cur[0]:
            continue
        sal = cur[1] / cur[2]
        son, fa = min(r1, r2), max(r1, r2)
        keep = []
        for coord, b in bnd[son]:
            lb = lab[b]
            if lb == son:
                continue
            if ucm.flat[coord] < sal:
                ucm.flat[coord] = sal
            if lb != fa:
                keep.append((coord, b))
        bnd[fa].extend(keep)
        bnd[son] = []
        for p in elements[son]:
            lab[p] = fa
        elements[fa].extend(elements[son])
        elements[son] = []
        nbr[fa] = {k: v for k, v in nbr[fa].items() if lab[k] == k}
        sn = {k: v for k, v in nbr[son].items() if lab[k] == k and lab[k] != fa}
        for k in sorted(sn):
            f = nbr[fa].setdefault(k, [0.0, 0.0, 0.0])
            g = nbr[k].setdefault(fa, [0.0, 0.0, 0.0])
            f[1] += sn[k][1]
            g[1] += sn[k][1]
            f[2] += sn[k][2]
            g[2] += sn[k][2]
        nbr[son] = {}
        for k in sorted(nbr[fa]):
            v = nbr[fa][k]
            d = v[1] / v[2]
            heapq.heappush(q, (d, k, fa))
            v[0] = d
            nbr[k].setdefault(fa, [0.0, 0.0, 0.0])[0] = d
    for x in range(0, GH, 2):
        for y in range(0, GW, 2):
            m = 0.0
            for u, v in ((x + 1, y), (x, y + 1), (x - 1, y), (x, y - 1)):
                if 0 <= u < GH and 0 <= v < GW and m < ucm[u, v]:
                    m = ucm[u, v]
            ucm[x, y] = m
    return ucm


def normalize(u):
    """NormalizeOutput (src/contours2ucm.cpp:191-249)."""
    z = (0.0 + 1.0 * -2.7487) + u * 11.1189
    v = 1.0 / (1.0 + np.exp(-z))
    v = (v - 0.0602) / (1.0 - 0.0602)
    return np.minimum(1.0, np.maximum(0.0, v))


def downsample(su):
    """the image-size map of Contours2Ucm (src/contours2ucm.cpp:476-486)"""
    GH, GW = su.shape
    out = np.zeros(((GH + 1) // 2, (GW + 1) // 2))
    out[:-1, :-1] = su[2::2, 2::2]
    return out


def labels_at_scale(ucm2, k):
    """UCM_generator::generateLabelsAtScaleK (src/UCMgenerator.cpp:120-161)"""
    l2, n = bwlabel(ucm2 <= k)
    return l2[1::2, 1::2] - 1, n
