#!/usr/bin/env python3
"""Writes tests/golden/ucm_cases.npz, the golden fixtures of the OWT-UCM
stage: seeded orientation planes and what the reference's own UCM sources
(src/contours2ucm.cpp, src/watershed.cpp, src/ucm_mean_pb.cpp,
src/MATLAB_functions.cpp, src/mex_contour_sides.cpp and lib_image's
contour_set), compiled into oracle/_ref by oracle/Makefile.ref, make of
them.  Run it where those sources are present:

    make -f oracle/Makefile.ref REF=<reference checkout>
    python tests/golden/make_golden_ucm.py

The quantised image comes from the oracle restatement (the reference
computes it inside CreateFinestPartition and does not expose it); every
other array is the reference's output.  The planes are float32 values, as
the library receives them, widened to float64 for the reference."""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "ucm-mpi-gpu_gb300"))
import pyoracle as po  # noqa: E402
import ucm_oracle as uo  # noqa: E402


def smooth_planes(H, W, seed, sigma):
    """8 smoothed-noise planes in [0, 1], squared (many small basins)"""
    from scipy.ndimage import gaussian_filter
    rng = np.random.default_rng(seed)
    g = np.stack([gaussian_filter(rng.random((H, W)), sigma) for _ in range(8)])
    g = (g - g.min()) / (g.max() - g.min())
    return (g ** 2).astype(np.float32)


def gpb_planes(H, W, seed):
    """orientation planes of the oracle's gPb of a synthetic image"""
    from gpb import synth
    img = synth.voronoi_image(H, W, max(3, H * W // 400), 8.0, synth.SEED_BASE + seed, lines=1)
    cb = synth.make_codebook(img, synth.SEED_BASE + seed, n_sample=1024)
    return po.globalpb(img, cb)["gpb_o"].astype(np.float32)


CASES = {
    "rand40x50": lambda: smooth_planes(40, 50, 1, 1.5),
    "rand80x64": lambda: smooth_planes(80, 64, 3, 1.2),
    "gpb48x64": lambda: gpb_planes(48, 64, 5),
    "tiny5x7": lambda: smooth_planes(5, 7, 11, 0.7),
    "flat32": lambda: np.full((8, 32, 32), 0.25, np.float32),
    "noise2x3": lambda: np.random.default_rng(23).random((8, 2, 3)).astype(np.float32),
    "noise4x9": lambda: np.random.default_rng(49).random((8, 4, 9)).astype(np.float32),
}


def run_case(L, planes):
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    g = np.ascontiguousarray(planes.astype(np.float64))
    H, W = g.shape[1:]
    q = uo.quantize(g)
    ws = np.zeros((H, W), np.int32)
    L.ref_ucm_watershed(P(q), H, W, P(ws))
    arcs = (ws == 0).astype(np.uint8)
    cv, ce, cp = H * W, 4 * H * W, 4 * H * W
    nv = np.zeros(1, np.int32)
    vert = np.zeros(2 * cv, np.int32)
    ed = np.zeros(2 * ce, np.int32)
    cm = np.zeros(ce, np.int32)
    off = np.zeros(ce + 1, np.int32)
    xy = np.zeros(2 * cp, np.int32)
    ne = L.ref_ucm_fit_contour(P(np.ascontiguousarray(arcs, np.float64)), H, W, cv, ce, cp, P(nv), P(vert), P(ed),
                               P(cm), P(off), P(xy))
    assert ne >= 0
    nc = int((cm[:ne] == 0).sum())  # completion edges follow the contour edges
    assert not cm[:nc].any()
    wswt = np.zeros((H, W))
    L.ref_ucm_finest_partition(P(g), H, W, P(wswt))
    w2 = np.zeros((2 * H + 1, 2 * W + 1))
    lab = np.zeros((H, W), np.int32)
    L.ref_ucm_super_clean(P(wswt), H, W, P(w2), P(lab))
    ucm2 = np.zeros((2 * H + 1, 2 * W + 1))
    L.ref_ucm_contours2ucm(P(g), H, W, 1, P(ucm2))
    ucm = np.zeros((H + 1, W + 1))
    L.ref_ucm_contours2ucm(P(g), H, W, 0, P(ucm))
    return {"planes": planes, "quant": q, "arcs": arcs, "vertices": vert[:2 * nv[0]].reshape(-1, 2),
            "edges": ed[:2 * nc].reshape(-1, 2), "off": off[:nc + 1], "pixels": xy[:2 * off[nc]].reshape(-1, 2),
            "wswt": wswt, "wswt2": w2, "labels": lab, "ucm2": ucm2, "ucm": ucm}


def main():
    if not po.ref_available():
        sys.exit("oracle/_ref/libgpbref.so is missing: build it with oracle/Makefile.ref first")
    L = po.ref()
    out = {}
    for name, make in CASES.items():
        for k, v in run_case(L, make()).items():
            out[name + "/" + k] = v
    path = os.path.join(HERE, "ucm_cases.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
