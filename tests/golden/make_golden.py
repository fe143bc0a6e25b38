#!/usr/bin/env python3
"""Writes the golden fixtures of tests/test_oracle_golden.py: small seeded
inputs and the outputs of the reference's own CPU cores (lib_image's
gaussian, hist_gradient_2D, Lab quantisation and oriented non-max
suppression; buildW's intervening-contour affinities; the Spectra
generalised eigensolver), compiled from the reference sources into
oracle/_ref by oracle/Makefile.ref.  Run it where those sources are
present:

    make -f oracle/Makefile.ref REF=<reference checkout>
    python tests/golden/make_golden.py

The fixtures carry the oracle's pins to machines without the reference."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import pyoracle as po  # noqa: E402

PI_REF = 3.1415926535


def main():
    if not po.ref_available():
        sys.exit("oracle/_ref/libgpbref.so is missing: build it with oracle/Makefile.ref first")
    out = {}
    # gaussian smoothing kernels (lib_image gaussian, deriv 0)
    for i, s in enumerate((2.5, 1.25, 0.7)):
        out["gauss%d_sigma" % i] = np.float64(s)
        out["gauss%d" % i] = po.ref_gaussian(s)
    # histogram gradients of mirrored label images
    for i, (r, kind) in enumerate([(3, "bg"), (5, "cg"), (10, None), (20, "bg"), (5, None)]):
        rng = np.random.default_rng(100 + i)
        lab = rng.integers(0, 25 if kind else 32, (19, 23)).astype(np.uint8)
        lab[3:11, 2:15] = 7
        lp = po.mirror(lab, 30)
        kern = {"bg": po.ref_gaussian(2.5), "cg": po.ref_gaussian(1.25), None: None}[kind]
        out["hg%d_lab" % i] = lab
        out["hg%d_r" % i] = np.int32(r)
        out["hg%d_kind" % i] = np.array(kind or "")
        out["hg%d" % i] = po.ref_hist_gradient_full(lp, r, kern)[:, 30:-30, 30:-30]
    # Lab quantisation of BGR colours (with the R/B order fixed)
    rng = np.random.default_rng(200)
    cols = rng.integers(0, 256, (20000, 3)).astype(np.uint8)
    cols = np.concatenate([cols, np.repeat(np.arange(256, dtype=np.uint8)[:, None], 3, 1),
                           np.array([[0, 0, 0], [255, 255, 255]], np.uint8)])
    s = 1.0 / 255.0
    out["lab_bgr"] = cols
    out["lab_bins"] = po.ref_lab_bins(cols[:, 2] * s, cols[:, 1] * s, cols[:, 0] * s)
    # oriented non-max suppression (then the x1.2 clip of multiscalePb)
    for i, shape in enumerate([(24, 30), (17, 33)]):
        rng = np.random.default_rng(300 + i)
        mo = rng.random((8,) + shape)
        mo[:, 6:12, 6:12] = 0.3
        a = mo.max(0)
        ind = mo.argmax(0) * PI_REF / 8
        rn = po.ref_nonmax_oriented(a, ind, PI_REF / 8)
        out["nm%d_mpbo" % i] = mo
        out["nm%d" % i] = np.where(1.2 * rn > 1, 1, rn)
    # buildW: CSR of the symmetrised affinity matrix
    for i, shape in enumerate([(16, 20), (13, 17)]):
        rng = np.random.default_rng(400 + i)
        m = np.clip(rng.random(shape) ** 3, 0, 1)
        m[3:12, 9] = 0.9
        m[2, :] = 1.0
        rowptr, colidx, vals = po.ref_buildW_csr(m)
        out["bw%d_mpb" % i] = m
        out["bw%d_rowptr" % i] = np.asarray(rowptr, np.int64)
        out["bw%d_cols" % i] = np.asarray(colidx, np.int64)
        out["bw%d_vals" % i] = np.asarray(vals, np.float64)
    # Spectra generalised eigenvalues (descending, as Spectra returns them)
    rng = np.random.default_rng(500)
    m = np.clip(rng.random((18, 21)) ** 3, 0, 1)
    m[:, 9] = 0.8
    rowptr, colidx, vals = po.ref_buildW_csr(m)
    nc, evr, _ = po.ref_spectra(rowptr, colidx, vals, 9, 24)
    out["eig_mpb"] = m
    out["eig_nconv"] = np.int32(nc)
    out["eig_vals"] = np.asarray(evr, np.float64)
    path = os.path.join(HERE, "reference_cores.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
