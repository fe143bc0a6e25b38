"""The oracle against golden outputs of the reference's own CPU cores
(tests/golden/reference_cores.npz, written by tests/golden/make_golden.py
from lib_image, buildW and Spectra compiled out of the reference sources).
Bit-exact where the reference's arithmetic is restated; eigenvalues to 1e-8
relative.  Needs no reference checkout."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_cores.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


@pytest.mark.parametrize("i", range(3))
def test_gaussian_kernel(orc, gold, i):
    assert np.array_equal(orc.gaussian_kernel(float(gold["gauss%d_sigma" % i])), gold["gauss%d" % i])


@pytest.mark.parametrize("i", range(5))
def test_hist_gradient(orc, gold, i):
    lab, r, kind = gold["hg%d_lab" % i], int(gold["hg%d_r" % i]), str(gold["hg%d_kind" % i])
    kern = {"bg": orc.gaussian_kernel(2.5), "cg": orc.gaussian_kernel(1.25), "": None}[kind]
    ours = orc.hist_gradient(orc.mirror(lab, 30), 30, r, kern)
    assert np.array_equal(ours, gold["hg%d" % i])


def test_lab_bins(orc, gold):
    cols = gold["lab_bgr"]
    q = orc.lab_bins(cols.reshape(1, -1, 3)).reshape(3, -1)
    assert np.array_equal(q, gold["lab_bins"])


@pytest.mark.parametrize("i", range(2))
def test_nonmax(orc, gold, i):
    assert np.array_equal(orc.nonmax(gold["nm%d_mpbo" % i], fix_clip_scale=0), gold["nm%d" % i])


def _csr_to_dia(rowptr, cols, vals, H, W, dy, dx):
    out = np.zeros((H, W, 81))
    lut = {(int(a), int(b)): k for k, (a, b) in enumerate(zip(dy, dx))}
    for p in range(H * W):
        y, x = divmod(p, W)
        for k in range(rowptr[p], rowptr[p + 1]):
            yy, xx = divmod(int(cols[k]), W)
            out[y, x, lut[(yy - y, xx - x)]] = vals[k]
    return out


@pytest.mark.parametrize("i", range(2))
def test_buildW(orc, gold, i):
    m = gold["bw%d_mpb" % i]
    dy, dx = orc.stencil()
    want = _csr_to_dia(gold["bw%d_rowptr" % i], gold["bw%d_cols" % i], gold["bw%d_vals" % i], m.shape[0], m.shape[1],
                       dy, dx)
    assert np.array_equal(orc.buildW(m), want)


def test_eigenvalues(orc, gold):
    ev, _, it, res = orc.eigs(orc.buildW(gold["eig_mpb"]), 9)
    assert int(gold["eig_nconv"]) == 9 and res.max() < 1e-9
    np.testing.assert_allclose(ev, gold["eig_vals"][::-1], rtol=1e-8, atol=1e-12)
