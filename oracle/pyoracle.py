"""ctypes bindings for the oracle (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
import this module; the product never does.  ``liborc.so`` is the FP64
restatement of the reference's CPU gPb path (gpb_oracle.c); ``_ref/
libgpbref.so`` (present only where the reference tree was available to build
it) wraps the reference's own lib_image / buildW / Spectra cores.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBORC = os.path.join(HERE, "liborc.so")
LIBREF = os.path.join(HERE, "_ref", "libgpbref.so")

_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_c = ctypes.c_int
_d = ctypes.c_double
_vp = ctypes.c_void_p


class OrcParams(ctypes.Structure):
    _fields_ = [
        ("fix_rb_swap", _c),
        ("fix_argmin", _c),
        ("nvec", _c),
        ("fix_clip_scale", _c),
        ("fix_eig_order", _c),
        ("damascene_weights", _c),
        ("sigmoid", _c),
        ("eig_tol", _d),
        ("eig_maxit", _c),
        ("threads", _c),
    ]


_orc = None
_ref = None


def orc():
    global _orc
    if _orc is None:
        if not os.path.exists(LIBORC):
            raise RuntimeError("oracle/liborc.so is not built (make -f oracle/Makefile)")
        L = ctypes.CDLL(LIBORC)
        L.orc_default_params.argtypes = [ctypes.POINTER(OrcParams)]
        L.orc_schmid_bank.argtypes = [_f64p]
        L.orc_grey_bgr.argtypes = [_u8p, _c, _c, _u8p]
        L.orc_texton_map.argtypes = [_u8p, _c, _c, _f32p, _c, _c, _u8p, _vp]
        L.orc_schmid_rings.argtypes = [_i32p, _i32p]
        L.orc_schmid_rings.restype = _c
        L.orc_lab_bins.argtypes = [_u8p, _c, _c, _c, _c, _u8p, _u8p, _u8p]
        L.orc_mirror_u8.argtypes = [_u8p, _c, _c, _c, _u8p]
        L.orc_slice_index.argtypes = [_c, _c, _c]
        L.orc_slice_index.restype = _c
        L.orc_gaussian_kernel.argtypes = [_d, _f64p]
        L.orc_gaussian_kernel.restype = _c
        L.orc_hist_gradient.argtypes = [_u8p, _c, _c, _c, _c, _vp, _c, _f64p, _vp, _c]
        L.orc_hist_gradient.restype = _c
        L.orc_local_cues.argtypes = [_u8p, _u8p, _c, _c, ctypes.POINTER(OrcParams), _f64p]
        L.orc_combine.argtypes = [_f64p, _c, _c, _f64p, _f64p]
        L.orc_nonmax.argtypes = [_f64p, _c, _c, _c, _f64p]
        L.orc_stencil.argtypes = [_i32p, _i32p]
        L.orc_buildW.argtypes = [_f64p, _c, _c, _f64p, _c]
        L.orc_eigs.argtypes = [_f64p, _c, _c, _c, _d, _c, _c, _f64p, _f64p, _vp]
        L.orc_eigs.restype = _c
        L.orc_oefilter.argtypes = [_d, _f64p]
        L.orc_spb.argtypes = [_f64p, _f64p, _f64p, _c, _c, _c, _f64p]
        L.orc_globalpb.argtypes = [_u8p, _c, _c, _f32p, _c, ctypes.POINTER(OrcParams)] + [_vp] * 9
        L.orc_globalpb.restype = _c
        _orc = L
    return _orc


def ref_available():
    return os.path.exists(LIBREF)


def ref():
    global _ref
    if _ref is None:
        L = ctypes.CDLL(LIBREF)
        L.ref_gaussian.argtypes = [_d, _f64p]
        L.ref_gaussian.restype = _c
        L.ref_hist_gradient.argtypes = [_u8p, _c, _c, _c, _vp, _c, _f64p]
        L.ref_lab_bins.argtypes = [_f64p, _f64p, _f64p, ctypes.c_long, _c, _u8p, _u8p, _u8p]
        L.ref_nonmax_oriented.argtypes = [_f64p, _f64p, _c, _c, _d, _f64p]
        L.ref_buildW.argtypes = [_f64p, _c, _c, _vp, _vp, _vp]
        L.ref_buildW.restype = ctypes.c_long
        L.ref_spectra_geigs.argtypes = [_c, _i64p, _i32p, _f64p, _c, _c, _f64p, _f64p]
        L.ref_spectra_geigs.restype = _c
        _ref = L
    return _ref


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_vp)


def params(**kw):
    p = OrcParams()
    orc().orc_default_params(ctypes.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


# ---------------------------------------------------------------- wrappers
def schmid_bank():
    F = np.zeros((13, 49, 49), np.float64)
    orc().orc_schmid_bank(F)
    return F


def grey_bgr(bgr):
    H, W, _ = bgr.shape
    g = np.zeros((H, W), np.uint8)
    orc().orc_grey_bgr(np.ascontiguousarray(bgr), H, W, g)
    return g


def texton_map(grey, codebook, fix_argmin=1, responses=False):
    H, W = grey.shape
    lab = np.zeros((H, W), np.uint8)
    cb = np.ascontiguousarray(codebook, np.float32)
    R = np.zeros((13, H, W), np.float64) if responses else None
    orc().orc_texton_map(np.ascontiguousarray(grey), H, W, cb, cb.shape[1], fix_argmin, lab, _ptr(R))
    return (lab, R) if responses else lab


def schmid_rings():
    ring_of = np.zeros(49 * 49, np.int32)
    ring_s = np.zeros(1200, np.int32)
    n = orc().orc_schmid_rings(ring_of, ring_s)
    return ring_of.reshape(49, 49), ring_s[:n]


def lab_bins(bgr, nbins=25, fix_rb=1):
    H, W, _ = bgr.shape
    q = np.zeros((3, H, W), np.uint8)
    orc().orc_lab_bins(np.ascontiguousarray(bgr), H, W, nbins, fix_rb, q[0], q[1], q[2])
    return q


def mirror(a, b):
    H, W = a.shape
    out = np.zeros((H + 2 * b, W + 2 * b), np.uint8)
    orc().orc_mirror_u8(np.ascontiguousarray(a, np.uint8), H, W, b, out)
    return out


def gaussian_kernel(sigma):
    k = np.zeros(256, np.float64)
    n = orc().orc_gaussian_kernel(sigma, k)
    return k[:n].copy()


def hist_gradient(lab_padded, border, r, kern=None, counts=False, threads=0):
    Hp, Wp = lab_padded.shape
    H, W = Hp - 2 * border, Wp - 2 * border
    out = np.zeros((8, H, W), np.float64)
    nb = int(lab_padded.max()) + 1
    cnt = np.zeros((H, W, 16, nb), np.int32) if counts else None
    k = None if kern is None else np.ascontiguousarray(kern, np.float64)
    orc().orc_hist_gradient(np.ascontiguousarray(lab_padded), Hp, Wp, border, r, _ptr(k),
                            0 if k is None else len(k), out, _ptr(cnt), threads)
    return (out, cnt) if counts else out


def local_cues(bgr, texton, p=None):
    H, W, _ = bgr.shape
    p = p or params()
    cues = np.zeros((12, 8, H, W), np.float64)
    orc().orc_local_cues(np.ascontiguousarray(bgr), np.ascontiguousarray(texton), H, W,
                         ctypes.byref(p), cues)
    return cues


def combine(cues, w):
    _, _, H, W = cues.shape
    out = np.zeros((8, H, W), np.float64)
    orc().orc_combine(np.ascontiguousarray(cues), H, W, np.ascontiguousarray(w, np.float64), out)
    return out


def nonmax(mpb_o, fix_clip_scale=1):
    _, H, W = mpb_o.shape
    out = np.zeros((H, W), np.float64)
    orc().orc_nonmax(np.ascontiguousarray(mpb_o), H, W, fix_clip_scale, out)
    return out


def stencil():
    dy = np.zeros(81, np.int32)
    dx = np.zeros(81, np.int32)
    orc().orc_stencil(dy, dx)
    return dy, dx


def buildW(mpb, threads=0):
    H, W = mpb.shape
    Wd = np.zeros((H, W, 81), np.float64)
    orc().orc_buildW(np.ascontiguousarray(mpb, np.float64), H, W, Wd, threads)
    return Wd


def eigs(Wd, nev=9, tol=1e-10, maxit=3000, threads=0):
    H, W, _ = Wd.shape
    ev = np.zeros(nev, np.float64)
    vec = np.zeros((nev, H * W), np.float64)
    res = np.zeros(nev, np.float64)
    it = orc().orc_eigs(np.ascontiguousarray(Wd), H, W, nev, tol, maxit, threads, ev, vec, _ptr(res))
    return ev, vec, it, res


def oefilter(theta):
    f = np.zeros(49, np.float64)
    orc().orc_oefilter(theta, f)
    return f.reshape(7, 7)


def spb(evals, evecs, dis, H, W, nvec=9):
    out = np.zeros((8, H, W), np.float64)
    orc().orc_spb(np.ascontiguousarray(evals, np.float64), np.ascontiguousarray(evecs, np.float64),
                  np.ascontiguousarray(dis, np.float64), H, W, nvec, out)
    return out


def globalpb(bgr, codebook, p=None, intermediates=False):
    """Whole oracle pipeline; returns a dict of float64 arrays."""
    H, W, _ = bgr.shape
    p = p or params()
    N = H * W
    r = {
        "gpb_o": np.zeros((8, H, W), np.float64),
        "nmax": np.zeros((H, W), np.float64),
        "texton": np.zeros((H, W), np.uint8),
    }
    if intermediates:
        r.update({
            "cues": np.zeros((12, 8, H, W), np.float64),
            "mpb": np.zeros((H, W), np.float64),
            "W": np.zeros((H, W, 81), np.float64),
            "evals": np.zeros(p.nvec, np.float64),
            "evecs": np.zeros((p.nvec, N), np.float64),
            "spb": np.zeros((8, H, W), np.float64),
        })
    cb = np.ascontiguousarray(codebook, np.float32)
    it = orc().orc_globalpb(np.ascontiguousarray(bgr), H, W, cb, cb.shape[1], ctypes.byref(p),
                            _ptr(r["gpb_o"]), _ptr(r["nmax"]), _ptr(r["texton"]),
                            _ptr(r.get("cues")), _ptr(r.get("mpb")), _ptr(r.get("W")),
                            _ptr(r.get("evals")), _ptr(r.get("evecs")), _ptr(r.get("spb")))
    r["matvecs"] = it
    return r


# ------------------------------------------------------------ reference
def ref_gaussian(sigma):
    k = np.zeros(256, np.float64)
    n = ref().ref_gaussian(sigma, k)
    return k[:n].copy()


def ref_hist_gradient_full(lab_padded, r, kern=None):
    Hp, Wp = lab_padded.shape
    out = np.zeros((8, Hp, Wp), np.float64)
    k = None if kern is None else np.ascontiguousarray(kern, np.float64)
    ref().ref_hist_gradient(np.ascontiguousarray(lab_padded), Hp, Wp, r, _ptr(k),
                            0 if k is None else len(k), out)
    return out


def ref_lab_bins(r, g, b, nbins=25):
    n = r.size
    q = np.zeros((3, n), np.uint8)
    ref().ref_lab_bins(np.ascontiguousarray(r, np.float64).ravel(),
                       np.ascontiguousarray(g, np.float64).ravel(),
                       np.ascontiguousarray(b, np.float64).ravel(), n, nbins, q[0], q[1], q[2])
    return q


def ref_nonmax_oriented(a, ind, tol):
    H, W = a.shape
    out = np.zeros((H, W), np.float64)
    ref().ref_nonmax_oriented(np.ascontiguousarray(a, np.float64), np.ascontiguousarray(ind, np.float64),
                              H, W, tol, out)
    return out


def ref_buildW_csr(mpb):
    H, W = mpb.shape
    m = np.ascontiguousarray(mpb, np.float64)
    nnz = ref().ref_buildW(m, H, W, None, None, None)
    rowptr = np.zeros(H * W + 1, np.int64)
    cols = np.zeros(nnz, np.int32)
    vals = np.zeros(nnz, np.float64)
    ref().ref_buildW(m, H, W, _ptr(rowptr), _ptr(cols), _ptr(vals))
    return rowptr, cols, vals


def ref_spectra(rowptr, cols, vals, nev, ncv):
    n = len(rowptr) - 1
    ev = np.zeros(nev, np.float64)
    vec = np.zeros((nev, n), np.float64)
    nc = ref().ref_spectra_geigs(n, rowptr, cols, vals, nev, ncv, ev, vec)
    return nc, ev, vec


def superpixel_features(bgr, texton, labels, n_labels, bin_step, K=None):
    """SPFeatures' per-superpixel rows (src/SPFeatures.cpp): texton histogram
    (genTextonFeatures pooling :260-275, only if K), grey-level histogram with
    bin = grey / bin_step (genIntensityHistograms :101-114), a zero column for
    the corner descriptor, mean B, G, R (genAverageFeatures :380-391);
    histograms / size * 10, means / size * (10 / 255), in that order."""
    grey = grey_bgr(bgr).astype(np.int64)
    nbins = 255 // bin_step + 1
    K = K or 0
    out = np.zeros((n_labels, K + nbins + 4), np.float64)
    lab = labels.ravel()
    ok = (lab >= 0) & (lab < n_labels)
    l = lab[ok]
    size = np.bincount(l, minlength=n_labels).astype(np.float64)
    cols = []
    if K:
        cols.append(np.zeros((n_labels, K)))
        np.add.at(cols[-1], (l, texton.ravel()[ok].astype(np.int64)), 1)
    hist = np.zeros((n_labels, nbins))
    np.add.at(hist, (l, grey.ravel()[ok] // bin_step), 1)
    cols.append(hist)
    nz = size > 0
    c0 = 0
    for c in cols:
        w = c.shape[1]
        out[nz, c0:c0 + w] = (c[nz] / size[nz][:, None]) * 10.0
        c0 += w
    c0 += 1  # the corner column stays zero
    px = bgr.reshape(-1, 3)[ok].astype(np.int64)
    for j in range(3):
        sm = np.zeros(n_labels)
        np.add.at(sm, l, px[:, j])
        out[nz, c0 + j] = (sm[nz] / size[nz]) * (10.0 / 255.0)
    return out
