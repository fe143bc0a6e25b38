"""Host-side mirror of the reference's gPb boundary over libgpb's C ABI.

``GlobalPbCuda`` mirrors ``GlobalPbCuda`` of src/globalPb.cpp:247-313 (a BGR
uint8 patch in, 8 orientation planes and the nonmax plane out, as float64
H x W arrays); ``compute_gpb`` mirrors ``computeGPb`` of
damascene/include/globalPb.h:35 (packed uint32 in, flat float32 buffers
out).  ``Context`` exposes the batched entry points.  Every call goes to the
CUDA library; there is no CPU path, and a missing library raises.
"""
import ctypes
import os

import numpy as np

from . import synth  # noqa: F401

_HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(_HERE, "libgpb.so")

(GPB_OK, GPB_ERR_ARG, GPB_ERR_CUDA, GPB_ERR_NOMEM, GPB_ERR_NOCONV, GPB_ERR_TIMEOUT, GPB_ERR_INTERNAL,
 GPB_ERR_TOO_LARGE) = range(8)
STATIC_MAX_PIXELS = 1 << 20   # gpb_texton_labels_static's scratch limit
STITCH_LAST, STITCH_INTERIOR, STITCH_BLEND = 0, 1, 2
UCM_QUANT, UCM_ARCS, UCM_WSWT, UCM_WSWT2, UCM_REGIONS = range(5)
COMPAT_CPU, COMPAT_DAMASCENE = 0, 1
EIG_LANCZOS, EIG_WARM, EIG_BLOCK, EIG_LEARNED = 0, 1, 2, 3
STAGES = {"texton": 0, "labbins": 1, "mpb_o": 2, "mpb": 3, "W": 4, "evals": 5, "evecs": 6,
          "spb": 7, "cues": 8, "gpb_o": 9, "counts": 10, "warm0": 11, "deg": 12}
WARMNET_PARAMS = 1609


class GpbError(RuntimeError):
    def __init__(self, status, what):
        super().__init__("%s: %s (status %d)" % (what, _lib().gpb_status_str(status).decode(), status))
        self.status = status


class Params(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("compat", ctypes.c_int), ("nvec", ctypes.c_int),
                ("eig_tol", ctypes.c_float), ("eig_max_matvecs", ctypes.c_int),
                ("krylov_dim", ctypes.c_int), ("krylov_keep", ctypes.c_int),
                ("eig_mode", ctypes.c_int), ("keep_intermediates", ctypes.c_int),
                ("cheb_degree", ctypes.c_int), ("warm_tol", ctypes.c_float),
                ("eig_gap_frac", ctypes.c_float)]


class Patch(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("packed_bgr", ctypes.c_void_p), ("stride", ctypes.c_size_t)]


class Result(ctypes.Structure):
    _fields_ = [("nmax", ctypes.c_void_p), ("orient", ctypes.c_void_p)]


class UcmInfo(ctypes.Structure):
    _fields_ = [("n_regions", ctypes.c_uint32), ("n_vertices", ctypes.c_uint32), ("n_edges", ctypes.c_uint32),
                ("n_artefacts", ctypes.c_uint32), ("fit_ok", ctypes.c_int32), ("ms_front", ctypes.c_double),
                ("ms_fit", ctypes.c_double), ("ms_mid", ctypes.c_double), ("ms_merge", ctypes.c_double),
                ("ms_total", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Stats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("ms_total", "ms_h2d", "ms_texton", "ms_cues", "ms_nms",
                                              "ms_buildw", "ms_eig", "ms_spb", "ms_d2h")] + [
        ("matvecs_max", ctypes.c_long), ("matvecs_total", ctypes.c_long), ("restarts", ctypes.c_int),
        ("max_residual", ctypes.c_float), ("texton_repaired", ctypes.c_long),
        ("gpu_launches", ctypes.c_int), ("spmv_ms", ctypes.c_double), ("orth_ms", ctypes.c_double),
        ("spmv_launches", ctypes.c_long), ("orth_launches", ctypes.c_long),
        ("spmv_bytes", ctypes.c_double), ("orth_bytes", ctypes.c_double), ("eig_fallback", ctypes.c_int),
        ("graph_replays", ctypes.c_int)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


_L = None


def _lib():
    global _L
    if _L is None:
        if not os.path.exists(LIBPATH):
            raise RuntimeError("libgpb.so is not built; run __graft_entry__.build() or "
                               "python ucm-mpi-gpu_gb300/gpb/build.py")
        L = ctypes.CDLL(LIBPATH)
        vp, c, sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t
        L.gpb_default_params.argtypes = [ctypes.POINTER(Params)]
        L.gpb_create.argtypes = [ctypes.POINTER(vp), ctypes.POINTER(Params)]
        L.gpb_create.restype = c
        L.gpb_destroy.argtypes = [vp]
        L.gpb_set_codebook.argtypes = [vp, vp, c]
        L.gpb_set_codebook.restype = c
        L.gpb_load_codebook_yml.argtypes = [vp, ctypes.c_char_p]
        L.gpb_load_codebook_yml.restype = c
        L.gpb_compute.argtypes = [vp, ctypes.c_uint32, ctypes.c_uint32, vp, ctypes.POINTER(vp),
                                  ctypes.POINTER(vp)]
        L.gpb_compute.restype = c
        L.gpb_compute_batch.argtypes = [vp, ctypes.POINTER(Patch), sz, ctypes.POINTER(Result)]
        L.gpb_compute_batch.restype = c
        L.gpb_compute_batch_device.argtypes = [vp, sz, vp, vp, vp, vp, vp, vp]
        L.gpb_compute_batch_device.restype = c
        L.gpb_fetch.argtypes = [vp, c, sz, vp, sz]
        L.gpb_fetch.restype = c
        L.gpb_last_stats.argtypes = [vp, ctypes.POINTER(Stats)]
        L.gpb_last_stats.restype = c
        L.gpb_tuning_report.argtypes = [vp, ctypes.c_char_p, sz]
        L.gpb_tuning_report.restype = sz
        L.gpb_learned_nparams.restype = sz
        L.gpb_learned_set.argtypes = [vp, vp, sz]
        L.gpb_learned_set.restype = c
        L.gpb_learned_get.argtypes = [vp, vp, sz]
        L.gpb_learned_get.restype = c
        L.gpb_learned_forward_device.argtypes = [vp, sz, vp, vp, vp, vp, vp]
        L.gpb_learned_forward_device.restype = c
        L.gpb_learned_grad_device.argtypes = [vp, sz, vp, vp, vp, vp, vp, ctypes.POINTER(ctypes.c_double), vp]
        L.gpb_learned_grad_device.restype = c
        L.gpb_learned_train_device.argtypes = [vp, sz, vp, vp, vp, vp, vp, c, c, ctypes.c_float, ctypes.c_uint64,
                                               vp]
        L.gpb_learned_train_device.restype = c
        L.gpb_device_count.restype = c
        L.gpb_status_str.argtypes = [c]
        L.gpb_status_str.restype = ctypes.c_char_p
        L.gpb_last_error.argtypes = [vp]
        L.gpb_last_error.restype = ctypes.c_char_p
        L.gpb_free.argtypes = [vp]
        L.gpb_stitch_device.argtypes = [vp, c, ctypes.c_uint32, ctypes.c_uint32, vp, sz, c, vp, vp]
        L.gpb_stitch_device.restype = c
        L.gpb_write_yml.argtypes = [ctypes.c_char_p, ctypes.c_char_p, vp, ctypes.c_uint32, ctypes.c_uint32]
        L.gpb_write_yml.restype = c
        L.gpb_write_png_minmax.argtypes = [ctypes.c_char_p, vp, ctypes.c_uint32, ctypes.c_uint32]
        L.gpb_write_png_minmax.restype = c
        L.gpb_superpixel_features.argtypes = [vp, sz, vp, ctypes.c_int32, c, c, vp]
        L.gpb_superpixel_features.restype = c
        L.gpb_warmnet_set.argtypes = [vp, vp, sz]
        L.gpb_warmnet_set.restype = c
        L.gpb_warmnet_capture.argtypes = [vp, c]
        L.gpb_warmnet_capture.restype = c
        L.gpb_warmnet_grad_device.argtypes = [vp, sz, vp, vp, vp, vp, vp, vp, vp, vp]
        L.gpb_warmnet_grad_device.restype = c
        L.gpb_texton_labels_static.argtypes = [vp, ctypes.c_uint32, ctypes.c_uint32, vp, vp, vp]
        L.gpb_texton_labels_static.restype = c
        u32, i32 = ctypes.c_uint32, ctypes.c_int32
        L.gpb_ucm.argtypes = [vp, u32, u32, vp, c, c, vp, ctypes.POINTER(UcmInfo)]
        L.gpb_ucm.restype = c
        L.gpb_ucm_batch.argtypes = [vp, sz, vp, vp, vp, c, c, vp, ctypes.POINTER(UcmInfo)]
        L.gpb_ucm_batch.restype = c
        L.gpb_ucm_fetch.argtypes = [vp, sz, c, vp, sz]
        L.gpb_ucm_fetch.restype = c
        L.gpb_ucm_fit_contours.argtypes = [vp, u32, u32, i32, i32, i32, vp, vp, vp, vp, vp]
        L.gpb_ucm_fit_contours.restype = i32
        L.gpb_ucm_mean_pb.argtypes = [vp, vp, u32, u32, vp]
        L.gpb_ucm_mean_pb.restype = c
        L.gpb_ucm_labels_at_scale.argtypes = [vp, u32, u32, ctypes.c_double, vp]
        L.gpb_ucm_labels_at_scale.restype = i32
        _L = L
    return _L


def default_params(**kw):
    p = Params()
    _lib().gpb_default_params(ctypes.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def learned_nparams():
    return int(_lib().gpb_learned_nparams())


def device_count():
    return _lib().gpb_device_count()


def _check(st, what, allow_noconv=False, h=None):
    if st == GPB_OK or (allow_noconv and st == GPB_ERR_NOCONV):
        return
    msg = _lib().gpb_last_error(h).decode() if h else ""
    raise GpbError(st, "%s [%s]" % (what, msg) if msg else what)


class Context:
    """One libgpb context (device buffers, stream, tables)."""

    def _ck(self, st, what, allow_noconv=False):
        _check(st, what, allow_noconv, self._h)

    def last_error(self):
        """the message of the most recent failed call on this context"""
        return _lib().gpb_last_error(self._h).decode() if self._h else ""

    def __init__(self, codebook=None, **params):
        self._h = ctypes.c_void_p()
        self.params = default_params(**params)
        self._ck(_lib().gpb_create(ctypes.byref(self._h), ctypes.byref(self.params)), "gpb_create")
        if codebook is not None:
            self.set_codebook(codebook)

    def close(self):
        if self._h:
            _lib().gpb_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_codebook(self, codebook):
        cb = np.ascontiguousarray(codebook, np.float32)
        if cb.ndim != 2 or cb.shape[0] != 13:
            raise ValueError("codebook must be 13 x K")
        self._ck(_lib().gpb_set_codebook(self._h, cb.ctypes.data, cb.shape[1]), "gpb_set_codebook")

    def load_codebook_yml(self, path):
        self._ck(_lib().gpb_load_codebook_yml(self._h, path.encode()), "gpb_load_codebook_yml")

    def compute_batch(self, packed_list):
        """packed_list: uint32 H x W arrays (B<<16|G<<8|R).  Returns a list of
        (nmax H x W, orient 8*H*W flat) float32 arrays in the context's layout."""
        n = len(packed_list)
        arrs = [np.ascontiguousarray(a, np.uint32) for a in packed_list]
        pt = (Patch * n)()
        res = (Result * n)()
        outs = []
        for i, a in enumerate(arrs):
            H, W = a.shape
            nm = np.empty((H, W), np.float32)
            orr = np.empty(8 * H * W, np.float32)
            outs.append((nm, orr))
            pt[i] = Patch(W, H, a.ctypes.data, W)
            res[i] = Result(nm.ctypes.data, orr.ctypes.data)
        st = _lib().gpb_compute_batch(self._h, pt, n, res)
        self._ck(st, "gpb_compute_batch", allow_noconv=True)
        self.last_status = st
        return outs

    def compute_batch_device(self, widths, heights, offsets, d_packed, d_nmax, d_orient):
        """Device-resident batch; the d_* arguments are raw device pointers."""
        n = len(widths)
        w = np.ascontiguousarray(widths, np.uint32)
        h = np.ascontiguousarray(heights, np.uint32)
        o = np.ascontiguousarray(offsets, np.uint64)
        st = _lib().gpb_compute_batch_device(self._h, n, w.ctypes.data, h.ctypes.data, o.ctypes.data,
                                             d_packed, d_nmax, d_orient)
        self._ck(st, "gpb_compute_batch_device", allow_noconv=True)
        self.last_status = st
        return st

    # ---- learned warm start (GPB_EIG_LEARNED)
    def learned_set(self, params):
        """gpb_learned_set: the network's weights (float32, learned_nparams());
        None drops them."""
        if params is None:
            self._ck(_lib().gpb_learned_set(self._h, None, 0), "gpb_learned_set")
            return
        w = np.ascontiguousarray(params, np.float32)
        self._ck(_lib().gpb_learned_set(self._h, w.ctypes.data, w.size), "gpb_learned_set")

    def learned_get(self):
        w = np.empty(learned_nparams(), np.float32)
        self._ck(_lib().gpb_learned_get(self._h, w.ctypes.data, w.size), "gpb_learned_get")
        return w

    @staticmethod
    def _sizes(shapes):
        h = np.ascontiguousarray([s[0] for s in shapes], np.uint32)
        w = np.ascontiguousarray([s[1] for s in shapes], np.uint32)
        return w, h

    def learned_forward_device(self, shapes, d_mpb, d_deg, d_y):
        """the 32 fields [H*W][32] per patch into device memory d_y; shapes:
        (H, W) per patch; d_mpb, d_deg: device arrays of H*W per patch."""
        w, h = self._sizes(shapes)
        self._ck(_lib().gpb_learned_forward_device(self._h, len(shapes), w.ctypes.data, h.ctypes.data, d_mpb, d_deg,
                                                   d_y), "gpb_learned_forward_device")

    def learned_grad_device(self, shapes, d_mpb, d_deg, d_v):
        """(loss summed over the patches, gradient) for the current weights."""
        w, h = self._sizes(shapes)
        loss = ctypes.c_double()
        g = np.empty(learned_nparams(), np.float32)
        self._ck(_lib().gpb_learned_grad_device(self._h, len(shapes), w.ctypes.data, h.ctypes.data, d_mpb, d_deg,
                                                d_v, ctypes.byref(loss), g.ctypes.data), "gpb_learned_grad_device")
        return loss.value, g

    def learned_train_device(self, shapes, d_mpb, d_deg, d_v, batch, epochs, lr, seed=0):
        """Adam on the context's weights; returns the mean loss per patch of
        each epoch."""
        w, h = self._sizes(shapes)
        hist = np.zeros(epochs, np.float64)
        self._ck(_lib().gpb_learned_train_device(self._h, len(shapes), w.ctypes.data, h.ctypes.data, d_mpb, d_deg,
                                                 d_v, batch, epochs, lr, seed, hist.ctypes.data),
                 "gpb_learned_train_device")
        return hist

    def tuning_report(self):
        """gpb_tuning_report: the autotuner's choice per shape bucket, as a dict
        key -> (chosen variant, [median ms per variant])."""
        n = _lib().gpb_tuning_report(self._h, None, 0)
        buf = ctypes.create_string_buffer(n + 1)
        _lib().gpb_tuning_report(self._h, buf, n + 1)
        out = {}
        for item in buf.value.decode().split("; "):
            if "=" not in item:
                continue
            k, rest = item.split("=", 1)
            ch, ms = rest.split(" (", 1)
            out[k] = (int(ch), [float(x) for x in ms.rstrip(")").split()])
        return out

    def fetch(self, stage, patch, shape, dtype):
        out = np.empty(shape, dtype)
        self._ck(_lib().gpb_fetch(self._h, STAGES[stage], patch, out.ctypes.data, out.nbytes), "gpb_fetch")
        return out

    def stitch_device(self, mode, width, height, places, d_nmax, d_orient, ramp=0):
        """gpb_stitch_device: whole-image planes (device pointers d_nmax,
        d_orient) from the last batch; places = [(x0, y0, ix, iy, iw, ih)] per
        patch, in batch order."""
        arr = np.ascontiguousarray(np.asarray(places, np.int32).reshape(-1, 6))
        self._ck(_lib().gpb_stitch_device(self._h, mode, width, height, arr.ctypes.data, arr.shape[0], ramp,
                                        d_nmax, d_orient), "gpb_stitch_device")

    def superpixel_features(self, patch, d_labels, n_labels, d_out, bin_step=8, with_textons=True):
        """gpb_superpixel_features: n_labels rows of [texton histogram |
        grey histogram | 0 | mean B G R] into the device doubles at d_out."""
        self._ck(_lib().gpb_superpixel_features(self._h, patch, d_labels, n_labels, bin_step, int(with_textons), d_out),
               "gpb_superpixel_features")

    def texton_labels_static(self, width, height, d_packed, d_labels, stream=None):
        """gpb_texton_labels_static: labels (L | a<<8 | b<<16 | texton<<24)
        of one device-resident packed image into d_labels, with no allocation;
        d_packed, d_labels and stream are raw device pointers / a stream
        handle.  Only enqueues work on the stream."""
        self._ck(_lib().gpb_texton_labels_static(self._h, width, height, d_packed, d_labels, stream),
               "gpb_texton_labels_static")

    def ucm(self, orient, double_size=True, d_orient=None, shape=None):
        """Contours2Ucm of 8 orientation planes: ``orient`` an (8, H, W) host
        array, or ``d_orient`` a device pointer with ``shape`` = (H, W).
        Returns the map (float64, (2H+1, 2W+1) or (H+1, W+1)) and the info
        dict of the call."""
        if d_orient is None:
            a = np.ascontiguousarray(orient, np.float32)
            if a.ndim != 3 or a.shape[0] != 8:
                raise ValueError("orient must be 8 x H x W")
            H, W = a.shape[1:]
            ptr, on_dev = a.ctypes.data, 0
        else:
            H, W = shape
            ptr, on_dev = d_orient, 1
        out = np.empty((2 * H + 1, 2 * W + 1) if double_size else (H + 1, W + 1), np.float64)
        info = UcmInfo()
        self._ck(_lib().gpb_ucm(self._h, W, H, ptr, on_dev, 1 if double_size else 0, out.ctypes.data,
                              ctypes.byref(info)), "gpb_ucm")
        self.last_ucm_shapes = [(H, W)]
        return out, info.as_dict()

    def ucm_batch(self, orients, double_size=True):
        """Contours2Ucm of several images in one call: ``orients`` a list of
        (8, H, W) host arrays.  Returns a list of (map, info dict)."""
        arrs = [np.ascontiguousarray(a, np.float32) for a in orients]
        n = len(arrs)
        ws = np.array([a.shape[2] for a in arrs], np.uint32)
        hs = np.array([a.shape[1] for a in arrs], np.uint32)
        outs = [np.empty((2 * h + 1, 2 * w + 1) if double_size else (h + 1, w + 1), np.float64)
                for h, w in zip(hs, ws)]
        ptr_in = (ctypes.c_void_p * n)(*[a.ctypes.data for a in arrs])
        ptr_out = (ctypes.c_void_p * n)(*[o.ctypes.data for o in outs])
        infos = (UcmInfo * n)()
        self._ck(_lib().gpb_ucm_batch(self._h, n, ws.ctypes.data, hs.ctypes.data, ptr_in, 0, 1 if double_size else 0,
                                    ptr_out, infos), "gpb_ucm_batch")
        self.last_ucm_shapes = [(int(h), int(w)) for h, w in zip(hs, ws)]
        return [(o, infos[i].as_dict()) for i, o in enumerate(outs)]

    def ucm_fetch(self, what, image=0):
        """an intermediate of image ``image`` of the last ucm call (UCM_* names)"""
        H, W = self.last_ucm_shapes[image]
        shape, dt = {UCM_QUANT: ((H, W), np.uint8), UCM_ARCS: ((H, W), np.uint8), UCM_WSWT: ((H, W), np.float32),
                     UCM_WSWT2: ((2 * H + 1, 2 * W + 1), np.float32), UCM_REGIONS: ((H, W), np.int32)}[what]
        out = np.empty(shape, dt)
        self._ck(_lib().gpb_ucm_fetch(self._h, image, what, out.ctypes.data, out.nbytes), "gpb_ucm_fetch")
        return out

    def warmnet_set(self, weights):
        """Switch the learned warm-start correction on (GPB_WARMNET_PARAMS
        float weights) or off (None)."""
        if weights is None:
            self._ck(_lib().gpb_warmnet_set(self._h, None, 0), "gpb_warmnet_set")
            return
        w = np.ascontiguousarray(weights, np.float32)
        self._ck(_lib().gpb_warmnet_set(self._h, w.ctypes.data, w.size), "gpb_warmnet_set")

    def warmnet_capture(self, on=True):
        self._ck(_lib().gpb_warmnet_capture(self._h, 1 if on else 0), "gpb_warmnet_capture")

    def warmnet_grad_device(self, widths, heights, d_xt, d_mpb, d_vt, weights):
        """Mean squared error and gradient of the correction net over patches
        held on the device (raw pointers); returns (loss, grad)."""
        w = np.ascontiguousarray(weights, np.float32)
        ws = np.ascontiguousarray(widths, np.uint32)
        hs = np.ascontiguousarray(heights, np.uint32)
        loss = ctypes.c_double()
        grad = np.empty(WARMNET_PARAMS, np.float32)
        self._ck(_lib().gpb_warmnet_grad_device(self._h, len(ws), ws.ctypes.data, hs.ctypes.data, d_xt, d_mpb, d_vt,
                                              w.ctypes.data, ctypes.byref(loss), grad.ctypes.data),
               "gpb_warmnet_grad_device")
        return loss.value, grad

    def stats(self):
        s = Stats()
        self._ck(_lib().gpb_last_stats(self._h, ctypes.byref(s)), "gpb_last_stats")
        return s.as_dict()


def ucm_fit_contours(bw):
    """fit_contour of a 0/1 watershed-arc map on the host: (vertices (V, 2),
    edges (E, 2), off (E+1,), pixels (P, 2)), or None where the chords
    cannot be made consistent."""
    b = np.ascontiguousarray(bw, np.uint8)
    H, W = b.shape
    cv, ce, cp = H * W, 4 * H * W, 4 * H * W
    nv = np.zeros(1, np.int32)
    vert = np.zeros(2 * cv, np.int32)
    ed = np.zeros(2 * ce, np.int32)
    off = np.zeros(ce + 1, np.int32)
    px = np.zeros(2 * cp, np.int32)
    ne = _lib().gpb_ucm_fit_contours(b.ctypes.data, W, H, cv, ce, cp, nv.ctypes.data, vert.ctypes.data,
                                     ed.ctypes.data, off.ctypes.data, px.ctypes.data)
    if ne == -2:
        return None
    if ne == -3:
        raise GpbError(GPB_ERR_NOMEM, "gpb_ucm_fit_contours")
    if ne < 0:
        raise GpbError(GPB_ERR_ARG, "gpb_ucm_fit_contours")
    return (vert[:2 * nv[0]].reshape(-1, 2), ed[:2 * ne].reshape(-1, 2), off[:ne + 1],
            px[:2 * off[ne]].reshape(-1, 2))


def ucm_mean_pb(ws_wt2, labels):
    """UcmMeanPb on the host: the (2H+1, 2W+1) map before calibration."""
    w = np.ascontiguousarray(ws_wt2, np.float64)
    lab = np.ascontiguousarray(labels, np.int32)
    H, W = lab.shape
    out = np.empty((2 * H + 1, 2 * W + 1), np.float64)
    _check(_lib().gpb_ucm_mean_pb(w.ctypes.data, lab.ctypes.data, W, H, out.ctypes.data), "gpb_ucm_mean_pb")
    return out


def ucm_labels_at_scale(ucm2, k):
    """generateLabelsAtScaleK: (labels H x W, number of regions)."""
    u = np.ascontiguousarray(ucm2, np.float64)
    H, W = (u.shape[0] - 1) // 2, (u.shape[1] - 1) // 2
    lab = np.empty((H, W), np.int32)
    n = _lib().gpb_ucm_labels_at_scale(u.ctypes.data, W, H, float(k), lab.ctypes.data)
    if n < 0:
        raise GpbError(GPB_ERR_ARG, "gpb_ucm_labels_at_scale")
    return lab, n


def write_piece_files(prefix, nmax, orient):
    """The reference's per-piece files (src/main.cpp:444-452) from host
    planes: <prefix>_gpb_nmax.png and .yml (matrix "gpb_nonmax") and
    <prefix>_gpb_orient_<o>.png for the 8 orientation planes."""
    nm = np.ascontiguousarray(nmax, np.float32)
    H, W = nm.shape
    ori = np.ascontiguousarray(orient, np.float32).reshape(8, H, W)
    L = _lib()
    _check(L.gpb_write_png_minmax((prefix + "_gpb_nmax.png").encode(), nm.ctypes.data, H, W), "gpb_write_png_minmax")
    _check(L.gpb_write_yml((prefix + "_gpb_nmax.yml").encode(), b"gpb_nonmax", nm.ctypes.data, H, W), "gpb_write_yml")
    for o in range(8):
        plane = np.ascontiguousarray(ori[o])
        _check(L.gpb_write_png_minmax(("%s_gpb_orient_%d.png" % (prefix, o)).encode(), plane.ctypes.data, H, W),
               "gpb_write_png_minmax")


def compute_gpb(ctx, packed):
    """computeGPb (damascene/include/globalPb.h:35) on one packed H x W patch:
    returns (hostGPb H*W, hostGPbAllConcat 8*H*W) as flat float32 arrays in
    the layout of the context's compat mode."""
    nm, orr = ctx.compute_batch([packed])[0]
    return nm.ravel(), orr


def GlobalPbCuda(ctx, image_patch, out_file="", n_orient=8, rank=0, rsz=1.0):
    """Mirror of GlobalPbCuda (src/globalPb.cpp:247-313): BGR uint8 H x W x 3
    patch in; returns (gPbOrient: list of n_orient float64 H x W planes,
    gPbNonmax: float64 H x W).  out_file and rsz are unused, as in the
    reference; rank selects nothing here (one context, one device)."""
    img = np.ascontiguousarray(image_patch, np.uint8)
    if img.ndim != 3 or img.shape[2] != 3:
        raise ValueError("expected an H x W x 3 BGR uint8 patch")
    H, W, _ = img.shape
    packed = synth.pack_bgr(img)
    nm, orr = ctx.compute_batch([packed])[0]
    if ctx.params.compat == COMPAT_DAMASCENE:
        # hostGPbAllConcat[o*rows*cols + j*rows + i] (src/globalPb.cpp:297)
        planes = orr.reshape(8, W, H).transpose(0, 2, 1)
    else:
        planes = orr.reshape(8, H, W)
    orient = [planes[o].astype(np.float64) for o in range(n_orient)]
    return orient, nm.reshape(H, W).astype(np.float64)
