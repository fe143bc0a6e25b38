"""Training and evaluation of the learned warm start (GPB_EIG_LEARNED).

Training data: synthetic patches (Voronoi images of 32-128 cells, noise
sigma 4-12, 0-2 lines), each labelled with the 9 eigenvectors the plain
cold-start Lanczos solver finds for it; the network sees the patch's mPb and
affinity degree.  Training runs on the GPU through the library's own
forward, backward and Adam kernels (gpb_learned_train_device).  Evaluation
runs held-out patches through the block eigensolver started from the
network, from a seeded random block (cold start), from the coarse-grid solve
(GPB_EIG_WARM) and through plain Lanczos, all to the same residual.

    python -m gpb.learned --train 2000 --size 256 --epochs 20 --out w.npy
    python -m gpb.learned --eval w.npy --n 32 --size 512
"""
import argparse
import json
import os
import time

import numpy as np

from . import synth

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "learned_weights.npy")


def images(n, size, seed):
    """n synthetic size x size images: Voronoi cells 32-128, sigma 4-12, 0-2 lines"""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        cells = int(rng.integers(32, 129))
        sigma = float(rng.uniform(4.0, 12.0))
        out.append(synth.voronoi_image(size, size, cells, sigma, synth.SEED_BASE + 104729 * seed + i,
                                       lines=int(rng.integers(0, 3))))
    return out


def make_dataset(n, size, seed, batch=16):
    """(shapes, mPb, degree, V) for n patches: device float32 tensors holding
    the patches back to back (V as [pixel][9], orthonormal per patch)."""
    import torch
    import gpb
    imgs = images(n, size, seed)
    cb = synth.make_codebook(imgs[0], synth.SEED_BASE + seed, n_sample=4096)
    ctx = gpb.Context(cb, eig_mode=gpb.EIG_LANCZOS, keep_intermediates=1)
    mpb, deg, vs, shapes = [], [], [], []
    for b0 in range(0, n, batch):
        chunk = imgs[b0:b0 + batch]
        ctx.compute_batch([synth.pack_bgr(im) for im in chunk])
        for i, im in enumerate(chunk):
            H, W = im.shape[:2]
            N = H * W
            mpb.append(ctx.fetch("mpb", i, (N,), np.float32))
            deg.append(ctx.fetch("deg", i, (N,), np.float32))
            ev = ctx.fetch("evecs", i, (ctx.params.nvec, N), np.float32)[:9].T.astype(np.float64)
            q, _ = np.linalg.qr(ev)
            vs.append(q.astype(np.float32))
            shapes.append((H, W))
    ctx.close()
    cat = lambda xs: torch.from_numpy(np.concatenate([x.ravel() for x in xs])).cuda()
    return shapes, cat(mpb), cat(deg), cat(vs)


def train(n=2000, size=256, epochs=20, batch=16, lr=1e-3, seed=0, log=print):
    """Trains from the oracle's initialisation; returns (weights, loss per epoch, seconds)."""
    import gpb
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle"))
    t0 = time.time()
    shapes, mpb, deg, v = make_dataset(n, size, seed)
    t_data = time.time() - t0
    log("dataset: %d patches of %d^2 in %.1f s" % (n, size, t_data))
    ctx = gpb.Context()
    ctx.learned_set(init_params(seed))
    t0 = time.time()
    hist = ctx.learned_train_device(shapes, mpb.data_ptr(), deg.data_ptr(), v.data_ptr(), batch, epochs, lr, seed)
    t_train = time.time() - t0
    log("training: %d epochs in %.1f s, loss per patch %s" % (epochs, t_train, np.round(hist, 4).tolist()))
    w = ctx.learned_get()
    ctx.close()
    return w, hist, {"data_s": t_data, "train_s": t_train}


def init_params(seed=0):
    """He-normal weights, zero biases, in the library's parameter layout."""
    import gpb
    rng = np.random.default_rng(seed)
    convs = [(16, 16), (16, 16), (16, 32), (32, 32), (32, 64), (64, 64), (64, 64), (64, 64),
             (128, 64), (64, 64), (96, 32), (32, 32), (48, 16), (16, 16), (16, 32)]
    out = []
    for k, (ci, co) in enumerate(convs):
        std = np.sqrt((1.0 if k == len(convs) - 1 else 2.0) / (9 * ci))
        out.append(rng.normal(0.0, std, co * 9 * ci))
        out.append(np.zeros(co))
    p = np.concatenate(out).astype(np.float32)
    assert p.size == gpb.learned_nparams()
    return p


def evaluate(weights, n=32, size=512, seed=77, batch=8, modes=None, tol=None, gap_frac=None):
    """Per eigensolver mode: eigensolver ms per patch (device events), matvecs,
    largest residual, over held-out patches; the learned and cold-start
    block solvers' gPb planes compared.  tol / gap_frac override eig_tol /
    eig_gap_frac (gap_frac 0: the residual criterion alone)."""
    import torch
    import gpb
    imgs = images(n, size, 1000 + seed)
    cb = synth.make_codebook(imgs[0], synth.SEED_BASE + seed, n_sample=4096)
    packed = [synth.pack_bgr(im) for im in imgs]
    modes = modes or {"learned": gpb.EIG_LEARNED, "cold_block": gpb.EIG_BLOCK, "coarse_warm": gpb.EIG_WARM,
                      "plain_lanczos": gpb.EIG_LANCZOS}
    res, planes = {}, {}
    over = {}
    if tol is not None:
        over["eig_tol"] = tol
    if gap_frac is not None:
        over["eig_gap_frac"] = gap_frac
    for name, mode in modes.items():
        ctx = gpb.Context(cb, eig_mode=mode, **over)
        if mode == gpb.EIG_LEARNED:
            ctx.learned_set(weights)
        ctx.compute_batch(packed[:batch])  # layout, autotuning, graphs
        torch.cuda.synchronize()
        eig_ms, mv, rmax, outs = 0.0, 0, 0.0, []
        for b0 in range(0, n, batch):
            outs += ctx.compute_batch(packed[b0:b0 + batch])
            st = ctx.stats()
            eig_ms += st["ms_eig"]
            mv += st["matvecs_total"]
            rmax = max(rmax, st["max_residual"])
        res[name] = {"eig_ms_per_patch": eig_ms / n, "matvecs_per_patch": mv / n, "max_residual": rmax,
                     "fallback": st["eig_fallback"]}
        planes[name] = outs
        ctx.close()
    if "learned" in planes and "cold_block" in planes:
        res["gpb_max_diff_learned_vs_cold"] = float(max(np.abs(a[1] - b[1]).max()
                                                        for a, b in zip(planes["learned"], planes["cold_block"])))
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=0)
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--out", default=WEIGHTS)
    ap.add_argument("--eval", default=None)
    ap.add_argument("--n", type=int, default=32)
    ap.add_argument("--report", default=None)
    ap.add_argument("--tol", type=float, default=None)
    ap.add_argument("--gap-frac", type=float, default=None)
    args = ap.parse_args()
    rep = {}
    if args.train:
        w, hist, t = train(args.train, args.size, args.epochs, args.batch, args.lr)
        np.save(args.out, w)
        rep["train"] = {"patches": args.train, "size": args.size, "epochs": args.epochs, "batch": args.batch,
                        "lr": args.lr, "loss_per_epoch": hist.tolist(), **t}
    if args.eval:
        rep["eval"] = evaluate(np.load(args.eval), n=args.n, size=512, tol=args.tol, gap_frac=args.gap_frac)
        print(json.dumps(rep["eval"]))
    if args.report:
        with open(args.report, "w") as f:
            json.dump(rep, f, indent=1)


if __name__ == "__main__":
    main()
