"""Training and evaluation of the learned warm-start correction (k_warmnet.cu).

The net refines the first 9 columns of the warm-start block (the
prolongated coarse Ritz vectors) before the fine block solve.  It is trained
on the GPU, with the library's own forward/backward kernels
(gpb_warmnet_grad_device) and Adam on the host, against the eigenvectors the
block solver converges to on synthetic patches: 256 x 256 Voronoi images of
32-128 cells, sigma 4-12.  Held-out 512 x 512 patches measure the gain.

    python -m gpb.warmnet --train N --epochs E --out weights.npy
    python -m gpb.warmnet --eval weights.npy
"""
import argparse
import json
import os
import time

import numpy as np

from . import synth

NPARAM = 1609
HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "warmnet_weights.npy")


def images(n, size, seed):
    """n synthetic images: Voronoi cells 32-128, noise sigma 4-12, 0-2 lines"""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        cells = int(rng.integers(32, 129))
        sigma = float(rng.uniform(4.0, 12.0))
        out.append(synth.voronoi_image(size, size, cells, sigma, synth.SEED_BASE + 7919 * seed + i,
                                       lines=int(rng.integers(0, 3))))
    return out


def collect(ctx, imgs):
    """Runs the warm solve on imgs with the start block captured; returns per
    image (x~ [N,9], mPb [N], v~ [N,9], H, W): RMS-1 start columns and their
    projections onto the span of the converged eigenvectors.  The targets
    depend on that span only, not on how it splits into eigenvectors, so
    clustered eigenvalues do not make them ambiguous."""
    ctx.warmnet_capture(True)
    ctx.compute_batch([synth.pack_bgr(im) for im in imgs])
    nvec = ctx.params.nvec
    data = []
    for i, im in enumerate(imgs):
        H, W = im.shape[:2]
        N = H * W
        x0 = ctx.fetch("warm0", i, (N, 9), np.float32).astype(np.float64)
        v = ctx.fetch("evecs", i, (nvec, N), np.float32)[:9].T.astype(np.float64)
        mpb = ctx.fetch("mpb", i, (N,), np.float32)
        nx = np.linalg.norm(x0, axis=0)
        nx[nx == 0] = 1.0
        xt = x0 / nx * np.sqrt(N)
        q, _ = np.linalg.qr(v)  # orthonormal basis of the eigenvectors' span
        vt = q @ (q.T @ xt)
        data.append((xt.astype(np.float32), mpb.astype(np.float32), vt.astype(np.float32), H, W))
    ctx.warmnet_capture(False)
    return data


def init_weights(seed=0, scale=0.005):
    rng = np.random.default_rng(seed)
    w = np.zeros(NPARAM, np.float32)
    w[:1440] = rng.normal(0.0, scale, 1440)
    w[1456:1600] = rng.normal(0.0, scale, 144)
    return w


def train(ctx, data, steps=300, lr=3e-3, seed=0, log=None):
    """Full-batch Adam over the training patches; returns (weights, history)."""
    import torch
    xt = torch.from_numpy(np.concatenate([d[0] for d in data])).cuda()
    mp = torch.from_numpy(np.concatenate([d[1] for d in data])).cuda()
    vt = torch.from_numpy(np.concatenate([d[2] for d in data])).cuda()
    ws = [d[4] for d in data]
    hs = [d[3] for d in data]
    w = init_weights(seed).astype(np.float64)
    m = np.zeros_like(w)
    v = np.zeros_like(w)
    b1, b2, eps = 0.9, 0.999, 1e-8
    hist = []
    for it in range(1, steps + 1):
        loss, g = ctx.warmnet_grad_device(ws, hs, xt.data_ptr(), mp.data_ptr(), vt.data_ptr(), w.astype(np.float32))
        g = g.astype(np.float64)
        m = b1 * m + (1 - b1) * g
        v = b2 * v + (1 - b2) * g * g
        w -= lr * (m / (1 - b1 ** it)) / (np.sqrt(v / (1 - b2 ** it)) + eps)
        hist.append(loss)
        if log and (it == 1 or it % 25 == 0):
            log("step %d loss %.5f" % (it, loss))
    return w.astype(np.float32), hist


def base_loss(data):
    """the loss of the uncorrected start (every weight 0)"""
    tot = sum(d[3] * d[4] for d in data) * 9
    return float(sum(((d[0].astype(np.float64) - d[2]) ** 2).sum() for d in data) / tot)


def evaluate(cb, imgs, weights):
    """Warm solves of imgs without and with the correction: per-patch matvecs,
    eigensolver time and the largest gPb difference between the two."""
    from . import Context, EIG_WARM
    res = {}
    outs = {}
    for tag, w in (("without", None), ("with", weights)):
        ctx = Context(cb, eig_mode=EIG_WARM)
        ctx.warmnet_set(w)
        packed = [synth.pack_bgr(im) for im in imgs]
        ctx.compute_batch(packed)  # warm-up
        t0 = time.perf_counter()
        outs[tag] = ctx.compute_batch(packed)
        st = ctx.stats()
        res[tag] = {"wall_ms": (time.perf_counter() - t0) * 1e3, "ms_eig": st["ms_eig"],
                    "matvecs_max": st["matvecs_max"], "max_residual": st["max_residual"]}
        ctx.close()
    res["max_gpb_diff"] = float(max(np.abs(a[0] - b[0]).max() for a, b in zip(outs["without"], outs["with"])))
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=0, help="number of 256 x 256 training patches")
    ap.add_argument("--steps", type=int, default=600)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--out", default=WEIGHTS)
    ap.add_argument("--eval", default=None, help="weights to evaluate on held-out 512 x 512 patches")
    ap.add_argument("--n-eval", type=int, default=8)
    args = ap.parse_args()
    from . import Context, EIG_WARM
    imgs = images(max(args.train, 1), 256, seed=1)
    cb = synth.make_codebook(imgs[0], synth.SEED_BASE + 1, n_sample=1024)
    if args.train:
        ctx = Context(cb, eig_mode=EIG_WARM)
        data = []
        for k in range(0, args.train, 16):
            data += collect(ctx, imgs[k:k + 16])
        print(json.dumps({"patches": len(data), "base_loss": base_loss(data)}), flush=True)
        w, hist = train(ctx, data, steps=args.steps, lr=args.lr, log=lambda s: print(s, flush=True))
        np.save(args.out, w)
        print(json.dumps({"final_loss": hist[-1], "first_loss": hist[0]}), flush=True)
        ctx.close()
    if args.eval:
        w = np.load(args.eval)
        ev = images(args.n_eval, 512, seed=2)
        print(json.dumps(evaluate(cb, ev, w)), flush=True)


if __name__ == "__main__":
    main()
