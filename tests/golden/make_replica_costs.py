"""Writes tests/golden/replica_costs.npz: the measured solve cost of every
patch of the uneven 4096^2 workload (64 patches) and of every fifth patch of
the 8192^2 workload, each solved alone (warm path, wall time of the call),
with the patch's pixel count and region count (gpb.replicas.regions).

    python tests/golden/make_replica_costs.py --measure costs.json   (on a GPU)
    python tests/golden/make_replica_costs.py costs.json             (anywhere)
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "ucm-mpi-gpu_gb300"))


def crops():
    from gpb import synth
    img, cb, boxes = synth.image_4096_uneven()
    out = [("config3", i, cb, np.ascontiguousarray(img[y0:y0 + h, x0:x0 + w])) for i, (y0, x0, h, w) in enumerate(boxes)]
    img, cb = synth.image_8192()
    bx = synth.grid_patches(8192, 8192, 16, 16, 5)
    for i in range(0, 256, 5):
        y0, x0, h, w = bx[i][:4]
        out.append(("config5", i, cb, np.ascontiguousarray(img[y0:y0 + h, x0:x0 + w])))
    return out


def measure(path):
    import gpb
    from gpb import synth
    rows = {"config3": [], "config5": []}
    ctx, last_cb = None, None
    for name, i, cb, crop in crops():
        if last_cb is not cb:
            if ctx:
                ctx.close()
            ctx = gpb.Context(cb, eig_mode=gpb.EIG_WARM)
            ctx.compute_batch([synth.pack_bgr(crop)])
            last_cb = cb
        ctx.compute_batch([synth.pack_bgr(crop)])
        st = ctx.stats()
        rows[name].append([i, crop.shape[0], crop.shape[1], st["ms_eig"], st["ms_total"], st["matvecs_max"]])
    ctx.close()
    with open(path, "w") as f:
        json.dump(rows, f)


def fixture(path):
    from gpb import replicas
    d = json.load(open(path))
    px, reg, ms, group = [], [], [], []
    by = {(name, i): crop for name, i, _, crop in crops()}
    for g, name in enumerate(("config3", "config5")):
        for i, h, w, ms_eig, ms_total, mv in d[name]:
            px.append(h * w)
            reg.append(replicas.regions(by[(name, i)]))
            ms.append(ms_total)
            group.append(g)
    np.savez(os.path.join(HERE, "replica_costs.npz"), pixels=np.array(px), regions=np.array(reg), ms=np.array(ms),
             group=np.array(group))


if __name__ == "__main__":
    if sys.argv[1] == "--measure":
        measure(sys.argv[2])
    else:
        fixture(sys.argv[1])
