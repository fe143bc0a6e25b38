"""CUDA graphs of the fixed launch chains: the stages before and after the
eigensolver, each block-solver filter and each Lanczos restart cycle.  A
chain runs directly the first time its layout is seen, is captured the
second time and replayed after that; every call must give the same bits as
direct launches (GPB_NO_GRAPHS=1)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _batch():
    from gpb import synth
    img = synth.voronoi_image(200, 260, 20, 8.0, synth.SEED_BASE + 21)
    cb = synth.make_codebook(img, synth.SEED_BASE + 21, n_sample=2048)
    boxes = [(0, 0, 64, 100), (20, 30, 97, 33), (100, 120, 100, 140), (5, 200, 40, 60)]
    return cb, [synth.pack_bgr(img[y:y + h, x:x + w]) for (y, x, h, w) in boxes]


def _env_context(cb, mode, var):
    import gpb
    os.environ[var] = "1"
    try:
        return gpb.Context(cb, eig_mode=mode)
    finally:
        del os.environ[var]


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_graph_replays_match_direct_launches(mode):
    import gpb
    cb, patches = _batch()
    direct = _env_context(cb, mode, "GPB_NO_GRAPHS")
    want = direct.compute_batch(patches)
    direct.compute_batch(patches)  # the first call also runs the autotuner's trials
    assert direct.stats()["graph_replays"] == 0
    launches = direct.stats()["gpu_launches"]
    direct.close()
    ctx = gpb.Context(cb, eig_mode=mode)
    for call in range(3):  # direct, captured, replayed
        got = ctx.compute_batch(patches)
        st = ctx.stats()
        for (nm_a, or_a), (nm_b, or_b) in zip(want, got):
            assert np.array_equal(nm_a, nm_b) and np.array_equal(or_a, or_b), call
        if call:
            assert st["gpu_launches"] == launches, call
    assert st["graph_replays"] > 0
    # another layout on the same context: its own graphs, the same bits
    sub = patches[1:3]
    want_sub = [ctx.compute_batch([p])[0] for p in sub]
    for _ in range(2):
        got = ctx.compute_batch(sub)
    for (nm_a, or_a), (nm_b, or_b) in zip(want_sub, got):
        assert np.abs(nm_a - nm_b).max() < 1e-6 and np.abs(or_a - or_b).max() < 1e-6
    ctx.close()


@pytest.mark.parametrize("mode", [1, 2])
def test_autotuner_settles_and_keeps_results(mode):
    """The autotuner tries every texton and block-step variant on real work,
    settles on one per shape bucket, and the results equal the untuned
    default variants bit for bit on every call."""
    import gpb
    cb, patches = _batch()
    ref = _env_context(cb, mode, "GPB_NO_TUNE")
    want = ref.compute_batch(patches)
    assert ref.tuning_report() == {}
    ref.close()
    ctx = gpb.Context(cb, eig_mode=mode)
    for call in range(4):  # the texton variants are all tried within the first call
        got = ctx.compute_batch(patches)
        for (nm_a, or_a), (nm_b, or_b) in zip(want, got):
            assert np.array_equal(nm_a, nm_b) and np.array_equal(or_a, or_b), call
    rep = ctx.tuning_report()
    tex = [k for k in rep if k.startswith("texton/")]
    steps = [k for k in rep if k.startswith("step/")]
    assert tex and steps, rep
    for k in tex:  # timed trials, or settled on the default for too few tiles
        ms = rep[k][1]
        assert rep[k][0] in (0, 1, 2) and len(ms) == 3, rep[k]
        assert min(ms) > 0 or (rep[k][0] == 1 and max(ms) < 0), rep[k]
    assert any(rep[k][0] >= 0 for k in steps), rep
    ctx.close()
