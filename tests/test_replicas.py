"""Replicas over a patch list: the cost-balanced split and the gather to
rank 0, with two gloo ranks on the host (the compute step is a stand-in:
no device work runs here)."""
import os
import socket

import numpy as np
import pytest


def _sizes():
    rng = np.random.default_rng(5)
    return [(int(h), int(w)) for h, w in rng.integers(200, 701, (64, 2))]


def test_partition_covers_and_balances():
    from gpb import replicas
    sizes = _sizes()
    for world in (1, 2, 3, 8):
        shares = replicas.partition(sizes, world)
        flat = sorted(i for s in shares for i in s)
        assert flat == list(range(len(sizes)))
        if world > 1:
            assert replicas.balance(sizes, shares) < 1.1
    with pytest.raises(ValueError):
        replicas.partition(sizes, 0)


def _stand_in(patches):
    # a deterministic per-patch result (what gpb_compute_batch would return)
    return [(p.astype(np.float32).mean(2), np.full(8, p.shape[0] * p.shape[1], np.float32)) for p in patches]


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    from gpb import replicas
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    rng = np.random.default_rng(9)
    patches = [rng.integers(0, 256, (h // 10, w // 10, 3), dtype=np.uint8) for h, w in _sizes()]
    pairs = replicas.run_share(_stand_in, patches, rank, world)
    out = replicas.gather(pairs, len(patches), rank, world)
    if rank == 0:
        want = _stand_in(patches)
        ok = all(np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) for a, b in zip(out, want))
        q.put(("ok" if ok else "mismatch", len(pairs)))
    else:
        q.put(("rank1", len(pairs)))
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_gather_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    res = dict(q.get(timeout=10) for _ in range(2))
    assert res["ok"] > 0 and res["rank1"] > 0 and res["ok"] + res["rank1"] == 64


def _fixture():
    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "replica_costs.npz"))
    return d["pixels"].astype(float), d["regions"].astype(float), d["ms"].astype(float), d["group"]


def _ranks(x):
    return np.argsort(np.argsort(x)).astype(float)


def test_cost_model_ranks_measured_costs():
    """The predicted cost ranks the measured solve times of 115 patches
    (solved one at a time on a GB300) at least as well as the pixel count."""
    from gpb import replicas
    px, reg, ms, _ = _fixture()
    model = px ** replicas.COST_EXP_PIXELS * (reg + 1) ** replicas.COST_EXP_REGIONS
    rho = lambda a, b: np.corrcoef(_ranks(a), _ranks(b))[0, 1]
    assert rho(model, ms) >= 0.9
    assert rho(model, ms) >= rho(px, ms)


def test_cost_split_balances_the_uneven_workload():
    """On the 64 uneven patches, 8 ranks split by predicted cost carry a
    smaller largest share of the measured time than a split by pixels."""
    from gpb import replicas
    px, reg, ms, group = _fixture()
    m = group == 0
    model = px[m] ** replicas.COST_EXP_PIXELS * (reg[m] + 1) ** replicas.COST_EXP_REGIONS
    sizes = [(int(p), 1) for p in px[m]]

    def worst(costs):
        loads = [ms[m][s].sum() for s in replicas.partition(sizes, 8, costs)]
        return max(loads) / np.mean(loads)
    assert worst(list(model)) < worst(None)


def test_predicted_cost_of_an_image():
    from gpb import replicas, synth
    a = synth.voronoi_image(96, 96, 4, 4.0, 1)
    b = synth.voronoi_image(96, 96, 60, 4.0, 1)
    assert replicas.regions(b) > replicas.regions(a)
    assert replicas.predicted_cost(b) > replicas.predicted_cost(a)
