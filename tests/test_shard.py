"""Batched worlds split across ranks (kizuriphysics3d_gb300.shard): the partition, and the metric
gather over a world_size-2 gloo process group on the CPU (the step itself is a stand-in here; on
GPUs each rank steps its range in its own context with no exchange on the step path)."""
import os
import socket

import numpy as np
import pytest

from kizuriphysics3d_gb300.shard import partition_worlds


def _check(sizes, n):
    r = partition_worlds(sizes, n)
    assert len(r) == n
    assert r[0][0] == 0 and r[-1][1] == len(sizes)
    for (a, b), (c, d) in zip(r, r[1:]):
        assert b == c and a <= b
    loads = [sum(sizes[a:b]) for a, b in r]
    # no contiguous split does better: the largest share is the optimum of the linear partition
    best = max(sizes) if sizes else 0
    lo = best
    while True:
        acc, pieces = 0, 1
        for s in sizes:
            if acc + s > lo:
                pieces, acc = pieces + 1, 0
            acc += s
        if pieces <= n:
            break
        lo += 1
    assert max(loads) == lo
    return r, loads


def test_partition_is_contiguous_complete_and_optimal():
    rng = np.random.default_rng(3)
    for n in (1, 2, 3, 4, 8):
        sizes = np.floor(np.exp(rng.uniform(np.log(8), np.log(512), 200))).astype(int).tolist()
        _check(sizes, n)


def test_partition_edge_cases():
    assert partition_worlds([], 3) == [(0, 0)] * 3
    assert partition_worlds([5], 2) == [(0, 1), (1, 1)]
    r, loads = _check([1, 1, 1, 100, 1, 1], 3)
    assert max(loads) == 100
    with pytest.raises(ValueError):
        partition_worlds([1, 2], 0)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, nranks, port, q):
    import torch.distributed as dist
    from kizuriphysics3d_gb300 import scenes
    from kizuriphysics3d_gb300.shard import run_shard
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=nranks)
    worlds = scenes.world_batch(24, seed=4242)

    def fake_step(scene, ids, steps):  # stands in for World(scene, world_ids=ids).step_fixed(n=steps)
        assert int(ids.max()) + 1 == len(set(ids.tolist()))
        return 10.0 + rank  # ms

    rng, total, slowest = run_shard(worlds, rank, nranks, fake_step, 5, pg=dist.group.WORLD)
    q.put((rank, rng, total, slowest))
    dist.destroy_process_group()


def test_world_split_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    from kizuriphysics3d_gb300 import scenes
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    worlds = scenes.world_batch(24, seed=4242)
    n_dyn = sum(w.num_dynamic for w in worlds)
    (r0, g0, t0, m0), (r1, g1, t1, m1) = out
    assert g0[1] == g1[0] and g0[0] == 0 and g1[1] == len(worlds)  # the two ranges cover every world once
    assert t0 == t1 == float(n_dyn * 5)  # whole-job body-steps, summed over the ranks
    assert m0 == m1 == 11.0  # the slowest rank's time
