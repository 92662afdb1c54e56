"""GPU parity on the two configurations stepped at scale: the batched worlds (4,096 independent
worlds in one context, here 32 of them) and the 200,000-box field.  Through the C-ABI, bit-exact.

Batched worlds: every world of a merged context - stepped through a replayed CUDA graph, after
the autotuner picked its launch shapes, and with either island-to-CTA order - must hold exactly
the bits of the same world stepped alone, and a few worlds are checked against the oracle.  Worlds
never interact: a body's pairs, constraints, islands and batches come from its own world only
(reference: each world is its own PhysicsWorld, src/World/PhysicsWorld.cpp:245-329).
"""
import os

import numpy as np
import pytest

from conftest import bits, oracle_blob

pytestmark = pytest.mark.gpu

WORLDS = 32
STEPS = 40


def _batch():
    from kizuriphysics3d_gb300 import scenes
    worlds = scenes.world_batch(WORLDS, seed=4242)
    merged, ids = scenes.merge_worlds(worlds)
    return worlds, merged, ids


def _alone_states(worlds, steps):
    from kizuriphysics3d_gb300 import World
    out = []
    for sc in worlds:
        with World(sc) as w:
            w.step_fixed(n=steps)
            out.append(w.state())
    return out


def test_batched_worlds_match_each_world_alone(oracle_lib, kzg_lib):
    from kizuriphysics3d_gb300 import World, resolve
    worlds, merged, ids = _batch()
    sizes = [len(w.bodies) for w in worlds]
    assert min(sizes) < 40 and max(sizes) > 200  # uneven, as in the 4,096-world batch
    with World(merged, resolved=resolve(merged), world_ids=ids) as gw:
        gw.set_graph(True)
        gw.step_fixed(n=5)
        before = gw.state()
        tuned = gw.autotune(steps_per_candidate=2)
        assert tuned["step_ms"] > 0.0
        assert np.array_equal(bits(gw.state()), bits(before)), "the tuner must leave the world as it was"
        gw.step_fixed(n=STEPS - 5)
        st = gw.state()
        assert gw.get_stats()["device_error"] == 0
    alone = _alone_states(worlds, STEPS)
    off = 0
    for w, (sc, a) in enumerate(zip(worlds, alone)):
        n = len(sc.bodies)
        assert np.array_equal(bits(st[off:off + n]), bits(a)), f"world {w} ({n} bodies) differs from the world alone"
        off += n
    for w in (0, 1, 7):  # a pyramid and two piles against the oracle's canonical pair order
        sc = worlds[w]
        ow = oracle_lib.OracleWorld(sc.to_bytes(), oracle_blob(sc, resolve(sc)), oracle_lib.PAIRS_CANONICAL)
        for _ in range(STEPS):
            ow.step(np.float32(sc.dt))
        assert np.array_equal(bits(alone[w]), bits(ow.state())), f"world {w} differs from the oracle"


@pytest.mark.parametrize("order", [0, 1])
def test_island_order_and_launch_shapes_keep_the_bits(order, kzg_lib):
    """Both island-to-CTA orders (island order, largest first) and extreme warp/CTA split points
    give the default launch shapes' bits, with and without graph replay."""
    from kizuriphysics3d_gb300 import World, resolve
    worlds, merged, ids = _batch()
    res = resolve(merged)
    with World(merged, resolved=res, world_ids=ids) as a, World(merged, resolved=res, world_ids=ids) as b:
        b.set_tuning(32, 128, island_order=order)
        b.set_graph(order == 1)
        for _ in range(3):
            a.step_fixed(n=5)
            b.step_fixed(n=5)
            assert np.array_equal(bits(a.state()), bits(b.state()))
        assert b.get_tuning()["island_order"] == order


def test_box_field_bit_exact_with_oracle(oracle_lib, kzg_lib):
    """The 200,000-box field (400 stacks of 500 unit boxes, jitter seed 7, 8 velocity + 2 position
    iterations): three steps against the multi-threaded oracle, bit for bit.  The oracle uses the
    mixed manifold-cache slot function here (same results; the reference's clusters so badly on
    neighbouring ids that one step takes minutes)."""
    from kizuriphysics3d_gb300 import World, resolve, scenes
    sc = scenes.stacks(20, 20, 500)
    res = resolve(sc)
    ow = oracle_lib.OracleWorld(sc.to_bytes(), oracle_blob(sc, res), oracle_lib.PAIRS_CANONICAL,
                                threads=os.cpu_count() or 1)
    ow.set_cache_hash(True)
    with World(sc, resolved=res) as gw:
        for s in range(3):
            ow.step(np.float32(sc.dt))
            gw.step_fixed()
            assert gw.compute_state_hash() == ow.hash(), f"step {s}"
            st, o = gw.get_stats(), ow.stats()
            assert (st["num_broadphase_pairs"], st["num_contact_constraints"], st["num_contact_points"],
                    st["num_islands"]) == (o["pairs"], o["constraints"], o["points"], o["islands"]), s
        assert np.array_equal(bits(gw.state()), bits(ow.state()))
        assert gw.get_stats()["device_error"] == 0
