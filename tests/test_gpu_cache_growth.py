"""The manifold cache grows as the reference's does (PhysicsWorld::GetOrCreateCached,
PhysicsWorld.cpp:418-433: entries never evicted, the table doubled past 0.7 load).  A context
started with a tiny table must give the same bits as one whose table never fills, in every way of
stepping: one step at a time, graph replay of many steps in one call, snapshot resume into a fresh
small table, and the autotuner (which holds a copy of the table)."""
import numpy as np
import pytest

from conftest import bits

pytestmark = pytest.mark.gpu

TINY = 256  # slots at creation


def _scene():
    from kizuriphysics3d_gb300 import scenes
    # projectiles crossing a box field: new pairs every step, so the entry count keeps rising
    return scenes.projectiles(n_shots=120, n_boxes=600, seed=21)


def test_tiny_table_grows_and_changes_nothing(kzg_lib):
    from kizuriphysics3d_gb300 import World, resolve
    sc = _scene()
    res = resolve(sc)
    with World(sc, resolved=res, max_cache_entries=TINY) as small, World(sc, resolved=res) as big:
        cap0 = big.get_stats()["cache_capacity"]
        for s in range(60):
            small.step_fixed()
            big.step_fixed()
            a, b = small.get_stats(), big.get_stats()
            assert a["device_error"] == 0 and b["device_error"] == 0
            assert a["cache_entries"] == b["cache_entries"], s
            # below 0.7 load before the step, so past it by at most this step's new entries
            assert a["cache_entries"] * 10 < a["cache_capacity"] * 7 + 10 * a["num_contact_constraints"], s
            if s % 10 == 9:
                assert np.array_equal(bits(small.state()), bits(big.state())), f"state differs at step {s}"
        st = small.get_stats()
        assert st["cache_capacity"] > TINY and st["cache_entries"] > TINY  # it did have to grow
        assert big.get_stats()["cache_capacity"] == cap0  # the default table never filled
        assert small.compute_state_hash() == big.compute_state_hash()


def test_graph_replay_grows_between_runs(kzg_lib):
    from kizuriphysics3d_gb300 import World, resolve
    sc = _scene()
    res = resolve(sc)
    with World(sc, resolved=res, max_cache_entries=TINY) as small, World(sc, resolved=res) as big:
        small.set_graph(True)
        big.set_graph(True)
        small.step_fixed(n=60)  # one call: replayed in runs, the table grown between them
        big.step_fixed(n=60)
        a = small.get_stats()
        assert a["device_error"] == 0
        assert a["cache_capacity"] > TINY
        assert a["cache_entries"] == big.get_stats()["cache_entries"]
        assert np.array_equal(bits(small.state()), bits(big.state()))


def test_snapshot_of_a_grown_table_loads_into_a_tiny_one(kzg_lib):
    from kizuriphysics3d_gb300 import World, resolve
    sc = _scene()
    res = resolve(sc)
    with World(sc, resolved=res, max_cache_entries=TINY) as a, \
            World(sc, resolved=res, max_cache_entries=TINY) as b:
        a.step_fixed(n=40)
        snap = a.snapshot()
        b.restore(snap)  # b's table takes the snapshot's capacity
        assert b.get_stats()["cache_capacity"] == a.get_stats()["cache_capacity"] > TINY
        for _ in range(20):
            a.step_fixed()
            b.step_fixed()
        assert b.get_stats()["cache_entries"] == a.get_stats()["cache_entries"]
        assert np.array_equal(bits(a.state()), bits(b.state()))


def test_autotune_on_a_tiny_table_leaves_the_world_unchanged(kzg_lib):
    from kizuriphysics3d_gb300 import World, resolve
    sc = _scene()
    res = resolve(sc)
    with World(sc, resolved=res, max_cache_entries=TINY) as a, World(sc, resolved=res) as ref:
        a.step_fixed(n=10)
        ref.step_fixed(n=10)
        a.autotune(steps_per_candidate=2)
        assert np.array_equal(bits(a.state()), bits(ref.state()))
        a.step_fixed(n=30)
        ref.step_fixed(n=30)
        assert np.array_equal(bits(a.state()), bits(ref.state()))
