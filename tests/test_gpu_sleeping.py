"""Sleeping on the GPU (WorldSettings::allowSleeping; UpdateSleeping, PhysicsWorld.cpp:866-951, and
the wake rule of BuildContactConstraints, :473-490) against the oracle, which the reference-traced
fixtures sleep_wake and pile120_sleep pin bit for bit (tests/test_oracle_golden.py).  Through the
C-ABI: state bits, the active list in its order, snapshots, SetBodyActive."""
import numpy as np
import pytest

from conftest import apply_golden_edits, bits, golden_edits, golden_resolved, load_golden, oracle_blob
from tests.golden.gen_golden import fixture_scenes

pytestmark = pytest.mark.gpu

FIXTURES = fixture_scenes()


def _worlds(name, mode):
    from kizuriphysics3d_gb300 import World
    from oracle import pykzo
    sc = FIXTURES[name][0]
    g = load_golden(name)
    res = golden_resolved(sc, g)
    ow = pykzo.OracleWorld(sc.to_bytes(), oracle_blob(sc, res), mode)
    return sc, g, res, ow, World(sc, resolved=res)


@pytest.mark.parametrize("name", ["sleep_wake", "pile120_sleep", "edits_sleep", "edits_nosleep"])
@pytest.mark.parametrize("mode", ["A", "B"])
def test_active_list_and_state_follow_the_oracle(name, mode, oracle_lib, kzg_lib):
    """Every step: the same bodies asleep, the active list in the same order (the reference's
    appends on waking and swap-removals on falling asleep), identical state bits.  The edit
    fixtures add the reference's body operations between steps (SetBodyActive, Add*, Set*), one
    of them with sleeping off: deactivated bodies there wait until a moving body touches them."""
    sc, g, res, ow, gw = _worlds(name, oracle_lib.PAIRS_TREE if mode == "A" else oracle_lib.PAIRS_CANONICAL)
    slept = woke = 0
    prev = None
    with gw:
        for s in range(FIXTURES[name][1]):
            apply_golden_edits(ow, g, s)
            apply_golden_edits(gw, g, s)
            if len(golden_edits(g, s)):
                prev = ow.activity()[1].copy()  # the flags the step starts from
            ow.step(np.float32(sc.dt))
            if mode == "A":
                gw.step_with_pairs(ow.pairs())
            else:
                gw.step_fixed()
            lst, flags, _ = ow.activity()
            assert np.array_equal(gw.active_bodies(), lst), f"active list differs at step {s}"
            assert np.array_equal(bits(gw.state()), bits(ow.state())), f"state differs at step {s}"
            assert gw.get_stats()["num_active_bodies"] == len(lst)
            if prev is not None:
                slept += int(((prev == 1) & (flags == 0)).sum())
                woke += int(((prev == 0) & (flags == 1)).sum())
            prev = flags.copy()
        assert gw.get_stats()["device_error"] == 0
    assert woke > 0 and (slept > 0 or not (sc.flags & 1))  # both directions (sleeping off: only edits deactivate)


def test_snapshot_with_sleeping_resumes_bit_exactly(kzg_lib):
    from kizuriphysics3d_gb300 import World
    sc = FIXTURES["sleep_wake"][0]
    g = load_golden("sleep_wake")
    res = golden_resolved(sc, g)
    with World(sc, resolved=res) as a, World(sc, resolved=res) as b:
        a.step_fixed(n=150)  # several bodies asleep by now
        assert len(a.active_bodies()) < len(sc.bodies)
        b.restore(a.snapshot())
        assert np.array_equal(a.active_bodies(), b.active_bodies())
        for _ in range(3):
            a.step_fixed(n=50)
            b.step_fixed(n=50)
            assert a.compute_state_hash() == b.compute_state_hash()
            assert np.array_equal(a.active_bodies(), b.active_bodies())


def test_set_bodies_active_matches_oracle(oracle_lib, kzg_lib):
    """PhysicsWorld::SetBodyActive in the middle of a run (both directions, ids in a given order),
    then 120 more steps: same active list and bits as the oracle."""
    sc, g, res, ow, gw = _worlds("sleep_wake", oracle_lib.PAIRS_CANONICAL)
    with gw:
        for _ in range(200):
            ow.step(np.float32(sc.dt))
            gw.step_fixed()
        lst, flags, _ = ow.activity()
        asleep = np.nonzero(flags == 0)[0][::-1].astype(np.uint32)  # wake in reverse slot order
        awake = lst[: max(1, len(lst) // 3)][::-1].copy()
        for ids, on in ((asleep, True), (awake, False)):
            ow.set_bodies_active(ids, on)
            gw.set_bodies_active(ids, on)
        assert np.array_equal(gw.active_bodies(), ow.activity()[0])
        for s in range(120):
            ow.step(np.float32(sc.dt))
            gw.step_fixed()
            assert np.array_equal(bits(gw.state()), bits(ow.state())), f"state differs at step {s}"
        assert np.array_equal(gw.active_bodies(), ow.activity()[0])


def test_sleeping_off_keeps_every_body_active(kzg_lib):
    from kizuriphysics3d_gb300 import World, scenes
    sc = scenes.pyramid(4)
    with World(sc) as w:
        w.step_fixed(n=120)
        assert len(w.active_bodies()) == len(sc.bodies)
        assert np.array_equal(w.active_bodies(), np.arange(len(sc.bodies), dtype=np.uint32))


def test_world_loaded_from_a_reference_kzp1_file(oracle_lib, kzg_lib):
    """A world the reference saved mid-run with SerializeWorld (sleep_wake after 300 steps, bodies
    asleep) loads with its sleeping bodies deactivated in slot order, as DeserializeWorld does, and
    then steps like the oracle loaded the same way."""
    import os
    from conftest import GOLDEN
    from kizuriphysics3d_gb300 import World, kzp1, resolve
    data = open(os.path.join(GOLDEN, "sleep_wake_step300.kzp1"), "rb").read()
    sc = kzp1.from_kzp1(data, template=FIXTURES["sleep_wake"][0])
    assert not sc.active.all()
    res = resolve(sc)
    ow = oracle_lib.OracleWorld(sc.to_bytes(), oracle_blob(sc, res), oracle_lib.PAIRS_CANONICAL)
    ow.set_bodies_active(np.nonzero(~sc.active)[0].astype(np.uint32), False)
    with World(sc, resolved=res) as gw:
        assert np.array_equal(gw.active_bodies(), ow.activity()[0])
        for s in range(150):
            ow.step(np.float32(sc.dt))
            gw.step_fixed()
            assert np.array_equal(bits(gw.state()), bits(ow.state())), f"state differs at step {s}"
            assert np.array_equal(gw.active_bodies(), ow.activity()[0]), f"active list differs at step {s}"


@pytest.mark.parametrize("name", ["edits_sleep", "edits_nosleep"])
def test_edit_fixtures_under_graph_replay(name, oracle_lib, kzg_lib):
    """The edit fixtures stepped from a captured graph, many steps per call between the edits: a
    deactivation switches the captured step to the active-list form and back once every body is
    active again, with the same bits as the oracle stepping one step at a time."""
    sc, g, res, ow, gw = _worlds(name, oracle_lib.PAIRS_CANONICAL)
    steps = FIXTURES[name][1]
    marks = sorted(set(int(s) for s in g["edits"]["step"])) + [steps]
    with gw:
        gw.set_graph(True)
        at = 0
        for m in marks:
            if m > at:
                gw.step_fixed(n=m - at)
                for s in range(at, m):
                    apply_golden_edits(ow, g, s)
                    ow.step(np.float32(sc.dt))
                at = m
                assert np.array_equal(bits(gw.state()), bits(ow.state())), f"state differs after step {m - 1}"
                lst, _, _ = ow.activity()
                assert np.array_equal(gw.active_bodies(), lst)
            if m < steps:
                apply_golden_edits(gw, g, m)
        assert gw.get_stats()["device_error"] == 0
