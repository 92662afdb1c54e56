"""The oracle (oracle/, a C restatement of the reference step) against the golden fixtures that the
reference engine itself produced (tests/golden/gen_golden.py).  CPU only."""
import numpy as np
import pytest

from conftest import apply_golden_edits, bits, golden_resolved, load_golden, oracle_blob
from tests.golden.gen_golden import fixture_scenes

FIXTURES = fixture_scenes()


@pytest.mark.parametrize("name", sorted(FIXTURES))
def test_oracle_matches_reference_every_step(name, oracle_lib):
    sc, steps, detail, ckpt = FIXTURES[name]
    g = load_golden(name)
    w = oracle_lib.OracleWorld(sc.to_bytes(), oracle_blob(sc, golden_resolved(sc, g)), oracle_lib.PAIRS_TREE)
    assert np.array_equal(bits(w.state()), bits(g["state0"]))
    im, iw = w.mass()
    assert np.array_equal(bits(iw), bits(g["inv_inertia_world"]))
    k = 0
    for s in range(steps):
        apply_golden_edits(w, g, s)  # body operations the reference run applied before this step
        w.step(np.float32(sc.dt))
        assert w.hash() == int(g["hashes"][s]), f"{name}: state hash differs at step {s}"
        st = w.stats()
        assert [st["pairs"], st["constraints"], st["points"], st["islands"]] == list(g["stats"][s]), s
        if s < detail:
            assert np.array_equal(w.pairs(), g[f"d{s}_pairs"])
            hdr, pts, fr = w.constraints()
            assert np.array_equal(hdr, g[f"d{s}_con_hdr"])
            assert np.array_equal(bits(fr), bits(g[f"d{s}_con_fr"]))
            assert np.array_equal(bits(pts), bits(g[f"d{s}_con_pts"]))
        if k < len(ckpt) and s == ckpt[k]:
            assert np.array_equal(bits(w.state()), bits(g["ckpt_states"][k])), f"{name}: state differs at {s}"
            k += 1


def test_oracle_thread_count_does_not_change_results(oracle_lib):
    sc, steps, _, _ = FIXTURES["pile200"]
    g = load_golden("pile200")
    blob = oracle_blob(sc, golden_resolved(sc, g))
    hs = []
    for threads in (1, 4):
        w = oracle_lib.OracleWorld(sc.to_bytes(), blob, oracle_lib.PAIRS_TREE, threads=threads)
        for _ in range(120):
            w.step(np.float32(sc.dt))
        hs.append(w.hash())
    assert hs[0] == hs[1] == int(g["hashes"][119])


def test_canonical_pairs_are_sorted_and_complete(oracle_lib):
    """Canonical mode finds every overlapping pair (the reference tree drops pairs whose leaf ids
    come out reversed in its traversal, BroadPhase.h:90-92) in MakePairKey order."""
    sc, _, _, _ = FIXTURES["pile200"]
    g = load_golden("pile200")
    blob = oracle_blob(sc, golden_resolved(sc, g))
    tree = oracle_lib.OracleWorld(sc.to_bytes(), blob, oracle_lib.PAIRS_TREE)
    canon = oracle_lib.OracleWorld(sc.to_bytes(), blob, oracle_lib.PAIRS_CANONICAL)
    tree.step(np.float32(sc.dt))
    canon.step(np.float32(sc.dt))
    pt, pc = tree.pairs(), canon.pairs()
    keys = (pc[:, 0].astype(np.uint64) << np.uint64(32)) | pc[:, 1].astype(np.uint64)
    assert np.all(np.diff(keys.astype(np.int64)) > 0)
    assert np.all(pc[:, 0] < pc[:, 1])
    st = set(map(tuple, np.sort(pt, axis=1)))
    assert st <= set(map(tuple, pc)), "the tree's pair set must be a subset of all overlapping pairs"


def _two_body_scene(shape_a, pos_a, shape_b, pos_b, motion_a=2, motion_b=2):
    from kizuriphysics3d_gb300 import scenes as S
    sc = S.Scene()
    ia = sc.add_shape(shape_a)
    ib = sc.add_shape(shape_b)
    sc.add_body(S.Body(ia, motion_a, pos=pos_a))
    sc.add_body(S.Body(ib, motion_b, pos=pos_b))
    return sc


def _collide(oracle_lib, sc, max_sep=0.02):
    from kizuriphysics3d_gb300.world import Resolved
    n = len(sc.bodies)
    res = Resolved({}, np.zeros(n, np.float32), np.zeros((n, 9), np.float32))
    w = oracle_lib.OracleWorld(sc.to_bytes(), oracle_blob(sc, res))
    return w.collide(0, 1, max_sep)


# Known-answer tests of the reference (tests/TestCollision.cpp:45-112), on the oracle.
def test_known_answer_sphere_sphere(oracle_lib):
    from kizuriphysics3d_gb300 import scenes as S
    m = _collide(oracle_lib, _two_body_scene(S.Shape(S.SHAPE_SPHERE, [1, 0, 0, 0]), (0, 0, 0),
                                             S.Shape(S.SHAPE_SPHERE, [1, 0, 0, 0]), (1.8, 0, 0)), 1.0e-1)
    assert m.shape[0] == 1
    assert abs(m[0, 9] - (-0.2)) < 1e-2 and abs(m[0, 6] - (-1.0)) < 1e-2


def test_known_answer_box_on_plane(oracle_lib):
    from kizuriphysics3d_gb300 import scenes as S
    m = _collide(oracle_lib, _two_body_scene(S.Shape(S.SHAPE_BOX, [1, 1, 1, 0]), (0, 0.9, 0),
                                             S.Shape(S.SHAPE_PLANE, [0, 1, 0, 0]), (0, 0, 0), 2, 0))
    assert m.shape[0] == 4 and abs(m[0, 9] + 0.1) < 1e-2


def test_known_answer_box_box(oracle_lib):
    from kizuriphysics3d_gb300 import scenes as S
    m = _collide(oracle_lib, _two_body_scene(S.Shape(S.SHAPE_BOX, [1, 1, 1, 0]), (0, 0, 0),
                                             S.Shape(S.SHAPE_BOX, [1, 1, 1, 0]), (0, 1.9, 0)))
    assert m.shape[0] >= 4 and m[0, 9] < 0


def test_known_answer_sphere_box(oracle_lib):
    from kizuriphysics3d_gb300 import scenes as S
    m = _collide(oracle_lib, _two_body_scene(S.Shape(S.SHAPE_SPHERE, [0.5, 0, 0, 0]), (1.4, 0, 0),
                                             S.Shape(S.SHAPE_BOX, [1, 1, 1, 0]), (0, 0, 0)))
    assert m.shape[0] == 1 and abs(m[0, 9] + 0.1) < 1e-2


def test_known_answer_separated(oracle_lib):
    from kizuriphysics3d_gb300 import scenes as S
    m = _collide(oracle_lib, _two_body_scene(S.Shape(S.SHAPE_BOX, [1, 1, 1, 0]), (0, 0, 0),
                                             S.Shape(S.SHAPE_BOX, [1, 1, 1, 0]), (10, 0, 0)))
    assert m.shape[0] == 0


def test_oracle_joint_trigonometry_modes(oracle_lib):
    """The oracle's joint trigonometry: the C library's float functions (default) reproduce the
    reference trace; double-evaluated values rounded to float (mode 1, the GPU kernels') give the same bits until
    the first call where the two differ, several steps into the joints fixture.  (After that the
    trajectories part quickly: the fixture's chain links press against each other.)"""
    sc, steps, _, _ = FIXTURES["joints_mix"]
    g = load_golden("joints_mix")
    blob = oracle_blob(sc, golden_resolved(sc, g))
    a = oracle_lib.OracleWorld(sc.to_bytes(), blob, oracle_lib.PAIRS_TREE)
    b = oracle_lib.OracleWorld(sc.to_bytes(), blob, oracle_lib.PAIRS_TREE)
    b.set_trig_mode(1)
    first = None
    for s in range(steps):
        a.step(np.float32(sc.dt))
        b.step(np.float32(sc.dt))
        assert a.hash() == int(g["hashes"][s])
        if first is None and a.hash() != b.hash():
            first = s
    assert first is not None and first >= 5


def test_joints_mix_is_ill_conditioned_in_the_reference_arithmetic(oracle_lib):
    """Why joints_mix is checked against the reference by bits only up to the first differing
    trigonometric rounding: its six-link chain, whose links touch each other, is so sensitive that a
    one-ulp change of one initial velocity, stepped with the reference's own arithmetic (the oracle
    in the reference's trigonometry mode), departs from the reference by more than 1e-2 relative
    within 30 steps.  No tolerance of the size the path allows survives that scene."""
    sc, steps, _, _ = FIXTURES["joints_mix"]
    g = load_golden("joints_mix")
    blob = oracle_blob(sc, golden_resolved(sc, g))
    base = oracle_lib.OracleWorld(sc.to_bytes(), blob, oracle_lib.PAIRS_TREE)
    pert = oracle_lib.OracleWorld(sc.to_bytes(), blob, oracle_lib.PAIRS_TREE)
    st = pert.state()
    st[7, 7] = np.nextafter(st[7, 7], np.float32(np.inf))  # last chain link: one ulp of its x velocity
    pert.set_state(st)
    dyn = np.array([b.motion == 2 for b in sc.bodies])
    worst = 0.0
    for s in range(30):
        base.step(np.float32(sc.dt))
        pert.step(np.float32(sc.dt))
        a, b = base.state()[dyn, 7:10].astype(np.float64), pert.state()[dyn, 7:10].astype(np.float64)
        worst = max(worst, float(np.max(np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(a, axis=1), 1e-3))))
    assert worst > 1e-2


def test_mixed_cache_slot_function_changes_no_result(oracle_lib):
    """The oracle's optional mixed manifold-cache slot function (used where the reference's
    clustered one makes a world too slow to step) gives the reference's results, bit for bit."""
    sc, _, _, _ = FIXTURES["pile200"]
    g = load_golden("pile200")
    w = oracle_lib.OracleWorld(sc.to_bytes(), oracle_blob(sc, golden_resolved(sc, g)), oracle_lib.PAIRS_TREE)
    w.set_cache_hash(True)
    for s in range(300):
        w.step(np.float32(sc.dt))
        assert w.hash() == int(g["hashes"][s]), s
