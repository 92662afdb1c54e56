"""GPU parity: the CUDA pipeline (through the C-ABI of libkzg.so) against the oracle and the
reference's golden fixtures.  The bar is bit-exact: identical ComputeStateHash after every step,
identical float bits of every body state, contact point and impulse.

Mode A feeds the GPU the reference's own broad-phase pair order (produced by the oracle's
restatement of the reference's dynamic AABB tree, itself pinned to the reference); mode B is the
production path with the GPU broad phase (canonical MakePairKey order) checked against the oracle
running the same pair order.
"""
import numpy as np
import pytest

from conftest import apply_golden_edits, bits, golden_resolved, load_golden, oracle_blob
from tests.golden.gen_golden import fixture_scenes

FIXTURES = fixture_scenes()
pytestmark = pytest.mark.gpu


def _pair_worlds(name, mode, oracle_lib, **kw):
    from kizuriphysics3d_gb300 import World
    sc = FIXTURES[name][0]
    g = load_golden(name)
    res = golden_resolved(sc, g)
    ow = oracle_lib.OracleWorld(sc.to_bytes(), oracle_blob(sc, res), mode, threads=kw.pop("threads", 1))
    gw = World(sc, resolved=res, **kw)
    return sc, g, ow, gw


# joints_mix: the joint kernels' trigonometry is evaluated in double and rounded to float, the reference's is the C
# library's float functions; that fixture has its own tests below.
@pytest.mark.parametrize("name", sorted(n for n in FIXTURES if n != "joints_mix"))
def test_mode_a_bit_exact_with_reference(name, oracle_lib, kzg_lib):
    sc, g, ow, gw = _pair_worlds(name, oracle_lib.PAIRS_TREE, oracle_lib)
    steps, detail = FIXTURES[name][1], FIXTURES[name][2]
    with gw:
        im, iw = gw.mass()
        assert np.array_equal(bits(iw), bits(g["inv_inertia_world"]))
        for s in range(steps):
            apply_golden_edits(ow, g, s)  # body operations of the reference run (edit fixtures)
            apply_golden_edits(gw, g, s)
            ow.step(np.float32(sc.dt))
            gw.step_with_pairs(ow.pairs())
            gs = gw.get_stats()
            # With sleeping on, numIslands is UpdateSleeping's count, which depends on the position
            # the reference's union-by-rank makes each root; it is counted that way on demand.
            assert [gs["num_broadphase_pairs"], gs["num_contact_constraints"], gs["num_contact_points"],
                    gs["num_islands"]] == list(g["stats"][s]), \
                f"{name}: WorldStats differ from the reference at step {s}"
            st = gw.state()
            if not np.array_equal(bits(st), bits(ow.state())):
                bad = np.argwhere(bits(st) != bits(ow.state()))
                pytest.fail(f"{name}: GPU state differs from the oracle at step {s}, first entries {bad[:4].tolist()}")
            assert gw.compute_state_hash() == int(g["hashes"][s]), f"{name}: hash differs from the reference at {s}"
            if s < detail:
                hdr, pts, fr = gw.contact_constraints()
                assert np.array_equal(hdr, g[f"d{s}_con_hdr"])
                assert np.array_equal(bits(fr), bits(g[f"d{s}_con_fr"]))
                assert np.array_equal(bits(pts), bits(g[f"d{s}_con_pts"]))
        assert gw.get_stats()["device_error"] == 0


@pytest.mark.parametrize("name,steps", [("pile200", 300), ("stacks2x2x20", 200), ("pyramid20", 200),
                                        ("ccd_shots", 120), ("ccd_threshold", 90), ("sleep_wake", 600),
                                        ("pile120_sleep", 480), ("edits_sleep", 480), ("edits_nosleep", 240),
                                        ("pyramid20_scalar", 300), ("pile200_scalar", 300)])
def test_mode_b_bit_exact_with_oracle(name, steps, oracle_lib, kzg_lib):
    sc, g, ow, gw = _pair_worlds(name, oracle_lib.PAIRS_CANONICAL, oracle_lib)
    with gw:
        for s in range(steps):
            apply_golden_edits(ow, g, s)
            apply_golden_edits(gw, g, s)
            ow.step(np.float32(sc.dt))
            gw.step_fixed()
            assert np.array_equal(gw.broadphase_pairs(), ow.pairs()), f"pair list differs at step {s}"
            assert np.array_equal(bits(gw.state()), bits(ow.state())), f"state differs at step {s}"
        hdr, pts, fr = gw.contact_constraints()
        ohdr, opts, ofr = ow.constraints()
        assert np.array_equal(hdr, ohdr) and np.array_equal(bits(pts), bits(opts))


def test_mode_b_larger_pile(oracle_lib, kzg_lib):
    from kizuriphysics3d_gb300 import World, resolve, scenes
    sc = scenes.pile(1500, seed=99, extent=6.0, y_range=(1.0, 20.0))
    res = resolve(sc)
    ow = oracle_lib.OracleWorld(sc.to_bytes(), oracle_blob(sc, res), oracle_lib.PAIRS_CANONICAL, threads=8)
    with World(sc, resolved=res) as gw:
        for s in range(150):
            ow.step(np.float32(sc.dt))
            gw.step_fixed()
        assert np.array_equal(bits(gw.state()), bits(ow.state()))
        assert gw.compute_state_hash() == ow.hash()


def test_mode_b_scalar_solver_larger_pile(oracle_lib, kzg_lib):
    """SolverSettings::useSIMDSolver = false on a 1,500-body pile: islands large enough for the
    CTA-wide schedule and solve, 150 steps bit-exact against the oracle's scalar sweep."""
    from kizuriphysics3d_gb300 import World, resolve, scenes
    sc = scenes.pile(1500, seed=99, extent=6.0, y_range=(1.0, 20.0))
    sc.flags |= scenes.WORLD_FLAG_SCALAR_SOLVER
    res = resolve(sc)
    ow = oracle_lib.OracleWorld(sc.to_bytes(), oracle_blob(sc, res), oracle_lib.PAIRS_CANONICAL, threads=8)
    with World(sc, resolved=res) as gw:
        for s in range(150):
            ow.step(np.float32(sc.dt))
            gw.step_fixed()
        assert np.array_equal(bits(gw.state()), bits(ow.state()))
        st, o = gw.get_stats(), ow.stats()
        assert st["num_batches"] == 0
        assert st["point_velocity_iterations"] == o["point_velocity_iterations"]


@pytest.mark.parametrize("scalar", [False, True])
def test_mode_b_settled_full_pile(scalar, oracle_lib, kzg_lib):
    """The 20,000-body random convex pile at its settled state (the bench snapshot): one giant
    island of ~100k contact points, so the schedule's open-batch table compacts and the solve runs
    the in-place big-island kernel.  Two steps, bit-exact against the oracle."""
    import os
    from kizuriphysics3d_gb300 import World, resolve, scenes
    snap = os.path.join(os.path.dirname(__file__), "..", "kizuriphysics3d_gb300", "data", "pile20000_step600.npz")
    sc = scenes.pile(20000, seed=1234)
    if scalar:  # the scalar solver's velocity levels through the same kernels
        sc.flags |= scenes.WORLD_FLAG_SCALAR_SOLVER
    with np.load(snap) as z:
        state = z["state"]
    for b, st in zip(sc.bodies, state):
        b.pos, b.rot, b.vel, b.ang = tuple(st[0:3]), tuple(st[3:7]), tuple(st[7:10]), tuple(st[10:13])
    res = resolve(sc)
    ow = oracle_lib.OracleWorld(sc.to_bytes(), oracle_blob(sc, res), oracle_lib.PAIRS_CANONICAL,
                                threads=os.cpu_count() or 1)
    with World(sc, resolved=res, max_pairs=48 * len(sc.bodies)) as gw:
        for s in range(2):
            ow.step(np.float32(sc.dt))
            gw.step_fixed()
            assert gw.compute_state_hash() == ow.hash(), f"step {s}"
        st = gw.get_stats()
        assert st["device_error"] == 0
        assert st["num_contact_points"] > 80000
        assert np.array_equal(bits(gw.state()), bits(ow.state()))


@pytest.mark.parametrize("name,steps", [("pile200", 120), ("pyramid20", 60)])
def test_residual_terminated_bit_exact_with_oracle(name, steps, oracle_lib, kzg_lib):
    """Residual-terminated velocity iterations (r <= 1e-4 m/s, cap 64): same iteration counts,
    same final residual and same state bits as the oracle running the same rule."""
    sc, g, ow, gw = _pair_worlds(name, oracle_lib.PAIRS_CANONICAL, oracle_lib)
    ow.set_residual(1e-4, 64)
    with gw:
        gw.set_residual(1e-4, 64)
        seen_iters = set()
        for s in range(steps):
            ow.step(np.float32(sc.dt))
            gw.step_fixed()
            o, st = ow.stats(), gw.get_stats()
            assert st["max_velocity_iterations_used"] == o["max_velocity_iterations"], f"step {s}"
            assert st["point_velocity_iterations"] == o["point_velocity_iterations"], f"step {s}"
            assert np.float32(st["final_residual"]).view(np.uint32) == np.float32(o["final_residual"]).view(np.uint32)
            assert gw.compute_state_hash() == ow.hash(), f"step {s}"
            seen_iters.add(st["max_velocity_iterations_used"])
        assert np.array_equal(bits(gw.state()), bits(ow.state()))
        assert len(seen_iters) > 1  # the stopping rule actually varied the iteration count


@pytest.mark.parametrize("mode", ["A", "B"])
def test_joints_bit_exact_with_oracle(mode, oracle_lib, kzg_lib):
    """Every joint type beside contacts (the joints_mix fixture), 180 steps, in both pair modes:
    bit-identical to the oracle evaluating sin / cos / acos / atan2 the way the joint kernels do
    (double precision rounded to float)."""
    sc, g, ow, gw = _pair_worlds("joints_mix", oracle_lib.PAIRS_TREE if mode == "A" else oracle_lib.PAIRS_CANONICAL,
                                 oracle_lib)
    ow.set_trig_mode(1)
    with gw:
        for s in range(FIXTURES["joints_mix"][1]):
            ow.step(np.float32(sc.dt))
            if mode == "A":
                gw.step_with_pairs(ow.pairs())
            else:
                gw.step_fixed()
            st, ost = gw.state(), ow.state()
            if not np.array_equal(bits(st), bits(ost)):
                bad = np.argwhere(bits(st) != bits(ost))
                pytest.fail(f"mode {mode}: state differs from the oracle at step {s}, first entries {bad[:4].tolist()}")
        assert gw.get_stats()["device_error"] == 0


def test_joints_match_reference_until_its_trigonometry_differs(oracle_lib, kzg_lib):
    """Against the reference's own trace: the GPU's state hash equals the reference's at every step
    before the first step where the C library's float sinf / cosf / acosf / atan2f (the reference's)
    and the double-evaluated values rounded to float (the GPU's) give different bits, found by running the oracle
    both ways."""
    sc, g, ow, gw = _pair_worlds("joints_mix", oracle_lib.PAIRS_TREE, oracle_lib)
    cw = oracle_lib.OracleWorld(sc.to_bytes(), oracle_blob(sc, golden_resolved(sc, g)), oracle_lib.PAIRS_TREE)
    cw.set_trig_mode(1)
    same = 0
    with gw:
        for s in range(FIXTURES["joints_mix"][1]):
            ow.step(np.float32(sc.dt))
            cw.step(np.float32(sc.dt))
            if ow.hash() != cw.hash():
                break
            gw.step_with_pairs(ow.pairs())
            assert gw.compute_state_hash() == int(g["hashes"][s]), f"hash differs from the reference at {s}"
            same += 1
    assert same >= 5


def test_joint_velocities_within_tolerance_of_reference(oracle_lib, kzg_lib):
    """Per-step velocities within 1e-4 relative of the reference's over 60 steps (the path's
    tolerance for floating point), on the reference-traced joints_single fixture: 48 single-joint
    systems of all six types with seeded motions and no contacts.  The reference's states of every
    step are in the fixture.  Relative error per body: |dv| / max(|v_ref|, 1e-3 m/s) for the linear
    and angular velocity."""
    sc, g, ow, gw = _pair_worlds("joints_single", oracle_lib.PAIRS_TREE, oracle_lib)
    dyn = np.array([b.motion == 2 for b in sc.bodies])
    exact = True
    with gw:
        for s in range(60):
            ow.step(np.float32(sc.dt))
            gw.step_with_pairs(ow.pairs())
            st, ref = gw.state(), g["ckpt_states"][s]
            for sl in (slice(7, 10), slice(10, 13)):
                dv = np.linalg.norm(st[dyn, sl].astype(np.float64) - ref[dyn, sl], axis=1)
                rel = dv / np.maximum(np.linalg.norm(ref[dyn, sl].astype(np.float64), axis=1), 1e-3)
                assert rel.max() <= 1e-4, f"step {s}: relative velocity error {rel.max():.3g}"
            exact = exact and np.array_equal(bits(st), bits(ref))
        assert gw.get_stats()["device_error"] == 0
    print("joints_single: bit-identical to the reference for all 60 steps" if exact else
          "joints_single: within 1e-4 relative, not bit-identical")


def _bullet_scene(flags):
    from kizuriphysics3d_gb300 import scenes
    sc = scenes.Scene(name="bullet")
    wall = sc.add_shape(scenes.Shape(scenes.SHAPE_BOX, [0.02, 2.0, 2.0, 0.0]))
    ball = sc.add_shape(scenes.Shape(scenes.SHAPE_SPHERE, [0.1, 0.0, 0.0, 0.0]))
    sc.gravity = (0.0, 0.0, 0.0)
    sc.add_body(scenes.Body(shape=wall, motion=scenes.MOTION_STATIC, pos=(0.0, 0.0, 0.0)))
    sc.add_body(scenes.Body(shape=ball, motion=scenes.MOTION_DYNAMIC, pos=(-3.0, 0.0, 0.0), vel=(120.0, 0.0, 0.0),
                            flags=flags, max_linear_velocity=500.0))
    return sc


def test_linear_cast_stops_a_bullet_at_a_thin_wall(kzg_lib):
    """A 0.1 m ball at 120 m/s (2 m per step) against a 4 cm static wall: the discrete body passes
    through between two steps; the LinearCast body's motion is clamped max_pen short of the cast
    hit every step (ClampMotionCCD), so it stays in front of the wall (x = -0.130 in the oracle)."""
    from kizuriphysics3d_gb300 import World, scenes
    xs = {}
    for flags in (0, scenes.BODY_FLAG_LINEAR_CAST):
        with World(_bullet_scene(flags)) as w:
            w.step_fixed(n=4)
            xs[flags] = float(w.state()[1][0])
            assert w.get_stats()["device_error"] == 0
    assert xs[0] > 2.0
    assert -0.2 < xs[scenes.BODY_FLAG_LINEAR_CAST] < -0.1


def _run_both(sc, steps, oracle_lib):
    """Step the GPU world and the oracle (joint trigonometry in double, rounded to float) side by side;
    returns the GPU's final state after checking every step bit for bit."""
    from kizuriphysics3d_gb300 import World, resolve
    res = resolve(sc)
    ow = oracle_lib.OracleWorld(sc.to_bytes(), oracle_blob(sc, res), oracle_lib.PAIRS_CANONICAL)
    ow.set_trig_mode(1)
    with World(sc, resolved=res) as w:
        for s in range(steps):
            ow.step(np.float32(sc.dt))
            w.step_fixed()
            assert np.array_equal(bits(w.state()), bits(ow.state())), f"{sc.name}: differs at step {s}"
        assert w.get_stats()["device_error"] == 0
        return w.state()


def test_reference_world_ccd_prevents_tunneling(oracle_lib, kzg_lib):
    """The reference's World_CCDPreventsTunneling (tests/TestWorld.cpp:250-279): a 0.1 m LinearCast
    sphere at 120 m/s toward a 10 cm static wall, no gravity; after 10 steps it is still behind."""
    from kizuriphysics3d_gb300 import scenes as S
    sc = S.Scene(name="ccd_tunneling")
    sc.gravity = (0.0, 0.0, 0.0)
    wall = sc.add_shape(S.Shape(S.SHAPE_BOX, [0.05, 5.0, 5.0, 0.0]))
    ball = sc.add_shape(S.Shape(S.SHAPE_SPHERE, [0.1, 0.0, 0.0, 0.0]))
    sc.add_body(S.Body(wall, S.MOTION_STATIC))
    sc.add_body(S.Body(ball, pos=(-5.0, 0.0, 0.0), vel=(120.0, 0.0, 0.0), gravity_factor=0.0,
                       flags=S.BODY_FLAG_ALLOW_SLEEPING | S.BODY_FLAG_LINEAR_CAST))
    st = _run_both(sc, 10, oracle_lib)
    assert st[1][0] < 0.0


def test_reference_world_point_constraint_pendulum(oracle_lib, kzg_lib):
    """The reference's World_PointConstraintPendulum (tests/TestWorld.cpp:186-213): a 0.3 m bob on a
    2 m point-joint rod from a static anchor swings for 2 s; the rod length holds within 0.15."""
    from kizuriphysics3d_gb300 import scenes as S
    sc = S.Scene(name="pendulum")
    anchor = sc.add_shape(S.Shape(S.SHAPE_SPHERE, [0.1, 0.0, 0.0, 0.0]))
    bob = sc.add_shape(S.Shape(S.SHAPE_SPHERE, [0.3, 0.0, 0.0, 0.0]))
    a = sc.add_body(S.Body(anchor, S.MOTION_STATIC, pos=(0.0, 5.0, 0.0)))
    b = sc.add_body(S.Body(bob, pos=(2.0, 5.0, 0.0)))
    sc.joints.append(S.Joint(S.JOINT_POINT, a, b, anchor_a=(0.0, 5.0, 0.0)))
    st = _run_both(sc, int(np.float32(2.0) / np.float32(1.0 / 60.0)), oracle_lib)
    assert abs(np.linalg.norm(st[1][0:3] - np.array([0.0, 5.0, 0.0])) - 2.0) < 0.15


def test_reference_world_distance_constraint(oracle_lib, kzg_lib):
    """The reference's World_DistanceConstraint (tests/TestWorld.cpp:215-233): a sphere hangs 2 m
    below a static one on a distance joint for 2 s; the distance holds within 0.15.  (The
    reference makes the upper body static after creating it dynamic, so it keeps a dynamic body's
    inverse mass; here it is created static.)"""
    from kizuriphysics3d_gb300 import scenes as S
    sc = S.Scene(name="distance")
    sph = sc.add_shape(S.Shape(S.SHAPE_SPHERE, [0.2, 0.0, 0.0, 0.0]))
    a = sc.add_body(S.Body(sph, S.MOTION_STATIC, pos=(0.0, 5.0, 0.0)))
    b = sc.add_body(S.Body(sph, pos=(0.0, 3.0, 0.0)))
    sc.joints.append(S.Joint(S.JOINT_DISTANCE, a, b, anchor_a=(0.0, 5.0, 0.0), anchor_b=(0.0, 3.0, 0.0), distance=2.0))
    st = _run_both(sc, int(np.float32(2.0) / np.float32(1.0 / 60.0)), oracle_lib)
    assert abs(np.linalg.norm(st[1][0:3] - np.array([0.0, 5.0, 0.0])) - 2.0) < 0.15


def test_graph_stepping_matches_direct_stepping(kzg_lib):
    """kzg_set_graph: steps replayed from one captured CUDA graph give the same bits as steps issued
    one by one, including after a settings change forces a new capture."""
    from kizuriphysics3d_gb300 import World, resolve, scenes
    sc = scenes.pile(600, seed=8, extent=4.0, y_range=(1.0, 12.0))
    res = resolve(sc)
    with World(sc, resolved=res) as a, World(sc, resolved=res) as b:
        b.set_graph(True)
        for chunk in (1, 7, 20, 20):
            a.step_fixed(n=chunk)
            b.step_fixed(n=chunk)
            assert a.compute_state_hash() == b.compute_state_hash()
        a.set_residual(1e-4, 64)
        b.set_residual(1e-4, 64)
        a.step_fixed(n=15)
        b.step_fixed(n=15)
        assert a.compute_state_hash() == b.compute_state_hash()
        assert np.array_equal(bits(a.state()), bits(b.state()))
        assert b.get_stats()["max_velocity_iterations_used"] == a.get_stats()["max_velocity_iterations_used"]


def test_many_linear_cast_bodies_bit_exact_with_oracle(oracle_lib, kzg_lib):
    """400 LinearCast projectiles among walls and boxes (the projectiles workload, scaled down):
    the GPU resolves the casts of independent bodies in parallel rounds and the ordered remainder in
    slot order; the result is the oracle's sequential one, bit for bit, for 40 steps."""
    from kizuriphysics3d_gb300 import World, resolve, scenes
    sc = scenes.projectiles(400, 600)
    res = resolve(sc)
    ow = oracle_lib.OracleWorld(sc.to_bytes(), oracle_blob(sc, res), oracle_lib.PAIRS_CANONICAL)
    with World(sc, resolved=res) as gw:
        for s in range(40):
            ow.step(np.float32(sc.dt))
            gw.step_fixed()
            assert np.array_equal(bits(gw.state()), bits(ow.state())), f"state differs at step {s}"
        assert gw.get_stats()["device_error"] == 0


def test_joint_field_bit_exact_with_oracle(oracle_lib, kzg_lib):
    """A field of 100 ten-link chains (the chains workload, scaled down): hundreds of joint islands
    with contacts, solved one CTA each, bit-identical to the oracle (trigonometry in double, rounded to float)
    for 40 steps."""
    from kizuriphysics3d_gb300 import World, resolve, scenes
    sc = scenes.chains(10, 10, 10)
    res = resolve(sc)
    ow = oracle_lib.OracleWorld(sc.to_bytes(), oracle_blob(sc, res), oracle_lib.PAIRS_CANONICAL)
    ow.set_trig_mode(1)
    with World(sc, resolved=res) as gw:
        for s in range(40):
            ow.step(np.float32(sc.dt))
            gw.step_fixed()
            assert np.array_equal(bits(gw.state()), bits(ow.state())), f"state differs at step {s}"
        assert gw.get_stats()["device_error"] == 0


def test_snapshot_resumes_bit_exactly(kzg_lib):
    """kzg_snapshot_save / load: a second context restored from a snapshot continues bit-exactly;
    restoring the body state alone (cold manifold cache) does not, which is what the cache part of
    the snapshot is for."""
    from kizuriphysics3d_gb300 import World, resolve, scenes
    sc = scenes.pile(500, seed=12, extent=4.0, y_range=(1.0, 10.0))
    res = resolve(sc)
    with World(sc, resolved=res) as a, World(sc, resolved=res) as b, World(sc, resolved=res) as c:
        a.step_fixed(n=60)
        snap, state60 = a.snapshot(), a.state()
        a.step_fixed(n=40)
        b.restore(snap)
        b.step_fixed(n=40)
        assert b.compute_state_hash() == a.compute_state_hash()
        assert np.array_equal(bits(b.state()), bits(a.state()))
        c.set_state(state60)
        c.step_fixed(n=40)
        assert c.compute_state_hash() != a.compute_state_hash()


def test_snapshot_with_joints_and_ccd_resumes_bit_exactly(kzg_lib):
    """The snapshot also carries the joints' accumulated impulses and prepared frames and the
    bodies' broad-phase fat bounds (continuous collision reads them): a world of joints resumes
    bit-exactly, and so does the CCD fixture."""
    from kizuriphysics3d_gb300 import World, resolve
    for name in ("joints_mix", "ccd_shots"):
        sc = FIXTURES[name][0]
        res = resolve(sc)
        with World(sc, resolved=res) as a, World(sc, resolved=res) as b:
            a.step_fixed(n=30)
            snap = a.snapshot()
            a.step_fixed(n=30)
            b.restore(snap)
            b.step_fixed(n=30)
            assert np.array_equal(bits(b.state()), bits(a.state())), name


def test_kzp1_world_steps_like_the_scene(kzg_lib):
    """A world loaded from KZP1 bytes of a box scene (no hulls to rebuild) steps to the same state
    as the scene it was written from."""
    from kizuriphysics3d_gb300 import World, kzp1, scenes
    sc = scenes.pyramid(6)
    back = kzp1.from_kzp1(kzp1.to_kzp1(sc), template=sc)
    with World(sc) as a, World(back) as b:
        a.step_fixed(n=50)
        b.step_fixed(n=50)
        assert a.compute_state_hash() == b.compute_state_hash()


def _facade_joint_scene(nx, nz, links):
    """The scene kizuriphysics3d_gb300/cpp/joints_example.cpp builds, through the Python API."""
    from kizuriphysics3d_gb300 import scenes as S
    f = S.f32
    sc = S.Scene(name="facade_joints")
    S._timed_settings(sc, 10, 2)
    S._ground(sc, 0.6)
    hook = sc.add_shape(S.Shape(S.SHAPE_BOX, [0.1, 0.1, 0.1, 0.0]))
    link = sc.add_shape(S.Shape(S.SHAPE_BOX, [0.1, 0.25, 0.1, 0.0]))
    ball = sc.add_shape(S.Shape(S.SHAPE_SPHERE, [0.1, 0.0, 0.0, 0.0]))
    for ix in range(nx):
        for iz in range(nz):
            c = ix * nz + iz
            x, z = f((ix - (nx - 1) * 0.5) * 1.5), f((iz - (nz - 1) * 0.5) * 1.5)
            prev = sc.add_body(S.Body(hook, S.MOTION_STATIC, pos=(x, f(6.1), z)))
            anchor = (x, 6.0, z)
            for k in range(links):
                y = f(6.0 - 0.5 * k - 0.25)
                b = sc.add_body(S.Body(link, pos=(x, y, z), vel=(f(((c % 5) - 2) * 0.5 * (k + 1) / links), 0.0,
                                                                  f(((c % 3) - 1) * 0.7 * (k + 1) / links))))
                if k % 3 == 2:
                    sc.joints.append(S.Joint(S.JOINT_HINGE, prev, b, anchor_a=anchor, axis_a=(0.0, 0.0, 1.0),
                                             axis_b=(0.0, 0.0, 1.0), lower=-0.8, upper=0.8, flags=S.JOINT_FLAG_LIMITS))
                else:
                    sc.joints.append(S.Joint(S.JOINT_POINT, prev, b, anchor_a=anchor))
                prev, anchor = b, (x, f(y - 0.25), z)
    sc.add_body(S.Body(ball, pos=(-5.0, 5.75, 0.0), vel=(80.0, 0.0, 0.0),
                       flags=S.BODY_FLAG_ALLOW_SLEEPING | S.BODY_FLAG_LINEAR_CAST))
    return sc


def test_cpp_facade_joints_and_ccd_match_python_api(kzg_lib):
    """Joints (PointConstraint, HingeConstraint with limits) and a LinearCast body created through
    the C++ facade step to the same state hash as the same scene through the Python API."""
    import os
    import subprocess
    from kizuriphysics3d_gb300 import World, build
    exe = os.path.join(build.OUT, "joints_example")
    out = subprocess.run([exe, "3", "3", "6", "60"], capture_output=True, text=True, check=True).stdout
    cpp_hash = int(out.split("hash")[1].split()[0], 16)
    with World(_facade_joint_scene(3, 3, 6)) as w:
        w.step_fixed(n=60)
        assert w.compute_state_hash() == cpp_hash


def test_hash_identical_run_to_run(kzg_lib):
    from kizuriphysics3d_gb300 import World, resolve, scenes
    sc = scenes.pile(800, seed=5, extent=4.0, y_range=(1.0, 12.0))
    res = resolve(sc)
    hashes = []
    for _ in range(2):
        with World(sc, resolved=res) as w:
            w.step_fixed(n=120)
            hashes.append(w.compute_state_hash())
    assert hashes[0] == hashes[1]


def test_full_size_box_field_properties(kzg_lib):
    """400 stacks x 500 unit boxes (the large-box-field workload) at full size: exact pair count,
    no device error, nothing tunnels through the plane, run-to-run identical state."""
    from kizuriphysics3d_gb300 import World, resolve, scenes
    sc = scenes.stacks(20, 20, 500)
    res = resolve(sc)
    hashes = []
    for _ in range(2):
        with World(sc, resolved=res, max_pairs=4 * len(sc.bodies)) as w:
            w.step_fixed()
            st = w.get_stats()
            assert st["num_broadphase_pairs"] == 400 * 499 + 400
            w.step_fixed(n=4)
            st = w.get_stats()
            assert st["device_error"] == 0
            # stacks never merge; exactly touching boxes may lose their tight-AABB overlap by
            # rounding (BroadPhase.cpp:375 keeps only overlapping pairs), which splits a stack
            assert st["num_islands"] >= 400
            s = w.state()
            assert float(s[1:, 1].min()) > 0.4
            hashes.append(w.compute_state_hash())
    assert hashes[0] == hashes[1]


def test_pair_capacity_overflow_is_reported(kzg_lib):
    from kizuriphysics3d_gb300 import World, capi, scenes
    sc = scenes.pyramid(8)
    with World(sc, max_pairs=4) as w:  # 8 bottom boxes touch the plane at step 0
        with pytest.raises(capi.KzgError) as e:
            w.step_fixed()
        assert e.value.status == -3


def test_stale_pair_ids_are_skipped(kzg_lib):
    from kizuriphysics3d_gb300 import World, scenes
    sc = scenes.pyramid(3)
    with World(sc) as w:
        w.step_with_pairs(np.array([[0, 1], [0xFF000001, 2], [999, 3]], np.uint32))
        hdr, _, _ = w.contact_constraints()
        assert all(h[0] < len(sc.bodies) and h[1] < len(sc.bodies) for h in hdr)


def test_cpp_facade_matches_python_api(kzg_lib):
    """The C++ facade (include/kizuri_gpu/PhysicsWorld.h) and the Python API step the same scene to
    the same state hash."""
    import os
    import subprocess
    from kizuriphysics3d_gb300 import World, build, scenes
    exe = os.path.join(build.OUT, "pyramid_example")
    out = subprocess.run([exe, "8", "60"], capture_output=True, text=True, check=True).stdout
    cpp_hash = int(out.split("hash")[1].split()[0], 16)
    with World(scenes.pyramid(8)) as w:
        w.step_fixed(n=60)
        assert w.compute_state_hash() == cpp_hash


def test_cpp_facade_body_operations_match_python_api_and_oracle(oracle_lib, kzg_lib):
    """The facade's reference-named body operations (AddImpulseAtPoint, SetLinearVelocity, AddForce,
    SetBodyRotation, SetBodyActive) halfway through the pyramid run, against the same edits through
    the Python API and the oracle."""
    import os
    import subprocess
    from kizuriphysics3d_gb300 import World, build, capi, make_edit, resolve, scenes
    exe = os.path.join(build.OUT, "pyramid_example")
    out = subprocess.run([exe, "8", "60", "1"], capture_output=True, text=True, check=True).stdout
    cpp_hash = int(out.split("hash")[1].split()[0], 16)
    cpp_active = int(out.split("active")[1].split()[0])
    sc = scenes.pyramid(8)
    res = resolve(sc)
    ow = oracle_lib.OracleWorld(sc.to_bytes(), oracle_blob(sc, res), oracle_lib.PAIRS_CANONICAL)
    with World(sc, resolved=res) as w:
        for s in range(60):
            if s == 30:
                top = len(sc.bodies) - 1
                t = w.state()[top]
                e = np.concatenate([
                    make_edit(capi.EDIT_ADD_IMPULSE_AT_POINT, top, (3.0, 0.0, 0.0, t[0], np.float32(t[1] + np.float32(0.5)),
                                                                     np.float32(t[2] + np.float32(0.3)))),
                    make_edit(capi.EDIT_SET_LINEAR_VELOCITY, 1, (0.0, 2.0, 0.0)),
                    make_edit(capi.EDIT_ADD_FORCE, 1, (0.0, 150.0, 0.0)),
                    make_edit(capi.EDIT_SET_ROTATION, 2, (0.0, 0.2, 0.0, 1.0)),
                    make_edit(capi.EDIT_DEACTIVATE, 3, (), wake=False)])
                w.edit_bodies(e)
                ow.edit_bodies(e)
            w.step_fixed()
            ow.step(np.float32(sc.dt))
        assert np.array_equal(bits(w.state()), bits(ow.state()))
        assert w.compute_state_hash() == cpp_hash == ow.hash()
        assert len(w.active_bodies()) == cpp_active
