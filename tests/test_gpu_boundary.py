"""The C-ABI's settings boundary on the GPU: reference settings the accelerated path cannot honour
are rejected, settings the reference ignores are accepted, and the bounded in-kernel wait's
give-up path (a poll limit small enough to run out) completes the step with unchanged results."""
import os

import numpy as np
import pytest

from conftest import bits

pytestmark = pytest.mark.gpu

KZG_DEVERR_WAIT = 16


def test_simd_and_scalar_solvers_agree(kzg_lib):
    """World_SIMDMatchesScalar (reference tests/TestWorld.cpp:302-328): four unit boxes stacked with
    small offsets on the ground, two seconds, once per SolverSettings::useSIMDSolver value: the box
    positions agree within 0.05 m, while the bits differ (the two paths are different solvers)."""
    from kizuriphysics3d_gb300 import World, scenes

    def run(simd):
        sc = scenes.Scene(name="simd_vs_scalar", flags=scenes.WORLD_FLAG_ALLOW_SLEEPING)
        plane = sc.add_shape(scenes.Shape(scenes.SHAPE_PLANE, [0.0, 1.0, 0.0, 0.0]))
        sc.add_body(scenes.Body(plane, scenes.MOTION_STATIC, friction=0.8))
        box = sc.add_shape(scenes.Shape(scenes.SHAPE_BOX, [0.5, 0.5, 0.5, 0.0]))
        for i in range(4):
            sc.add_body(scenes.Body(box, pos=(scenes.f32(i * 0.05), scenes.f32(1.0 + i * 1.02), 0.0), friction=0.6))
        with World(sc) as w:
            w.set_solver(use_simd_solver=1 if simd else 0)
            w.step_fixed(n=int(2.0 / (1.0 / 60.0)))
            assert w.get_stats()["device_error"] == 0
            return w.state()[1:, 0:3].copy()

    a, b = run(False), run(True)
    assert np.all(np.linalg.norm(a.astype(np.float64) - b, axis=1) <= 0.05)
    assert not np.array_equal(bits(a), bits(b))


def test_split_impulse_flag_changes_nothing(kzg_lib):
    """SolverSettings::useSplitImpulse is read nowhere by the reference (ContactSolver.h:75): both
    values give identical bits."""
    from kizuriphysics3d_gb300 import World, scenes
    sc = scenes.pyramid(8)
    with World(sc) as a, World(sc) as b:
        a.set_solver(use_split_impulse=1)
        b.set_solver(use_split_impulse=0)
        a.step_fixed(n=60)
        b.step_fixed(n=60)
        assert np.array_equal(bits(a.state()), bits(b.state()))


def _settled_pile():
    from kizuriphysics3d_gb300 import resolve, scenes
    snap = os.path.join(os.path.dirname(__file__), "..", "kizuriphysics3d_gb300", "data", "pile20000_step600.npz")
    sc = scenes.pile(20000, seed=1234)
    with np.load(snap) as z:
        state = z["state"]
    for b, st in zip(sc.bodies, state):
        b.pos, b.rot, b.vel, b.ang = tuple(st[0:3]), tuple(st[3:7]), tuple(st[7:10]), tuple(st[10:13])
    return sc, resolve(sc)


def test_wait_that_runs_out_completes_the_step(kzg_lib):
    """The settled 20,000-body pile's giant island streams its velocity level sweep behind the first
    fit (the one in-kernel wait).  With a poll limit of 1 the wait runs out: KZG_DEVERR_WAIT is
    reported in the stats, the step still returns KZG_OK, its result is bit-identical to the
    default limit's, and the next step with the default limit runs clean."""
    from kizuriphysics3d_gb300 import World
    sc, res = _settled_pile()
    with World(sc, resolved=res, max_pairs=48 * len(sc.bodies)) as short, \
            World(sc, resolved=res, max_pairs=48 * len(sc.bodies)) as normal:
        short.set_wait_limit(1)
        short.step_fixed()  # raises on any status but KZG_OK
        normal.step_fixed()
        st = short.get_stats()
        assert st["device_error"] & KZG_DEVERR_WAIT
        assert st["device_error"] & ~KZG_DEVERR_WAIT == 0
        assert normal.get_stats()["device_error"] == 0
        assert np.array_equal(bits(short.state()), bits(normal.state()))
        short.set_wait_limit(0)  # back to the default
        short.step_fixed()
        normal.step_fixed()
        assert short.get_stats()["device_error"] == 0
        assert short.compute_state_hash() == normal.compute_state_hash()


def test_host_transfers_through_staging(kzg_lib):
    """kzg_download_transforms equals the position and rotation columns of the state, and forces
    uploaded from a host array act exactly as the same forces added through AddForce / AddTorque
    (a twin world), for a range that starts past slot 0."""
    from kizuriphysics3d_gb300 import World, capi, make_edit, scenes
    sc = scenes.pile(300, seed=31, extent=3.0, y_range=(1.0, 10.0))
    with World(sc) as a, World(sc) as b:
        a.step_fixed(n=5)
        b.step_fixed(n=5)
        tr = a.transforms()
        st = a.state()
        assert np.array_equal(bits(tr[:, 0:3]), bits(st[:, 0:3])) and np.array_equal(bits(tr[:, 3:7]), bits(st[:, 3:7]))
        rng = np.random.default_rng(5)
        ft = np.zeros((a.n, 6), np.float32)
        ft[1:] = rng.normal(0.0, 50.0, (a.n - 1, 6)).astype(np.float32)
        ft[1::7] = 0.0
        a.upload_forces(ft)
        edits = np.concatenate([np.concatenate([make_edit(capi.EDIT_ADD_FORCE, i, ft[i, 0:3], wake=False),
                                                make_edit(capi.EDIT_ADD_TORQUE, i, ft[i, 3:6], wake=False)])
                                for i in range(1, a.n)])
        b.edit_bodies(edits)
        a.step_fixed()
        b.step_fixed()
        assert np.array_equal(bits(a.state()), bits(b.state()))
