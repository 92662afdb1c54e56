"""Generate the golden fixtures in tests/golden/ from the reference engine itself.

Runs only where the reference sources exist (this script builds oracle/_ref/ref_trace from them
with oracle/Makefile.ref).  For every fixture scene it records what the unmodified reference
computed: the ComputeStateHash value after every step, the full body state at checkpoint steps,
the broad-phase pair list and contact constraints of the first steps, WorldStats counters, the
resolved mass properties and every hull as built by ConvexHullShape::Create.

    python tests/golden/gen_golden.py --ref <reference checkout> [--only NAME ...]

(--ref defaults to the KIZURI_REFERENCE environment variable.)
"""
from __future__ import annotations

import argparse
import math
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from kizuriphysics3d_gb300 import scenes  # noqa: E402
from oracle import trace as T  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def fixture_scenes():
    """name -> (scene, steps, detail steps, checkpoint steps)."""
    out = {}
    out["pyramid20"] = (scenes.pyramid(20), 600, 2, [0, 1, 2, 9, 59, 119, 299, 599])
    out["pile200"] = (scenes.pile(200, seed=1234, extent=3.0, y_range=(2.0, 12.0)), 600, 2, [0, 1, 59, 299, 599])
    out["stacks2x2x20"] = (scenes.stacks(2, 2, 20), 300, 2, [0, 1, 59, 299])
    out["pile64_nows"] = (_nows(scenes.pile(64, seed=77, extent=1.5, y_range=(1.0, 5.0))), 240, 2, [0, 59, 239])
    out["pyramid4_tests"] = (_reference_test_pyramid(), 240, 2, [0, 239])
    out["ccd_shots"] = (_ccd_shots(), 120, 2, [0, 1, 29, 59, 119])
    out["joints_mix"] = (_joints_mix(), 180, 2, [0, 1, 59, 179])
    out["ccd_threshold"] = (_ccd_threshold(), 90, 2, [0, 1, 29, 89])
    out["joints_single"] = (_joints_single(), 60, 2, list(range(60)))
    out["sleep_wake"] = (_sleep_wake(), 600, 2, [0, 59, 119, 239, 359, 479, 599])
    out["pile120_sleep"] = (_sleeping(scenes.pile(120, seed=55, extent=2.5, y_range=(1.0, 8.0)), "pile120_sleep"),
                            480, 2, [0, 119, 239, 479])
    out["pyramid20_scalar"] = (_scalar(scenes.pyramid(20), "pyramid20_scalar"), 300, 2, [0, 1, 59, 299])
    out["pile200_scalar"] = (_scalar(scenes.pile(200, seed=1234, extent=3.0, y_range=(2.0, 12.0)), "pile200_scalar"),
                             300, 2, [0, 1, 59, 299])
    out["edits_sleep"] = (_edits_sleep_scene(), 480, 2, [0, 20, 45, 199, 200, 299, 479])
    out["edits_nosleep"] = (_edits_nosleep_scene(), 240, 2, [0, 40, 41, 119, 120, 239])
    return out


# Body operations between steps (PhysicsWorld.cpp:109-205), applied by the reference through its own
# methods: name -> list of (step, op, slot, wake, operands, stale).  Op numbers are kzg_body_edit's.
(E_POS, E_ROT, E_XFORM, E_LINV, E_ANGV, E_FORCE, E_FORCE_AT, E_TORQUE, E_IMP, E_IMP_AT, E_ACT, E_DEACT) = range(12)
EDIT_DTYPE = np.dtype([("step", "<u4"), ("op", "<u4"), ("slot", "<u4"), ("wake", "<u4"), ("v", "<f4", (8,))])


def edit_schedules():
    """Fixture name -> its edit records (EDIT_DTYPE; slot bit 31: a stale BodyID of that slot)."""
    f = scenes.f32
    top_y = f(0.5 + 2 * 1.02)
    sleep = [  # edits_sleep: slots 1-6 pyramid, 7-9 stack, 10-13 spheres, 14 box, 15 kinematic, 16 capsule
        (20, E_IMP_AT, 6, 1, (2.0, 0.0, 0.0, 0.0, f(top_y + 0.5), 0.3)),
        (20, E_LINV, 10, 1, (0.0, 4.0, 0.0)),
        (20, E_FORCE, 7, 1, (0.0, 900.0, 0.0)),
        (20, E_TORQUE, 8, 1, (0.0, 30.0, 0.0)),
        (20, E_IMP, 0, 1, (1.0, 0.0, 0.0)),  # static ground: Apply* ignores it, wake keeps it active
        (45, E_ROT, 14, 1, (0.0, 0.5, 0.0, 1.0)),  # not normalised: SetBodyRotation normalises
        (45, E_POS, 11, 0, (-5.5, 3.0, 4.0)),
        (45, E_ANGV, 16, 1, (0.0, 3.0, 0.0)),
        (45, E_FORCE_AT, 16, 1, (0.0, 0.0, 200.0, -3.7, 0.2, 4.0)),
        (200, E_DEACT, 12, 0, ()),
        (200, E_IMP, 13, 0, (0.0, 0.0, 3.0)),  # on a body that may be asleep, without waking it
        (200, E_XFORM, 2, 1, (f(1.02), f(0.7), 0.0, 0.0, 0.0, 0.0998, 0.995)),
        (200, E_ACT, 0, 0, ()),  # ActivateBody on a static body: it joins the active list
        (260, E_LINV, 15, 1, (1.0, 0.0, 0.0)),  # kinematic pusher towards the stack
        (300, E_DEACT, 15, 0, ()),  # a deactivated kinematic body stops (velocities zeroed)
        (340, E_LINV, 14, 1, (0.0, 10.0, 0.0), True),  # stale id: skipped
        (340, E_ACT, 15, 0, ()),
        (340, E_LINV, 15, 1, (-1.0, 0.0, 0.0)),
        (400, E_FORCE, 9, 1, (0.0, 2000.0, 0.0)),
    ]
    nosleep = [  # edits_nosleep: 80-body pile, sleeping off; deactivated bodies wait until touched
        (40, E_DEACT, 5, 0, ()),
        (40, E_DEACT, 17, 0, ()),
        (40, E_DEACT, 33, 0, ()),
        (40, E_DEACT, 50, 0, ()),
        (40, E_LINV, 60, 0, (0.0, 6.0, 0.0)),
        (120, E_DEACT, 71, 0, ()),
        (120, E_IMP_AT, 8, 1, (0.0, 3.0, 0.0, 0.0, 0.0, 0.0)),
        (120, E_ACT, 17, 0, ()),
        (120, E_XFORM, 40, 1, (0.0, 6.0, 0.0, 0.0, 0.0, 0.0, 1.0)),  # dropped onto the pile again
    ]
    out = {}
    for name, lst in (("edits_sleep", sleep), ("edits_nosleep", nosleep)):
        e = np.zeros(len(lst), EDIT_DTYPE)
        for k, rec in enumerate(lst):
            step, op, slot, wake, vals = rec[:5]
            stale = len(rec) > 5 and rec[5]
            e[k]["step"], e[k]["op"], e[k]["wake"] = step, op, wake
            e[k]["slot"] = slot | (0x80000000 if stale else 0)
            e[k]["v"][:len(vals)] = np.asarray(vals, np.float32)
        out[name] = e
    return out


def _edits_sleep_scene():
    """Sleeping on; a 3-row pyramid, a 3-box stack, four spheres, a free box, a kinematic box and a
    capsule, poked by the edit schedule while they fall asleep and wake."""
    S = scenes
    f = S.f32
    sc = S.Scene(name="edits_sleep")
    S._timed_settings(sc, 10, 2)
    sc.flags |= S.WORLD_FLAG_ALLOW_SLEEPING
    S._ground(sc, 0.6)
    box = sc.add_shape(S.Shape(S.SHAPE_BOX, [0.5, 0.5, 0.5, 0.0]))
    ball = sc.add_shape(S.Shape(S.SHAPE_SPHERE, [0.3, 0.0, 0.0, 0.0]))
    cap = sc.add_shape(S.Shape(S.SHAPE_CAPSULE, [0.3, 0.2, 0.0, 0.0]))
    for r in range(3):
        n = 3 - r
        for i in range(n):
            sc.add_body(S.Body(box, pos=(f((i - (n - 1) * 0.5) * 1.02), f(0.5 + r * 1.02), 0.0), friction=0.6))
    for k in range(3):
        sc.add_body(S.Body(box, pos=(6.0, f(0.5 + 1.01 * k), -4.0), friction=0.6))
    for k in range(4):
        sc.add_body(S.Body(ball, pos=(f(-6.0 + 0.61 * k), 0.3, 4.0), friction=0.6))
    sc.add_body(S.Body(box, pos=(-6.0, 0.5, -3.0), friction=0.6))
    sc.add_body(S.Body(box, S.MOTION_KINEMATIC, pos=(3.0, 0.6, -4.0)))
    sc.add_body(S.Body(cap, pos=(-4.0, 0.2, 4.0), rot=(0.0, 0.0, f(0.7071068), f(0.7071068)), friction=0.6))
    return sc


def _edits_nosleep_scene():
    sc = scenes.pile(80, seed=909, extent=2.0, y_range=(1.0, 6.0))
    sc.name = "edits_nosleep"
    return sc


def kzp1_fixtures():
    """Fixture scene -> step count after which the reference saves the world as KZP1."""
    return {"pile200": 0, "sleep_wake": 300, "ccd_threshold": 30}


def _scalar(sc, name):
    """SolverSettings::useSIMDSolver = false: velocity iterations over the constraints in order with
    the scalar SolveContactVelocity (PhysicsWorld.cpp:723-727, ContactSolver.cpp:136-181)."""
    sc.flags |= scenes.WORLD_FLAG_SCALAR_SOLVER
    sc.name = name
    return sc


def _sleeping(sc, name):
    sc.flags |= scenes.WORLD_FLAG_ALLOW_SLEEPING
    sc.name = name
    return sc


def _sleep_wake():
    """Sleeping on (WorldSettings::allowSleeping, UpdateSleeping PhysicsWorld.cpp:866-951): small
    structures settle and fall asleep, then are woken - a box dropped onto a sleeping pyramid, a
    kinematic box pushing into a sleeping stack (a moving kinematic body wakes what it touches,
    :473-490), a sphere dropped into sleeping spheres - beside a body that may not sleep."""
    S = scenes
    sc = S.Scene(name="sleep_wake")
    S._timed_settings(sc, 10, 2)
    sc.flags |= S.WORLD_FLAG_ALLOW_SLEEPING
    S._ground(sc, 0.6)
    box = sc.add_shape(S.Shape(S.SHAPE_BOX, [0.5, 0.5, 0.5, 0.0]))
    small = sc.add_shape(S.Shape(S.SHAPE_BOX, [0.3, 0.3, 0.3, 0.0]))
    ball = sc.add_shape(S.Shape(S.SHAPE_SPHERE, [0.3, 0.0, 0.0, 0.0]))
    f = S.f32
    for r in range(4):  # 4-row pyramid (the World_PyramidRest layout)
        n = 4 - r
        for i in range(n):
            sc.add_body(S.Body(box, pos=(f((i - (n - 1) * 0.5) * 1.02), f(0.5 + r * 1.02), 0.0), friction=0.6))
    for k in range(3):  # a stack
        sc.add_body(S.Body(box, pos=(8.0, f(0.5 + 1.01 * k), 0.0), friction=0.6))
    for k in range(5):  # loose spheres in a row
        sc.add_body(S.Body(ball, pos=(f(-6.0 + 0.61 * k), 0.3, 4.0), friction=0.6))
    sc.add_body(S.Body(small, pos=(3.0, 0.3, 4.0), friction=0.6, flags=0))  # may not sleep
    sc.add_body(S.Body(small, pos=(0.05, 22.0, 0.1), friction=0.6))  # lands on the pyramid at ~2.1 s
    sc.add_body(S.Body(ball, pos=(-4.8, 45.0, 4.0), friction=0.6))  # lands among the spheres at ~3 s
    # kinematic pusher: reaches the stack after ~4 s
    sc.add_body(S.Body(small, S.MOTION_KINEMATIC, pos=(4.0, 0.6, 0.0), vel=(0.8, 0.0, 0.0)))
    return sc


def _joints_single(copies: int = 8):
    """Single-joint systems of every joint type (Constraints.h:41-277), `copies` of each with seeded
    initial motions: a body on a point joint, a hinge door with limits and a motor, a slider with
    limits and a six-dof joint hang from static posts; fixed and distance pairs tumble in free
    flight.  Dynamic bodies collide with the ground layer only and stay clear of it for 60 steps,
    so no contact appears or vanishes.  Single-joint systems are well conditioned: a one-rounding-
    step difference in a joint's trigonometry stays a small perturbation, which makes this the
    scene on which per-step velocities are compared with the reference at 1e-4 relative."""
    S = scenes
    sc = S.Scene(name="joints_single")
    S._timed_settings(sc, 10, 2)
    S._ground(sc, 0.6)
    post = sc.add_shape(S.Shape(S.SHAPE_BOX, [0.1, 0.1, 0.1, 0.0]))
    cube = sc.add_shape(S.Shape(S.SHAPE_BOX, [0.3, 0.2, 0.25, 0.0]))
    door = sc.add_shape(S.Shape(S.SHAPE_BOX, [0.5, 0.8, 0.05, 0.0]))
    ball = sc.add_shape(S.Shape(S.SHAPE_SPHERE, [0.25, 0.0, 0.0, 0.0]))
    st = S.MOTION_STATIC
    f = scenes.f32
    rng = np.random.default_rng(2024)
    J = []

    def dyn(shape, pos, vel=(0.0, 0.0, 0.0), ang=(0.0, 0.0, 0.0)):
        return sc.add_body(S.Body(shape, pos=tuple(f(x) for x in pos), vel=tuple(f(x) for x in vel),
                                  ang=tuple(f(x) for x in ang), layer=2, mask=1))

    def fixed_post(pos):
        return sc.add_body(S.Body(post, st, pos=pos, layer=4))

    for k in range(copies):
        z = 3.0 * k
        r = rng.uniform(-1.0, 1.0, 12)
        p = fixed_post((0.0, 8.0, z))  # pendulum on a point joint, swinging in 3-D
        b = dyn(cube, (0.9, 7.5, z + 0.2), vel=(0.0, 0.0, 1.2 * r[0]), ang=(0.3 * r[1], 0.0, 0.4 * r[2]))
        J.append(S.Joint(S.JOINT_POINT, p, b, anchor_a=(0.0, 8.0, z)))
        p = fixed_post((4.0, 8.0, z))  # hinge door with limits and a motor
        b = dyn(door, (4.6, 8.0, z), ang=(0.0, 1.5 * r[3], 0.0))
        J.append(S.Joint(S.JOINT_HINGE, p, b, anchor_a=(4.1, 8.0, z), axis_a=(0.0, 1.0, 0.0),
                         axis_b=(0.0, 1.0, 0.0), lower=-1.0, upper=1.0, motor_target=f(2.0 * r[4]), motor_max=5.0,
                         flags=S.JOINT_FLAG_LIMITS | S.JOINT_FLAG_MOTOR))
        p = fixed_post((8.0, 8.0, z))  # slider with limits along a tilted axis
        b = dyn(cube, (8.5, 8.0, z), vel=(0.5 * r[5], 0.0, 0.0))
        J.append(S.Joint(S.JOINT_SLIDER, p, b, anchor_a=(8.5, 8.0, z), axis_a=(0.8, -0.6, 0.0), lower=-0.6,
                         upper=0.9, flags=S.JOINT_FLAG_LIMITS))
        p = fixed_post((12.0, 8.0, z))  # six-dof: fixed, limited and motorised axes
        b = dyn(cube, (12.0, 8.0, z + 0.6), ang=(0.5 * r[6], 1.0 * r[7], 0.0))
        c, s_ = math.cos(0.3), math.sin(0.3)
        J.append(S.Joint(S.JOINT_SIXDOF, p, b, anchor_a=(12.0, 8.0, z + 0.6), rotation=(0.0, s_, 0.0, c),
                         axis_modes=(2 << 0) | (2 << 2) | (1 << 4) | (2 << 6), motor_mask=(1 << 2) | (1 << 4),
                         six_motor=(0.0, 0.0, 0.5, 0.0, 0.0, 3.0, 0.0, 1.5, 0.0, 0.0, 2.0, 0.0)))
        f1 = dyn(cube, (16.0, 9.0, z), vel=(0.0, 2.0, 0.0), ang=(0.3 * r[8], 0.0, 0.2))  # fixed pair, tumbling
        f2 = dyn(cube, (16.62, 9.1, z), vel=(0.0, 2.0, 0.0))
        J.append(S.Joint(S.JOINT_FIXED, f1, f2, anchor_a=(16.31, 9.05, z)))
        d1 = dyn(ball, (20.0, 9.0, z), vel=(0.0, 3.0, 1.0 * r[9]))  # distance pair, tumbling
        d2 = dyn(ball, (21.0, 9.5, z), vel=(0.0, 1.0, -1.0), ang=(0.0, 2.0 * r[10], 0.0))
        J.append(S.Joint(S.JOINT_DISTANCE, d1, d2, anchor_a=(20.0, 9.0, z), anchor_b=(21.0, 9.5, z), distance=1.2))
    sc.joints = J
    return sc


def _ccd_threshold():
    """The CCD shots with BodySettings::ccdMotionThreshold (Body.h:70) set on every other
    LinearCast body, between the shortest and longest step displacement of the shots: bodies moving
    less than their threshold in a step are not clamped (PhysicsWorld.cpp:807) and may tunnel."""
    sc = _ccd_shots()
    sc.name = "ccd_threshold"
    k = 0
    for b in sc.bodies:
        if b.flags & scenes.BODY_FLAG_LINEAR_CAST:
            if k % 2:
                b.ccd_motion_threshold = 0.7
            k += 1
    return sc


def _joints_mix():
    """Every joint type (Constraints.h:41-277) beside contacts: a point-joint chain hanging from
    a static post, a motorised hinge door with limits, sliders with limits and with a motor, a
    fixed pair and a distance pair falling onto the ground (contacts and joints in one island), a
    six-dof joint with fixed, limited and motorised axes, and a disabled joint."""
    S = scenes
    sc = S.Scene(name="joints_mix")
    S._timed_settings(sc, 10, 2)
    S._ground(sc, 0.6)
    post = sc.add_shape(S.Shape(S.SHAPE_BOX, [0.1, 2.0, 0.1, 0.0]))
    link = sc.add_shape(S.Shape(S.SHAPE_BOX, [0.1, 0.25, 0.1, 0.0]))
    door = sc.add_shape(S.Shape(S.SHAPE_BOX, [0.5, 0.8, 0.05, 0.0]))
    cube = sc.add_shape(S.Shape(S.SHAPE_BOX, [0.3, 0.3, 0.3, 0.0]))
    ball = sc.add_shape(S.Shape(S.SHAPE_SPHERE, [0.25, 0.0, 0.0, 0.0]))
    cap = sc.add_shape(S.Shape(S.SHAPE_CAPSULE, [0.3, 0.15, 0.0, 0.0]))
    st = S.MOTION_STATIC
    J = []
    # chain: static post at x=0 (top at y=4), 6 links hanging beside it from x=0.4, swinging
    p0 = sc.add_body(S.Body(post, st, pos=(0.0, 2.0, 0.0)))
    prev, anchor = p0, (0.4, 4.0, 0.0)
    for k in range(6):
        y = 4.0 - 0.5 * k - 0.25
        b = sc.add_body(S.Body(link, pos=(0.4, y, 0.0), vel=(1.5 if k == 5 else 0.0, 0.0, 0.5)))
        J.append(S.Joint(S.JOINT_POINT, prev, b, anchor_a=anchor))
        prev, anchor = b, (0.4, y - 0.25, 0.0)
    # hinge door on a second post, limited to +-1 rad, motor driving it
    p1 = sc.add_body(S.Body(post, st, pos=(3.0, 2.0, 0.0)))
    d = sc.add_body(S.Body(door, pos=(3.6, 2.0, 0.0)))
    J.append(S.Joint(S.JOINT_HINGE, p1, d, anchor_a=(3.1, 2.0, 0.0), axis_a=(0.0, 1.0, 0.0), axis_b=(0.0, 1.0, 0.0),
                     lower=-1.0, upper=1.0, motor_target=2.0, motor_max=5.0,
                     flags=S.JOINT_FLAG_LIMITS | S.JOINT_FLAG_MOTOR))
    # second door: limits only, pushed
    p2 = sc.add_body(S.Body(post, st, pos=(-3.0, 2.0, 0.0)))
    d2 = sc.add_body(S.Body(door, pos=(-2.4, 2.0, 0.0), ang=(0.0, 3.0, 0.0)))
    J.append(S.Joint(S.JOINT_HINGE, p2, d2, anchor_a=(-2.9, 2.0, 0.0), axis_a=(0.0, 1.0, 0.0),
                     axis_b=(0.0, 1.0, 0.0), lower=-0.5, upper=0.5, flags=S.JOINT_FLAG_LIMITS))
    # sliders along x from a static post: one limited, one motorised
    p3 = sc.add_body(S.Body(post, st, pos=(0.0, 2.0, 3.0)))
    s1 = sc.add_body(S.Body(cube, pos=(0.8, 3.0, 3.0), vel=(2.0, 0.0, 0.0)))
    J.append(S.Joint(S.JOINT_SLIDER, p3, s1, anchor_a=(0.8, 3.0, 3.0), axis_a=(1.0, 0.0, 0.0), lower=-0.5,
                     upper=0.6, flags=S.JOINT_FLAG_LIMITS))
    s2 = sc.add_body(S.Body(cube, pos=(-0.8, 1.5, 3.0)))
    J.append(S.Joint(S.JOINT_SLIDER, p3, s2, anchor_a=(-0.8, 1.5, 3.0), axis_a=(-1.0, 0.2, 0.0), motor_target=1.0,
                     motor_max=20.0, flags=S.JOINT_FLAG_MOTOR))
    # fixed pair and distance pair dropped onto the ground
    f1 = sc.add_body(S.Body(cube, pos=(5.0, 1.5, 3.0), ang=(0.3, 0.0, 0.2)))
    f2 = sc.add_body(S.Body(cube, pos=(5.62, 1.6, 3.0)))
    J.append(S.Joint(S.JOINT_FIXED, f1, f2, anchor_a=(5.31, 1.55, 3.0)))
    b1 = sc.add_body(S.Body(ball, pos=(-5.0, 2.0, 3.0), vel=(0.0, 0.0, 1.0)))
    b2 = sc.add_body(S.Body(cap, pos=(-4.0, 2.5, 3.0)))
    J.append(S.Joint(S.JOINT_DISTANCE, b1, b2, anchor_a=(-5.0, 2.0, 3.0), anchor_b=(-4.0, 2.5, 3.0), distance=1.2))
    # point joint with local anchors between a cube and the second chain link
    c3 = sc.add_body(S.Body(cube, pos=(1.3, 3.2, -0.2)))
    J.append(S.Joint(S.JOINT_POINT, 3, c3, anchor_a=(0.1, 0.0, 0.0), anchor_b=(-0.4, 0.0, 0.0),
                     flags=S.JOINT_FLAG_LOCAL_ANCHORS))
    # six-dof: linear x,y fixed, z limited, angular x fixed; linear z motor, angular y motor
    p4 = sc.add_body(S.Body(post, st, pos=(3.0, 2.0, -3.0)))
    x6 = sc.add_body(S.Body(cube, pos=(3.0, 3.0, -2.4), ang=(0.5, 1.0, 0.0)))
    c, s_ = math.cos(0.3), math.sin(0.3)
    J.append(S.Joint(S.JOINT_SIXDOF, p4, x6, anchor_a=(3.0, 3.0, -2.4), rotation=(0.0, s_, 0.0, c),
                     axis_modes=(2 << 0) | (2 << 2) | (1 << 4) | (2 << 6), motor_mask=(1 << 2) | (1 << 4),
                     six_motor=(0.0, 0.0, 0.5, 0.0, 0.0, 3.0, 0.0, 1.5, 0.0, 0.0, 2.0, 0.0)))
    # a disabled joint (never prepared, solved or islanded)
    J.append(S.Joint(S.JOINT_POINT, f1, b1, anchor_a=(0.0, 1.0, 3.0), flags=S.JOINT_FLAG_DISABLED))
    sc.joints = J
    return sc


def _ccd_shots():
    """Continuous collision (PhysicsWorld.cpp:804-852): small LinearCast spheres and boxes fired
    down at a thin static slab and sideways at a static wall fast enough to pass through them in
    one step, beside a few discrete boxes; ground plane below."""
    import numpy as np
    sc = scenes.Scene(name="ccd_shots")
    scenes._timed_settings(sc, 10, 2)
    scenes._ground(sc, 0.5)
    slab = sc.add_shape(scenes.Shape(scenes.SHAPE_BOX, [3.0, 0.05, 3.0, 0.0]))
    wall = sc.add_shape(scenes.Shape(scenes.SHAPE_BOX, [0.05, 2.0, 3.0, 0.0]))
    ball = sc.add_shape(scenes.Shape(scenes.SHAPE_SPHERE, [0.1, 0.0, 0.0, 0.0]))
    cube = sc.add_shape(scenes.Shape(scenes.SHAPE_BOX, [0.12, 0.12, 0.12, 0.0]))
    big = sc.add_shape(scenes.Shape(scenes.SHAPE_BOX, [0.4, 0.4, 0.4, 0.0]))
    f = scenes.f32
    sc.add_body(scenes.Body(slab, scenes.MOTION_STATIC, pos=(0.0, 3.0, 0.0)))
    sc.add_body(scenes.Body(wall, scenes.MOTION_STATIC, pos=(6.0, 2.0, 0.0)))
    rng = np.random.default_rng(31)
    lc = scenes.BODY_FLAG_ALLOW_SLEEPING | scenes.BODY_FLAG_LINEAR_CAST
    for k in range(12):  # dropped through the slab
        x, z = rng.uniform(-2.5, 2.5, 2)
        vy = -f(rng.uniform(25.0, 45.0))
        sc.add_body(scenes.Body(ball if k % 2 else cube, pos=(f(x), f(rng.uniform(4.0, 6.0)), f(z)),
                                vel=(0.0, vy, 0.0), flags=lc))
    for k in range(8):  # fired at the wall
        y, z = rng.uniform(0.4, 3.5), rng.uniform(-2.5, 2.5)
        vx = f(rng.uniform(30.0, 60.0))
        sc.add_body(scenes.Body(cube if k % 2 else ball, pos=(f(rng.uniform(1.0, 3.0)), f(y), f(z)),
                                vel=(vx, 0.0, 0.0), flags=lc))
    for k in range(6):  # discrete boxes resting and falling
        sc.add_body(scenes.Body(big, pos=(f(-4.0 + 1.1 * k), f(0.4 + 0.9 * (k % 2)), f(-4.0))))
    return sc


def _nows(sc):
    sc.flags |= scenes.WORLD_FLAG_NO_WARM_START
    sc.name += "_nows"
    return sc


def _reference_test_pyramid():
    """World_PyramidRest (tests/TestWorld.cpp:103-128) with the reference test's materials and the
    reference default solver settings (16 velocity / 6 position iterations)."""
    sc = scenes.pyramid(4, friction=0.6, vel_iters=16, pos_iters=6)
    sc.bodies[0].friction = 0.8  # AddGround uses friction 0.8 (TestWorld.cpp:16)
    sc.name = "pyramid4_tests"
    return sc


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("KIZURI_REFERENCE"),
                    help="the reference's source checkout (default: $KIZURI_REFERENCE)")
    ap.add_argument("--only", nargs="*", default=None, help="fixture names to (re)generate (default: all)")
    args = ap.parse_args()
    if not args.ref:
        ap.error("give --ref or set KIZURI_REFERENCE to the reference's source checkout")
    subprocess.run(["make", "-s", "-f", os.path.join(ROOT, "oracle", "Makefile.ref"), f"REF={args.ref}", "-j8"],
                   check=True)
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_trace")
    with tempfile.TemporaryDirectory() as td:
        for name, (sc, steps, detail, ckpt) in fixture_scenes().items():
            if args.only and name not in args.only:
                continue
            sp = os.path.join(td, name + ".kzsc")
            tp = os.path.join(td, name + ".kztr")
            sc.save(sp)
            cmd = [exe, sp, tp, str(steps), str(detail)]
            edits = edit_schedules().get(name)
            if edits is not None:
                ep = os.path.join(td, name + ".edits")
                with open(ep, "wb") as fh:
                    fh.write(np.uint32(len(edits)).tobytes() + edits.tobytes())
                cmd += ["--edits", ep]
            subprocess.run(cmd, check=True)
            tr = T.read_trace(tp)
            fx = dict(hashes=tr.hashes, stats=tr.stats, packed=tr.packed, inv_mass=tr.inv_mass,
                      inv_inertia_local=tr.inv_inertia_local, inv_inertia_world=tr.inv_inertia_world,
                      state0=tr.state0, ckpt_steps=np.array(ckpt, np.int32),
                      ckpt_states=np.stack([tr.states[s] for s in ckpt]))
            if edits is not None:
                fx["edits"] = edits
            for si, hull in tr.hulls.items():
                fx[f"hull{si}_verts"] = hull.verts
                fx[f"hull{si}_sizes"] = hull.sizes
                fx[f"hull{si}_idx"] = hull.idx
            for d, det in enumerate(tr.detail):
                fx[f"d{d}_pairs"] = det.pairs
                fx[f"d{d}_con_hdr"] = det.con_hdr
                fx[f"d{d}_con_fr"] = det.con_fr
                fx[f"d{d}_con_pts"] = det.con_pts
            np.savez_compressed(os.path.join(HERE, name + ".npz"), **fx)
            print(f"{name}: {steps} steps, final hash {int(tr.hashes[-1]):016x}")
        for name, nsteps in kzp1_fixtures().items():  # worlds saved by the reference's SerializeWorld
            if args.only and name not in args.only:
                continue
            sc = fixture_scenes()[name][0]
            sp, tp = os.path.join(td, name + ".kzsc"), os.path.join(td, name + ".kztr")
            sc.save(sp)
            out = os.path.join(HERE, f"{name}_step{nsteps}.kzp1")
            subprocess.run([exe, sp, tp, str(nsteps), "0", "--kzp1", out], check=True)
            print(f"{out}: written by the reference after {nsteps} steps")


if __name__ == "__main__":
    main()
