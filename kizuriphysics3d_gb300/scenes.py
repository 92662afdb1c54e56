"""Seeded scene definitions and the binary scene format shared by every consumer.

A scene is the full input of a simulation: world/solver settings, a shape table and
a body list in creation order.  The same scene bytes feed

* the GPU world (``kizuriphysics3d_gb300.World.from_scene``),
* the CPU oracle (``oracle/``), and
* the reference trace tool built from the reference's own sources (``oracle/ref_trace.cpp``),

so that all three simulate bit-identical inputs.  Random draws use numpy's legacy
``RandomState`` (MT19937, stream-stable across numpy versions and platforms); every
value is computed in float64 and rounded once to float32, exactly like the
reference's ``Real(...)`` conversions of double expressions.

Layouts follow the configurations the reference is benchmarked on:

* ``pyramid`` - the ``World_PyramidRest`` layout (tests/TestWorld.cpp:108-119) scaled to
  ``rows`` rows; 20 rows = 210 unit boxes.
* ``pile`` - random convex pile: sphere / box / capsule / 16-point hull by ``i % 4``,
  uniform SO(3) orientation (Shoemake), positions in [-X,X]x[2,Ymax]x[-X,X].
* ``stacks`` - ``nx*nz`` stacks of ``height`` unit boxes on a 2 m grid with seeded
  lateral jitter.

Shape parameters follow the reference constructors (include/Kizuri/Geometry/Shape.h):
sphere (radius), box (half extents), capsule (halfHeight, radius) - note the argument
order of ``CapsuleShape(halfHeight, radius)`` at Shape.h:206 - plane (normal, distance)
and hull (input point cloud, hull built by ``ConvexHullShape::Create`` semantics).
"""
from __future__ import annotations

import math
import struct
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

# ShapeType numbering of include/Kizuri/Geometry/Shape.h:13-25.
SHAPE_SPHERE = 0
SHAPE_BOX = 1
SHAPE_CAPSULE = 2
SHAPE_HULL = 4
SHAPE_PLANE = 8

# MotionType numbering of include/Kizuri/Body/Body.h:37-41.
MOTION_STATIC = 0
MOTION_KINEMATIC = 1
MOTION_DYNAMIC = 2

BODY_FLAG_SENSOR = 1
BODY_FLAG_ALLOW_SLEEPING = 2
BODY_FLAG_LINEAR_CAST = 4   # MotionQuality::LinearCast: continuous collision clamps the motion (Body.h:46-67)

WORLD_FLAG_ALLOW_SLEEPING = 1
WORLD_FLAG_VELOCITY_BIAS = 2
WORLD_FLAG_NO_WARM_START = 4   # the reference's KZ_NOWS environment switch (PhysicsWorld.cpp:493)
WORLD_FLAG_SCALAR_SOLVER = 8   # SolverSettings::useSIMDSolver = false (ContactSolver.h:77)

SCENE_MAGIC = 0x4353_5A4B  # 'KZSC'
SCENE_VERSION = 2  # 2 adds the world's sleep thresholds and each body's CCD motion threshold; 1 is still read

F32 = np.float32


def f32(x: float) -> float:
    """Round a float64 value to the nearest float32 (the reference's Real(double))."""
    return float(np.float32(x))


@dataclass
class Shape:
    type: int
    params: List[float] = field(default_factory=lambda: [0.0, 0.0, 0.0, 0.0])
    points: Optional[np.ndarray] = None  # (n,3) float32 hull input cloud


@dataclass
class Body:
    shape: int
    motion: int = MOTION_DYNAMIC
    pos: tuple = (0.0, 0.0, 0.0)
    rot: tuple = (0.0, 0.0, 0.0, 1.0)
    vel: tuple = (0.0, 0.0, 0.0)
    ang: tuple = (0.0, 0.0, 0.0)
    # BodySettings defaults, include/Kizuri/Body/Body.h:62-90
    friction: float = 0.5
    restitution: float = 0.0
    linear_damping: float = 0.05
    angular_damping: float = 0.05
    gravity_factor: float = 1.0
    max_linear_velocity: float = 500.0
    max_angular_velocity: float = 50.0
    density: float = 1000.0
    mass_override: float = 0.0
    layer: int = 1
    mask: int = 0xFFFFFFFF
    flags: int = BODY_FLAG_ALLOW_SLEEPING
    ccd_motion_threshold: float = 0.0  # BodySettings::ccdMotionThreshold (Body.h:70)


# Joint types (include/Kizuri/Constraint/Constraints.h:41-277)
JOINT_POINT, JOINT_DISTANCE, JOINT_FIXED, JOINT_HINGE, JOINT_SLIDER, JOINT_SIXDOF = range(6)
JOINT_FLAG_DISABLED = 1       # Constraint::SetEnabled(false)
JOINT_FLAG_LIMITS = 2         # Hinge/SliderConstraint::SetLimits(lower, upper)
JOINT_FLAG_MOTOR = 4          # Hinge/SliderConstraint::SetMotor(target, max)
JOINT_FLAG_LOCAL_ANCHORS = 8  # PointConstraint(a, b, localAnchorA, localAnchorB)
AXIS_FREE, AXIS_LIMITED, AXIS_FIXED = 0, 1, 2  # SixDOFConstraint::AxisMode
JOINT_RECORD = struct.Struct("<4I21f2I12f")


@dataclass
class Joint:
    """One joint as the reference's constructors take it: world-space anchors and axes at the
    bodies' creation poses.  anchor_b is DistanceConstraint's second anchor (or PointConstraint's
    local anchor B with JOINT_FLAG_LOCAL_ANCHORS); axis_b is HingeConstraint's axis on B; rotation
    is SixDOFConstraint's world frame; axis_modes packs 2 bits per axis (linear x,y,z then
    angular x,y,z); motor_mask bit k / 3+k enables SixDOF linear / angular motor k."""
    type: int
    body_a: int
    body_b: int
    anchor_a: tuple = (0.0, 0.0, 0.0)
    anchor_b: tuple = (0.0, 0.0, 0.0)
    axis_a: tuple = (0.0, 1.0, 0.0)
    axis_b: tuple = (0.0, 1.0, 0.0)
    rotation: tuple = (0.0, 0.0, 0.0, 1.0)
    distance: float = 0.0
    lower: float = 0.0
    upper: float = 0.0
    motor_target: float = 0.0
    motor_max: float = 0.0
    flags: int = 0
    axis_modes: int = 0
    motor_mask: int = 0
    six_motor: tuple = (0.0,) * 12  # linear targets[3], linear max[3], angular targets[3], angular max[3]

    def to_bytes(self) -> bytes:
        fl = [f32(x) for x in (*self.anchor_a, *self.anchor_b, *self.axis_a, *self.axis_b, *self.rotation,
                               self.distance, self.lower, self.upper, self.motor_target, self.motor_max)]
        return JOINT_RECORD.pack(self.type, self.body_a, self.body_b, self.flags, *fl, self.axis_modes,
                                 self.motor_mask, *[f32(x) for x in self.six_motor])

    @staticmethod
    def from_values(v) -> "Joint":
        f = v[4:25]
        return Joint(v[0], v[1], v[2], tuple(f[0:3]), tuple(f[3:6]), tuple(f[6:9]), tuple(f[9:12]),
                     tuple(f[12:16]), f[16], f[17], f[18], f[19], f[20], v[3], v[25], v[26], tuple(v[27:39]))


@dataclass
class Scene:
    """World settings + shapes + bodies.  Settings defaults are WorldSettings /
    SolverSettings (PhysicsWorld.h:20-43, ContactSolver.h:67-82) except that sleeping
    is off, which is how every timed and parity run is configured."""
    name: str = "scene"
    gravity: tuple = (0.0, -9.81, 0.0)
    dt: float = 1.0 / 60.0
    velocity_iterations: int = 16
    position_iterations: int = 6
    flags: int = 0
    baumgarte: float = 0.2
    penetration_slop: float = 0.005
    restitution_threshold: float = 1.0
    max_bias_velocity: float = 3.0
    warm_start_factor: float = 1.0
    # WorldSettings sleep thresholds (PhysicsWorld.h:25-27), used with WORLD_FLAG_ALLOW_SLEEPING
    sleep_time_threshold: float = 0.5
    sleep_linear_threshold: float = 0.05
    sleep_angular_threshold: float = 0.1
    shapes: List[Shape] = field(default_factory=list)
    bodies: List[Body] = field(default_factory=list)
    joints: List[Joint] = field(default_factory=list)

    # -- construction helpers -------------------------------------------------
    def add_shape(self, shape: Shape) -> int:
        self.shapes.append(shape)
        return len(self.shapes) - 1

    def add_body(self, body: Body) -> int:
        self.bodies.append(body)
        return len(self.bodies) - 1

    @property
    def num_dynamic(self) -> int:
        return sum(1 for b in self.bodies if b.motion == MOTION_DYNAMIC)

    # -- binary format ----------------------------------------------------------
    def to_bytes(self) -> bytes:
        out = bytearray()
        out += struct.pack("<II", SCENE_MAGIC, SCENE_VERSION)
        out += struct.pack("<3ff", *[f32(g) for g in self.gravity], f32(self.dt))
        out += struct.pack("<III", self.velocity_iterations, self.position_iterations, self.flags)
        out += struct.pack("<5f", f32(self.baumgarte), f32(self.penetration_slop),
                           f32(self.restitution_threshold), f32(self.max_bias_velocity),
                           f32(self.warm_start_factor))
        out += struct.pack("<3f", f32(self.sleep_time_threshold), f32(self.sleep_linear_threshold),
                           f32(self.sleep_angular_threshold))
        out += struct.pack("<I", len(self.shapes))
        for s in self.shapes:
            p = list(s.params) + [0.0] * (4 - len(s.params))
            pts = np.zeros((0, 3), F32) if s.points is None else np.asarray(s.points, F32).reshape(-1, 3)
            out += struct.pack("<I4fI", s.type, *[f32(x) for x in p[:4]], pts.shape[0])
            out += pts.astype("<f4").tobytes()
        out += struct.pack("<I", len(self.bodies))
        for b in self.bodies:
            out += struct.pack("<II", b.shape, b.motion)
            out += struct.pack("<3f4f3f3f", *[f32(x) for x in (*b.pos, *b.rot, *b.vel, *b.ang)])
            out += struct.pack("<9f", *[f32(x) for x in (
                b.friction, b.restitution, b.linear_damping, b.angular_damping, b.gravity_factor,
                b.max_linear_velocity, b.max_angular_velocity, b.density, b.mass_override)])
            out += struct.pack("<III", b.layer & 0xFFFFFFFF, b.mask & 0xFFFFFFFF, b.flags)
            out += struct.pack("<f", f32(b.ccd_motion_threshold))
        if self.joints:  # optional trailing section
            out += struct.pack("<I", len(self.joints))
            for j in self.joints:
                out += j.to_bytes()
        return bytes(out)

    def save(self, path: str) -> None:
        with open(path, "wb") as fh:
            fh.write(self.to_bytes())

    @staticmethod
    def from_bytes(data: bytes, name: str = "scene") -> "Scene":
        off = 0

        def take(fmt):
            nonlocal off
            vals = struct.unpack_from(fmt, data, off)
            off += struct.calcsize(fmt)
            return vals

        magic, version = take("<II")
        if magic != SCENE_MAGIC or version not in (1, 2):
            raise ValueError("not a KZSC v1/v2 scene")
        sc = Scene(name=name)
        gx, gy, gz, dt = take("<3ff")
        sc.gravity, sc.dt = (gx, gy, gz), dt
        sc.velocity_iterations, sc.position_iterations, sc.flags = take("<III")
        (sc.baumgarte, sc.penetration_slop, sc.restitution_threshold,
         sc.max_bias_velocity, sc.warm_start_factor) = take("<5f")
        if version >= 2:
            sc.sleep_time_threshold, sc.sleep_linear_threshold, sc.sleep_angular_threshold = take("<3f")
        (ns,) = take("<I")
        for _ in range(ns):
            t, p0, p1, p2, p3, n = take("<I4fI")
            pts = None
            if n:
                pts = np.frombuffer(data, "<f4", 3 * n, off).reshape(n, 3).astype(F32)
                off += 12 * n
            sc.shapes.append(Shape(t, [p0, p1, p2, p3], pts))
        (nb,) = take("<I")
        for _ in range(nb):
            shape, motion = take("<II")
            v = take("<3f4f3f3f")
            m = take("<9f")
            layer, mask, flags = take("<III")
            (thr,) = take("<f") if version >= 2 else (0.0,)
            sc.bodies.append(Body(shape, motion, v[0:3], v[3:7], v[7:10], v[10:13], *m,
                                  layer=layer, mask=mask, flags=flags, ccd_motion_threshold=thr))
        if off < len(data):
            (nj,) = take("<I")
            for _ in range(nj):
                sc.joints.append(Joint.from_values(JOINT_RECORD.unpack_from(data, off)))
                off += JOINT_RECORD.size
        return sc


# ---------------------------------------------------------------------------
# Scene builders
# ---------------------------------------------------------------------------
def _ground(sc: Scene, friction: float) -> None:
    """Static plane y = 0 at the origin (PlaneShape(Plane(UnitY, 0)))."""
    s = sc.add_shape(Shape(SHAPE_PLANE, [0.0, 1.0, 0.0, 0.0]))
    sc.add_body(Body(s, MOTION_STATIC, friction=friction))


def _timed_settings(sc: Scene, vel: int, pos: int) -> None:
    sc.velocity_iterations = vel
    sc.position_iterations = pos
    sc.flags = 0  # allowSleeping = false for every timed and parity run


def pyramid(rows: int = 20, friction: float = 0.6, vel_iters: int = 10, pos_iters: int = 2,
            spacing: float = 1.02, z: float = 0.0) -> Scene:
    """Row r holds rows-r unit boxes at x=(i-(n-1)/2)*1.02, y=0.5+r*1.02 (TestWorld.cpp:108-119)."""
    sc = Scene(name=f"pyramid{rows}")
    _timed_settings(sc, vel_iters, pos_iters)
    _ground(sc, friction)
    box = sc.add_shape(Shape(SHAPE_BOX, [0.5, 0.5, 0.5, 0.0]))
    for row in range(rows):
        n = rows - row
        y = 0.5 + row * spacing
        for i in range(n):
            x = (i - (n - 1) * 0.5) * spacing
            sc.add_body(Body(box, pos=(f32(x), f32(y), f32(z)), friction=friction))
    return sc


def stacks(nx: int = 20, nz: int = 20, height: int = 500, pitch: float = 2.0, seed: int = 7,
           friction: float = 0.6, vel_iters: int = 8, pos_iters: int = 2, jitter: float = 0.01) -> Scene:
    """nx*nz stacks of ``height`` unit boxes, vertical pitch 1 m, lateral jitter U[-j,j]."""
    sc = Scene(name=f"stacks{nx}x{nz}x{height}")
    _timed_settings(sc, vel_iters, pos_iters)
    _ground(sc, friction)
    box = sc.add_shape(Shape(SHAPE_BOX, [0.5, 0.5, 0.5, 0.0]))
    rng = np.random.RandomState(seed)
    jit = rng.random_sample((nx * nz, height, 2)) * (2.0 * jitter) - jitter
    for ix in range(nx):
        for iz in range(nz):
            s = ix * nz + iz
            cx = (ix - (nx - 1) * 0.5) * pitch
            cz = (iz - (nz - 1) * 0.5) * pitch
            for k in range(height):
                sc.add_body(Body(box, pos=(f32(cx + jit[s, k, 0]), f32(0.5 + k * 1.0),
                                           f32(cz + jit[s, k, 1])), friction=friction))
    return sc


def chains(nx: int = 40, nz: int = 40, links: int = 10, pitch: float = 1.5, seed: int = 5,
           vel_iters: int = 10, pos_iters: int = 2) -> Scene:
    """A joint workload: nx*nz static hooks 6 m up, each holding a chain of ``links`` boxes
    (0.2 x 0.5 x 0.2 m) joined by point joints, every third joint a hinge about z with +-0.8 rad
    limits; the chains start straight down with a random push, swing, and hit their neighbours
    and the ground plane."""
    sc = Scene(name=f"chains{nx}x{nz}x{links}")
    _timed_settings(sc, vel_iters, pos_iters)
    _ground(sc, 0.6)
    hook = sc.add_shape(Shape(SHAPE_BOX, [0.1, 0.1, 0.1, 0.0]))
    link = sc.add_shape(Shape(SHAPE_BOX, [0.1, 0.25, 0.1, 0.0]))
    rng = np.random.RandomState(seed)
    push = rng.uniform(-2.0, 2.0, (nx * nz, 2))
    top = 6.0
    for ix in range(nx):
        for iz in range(nz):
            c = ix * nz + iz
            x = f32((ix - (nx - 1) * 0.5) * pitch)
            z = f32((iz - (nz - 1) * 0.5) * pitch)
            prev = sc.add_body(Body(hook, MOTION_STATIC, pos=(x, f32(top + 0.1), z)))
            anchor = (x, f32(top), z)
            for k in range(links):
                y = f32(top - 0.5 * k - 0.25)
                b = sc.add_body(Body(link, pos=(x, y, z), vel=(f32(push[c, 0] * (k + 1) / links), 0.0,
                                                                f32(push[c, 1] * (k + 1) / links))))
                if k % 3 == 2:
                    sc.joints.append(Joint(JOINT_HINGE, prev, b, anchor_a=anchor, axis_a=(0.0, 0.0, 1.0),
                                           axis_b=(0.0, 0.0, 1.0), lower=-0.8, upper=0.8, flags=JOINT_FLAG_LIMITS))
                else:
                    sc.joints.append(Joint(JOINT_POINT, prev, b, anchor_a=anchor))
                prev, anchor = b, (x, f32(y - 0.25), z)
    return sc


def projectiles(n_shots: int = 2000, n_boxes: int = 4000, seed: int = 9) -> Scene:
    """A continuous-collision workload: LinearCast spheres and small boxes fired at 40-80 m/s at
    thin static walls (5 cm) beside a field of resting boxes, ground plane below."""
    sc = Scene(name=f"projectiles{n_shots}")
    _timed_settings(sc, 10, 2)
    _ground(sc, 0.6)
    wall = sc.add_shape(Shape(SHAPE_BOX, [0.025, 2.0, 8.0, 0.0]))
    ball = sc.add_shape(Shape(SHAPE_SPHERE, [0.1, 0.0, 0.0, 0.0]))
    cube = sc.add_shape(Shape(SHAPE_BOX, [0.1, 0.1, 0.1, 0.0]))
    box = sc.add_shape(Shape(SHAPE_BOX, [0.4, 0.4, 0.4, 0.0]))
    rng = np.random.RandomState(seed)
    for k in range(8):
        sc.add_body(Body(wall, MOTION_STATIC, pos=(f32(-28.0 + 8.0 * k), 2.0, 0.0)))
    side = int(math.ceil(math.sqrt(n_boxes)))
    for i in range(n_boxes):
        sc.add_body(Body(box, pos=(f32(-30.0 + 60.0 * (i % side) / side), 0.4, f32(10.0 + 40.0 * (i // side) / side))))
    lc = BODY_FLAG_ALLOW_SLEEPING | BODY_FLAG_LINEAR_CAST
    for i in range(n_shots):
        x = f32(rng.uniform(-30.0, 30.0))
        sc.add_body(Body(ball if i % 2 else cube, pos=(x, f32(rng.uniform(0.5, 3.5)), f32(rng.uniform(-7.0, 7.0))),
                         vel=(f32(rng.choice([-1.0, 1.0]) * rng.uniform(40.0, 80.0)), 0.0, 0.0), flags=lc))
    return sc


def _shoemake(u1: float, u2: float, u3: float) -> tuple:
    """Uniform random rotation (Shoemake 1992), returned as float32 (x, y, z, w)."""
    a = math.sqrt(1.0 - u1)
    b = math.sqrt(u1)
    t2 = 2.0 * math.pi * u2
    t3 = 2.0 * math.pi * u3
    return (f32(a * math.sin(t2)), f32(a * math.cos(t2)), f32(b * math.sin(t3)), f32(b * math.cos(t3)))


def pile(n: int = 20000, seed: int = 1234, extent: float = 20.0, y_range=(2.0, 100.0),
         friction: float = 0.6, vel_iters: int = 10, pos_iters: int = 2, hull_points: int = 16) -> Scene:
    """Random convex pile: body i is a sphere / box / capsule / hull by i % 4.

    Radii r~U[0.2,0.6]; half extents ~U[0.2,0.5]^3; capsule r~U[0.15,0.4], halfHeight~U[0.2,0.6];
    hull = 16 points uniform on the unit sphere scaled by U[0.3,0.7].  One shape per body.
    """
    sc = Scene(name=f"pile{n}_s{seed}")
    _timed_settings(sc, vel_iters, pos_iters)
    _ground(sc, friction)
    rng = np.random.RandomState(seed)
    for i in range(n):
        kind = i % 4
        if kind == 0:
            r = 0.2 + 0.4 * rng.random_sample()
            shape = Shape(SHAPE_SPHERE, [f32(r), 0.0, 0.0, 0.0])
        elif kind == 1:
            h = 0.2 + 0.3 * rng.random_sample(3)
            shape = Shape(SHAPE_BOX, [f32(h[0]), f32(h[1]), f32(h[2]), 0.0])
        elif kind == 2:
            r = 0.15 + 0.25 * rng.random_sample()
            hh = 0.2 + 0.4 * rng.random_sample()
            shape = Shape(SHAPE_CAPSULE, [f32(hh), f32(r), 0.0, 0.0])
        else:
            g = rng.standard_normal((hull_points, 3))
            g /= np.linalg.norm(g, axis=1, keepdims=True)
            scale = 0.3 + 0.4 * rng.random_sample()
            shape = Shape(SHAPE_HULL, [0.0] * 4, (g * scale).astype(F32))
        s = sc.add_shape(shape)
        u = rng.random_sample(3)
        rot = _shoemake(u[0], u[1], u[2])
        p = rng.random_sample(3)
        pos = (f32(-extent + 2 * extent * p[0]), f32(y_range[0] + (y_range[1] - y_range[0]) * p[1]),
               f32(-extent + 2 * extent * p[2]))
        sc.add_body(Body(s, pos=pos, rot=rot, friction=friction))
    return sc


def world_batch(num_worlds: int = 4096, seed: int = 4242, lo: int = 8, hi: int = 512) -> List[Scene]:
    """Independent worlds with log-uniform body counts in [lo, hi]: even worlds are pyramids
    (largest r with r(r+1)/2 <= N), odd worlds are convex piles with the xz extent scaled by
    sqrt(N/20000)."""
    rng = np.random.RandomState(seed)
    worlds = []
    for w in range(num_worlds):
        nb = int(math.floor(math.exp(math.log(lo) + (math.log(hi) - math.log(lo)) * rng.random_sample())))
        nb = max(lo, min(hi, nb))
        if w % 2 == 0:
            r = int((math.isqrt(8 * nb + 1) - 1) // 2)
            sc = pyramid(rows=max(r, 1))
        else:
            sc = pile(n=nb, seed=seed + w, extent=max(20.0 * math.sqrt(nb / 20000.0), 1.0))
        sc.name = f"world{w}"
        worlds.append(sc)
    return worlds


def merge_worlds(worlds: List[Scene]):
    """Independent worlds as one scene plus a world id per body: shape tables are concatenated
    (bodies re-indexed), world and solver settings are taken from the first world (all must agree).
    Bodies of different worlds never interact (the broad phase keys its cells and its plane lists by
    world)."""
    if not worlds:
        raise ValueError("no worlds")
    first = worlds[0]
    keys = ("gravity", "dt", "velocity_iterations", "position_iterations", "flags", "baumgarte",
            "penetration_slop", "restitution_threshold", "max_bias_velocity", "warm_start_factor",
            "sleep_time_threshold", "sleep_linear_threshold", "sleep_angular_threshold")
    out = Scene(name=f"{len(worlds)} worlds", **{k: getattr(first, k) for k in keys})
    ids = []
    for w, sc in enumerate(worlds):
        if any(getattr(sc, k) != getattr(first, k) for k in keys):
            raise ValueError(f"world {w} has different settings")
        base = len(out.shapes)
        out.shapes.extend(sc.shapes)
        for b in sc.bodies:
            nb = Body(**{f: getattr(b, f) for f in b.__dataclass_fields__})
            nb.shape = b.shape + base
            out.bodies.append(nb)
            ids.append(w)
    return out, np.asarray(ids, np.uint32)
