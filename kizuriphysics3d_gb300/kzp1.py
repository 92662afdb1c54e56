"""KZP1 world files: the reference's binary save format (SerializeWorld / DeserializeWorld,
src/Serialization/Serializer.cpp:11-12, 123-237), read and written for this package's scenes.

A file holds bodies only (no world settings): magic 'KZP1' (0x31505A4B), version 1, a body count,
then per body in slot order its shape (u8 ShapeType + parameters; a hull as its vertex count and
vertices, rebuilt with ConvexHullShape::Create on load), its BodySettings (position, rotation,
velocities, motion type and quality, CCD threshold, friction, restitution, damping, gravity factor,
velocity limits, layer, mask, sleeping and sensor flags, user data, mass override, density) and an
active flag.  Little-endian, floats as FP32, vectors as 3 (4 for quaternions) floats.

Cylinders, meshes, compounds and height fields are not part of the accelerated path: reading a file
with one raises, like the reference's writer refuses the last three.
"""
from __future__ import annotations

import copy
import struct
from typing import Optional

import numpy as np

from . import scenes
from .scenes import Body, Scene, Shape

MAGIC = 0x31505A4B
VERSION = 1
_CYLINDER = 3


def _shape_bytes(sh: Shape, hull_vertices) -> bytes:
    t = sh.type
    out = struct.pack("<B", t)
    p = [float(np.float32(v)) for v in sh.params]
    if t == scenes.SHAPE_SPHERE:
        out += struct.pack("<f", p[0])
    elif t == scenes.SHAPE_BOX:
        out += struct.pack("<3f", *p[:3])
    elif t == scenes.SHAPE_CAPSULE:  # CapsuleShape(halfHeight, radius)
        out += struct.pack("<2f", p[0], p[1])
    elif t == scenes.SHAPE_PLANE:  # normal xyz, distance
        out += struct.pack("<4f", *p[:4])
    elif t == scenes.SHAPE_HULL:
        v = np.ascontiguousarray(hull_vertices, np.float32).reshape(-1, 3)
        out += struct.pack("<I", v.shape[0]) + v.tobytes()
    else:
        raise ValueError(f"shape type {t} cannot be written to KZP1")
    return out


def to_kzp1(scene: Scene, state: Optional[np.ndarray] = None, active: Optional[np.ndarray] = None,
            inv_mass: Optional[np.ndarray] = None) -> bytes:
    """KZP1 bytes of a scene's bodies (at `state`, 13 floats per body, when given), as the
    reference's SerializeWorld writes them: BodySettings captured from the body (Body::CaptureSettings,
    Body.h:237-262: a dynamic body's mass as its mass override, density 0) and the active flag.
    `active` (one flag per body; default all active) and `inv_mass` (the resolved inverse masses;
    default: the scene's own mass override and density are written) make the bytes those of the
    reference's file for the same world."""
    from .world import build_hull
    hulls = {}
    out = bytearray(struct.pack("<III", MAGIC, VERSION, len(scene.bodies)))
    for i, b in enumerate(scene.bodies):
        sh = scene.shapes[b.shape]
        hv = None
        if sh.type == scenes.SHAPE_HULL:
            if b.shape not in hulls:  # the reference writes the hull's points, i.e. its vertices
                hulls[b.shape] = build_hull(np.asarray(sh.points, np.float32)).verts
            hv = hulls[b.shape]
        out += _shape_bytes(sh, hv)
        pos, rot, vel, ang = b.pos, b.rot, b.vel, b.ang
        if state is not None:
            st = state[i]
            pos, rot, vel, ang = st[0:3], st[3:7], st[7:10], st[10:13]
        f = lambda xs: [float(np.float32(x)) for x in xs]
        out += struct.pack("<3f4f3f3f", *f(pos), *f(rot), *f(vel), *f(ang))
        quality = 1 if b.flags & scenes.BODY_FLAG_LINEAR_CAST else 0  # MotionQuality::LinearCast = 1
        out += struct.pack("<BBf", b.motion, quality, float(np.float32(b.ccd_motion_threshold)))
        out += struct.pack("<7f", *f([b.friction, b.restitution, b.linear_damping, b.angular_damping,
                                      b.gravity_factor, b.max_linear_velocity, b.max_angular_velocity]))
        out += struct.pack("<II", b.layer & 0xFFFFFFFF, b.mask & 0xFFFFFFFF)
        out += struct.pack("<BB", 1 if b.flags & scenes.BODY_FLAG_ALLOW_SLEEPING else 0,
                           1 if b.flags & scenes.BODY_FLAG_SENSOR else 0)
        out += struct.pack("<Q", 0)  # userData
        if inv_mass is not None:  # GetMass() = 1 / inverseMass of a dynamic body (Body.h:168), else 0
            im = np.float32(inv_mass[i])
            mass = float(np.float32(1.0) / im) if b.motion == scenes.MOTION_DYNAMIC and im > 0 else 0.0
            out += struct.pack("<2f", mass, 0.0)
        else:
            out += struct.pack("<2f", *f([b.mass_override, b.density]))
        out += struct.pack("<B", 1 if active is None or active[i] else 0)
    return bytes(out)


class _Reader:
    def __init__(self, data: bytes):
        self.d, self.o = memoryview(data), 0

    def take(self, fmt: str):
        n = struct.calcsize(fmt)
        if self.o + n > len(self.d):
            raise ValueError("truncated KZP1 data")
        v = struct.unpack_from(fmt, self.d, self.o)
        self.o += n
        return v


def from_kzp1(data: bytes, template: Optional[Scene] = None) -> Scene:
    """A scene with the file's bodies; world and solver settings come from `template` (defaults:
    the reference's WorldSettings / SolverSettings).  Identical shapes are shared.  The bodies'
    active flags are in the returned scene's `active` array; a World built from the scene
    deactivates the inactive ones in slot order, as DeserializeWorld does (Serializer.cpp:214-232)."""
    r = _Reader(data)
    magic, version, count = r.take("<III")
    if magic != MAGIC or version != VERSION:
        raise ValueError("not a KZP1 version 1 file")
    sc = copy.copy(template) if template is not None else Scene(name="kzp1")
    sc.shapes, sc.bodies = [], []
    seen = {}
    active = []
    for _ in range(count):
        (t,) = r.take("<B")
        if t == scenes.SHAPE_SPHERE:
            key = (t, r.take("<f"))
            sh = Shape(t, [key[1][0], 0.0, 0.0, 0.0])
        elif t == scenes.SHAPE_BOX:
            key = (t, r.take("<3f"))
            sh = Shape(t, list(key[1]) + [0.0])
        elif t == scenes.SHAPE_CAPSULE:
            key = (t, r.take("<2f"))
            sh = Shape(t, list(key[1]) + [0.0, 0.0])
        elif t == scenes.SHAPE_PLANE:
            key = (t, r.take("<4f"))
            sh = Shape(t, list(key[1]))
        elif t == scenes.SHAPE_HULL:
            (nv,) = r.take("<I")
            if nv > 100000:
                raise ValueError("hull vertex count out of range")
            pts = np.asarray(r.take(f"<{3 * nv}f"), np.float32).reshape(nv, 3)
            key = (t, pts.tobytes())
            sh = Shape(t, [0.0, 0.0, 0.0, 0.0], pts)
        else:
            raise ValueError(f"KZP1 shape type {t} ({'cylinder' if t == _CYLINDER else 'unsupported'}) "
                             "is outside the accelerated path")
        if key not in seen:
            seen[key] = sc.add_shape(sh)
        pos = r.take("<3f"); rot = r.take("<4f"); vel = r.take("<3f"); ang = r.take("<3f")
        motion, quality, ccd = r.take("<BBf")
        fr, rs, ld, ad, gf, ml, ma = r.take("<7f")
        layer, mask = r.take("<II")
        sleep, sensor = r.take("<BB")
        r.take("<Q")
        mass_override, density = r.take("<2f")
        (act,) = r.take("<B")
        active.append(act != 0)
        flags = ((scenes.BODY_FLAG_ALLOW_SLEEPING if sleep else 0) | (scenes.BODY_FLAG_SENSOR if sensor else 0) |
                 (scenes.BODY_FLAG_LINEAR_CAST if quality == 1 else 0))
        sc.add_body(Body(shape=seen[key], motion=motion, pos=pos, rot=rot, vel=vel, ang=ang, friction=fr,
                         restitution=rs, linear_damping=ld, angular_damping=ad, gravity_factor=gf,
                         max_linear_velocity=ml, max_angular_velocity=ma, density=density,
                         mass_override=mass_override, layer=layer, mask=mask, flags=flags,
                         ccd_motion_threshold=ccd))
    if r.o != len(r.d):
        raise ValueError("trailing bytes after the last KZP1 body")
    sc.active = np.asarray(active, bool)
    return sc
