"""Reader for the binary traces written by oracle/ref_trace.cpp (test infrastructure).

A trace holds what the reference engine computed for one scene: per-body packed ids and mass
properties, every hull as built by ``ConvexHullShape::Create`` (Shapes.cpp:331-471), the
initial state, and per step the ``ComputeStateHash`` value, the WorldStats counters, the full
body state and - for the first ``detail`` steps - the broad-phase pair list (reference order)
and every contact constraint after the solve.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field
from typing import Dict, List

import numpy as np

PT_FLOATS = 39  # same layout as KZO_PT_FLOATS in oracle/kzo.h


@dataclass
class Hull:
    verts: np.ndarray      # (n,3) float32
    sizes: np.ndarray      # (f,) uint8
    idx: np.ndarray        # (k,) uint32
    volume: float


@dataclass
class StepDetail:
    pairs: np.ndarray        # (p,2) uint32 packed ids, reference order
    con_hdr: np.ndarray      # (c,3) uint32 packed A, packed B, numPoints
    con_fr: np.ndarray       # (c,2) float32 friction, restitution
    con_pts: np.ndarray      # (c,8,PT_FLOATS) float32


@dataclass
class Trace:
    n_bodies: int
    n_steps: int
    packed: np.ndarray            # (n,) uint32
    inv_mass: np.ndarray          # (n,) float32
    inv_inertia_local: np.ndarray  # (n,9) float32 column-major
    inv_inertia_world: np.ndarray  # (n,9) float32 column-major (at creation)
    hulls: Dict[int, Hull]
    state0: np.ndarray            # (n,13)
    hashes: np.ndarray            # (steps,) uint64
    stats: np.ndarray             # (steps,4) pairs, constraints, points, islands
    states: np.ndarray            # (steps,n,13)
    detail: List[StepDetail] = field(default_factory=list)
    ms_total: float = 0.0


def read_trace(path: str) -> Trace:
    data = open(path, "rb").read()
    off = 0

    def take(fmt):
        nonlocal off
        v = struct.unpack_from(fmt, data, off)
        off += struct.calcsize(fmt)
        return v

    def arr(dtype, count):
        nonlocal off
        a = np.frombuffer(data, dtype, count, off).copy()
        off += a.nbytes
        return a

    magic, ver, nb, steps, detail = take("<5I")
    assert magic == 0x52545A4B and ver == 1, "not a KZTR v1 trace"
    packed = np.zeros(nb, np.uint32)
    inv_mass = np.zeros(nb, np.float32)
    iil = np.zeros((nb, 9), np.float32)
    iiw = np.zeros((nb, 9), np.float32)
    for i in range(nb):
        packed[i], = take("<I")
        inv_mass[i], = take("<f")
        iil[i] = arr("<f4", 9)
        iiw[i] = arr("<f4", 9)
    (nh,) = take("<I")
    hulls = {}
    for _ in range(nh):
        si, nv = take("<II")
        verts = arr("<f4", 3 * nv).reshape(nv, 3)
        (nf,) = take("<I")
        sizes = arr("u1", nf)
        (ni,) = take("<I")
        idx = arr("<u4", ni)
        (vol,) = take("<f")
        hulls[si] = Hull(verts, sizes, idx, vol)
    state0 = arr("<f4", 13 * nb).reshape(nb, 13)
    hashes = np.zeros(steps, np.uint64)
    stats = np.zeros((steps, 4), np.uint32)
    states = np.zeros((steps, nb, 13), np.float32)
    det = []
    for s in range(steps):
        (si,) = take("<I")
        assert si == s
        (hashes[s],) = take("<Q")
        stats[s] = take("<4I")
        states[s] = arr("<f4", 13 * nb).reshape(nb, 13)
        if s < detail:
            (np_,) = take("<I")
            pairs = arr("<u4", 2 * np_).reshape(np_, 2)
            (nc,) = take("<I")
            hdr = np.zeros((nc, 3), np.uint32)
            fr = np.zeros((nc, 2), np.float32)
            pts = np.zeros((nc, 8, PT_FLOATS), np.float32)
            for c in range(nc):
                hdr[c] = take("<3I")
                fr[c] = take("<2f")
                for p in range(hdr[c, 2]):
                    pts[c, p] = arr("<f4", PT_FLOATS)
            det.append(StepDetail(pairs, hdr, fr, pts))
    (ms,) = take("<d")
    return Trace(nb, steps, packed, inv_mass, iil, iiw, hulls, state0, hashes, stats, states, det, ms)


def resolved_blob(scene, hulls: Dict[int, Hull], inv_mass: np.ndarray, inv_inertia_local: np.ndarray) -> bytes:
    """Resolved setup data for kzo_create: built hulls (shape order) then per-body mass."""
    out = bytearray()
    for si, s in enumerate(scene.shapes):
        if s.type != 4:
            continue
        h = hulls[si]
        out += struct.pack("<I", h.verts.shape[0]) + np.asarray(h.verts, "<f4").tobytes()
        out += struct.pack("<I", len(h.sizes)) + np.asarray(h.sizes, "u1").tobytes()
        out += b"\0" * ((4 - len(out) % 4) % 4)
        out += struct.pack("<I", len(h.idx)) + np.asarray(h.idx, "<u4").tobytes()
    for i in range(len(scene.bodies)):
        out += struct.pack("<f", float(inv_mass[i])) + np.asarray(inv_inertia_local[i], "<f4").tobytes()
    return bytes(out)
