"""Python host API over the C-ABI: a device-resident world built from a scene.

Mirrors the reference's PhysicsWorld surface (include/Kizuri/World/PhysicsWorld.h:82-239):
``step_fixed`` = StepFixed, ``compute_state_hash`` = ComputeStateHash, ``get_stats`` = GetStats,
``contact_constraints`` = GetContactConstraints, ``broadphase_pairs`` = GetBroadPhase().GetPairs().
Mass properties and hulls are resolved on the host exactly as BodyManager::CreateBody and
ConvexHullShape::Create do (kzg_mass_properties / kzg_hull_build).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from . import capi
from .scenes import (Scene, SHAPE_HULL, WORLD_FLAG_ALLOW_SLEEPING, WORLD_FLAG_NO_WARM_START,
                     WORLD_FLAG_SCALAR_SOLVER, WORLD_FLAG_VELOCITY_BIAS)

PT_FLOATS = 39


@dataclass
class HullData:
    verts: np.ndarray   # (n,3) float32, ConvexHullShape point order
    sizes: np.ndarray   # (f,) uint8
    idx: np.ndarray     # (k,) uint32


@dataclass
class Resolved:
    """Host-resolved setup: built hulls (per hull shape index) and per-body mass."""
    hulls: Dict[int, HullData] = field(default_factory=dict)
    inv_mass: np.ndarray = None
    inv_inertia_local: np.ndarray = None


def build_hull(points: np.ndarray, max_points: int = 256) -> HullData:
    L = capi.load()
    p = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    cap_f = 2 * p.shape[0] + 8
    ov = np.zeros((p.shape[0], 3), np.float32)
    osz = np.zeros(cap_f, np.uint8)
    oidx = np.zeros(3 * cap_f, np.uint32)
    nv, nf, ni = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
    capi.check(L.kzg_hull_build(capi.ptr(p), p.shape[0], max_points, capi.ptr(ov), ctypes.byref(nv), capi.ptr(osz),
                                ctypes.byref(nf), capi.ptr(oidx), ctypes.byref(ni), cap_f))
    return HullData(ov[:nv.value].copy(), osz[:nf.value].copy(), oidx[:ni.value].copy())


def _shape_table(scene: Scene, hulls: Dict[int, HullData]):
    descs = (capi.KzgShapeDesc * max(1, len(scene.shapes)))()
    verts, sizes, idx = [], [], []
    nv = nf = ni = 0
    for i, s in enumerate(scene.shapes):
        d = descs[i]
        d.type = s.type
        for k in range(4):
            d.params[k] = float(np.float32(s.params[k])) if k < len(s.params) else 0.0
        if s.type == SHAPE_HULL:
            h = hulls[i]
            d.first_vertex, d.num_vertices = nv, h.verts.shape[0]
            d.first_face, d.num_faces = nf, h.sizes.shape[0]
            d.first_index, d.num_indices = ni, h.idx.shape[0]
            verts.append(h.verts)
            sizes.append(h.sizes)
            idx.append(h.idx)
            nv += h.verts.shape[0]
            nf += h.sizes.shape[0]
            ni += h.idx.shape[0]
    V = np.concatenate(verts).astype(np.float32) if verts else np.zeros((0, 3), np.float32)
    S = np.concatenate(sizes).astype(np.uint8) if sizes else np.zeros(0, np.uint8)
    I = np.concatenate(idx).astype(np.uint32) if idx else np.zeros(0, np.uint32)
    return descs, np.ascontiguousarray(V), np.ascontiguousarray(S), np.ascontiguousarray(I)


def make_edit(op: int, packed_id: int, values=(), wake: bool = True) -> np.ndarray:
    """One kzg_body_edit record: `values` fills the operands in the order include/kzg.h gives."""
    e = np.zeros(1, capi.EDIT_DTYPE)
    e["op"], e["body"], e["wake"] = op, packed_id, int(bool(wake))
    v = np.asarray(values, np.float32).reshape(-1)
    e["v"][0, :v.size] = v
    return e


def resolve(scene: Scene) -> Resolved:
    """Build every hull and every body's mass properties on the host (no GPU needed)."""
    L = capi.load()
    hulls = {i: build_hull(s.points) for i, s in enumerate(scene.shapes) if s.type == SHAPE_HULL}
    descs, V, S, I = _shape_table(scene, hulls)
    n = len(scene.bodies)
    im = np.zeros(n, np.float32)
    iil = np.zeros((n, 9), np.float32)
    out_im = ctypes.c_float()
    out_i = np.zeros(9, np.float32)
    cache = {}
    for b_i, b in enumerate(scene.bodies):
        key = (b.shape, b.motion, np.float32(b.density).item(), np.float32(b.mass_override).item())
        if key not in cache:
            capi.check(L.kzg_mass_properties(ctypes.byref(descs[b.shape]), capi.ptr(V), capi.ptr(S), capi.ptr(I),
                                             b.motion, np.float32(b.density), np.float32(b.mass_override),
                                             ctypes.byref(out_im), capi.ptr(out_i)))
            cache[key] = (out_im.value, out_i.copy())
        im[b_i], iil[b_i] = cache[key]
    return Resolved(hulls, im, iil)


class World:
    """One device-resident world (or batch of independent worlds via ``world_ids``)."""

    def __init__(self, scene: Scene, resolved: Optional[Resolved] = None, world_ids: Optional[np.ndarray] = None,
                 max_pairs: Optional[int] = None, max_cache_entries: Optional[int] = None, device: int = 0):
        L = capi.load()
        self.scene = scene
        self.resolved = resolved or resolve(scene)
        n = len(scene.bodies)
        self.n = n
        descs, V, S, I = _shape_table(scene, self.resolved.hulls)
        cfg = capi.KzgConfig()
        cfg.max_bodies = max(n, 1)
        cfg.max_shapes = max(len(scene.shapes), 1)
        cfg.max_hull_vertices = max(V.shape[0], 1)
        cfg.max_hull_indices = max(I.shape[0], 1)
        cfg.max_pairs = int(max_pairs or max(16 * n, 4096))
        cache = int(max_cache_entries or 1 << max(12, int(np.ceil(np.log2(max(64 * n, 4096))))))
        cfg.max_cache_entries = cache
        cfg.device = device
        cfg.max_joints = len(getattr(scene, "joints", []))
        h = ctypes.c_void_p()
        capi.check(L.kzg_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        ws, ss = capi.KzgWorldSettings(), capi.KzgSolverSettings()
        L.kzg_default_settings(ctypes.byref(ws), ctypes.byref(ss))
        for k in range(3):
            ws.gravity[k] = float(np.float32(scene.gravity[k]))
        ws.allow_sleeping = int(bool(scene.flags & WORLD_FLAG_ALLOW_SLEEPING))
        ws.warm_start = 0 if scene.flags & WORLD_FLAG_NO_WARM_START else 1
        ws.sleep_time_threshold = float(np.float32(scene.sleep_time_threshold))
        ws.sleep_linear_threshold = float(np.float32(scene.sleep_linear_threshold))
        ws.sleep_angular_threshold = float(np.float32(scene.sleep_angular_threshold))
        ss.velocity_iterations = scene.velocity_iterations
        ss.position_iterations = scene.position_iterations
        ss.baumgarte = scene.baumgarte
        ss.penetration_slop = scene.penetration_slop
        ss.restitution_threshold = scene.restitution_threshold
        ss.max_bias_velocity = scene.max_bias_velocity
        ss.warm_start_factor = scene.warm_start_factor
        ss.use_velocity_bias = int(bool(scene.flags & WORLD_FLAG_VELOCITY_BIAS))
        ss.use_simd_solver = 0 if scene.flags & WORLD_FLAG_SCALAR_SOLVER else 1
        self._check(L.kzg_set_world_settings(h, ctypes.byref(ws)))
        self._check(L.kzg_set_solver_settings(h, ctypes.byref(ss)))
        self._ss = ss
        self._check(L.kzg_upload_shapes(h, descs, len(scene.shapes), capi.ptr(V), V.shape[0], capi.ptr(S), S.shape[0],
                                        capi.ptr(I), I.shape[0]))
        bodies = scene.bodies
        arr = {}

        def col(name, vals, dt=np.float32):
            a = np.ascontiguousarray(np.asarray(vals, dt))
            arr[name] = a
            return capi.ptr(a)

        soa = capi.KzgBodySoa()
        soa.shape = col("shape", [b.shape for b in bodies], np.uint32)
        soa.motion = col("motion", [b.motion for b in bodies], np.uint32)
        soa.flags = col("flags", [b.flags for b in bodies], np.uint32)
        soa.position = col("position", [b.pos for b in bodies])
        soa.rotation = col("rotation", [b.rot for b in bodies])
        soa.linear_velocity = col("lv", [b.vel for b in bodies])
        soa.angular_velocity = col("av", [b.ang for b in bodies])
        soa.friction = col("fr", [b.friction for b in bodies])
        soa.restitution = col("rs", [b.restitution for b in bodies])
        soa.linear_damping = col("ld", [b.linear_damping for b in bodies])
        soa.angular_damping = col("ad", [b.angular_damping for b in bodies])
        soa.gravity_factor = col("gf", [b.gravity_factor for b in bodies])
        soa.max_linear_velocity = col("ml", [b.max_linear_velocity for b in bodies])
        soa.max_angular_velocity = col("ma", [b.max_angular_velocity for b in bodies])
        soa.inv_mass = col("im", self.resolved.inv_mass)
        soa.inv_inertia_local = col("iil", self.resolved.inv_inertia_local)
        soa.object_layer = col("layer", [b.layer for b in bodies], np.uint32)
        soa.collision_mask = col("mask", [b.mask for b in bodies], np.uint32)
        soa.world_id = col("world", world_ids if world_ids is not None else np.zeros(n), np.uint32)
        soa.ccd_motion_threshold = col("ccdthr", [b.ccd_motion_threshold for b in bodies])
        first = ctypes.c_uint32()
        self._check(L.kzg_add_bodies(h, n, ctypes.byref(soa), ctypes.byref(first)))
        if getattr(scene, "joints", None):
            self.add_joints(scene.joints)
        inactive = getattr(scene, "active", None)
        if inactive is not None and not np.all(inactive):  # a loaded KZP1 file's sleeping bodies
            self.set_bodies_active(np.nonzero(~np.asarray(inactive, bool))[0].astype(np.uint32), False)
        self.dt = float(np.float32(scene.dt))

    def add_joints(self, joints) -> int:
        """Create joints (scenes.Joint records) at the bodies' current poses (PhysicsWorld::AddConstraint);
        returns the first one's index."""
        arr = (capi.KzgJointDesc * len(joints))()
        for d, j in zip(arr, joints):
            d.type, d.body_a, d.body_b, d.flags = j.type, j.body_a, j.body_b, j.flags
            for k in range(3):
                d.anchor_a[k], d.anchor_b[k] = j.anchor_a[k], j.anchor_b[k]
                d.axis_a[k], d.axis_b[k] = j.axis_a[k], j.axis_b[k]
            for k in range(4):
                d.rotation[k] = j.rotation[k]
            d.distance, d.lower, d.upper, d.motor_target, d.motor_max = (j.distance, j.lower, j.upper,
                                                                         j.motor_target, j.motor_max)
            d.axis_modes, d.motor_mask = j.axis_modes, j.motor_mask
            for k in range(12):
                d.six_motor[k] = j.six_motor[k]
        first = ctypes.c_uint32()
        self._check(capi.load().kzg_add_joints(self._h, len(joints), arr, ctypes.byref(first)))
        return first.value

    # -- settings ----------------------------------------------------------------------------
    def set_solver(self, **fields):
        """Change SolverSettings fields (kzg_solver_settings names) for the following steps."""
        for k, v in fields.items():
            if not hasattr(self._ss, k):
                raise AttributeError(f"kzg_solver_settings has no field {k}")
            setattr(self._ss, k, v)
        self._check(capi.load().kzg_set_solver_settings(self._h, ctypes.byref(self._ss)))

    def snapshot(self) -> bytes:
        """Device state and manifold cache (kzg_snapshot_save): restore() resumes bit-exactly."""
        L = capi.load()
        n = ctypes.c_size_t()
        self._check(L.kzg_snapshot_size(self._h, ctypes.byref(n)))
        buf = np.zeros(n.value, np.uint8)
        self._check(L.kzg_snapshot_save(self._h, capi.ptr(buf), n.value))
        return buf.tobytes()

    def restore(self, snap: bytes):
        buf = np.frombuffer(snap, np.uint8).copy()
        self._check(capi.load().kzg_snapshot_load(self._h, capi.ptr(buf), buf.size))

    def set_graph(self, enabled: bool = True):
        """Step through a captured CUDA graph (step_fixed(n) then launches n steps back to back)."""
        self._check(capi.load().kzg_set_graph(self._h, int(bool(enabled))))

    def set_tuning(self, small_island_constraints: int, warp_island_bodies: int, island_order: int = 0):
        """Launch shapes (bit-identical results): warp/CTA split points and the island-to-CTA order
        (0 island order, 1 largest first)."""
        t = capi.KzgTuning(small_island_constraints, warp_island_bodies, 0.0, island_order)
        self._check(capi.load().kzg_set_tuning(self._h, ctypes.byref(t)))

    def get_tuning(self) -> dict:
        t = capi.KzgTuning()
        self._check(capi.load().kzg_get_tuning(self._h, ctypes.byref(t)))
        return {n: getattr(t, n) for n, _ in capi.KzgTuning._fields_}

    def set_wait_limit(self, polls: int):
        """Poll limit of the bounded in-kernel waits (0 = the default 2^26)."""
        self._check(capi.load().kzg_set_wait_limit(self._h, int(polls)))

    def autotune(self, steps_per_candidate: int = 3, dt: Optional[float] = None) -> dict:
        """Pick the fastest launch shapes, each timed from the world's current state; the world is
        restored afterwards, so it does not advance."""
        t = capi.KzgTuning()
        self._check(capi.load().kzg_autotune(self._h, np.float32(self.dt if dt is None else dt),
                                             int(steps_per_candidate), ctypes.byref(t)))
        return {n: getattr(t, n) for n, _ in capi.KzgTuning._fields_}

    def set_residual(self, tolerance: float, max_iterations: int = 64):
        """Residual-terminated velocity iterations: an island stops once its relative impulse change
        sum|dImpulse| / sum|impulse| of one iteration is <= tolerance (0 = the fixed count)."""
        self.set_solver(residual_tolerance=float(tolerance), max_velocity_iterations=int(max_iterations))

    # -- lifetime ----------------------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            capi.load().kzg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, status):
        capi.check(status, self._h)

    # -- stepping (PhysicsWorld::StepFixed) --------------------------------------------------
    def step_fixed(self, dt: Optional[float] = None, n: int = 1):
        self._check(capi.load().kzg_step(self._h, np.float32(self.dt if dt is None else dt), n))

    def step_with_pairs(self, pairs: np.ndarray, dt: Optional[float] = None):
        p = np.ascontiguousarray(pairs, np.uint32).reshape(-1, 2)
        self._check(capi.load().kzg_step_with_pairs(self._h, capi.ptr(p), p.shape[0],
                                                     np.float32(self.dt if dt is None else dt)))

    def synchronize(self):
        self._check(capi.load().kzg_synchronize(self._h))

    # -- state -----------------------------------------------------------------------------
    def state(self) -> np.ndarray:
        out = np.zeros((self.n, 13), np.float32)
        self._check(capi.load().kzg_download_state(self._h, capi.ptr(out), 0, self.n))
        return out

    def set_state(self, s: np.ndarray):
        s = np.ascontiguousarray(s, np.float32).reshape(self.n, 13)
        self._check(capi.load().kzg_upload_state(self._h, capi.ptr(s), 0, self.n))

    def transforms(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        if out is None:
            out = np.zeros((self.n, 7), np.float32)
        self._check(capi.load().kzg_download_transforms(self._h, capi.ptr(out), 0, self.n))
        return out

    def upload_forces(self, force_torque: np.ndarray):
        ft = np.ascontiguousarray(force_torque, np.float32).reshape(self.n, 6)
        self._check(capi.load().kzg_upload_forces(self._h, capi.ptr(ft), 0, self.n))

    def mass(self):
        im = np.zeros(self.n, np.float32)
        iw = np.zeros((self.n, 9), np.float32)
        self._check(capi.load().kzg_download_mass(self._h, capi.ptr(im), capi.ptr(iw)))
        return im, iw

    # -- sleeping (PhysicsWorld::SetBodyActive / GetNumActiveBodies) ------------------------------
    def active_bodies(self) -> np.ndarray:
        """The active list: packed BodyIDs in the reference's order."""
        L = capi.load()
        n = ctypes.c_uint32()
        self._check(L.kzg_get_active_bodies(self._h, None, 0, ctypes.byref(n)))
        out = np.zeros(max(n.value, 1), np.uint32)
        if n.value:
            self._check(L.kzg_get_active_bodies(self._h, capi.ptr(out), n.value, ctypes.byref(n)))
        return out[:n.value]

    def set_bodies_active(self, packed_ids, active: bool):
        ids = np.ascontiguousarray(packed_ids, np.uint32).reshape(-1)
        self._check(capi.load().kzg_set_bodies_active(self._h, capi.ptr(ids), ids.size, int(bool(active))))

    def edit_bodies(self, edits: np.ndarray):
        """kzg_edit_bodies: PhysicsWorld's SetBody*/Add*/Activate/Deactivate operations, applied in
        order; `edits` is an array of capi.EDIT_DTYPE records (see make_edit)."""
        e = np.ascontiguousarray(edits, capi.EDIT_DTYPE).reshape(-1)
        self._check(capi.load().kzg_edit_bodies(self._h, capi.ptr(e), e.size))

    # -- diagnostics ----------------------------------------------------------------------------
    def compute_state_hash(self) -> int:
        h = ctypes.c_uint64()
        self._check(capi.load().kzg_state_hash(self._h, ctypes.byref(h)))
        return int(h.value)

    def get_stats(self) -> dict:
        s = capi.KzgStats()
        self._check(capi.load().kzg_get_stats(self._h, ctypes.byref(s)))
        return {name: getattr(s, name) for name, _ in capi.KzgStats._fields_}

    def broadphase_pairs(self) -> np.ndarray:
        L = capi.load()
        n = ctypes.c_uint32()
        self._check(L.kzg_num_pairs(self._h, ctypes.byref(n)))
        out = np.zeros((n.value, 2), np.uint32)
        if n.value:
            self._check(L.kzg_download_pairs(self._h, capi.ptr(out), n.value))
        return out

    def contact_constraints(self):
        L = capi.load()
        n = ctypes.c_uint32()
        self._check(L.kzg_num_constraints(self._h, ctypes.byref(n)))
        hdr = np.zeros((n.value, 3), np.uint32)
        fr = np.zeros((n.value, 2), np.float32)
        pts = np.zeros((n.value, 8, PT_FLOATS), np.float32)
        if n.value:
            self._check(L.kzg_download_constraints(self._h, capi.ptr(hdr), capi.ptr(fr), capi.ptr(pts), n.value))
        return hdr, pts, fr

    # -- learned warm start ------------------------------------------------------------------
    def mlp_set_params(self, theta: np.ndarray, mean: np.ndarray, std: np.ndarray):
        th = np.ascontiguousarray(theta, np.float32).reshape(-1)
        if th.size != capi.MLP_PARAMS:
            raise ValueError(f"expected {capi.MLP_PARAMS} parameters, got {th.size}")
        mu = np.ascontiguousarray(mean, np.float32).reshape(-1)
        sd = np.ascontiguousarray(std, np.float32).reshape(-1)
        self._check(capi.load().kzg_mlp_set_params(self._h, capi.ptr(th), capi.ptr(mu), capi.ptr(sd)))

    def mlp_get_params(self):
        th = np.zeros(capi.MLP_PARAMS, np.float32)
        mu = np.zeros(capi.MLP_FEATURES, np.float32)
        sd = np.zeros(capi.MLP_FEATURES, np.float32)
        self._check(capi.load().kzg_mlp_get_params(self._h, capi.ptr(th), capi.ptr(mu), capi.ptr(sd)))
        return th, mu, sd

    def mlp_enable(self, on: bool = True):
        self._check(capi.load().kzg_mlp_enable(self._h, int(bool(on))))

    def mlp_set_blend(self, normal: float, tangent: float):
        self._check(capi.load().kzg_mlp_set_blend(self._h, np.float32(normal), np.float32(tangent)))

    def mlp_set_quantile(self, tau: float):
        self._check(capi.load().kzg_mlp_set_quantile(self._h, np.float32(tau)))

    def mlp_log_begin(self, capacity: int):
        self._check(capi.load().kzg_mlp_log_begin(self._h, int(capacity)))

    def mlp_log_fetch(self) -> np.ndarray:
        L = capi.load()
        n = ctypes.c_uint32()
        self._check(L.kzg_mlp_log_fetch(self._h, None, 0, ctypes.byref(n)))
        out = np.zeros((n.value, capi.MLP_LOG_FLOATS), np.float32)
        if n.value:
            self._check(L.kzg_mlp_log_fetch(self._h, capi.ptr(out), n.value, ctypes.byref(n)))
        return out

    def mlp_set_dataset(self, samples: np.ndarray):
        s = np.ascontiguousarray(samples, np.float32).reshape(-1, capi.MLP_LOG_FLOATS)
        self._check(capi.load().kzg_mlp_set_dataset(self._h, capi.ptr(s), s.shape[0]))

    def mlp_gradient(self, first: int, count: int):
        g = np.zeros(capi.MLP_PARAMS, np.float32)
        loss = ctypes.c_float()
        self._check(capi.load().kzg_mlp_gradient(self._h, first, count, capi.ptr(g), ctypes.byref(loss)))
        return g, loss.value

    def mlp_train_step(self, first: int, count: int, lr: float) -> float:
        loss = ctypes.c_float()
        self._check(capi.load().kzg_mlp_train_step(self._h, first, count, np.float32(lr), ctypes.byref(loss)))
        return loss.value

    def mlp_predict(self, first: int, count: int) -> np.ndarray:
        out = np.zeros((count, 3), np.float32)
        self._check(capi.load().kzg_mlp_predict(self._h, first, count, capi.ptr(out)))
        return out

    # reference-style aliases
    StepFixed = step_fixed
    ComputeStateHash = compute_state_hash
    GetStats = get_stats
