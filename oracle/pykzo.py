"""ctypes binding of the oracle library (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module; the
product never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libkzo.so")

PAIRS_TREE = 0
PAIRS_CANONICAL = 1
PAIRS_EXTERNAL = 2

# kzo_body_edit (kzo.h): op, packed body id, wake, reserved, 8 operands
EDIT_DTYPE = np.dtype([("op", "<u4"), ("body", "<u4"), ("wake", "<u4"), ("reserved", "<u4"), ("v", "<f4", (8,))])
PT_FLOATS = 39

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (seconds)."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-f", os.path.join(HERE, "Makefile")], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        vp, u32, f32, sz = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_float, ctypes.c_size_t
        L.kzo_create.restype = vp
        L.kzo_create.argtypes = [ctypes.c_char_p, sz, ctypes.c_char_p, sz]
        L.kzo_destroy.argtypes = [vp]
        L.kzo_error.restype = ctypes.c_char_p
        L.kzo_set_threads.argtypes = [vp, ctypes.c_int]
        L.kzo_set_pair_mode.argtypes = [vp, ctypes.c_int]
        L.kzo_set_schedule_stats.argtypes = [vp, ctypes.c_int]
        L.kzo_set_residual.argtypes = [vp, f32, u32]
        L.kzo_set_trig_mode.argtypes = [vp, ctypes.c_int]
        L.kzo_set_cache_hash.argtypes = [vp, ctypes.c_int]
        L.kzo_num_active.restype = u32
        L.kzo_num_active.argtypes = [vp]
        L.kzo_get_activity.argtypes = [vp, vp, vp, vp]
        L.kzo_shared_sleepers.restype = u32
        L.kzo_shared_sleepers.argtypes = [vp]
        L.kzo_set_bodies_active.argtypes = [vp, vp, u32, ctypes.c_int]
        L.kzo_edit_bodies.argtypes = [vp, vp, u32]
        L.kzo_set_external_pairs.argtypes = [vp, vp, u32]
        L.kzo_step.argtypes = [vp, f32]
        L.kzo_num_bodies.restype = u32
        L.kzo_num_bodies.argtypes = [vp]
        L.kzo_get_state.argtypes = [vp, vp]
        L.kzo_set_state.argtypes = [vp, vp]
        L.kzo_hash.restype = ctypes.c_uint64
        L.kzo_hash.argtypes = [vp]
        L.kzo_num_pairs.restype = u32
        L.kzo_num_pairs.argtypes = [vp]
        L.kzo_get_pairs.argtypes = [vp, vp]
        L.kzo_num_constraints.restype = u32
        L.kzo_num_constraints.argtypes = [vp]
        L.kzo_get_constraints.argtypes = [vp, vp, vp, vp]
        L.kzo_get_stats.argtypes = [vp, vp]
        L.kzo_get_mass.argtypes = [vp, vp, vp]
        L.kzo_collide_bodies.restype = u32
        L.kzo_collide_bodies.argtypes = [vp, u32, u32, f32, vp]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


class OracleWorld:
    """One oracle world built from scene bytes and resolved setup (hulls + mass)."""

    def __init__(self, scene_bytes: bytes, resolved: bytes, pair_mode: int = PAIRS_TREE, threads: int = 1):
        L = lib()
        self._w = L.kzo_create(scene_bytes, len(scene_bytes), resolved, len(resolved))
        if not self._w:
            raise RuntimeError("oracle: " + L.kzo_error().decode())
        L.kzo_set_pair_mode(self._w, pair_mode)
        L.kzo_set_threads(self._w, threads)
        self.n = L.kzo_num_bodies(self._w)

    def close(self):
        if self._w:
            lib().kzo_destroy(self._w)
            self._w = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_pair_mode(self, mode: int):
        lib().kzo_set_pair_mode(self._w, mode)

    def set_threads(self, n: int):
        lib().kzo_set_threads(self._w, n)

    def set_schedule_stats(self, on: bool):
        lib().kzo_set_schedule_stats(self._w, int(on))

    def set_trig_mode(self, mode: int):
        """0: the C library's float trigonometry (the reference's); 1: double precision rounded to
        float (the GPU's joint kernels)."""
        lib().kzo_set_trig_mode(self._w, int(mode))

    def set_cache_hash(self, mixed: bool):
        """Mixed manifold-cache slot function (same results; avoids the reference's clustering)."""
        lib().kzo_set_cache_hash(self._w, int(mixed))

    def activity(self):
        """(active list in order, per-body active flags, per-body sleep timers)."""
        n = lib().kzo_num_active(self._w)
        lst = np.zeros(max(n, 1), np.uint32)
        fl = np.zeros(self.n, np.uint8)
        tm = np.zeros(self.n, np.float32)
        lib().kzo_get_activity(self._w, _ptr(lst), _ptr(fl), _ptr(tm))
        return lst[:n], fl, tm

    def set_bodies_active(self, packed_ids, active: bool):
        ids = np.ascontiguousarray(packed_ids, np.uint32).reshape(-1)
        lib().kzo_set_bodies_active(self._w, _ptr(ids), ids.size, int(bool(active)))

    def edit_bodies(self, edits: np.ndarray):
        """kzo_edit_bodies: a structured array of EDIT_DTYPE records, applied in order."""
        e = np.ascontiguousarray(edits, EDIT_DTYPE).reshape(-1)
        lib().kzo_edit_bodies(self._w, _ptr(e), e.size)

    def shared_sleepers(self) -> int:
        return int(lib().kzo_shared_sleepers(self._w))

    def set_residual(self, tol: float, cap: int = 64):
        lib().kzo_set_residual(self._w, np.float32(tol), cap)

    def set_external_pairs(self, pairs: np.ndarray):
        p = np.ascontiguousarray(pairs, np.uint32)
        lib().kzo_set_external_pairs(self._w, _ptr(p), p.shape[0])

    def step(self, dt: float):
        lib().kzo_step(self._w, dt)

    def state(self) -> np.ndarray:
        out = np.zeros((self.n, 13), np.float32)
        lib().kzo_get_state(self._w, _ptr(out))
        return out

    def set_state(self, s: np.ndarray):
        s = np.ascontiguousarray(s, np.float32)
        lib().kzo_set_state(self._w, _ptr(s))

    def hash(self) -> int:
        return int(lib().kzo_hash(self._w))

    def pairs(self) -> np.ndarray:
        n = lib().kzo_num_pairs(self._w)
        out = np.zeros((n, 2), np.uint32)
        if n:
            lib().kzo_get_pairs(self._w, _ptr(out))
        return out

    def constraints(self):
        n = lib().kzo_num_constraints(self._w)
        hdr = np.zeros((n, 3), np.uint32)
        pts = np.zeros((n, 8, PT_FLOATS), np.float32)
        fr = np.zeros((n, 2), np.float32)
        if n:
            lib().kzo_get_constraints(self._w, _ptr(hdr), _ptr(pts), _ptr(fr))
        return hdr, pts, fr

    def stats(self) -> dict:
        o = np.zeros(13, np.uint32)
        lib().kzo_get_stats(self._w, _ptr(o))
        keys = ["pairs", "constraints", "points", "islands", "batches", "max_vel_levels",
                "max_bias_levels", "max_island_points", "sum_vel_levels", "max_open_batches",
                "max_velocity_iterations", "point_velocity_iterations"]
        d = dict(zip(keys, (int(x) for x in o[:12])))
        d["final_residual"] = float(o[12:13].view(np.float32)[0])
        return d

    def mass(self):
        im = np.zeros(self.n, np.float32)
        iw = np.zeros((self.n, 9), np.float32)
        lib().kzo_get_mass(self._w, _ptr(im), _ptr(iw))
        return im, iw

    def collide(self, a: int, b: int, max_sep: float = 0.02) -> np.ndarray:
        out = np.zeros((8, 11), np.float32)
        n = lib().kzo_collide_bodies(self._w, a, b, max_sep, _ptr(out))
        return out[:n]
