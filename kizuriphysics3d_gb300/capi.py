"""ctypes binding of libkzg.so (include/kzg.h).

The library is loaded from the package's in-tree build directory.  There is no fallback: if the
library is missing, or no CUDA device is present when a world is created, the call raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

HERE = os.path.dirname(os.path.abspath(__file__))

KZG_OK = 0
MLP_FEATURES = 24
MLP_PARAMS = 5955
MLP_LOG_FLOATS = 30
ERRORS = {-1: "KZG_ERR_INVALID", -2: "KZG_ERR_CUDA", -3: "KZG_ERR_CAPACITY", -4: "KZG_ERR_UNSUPPORTED",
          -5: "KZG_ERR_DEVICE"}

u32, f32, vp = ctypes.c_uint32, ctypes.c_float, ctypes.c_void_p


class KzgConfig(ctypes.Structure):
    _fields_ = [("max_bodies", u32), ("max_shapes", u32), ("max_hull_vertices", u32), ("max_hull_indices", u32),
                ("max_pairs", u32), ("max_cache_entries", u32), ("device", ctypes.c_int),
                ("max_joints", u32)]


class KzgSolverSettings(ctypes.Structure):
    _fields_ = [("velocity_iterations", u32), ("position_iterations", u32), ("baumgarte", f32),
                ("penetration_slop", f32), ("restitution_threshold", f32), ("max_bias_velocity", f32),
                ("warm_start_factor", f32), ("use_velocity_bias", ctypes.c_int), ("schedule", ctypes.c_int),
                ("residual_tolerance", f32), ("max_velocity_iterations", u32), ("use_split_impulse", ctypes.c_int),
                ("use_simd_solver", ctypes.c_int)]


class KzgWorldSettings(ctypes.Structure):
    _fields_ = [("gravity", f32 * 3), ("fixed_timestep", f32), ("allow_sleeping", ctypes.c_int),
                ("warm_start", ctypes.c_int), ("use_ccd", ctypes.c_int), ("ccd_max_penetration", f32),
                ("sleep_time_threshold", f32), ("sleep_linear_threshold", f32), ("sleep_angular_threshold", f32)]


class KzgShapeDesc(ctypes.Structure):
    _fields_ = [("type", u32), ("params", f32 * 4), ("first_vertex", u32), ("num_vertices", u32),
                ("first_face", u32), ("num_faces", u32), ("first_index", u32), ("num_indices", u32)]


class KzgBodySoa(ctypes.Structure):
    _fields_ = [(n, vp) for n in ("shape", "motion", "flags", "position", "rotation", "linear_velocity",
                                   "angular_velocity", "friction", "restitution", "linear_damping",
                                   "angular_damping", "gravity_factor", "max_linear_velocity",
                                   "max_angular_velocity", "inv_mass", "inv_inertia_local", "object_layer",
                                   "collision_mask", "world_id", "ccd_motion_threshold")]


class KzgTuning(ctypes.Structure):
    _fields_ = [("small_island_constraints", u32), ("warp_island_bodies", u32), ("step_ms", f32),
                ("island_order", u32)]


# kzg_body_edit (include/kzg.h) as a numpy record: op, packed BodyID, wake, reserved, 8 operands
EDIT_DTYPE = np.dtype([("op", "<u4"), ("body", "<u4"), ("wake", "<u4"), ("reserved", "<u4"), ("v", "<f4", (8,))])
(EDIT_SET_POSITION, EDIT_SET_ROTATION, EDIT_SET_TRANSFORM, EDIT_SET_LINEAR_VELOCITY, EDIT_SET_ANGULAR_VELOCITY,
 EDIT_ADD_FORCE, EDIT_ADD_FORCE_AT_POINT, EDIT_ADD_TORQUE, EDIT_ADD_IMPULSE, EDIT_ADD_IMPULSE_AT_POINT,
 EDIT_ACTIVATE, EDIT_DEACTIVATE) = range(12)


class KzgStats(ctypes.Structure):
    _fields_ = [(n, u32) for n in ("num_bodies", "num_broadphase_pairs", "num_contact_constraints",
                                   "num_contact_points", "num_islands", "num_batches", "max_velocity_levels",
                                   "max_bias_levels", "cache_entries", "device_error", "kernel_launches",
                                   "max_velocity_iterations_used", "point_velocity_iterations")] + \
               [(n, f32) for n in ("broadphase_ms", "narrowphase_ms", "constraints_ms", "schedule_ms", "solve_ms",
                                   "integrate_ms", "step_ms", "final_residual")] + [("num_active_bodies", u32), ("cache_capacity", u32), ("num_epa_pairs", u32)]


class KzgJointDesc(ctypes.Structure):
    _fields_ = [("type", u32), ("body_a", u32), ("body_b", u32), ("flags", u32), ("anchor_a", f32 * 3),
                ("anchor_b", f32 * 3), ("axis_a", f32 * 3), ("axis_b", f32 * 3), ("rotation", f32 * 4),
                ("distance", f32), ("lower", f32), ("upper", f32), ("motor_target", f32), ("motor_max", f32),
                ("axis_modes", u32), ("motor_mask", u32), ("six_motor", f32 * 12)]


EXPORTS = ["kzg_create", "kzg_destroy", "kzg_last_error", "kzg_set_stream", "kzg_synchronize",
           "kzg_set_world_settings", "kzg_set_solver_settings", "kzg_default_settings", "kzg_upload_shapes",
           "kzg_add_bodies", "kzg_add_joints", "kzg_step", "kzg_step_with_pairs", "kzg_download_state", "kzg_upload_state",
           "kzg_download_transforms", "kzg_upload_forces", "kzg_download_mass", "kzg_state_hash", "kzg_get_stats",
           "kzg_num_pairs", "kzg_download_pairs", "kzg_num_constraints", "kzg_download_constraints",
           "kzg_hull_build", "kzg_mass_properties"]

_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libkzg.so (building it first when absent and nvcc is available)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"libkzg.so not built ({path}); run kizuriphysics3d_gb300.build.build()")
        _build.build()
    L = ctypes.CDLL(path)
    st = ctypes.c_int
    P = ctypes.POINTER
    L.kzg_create.argtypes = [P(KzgConfig), P(vp)]
    L.kzg_create.restype = st
    L.kzg_destroy.argtypes = [vp]
    L.kzg_last_error.argtypes = [vp]
    L.kzg_last_error.restype = ctypes.c_char_p
    L.kzg_set_stream.argtypes = [vp, vp]
    L.kzg_synchronize.argtypes = [vp]
    L.kzg_set_world_settings.argtypes = [vp, P(KzgWorldSettings)]
    L.kzg_set_solver_settings.argtypes = [vp, P(KzgSolverSettings)]
    L.kzg_default_settings.argtypes = [P(KzgWorldSettings), P(KzgSolverSettings)]
    L.kzg_default_settings.restype = None
    L.kzg_upload_shapes.argtypes = [vp, P(KzgShapeDesc), u32, vp, u32, vp, u32, vp, u32]
    L.kzg_add_bodies.argtypes = [vp, u32, P(KzgBodySoa), P(u32)]
    L.kzg_add_joints.argtypes = [vp, u32, P(KzgJointDesc), P(u32)]
    L.kzg_step.argtypes = [vp, f32, u32]
    L.kzg_step_with_pairs.argtypes = [vp, vp, u32, f32]
    L.kzg_download_state.argtypes = [vp, vp, u32, u32]
    L.kzg_upload_state.argtypes = [vp, vp, u32, u32]
    L.kzg_download_transforms.argtypes = [vp, vp, u32, u32]
    L.kzg_upload_forces.argtypes = [vp, vp, u32, u32]
    L.kzg_download_mass.argtypes = [vp, vp, vp]
    L.kzg_state_hash.argtypes = [vp, P(ctypes.c_uint64)]
    L.kzg_get_stats.argtypes = [vp, P(KzgStats)]
    L.kzg_num_pairs.argtypes = [vp, P(u32)]
    L.kzg_download_pairs.argtypes = [vp, vp, u32]
    L.kzg_num_constraints.argtypes = [vp, P(u32)]
    L.kzg_download_constraints.argtypes = [vp, vp, vp, vp, u32]
    L.kzg_hull_build.argtypes = [vp, u32, u32, vp, P(u32), vp, P(u32), vp, P(u32), u32]
    L.kzg_mass_properties.argtypes = [P(KzgShapeDesc), vp, vp, vp, u32, f32, f32, P(f32), vp]
    L.kzg_state_hash_noalloc.argtypes = [vp, vp, u32, vp, P(ctypes.c_uint64), P(ctypes.c_char_p)]
    L.kzg_set_graph.argtypes = [vp, ctypes.c_int]
    L.kzg_snapshot_size.argtypes = [vp, ctypes.POINTER(ctypes.c_size_t)]
    L.kzg_snapshot_save.argtypes = [vp, vp, ctypes.c_size_t]
    L.kzg_snapshot_load.argtypes = [vp, vp, ctypes.c_size_t]
    L.kzg_set_tuning.argtypes = [vp, P(KzgTuning)]
    L.kzg_get_tuning.argtypes = [vp, P(KzgTuning)]
    L.kzg_autotune.argtypes = [vp, f32, u32, P(KzgTuning)]
    L.kzg_set_wait_limit.argtypes = [vp, u32]
    L.kzg_set_bodies_active.argtypes = [vp, vp, u32, ctypes.c_int]
    L.kzg_get_active_bodies.argtypes = [vp, vp, u32, P(u32)]
    L.kzg_edit_bodies.argtypes = [vp, vp, u32]
    L.kzg_mlp_set_params.argtypes = [vp, vp, vp, vp]
    L.kzg_mlp_get_params.argtypes = [vp, vp, vp, vp]
    L.kzg_mlp_enable.argtypes = [vp, ctypes.c_int]
    L.kzg_mlp_set_blend.argtypes = [vp, f32, f32]
    L.kzg_mlp_set_quantile.argtypes = [vp, f32]
    L.kzg_mlp_log_begin.argtypes = [vp, u32]
    L.kzg_mlp_log_fetch.argtypes = [vp, vp, u32, P(u32)]
    L.kzg_mlp_set_dataset.argtypes = [vp, vp, u32]
    L.kzg_mlp_gradient.argtypes = [vp, u32, u32, vp, P(f32)]
    L.kzg_mlp_train_step.argtypes = [vp, u32, u32, f32, P(f32)]
    L.kzg_mlp_predict.argtypes = [vp, u32, u32, vp]
    _lib = L
    return L


def ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


class KzgError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{ERRORS.get(status, status)}: {msg}")
        self.status = status


def check(status: int, handle=None) -> None:
    if status != KZG_OK:
        raise KzgError(status, load().kzg_last_error(handle).decode(errors="replace"))
