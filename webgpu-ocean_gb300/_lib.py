"""ctypes bindings of libmpm.so (declarations: include/mpm.h).

The library is built in-tree by build.py.  Loading never falls back to
anything else: if libmpm.so is missing or fails to load, the import error
propagates.
"""
from __future__ import annotations

import ctypes
import os
import re

from . import build as _build

HEADER = os.path.join(_build.INCLUDE, "mpm.h")

MPM_OK = 0
MPM_E_INVALID = -1
MPM_E_CAPACITY = -2
MPM_E_GRID_CAPACITY = -3
MPM_E_CUDA = -4
MPM_E_NO_DEVICE = -5
MPM_E_STATE = -6
MPM_E_NONFINITE = -7

MPM_ENGINE_SORTED = 0
MPM_ENGINE_DISPATCH = 1

MPM_TAPE_FIXED_POINT = 0
MPM_TAPE_FP64 = 1

MPM_RENDER_COLOR = 0
MPM_RENDER_COLOR8 = 1
MPM_RENDER_DEPTH = 2
MPM_RENDER_THICKNESS = 3

KERNELS = {
    "clearGrid": 0,
    "p2g_1": 1,
    "p2g_2": 2,
    "updateGrid": 3,
    "g2p": 4,
    "copyPosition": 5,
}


class Params(ctypes.Structure):
    """mpm_params: the pipeline override constants (mls-mpm/mls-mpm.ts:53-59)."""
    _fields_ = [
        ("stiffness", ctypes.c_float),
        ("rest_density", ctypes.c_float),
        ("dynamic_viscosity", ctypes.c_float),
        ("dt", ctypes.c_float),
        ("fixed_point_multiplier", ctypes.c_float),
    ]


class SceneDesc(ctypes.Structure):
    """mpm_scene_desc: one scene of a batch."""
    _fields_ = [
        ("num_particles", ctypes.c_int),
        ("init_box", ctypes.c_float * 3),
        ("real_box", ctypes.c_float * 3),
        ("stiffness", ctypes.c_float),
        ("rest_density", ctypes.c_float),
        ("dynamic_viscosity", ctypes.c_float),
        ("dt", ctypes.c_float),
        ("fixed_point_multiplier", ctypes.c_float),
        ("gravity", ctypes.c_float * 3),
    ]


class RenderUniforms(ctypes.Structure):
    """mpm_render_uniforms: RenderUniforms of common.ts:1-9 (272 bytes),
    4x4 matrices by columns."""
    _fields_ = [
        ("texel_size", ctypes.c_float * 2),
        ("sphere_size", ctypes.c_float),
        ("pad", ctypes.c_float),
        ("inv_projection_matrix", ctypes.c_float * 16),
        ("projection_matrix", ctypes.c_float * 16),
        ("view_matrix", ctypes.c_float * 16),
        ("inv_view_matrix", ctypes.c_float * 16),
    ]


class KernelStat(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char_p), ("launches", ctypes.c_int64),
                ("timed_launches", ctypes.c_int64), ("total_ms", ctypes.c_double)]


class Health(ctypes.Structure):
    _fields_ = [("nonfinite_particles", ctypes.c_int64),
                ("out_of_range_accesses", ctypes.c_int64)]


_lib = None


def declared_functions() -> list[str]:
    """Names of every function include/mpm.h declares."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mpm_[a-z0-9_]+)\s*\(", text)))


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_missing:
        path = _build.build()
    if not os.path.exists(path):
        raise ImportError(f"libmpm.so not built ({path}); run build()")
    L = ctypes.CDLL(path)
    vp, i32, i64, f32 = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_float
    fp, dp, ip = ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int32)
    sig = {
        "mpm_default_params": (None, [ctypes.POINTER(Params)]),
        "mpm_create": (i32, [ctypes.POINTER(Params), i32, i32, i32, i32, f32, vp, ctypes.c_size_t,
                             ctypes.POINTER(vp)]),
        "mpm_destroy": (i32, [vp]),
        "mpm_reset_dambreak": (i32, [vp, i32, dp, ctypes.c_uint64]),
        "mpm_upload": (i32, [vp, fp, i32, fp]),
        "mpm_step": (i32, [vp, i32, vp]),
        "mpm_set_real_box": (i32, [vp, fp]),
        "mpm_num_particles": (i32, [vp]),
        "mpm_grid_count": (i64, [vp]),
        "mpm_render_diameter": (f32, [vp]),
        "mpm_posvel_device_ptr": (vp, [vp]),
        "mpm_download_particles": (i32, [vp, fp]),
        "mpm_download_grid": (i32, [vp, ip]),
        "mpm_download_posvel": (i32, [vp, fp, vp]),
        "mpm_download_posvel_async": (i32, [vp, fp, vp]),
        "mpm_wait_posvel": (i32, [vp, vp]),
        "mpm_dispatch": (i32, [vp, i32, vp]),
        "mpm_set_engine": (i32, [vp, i32]),
        "mpm_get_engine": (i32, [vp]),
        "mpm_synchronize": (i32, [vp]),
        "mpm_check_health": (i32, [vp, ctypes.POINTER(Health)]),
        "mpm_error_string": (ctypes.c_char_p, [i32]),
        "mpm_last_error": (ctypes.c_char_p, []),
        "mpm_scene_dambreak": (i32, [fp, i32, dp, ctypes.c_uint64]),
        "mpm_scene_lattice": (i32, [fp, i32, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_uint64]),
        "mpm_probe_conversions": (i32, [fp, i32, f32, ip, fp]),
        "mpm_probe_packed": (i32, [fp, fp, i32, fp]),
        "mpm_count_nonfinite_noalloc": (i32, [vp, i32, i32, vp, vp]),
        "mpm_set_profiling": (i32, [vp, i32]),
        "mpm_kernel_stats": (i32, [vp, ctypes.POINTER(KernelStat), i32]),
        "mpm_launch_count": (i64, [vp]),
        "mpm_set_gravity": (i32, [vp, fp]),
        "mpm_set_graph": (i32, [vp, i32]),
        "mpm_set_task_size": (i32, [vp, i32]),
        "mpm_get_task_size": (i32, [vp]),
        "mpm_autotune": (i32, [vp, i32, ctypes.POINTER(ctypes.c_int)]),
        "mpm_batch_set_task_size": (i32, [vp, i32]),
        "mpm_batch_get_task_size": (i32, [vp]),
        "mpm_set_lane_table_min": (i32, [vp, i32]),
        "mpm_get_lane_table_min": (i32, [vp]),
        "mpm_batch_set_lane_table_min": (i32, [vp, i32]),
        "mpm_batch_get_lane_table_min": (i32, [vp]),
        "mpm_set_task_threads": (i32, [vp, i32]),
        "mpm_get_task_threads": (i32, [vp]),
        "mpm_batch_set_task_threads": (i32, [vp, i32]),
        "mpm_batch_get_task_threads": (i32, [vp]),
        "mpm_set_bin_pairing": (i32, [vp, i32]),
        "mpm_get_bin_pairing": (i32, [vp]),
        "mpm_batch_set_bin_pairing": (i32, [vp, i32]),
        "mpm_batch_get_bin_pairing": (i32, [vp]),
        "mpm_batch_autotune": (i32, [vp, i32, ctypes.POINTER(ctypes.c_int)]),
        "mpm_batch_create": (i32, [ctypes.POINTER(SceneDesc), i32, fp, ctypes.POINTER(vp)]),
        "mpm_batch_destroy": (i32, [vp]),
        "mpm_batch_num_scenes": (i32, [vp]),
        "mpm_batch_num_particles": (i64, [vp]),
        "mpm_batch_step": (i32, [vp, i32, vp]),
        "mpm_batch_upload": (i32, [vp, fp]),
        "mpm_batch_set_scene": (i32, [vp, i32, ctypes.POINTER(SceneDesc)]),
        "mpm_batch_set_graph": (i32, [vp, i32]),
        "mpm_batch_download_particles": (i32, [vp, fp]),
        "mpm_batch_download_grid": (i32, [vp, i32, ip]),
        "mpm_batch_posvel_device_ptr": (vp, [vp]),
        "mpm_batch_check_health": (i32, [vp, ctypes.POINTER(Health)]),
        "mpm_batch_launch_count": (i64, [vp]),
        "mpm_batch_set_profiling": (i32, [vp, i32]),
        "mpm_batch_kernel_stats": (i32, [vp, ctypes.POINTER(KernelStat), i32]),
        "mpm_adjoint_create": (i32, [ctypes.POINTER(SceneDesc), i32, i32, i32, ctypes.POINTER(vp)]),
        "mpm_adjoint_destroy": (i32, [vp]),
        "mpm_adjoint_set_tape": (i32, [vp, i32]),
        "mpm_adjoint_set_scene": (i32, [vp, i32, ctypes.POINTER(SceneDesc)]),
        "mpm_forward_ckpt": (i32, [vp, fp, i32, vp]),
        "mpm_adjoint_state": (i32, [vp, i32, fp]),
        "mpm_backward": (i32, [vp, fp, ip, i32, fp, dp, vp]),
        "mpm_backward_list": (i32, [vp, ctypes.POINTER(fp), ip, i32, fp, dp, vp]),
        "mpm_adjoint_set_observations": (i32, [vp, i32, ip, ctypes.POINTER(fp)]),
        "mpm_adjoint_observation_loss": (i32, [vp, dp, vp]),
        "mpm_backward_observed": (i32, [vp, fp, dp, vp]),
        "mpm_renderer_create": (i32, [i32, i32, f32, f32, ctypes.POINTER(vp)]),
        "mpm_renderer_destroy": (i32, [vp]),
        "mpm_renderer_set_envmap": (i32, [vp, i32, fp]),
        "mpm_renderer_execute": (i32, [vp, vp, i32, ctypes.POINTER(RenderUniforms), vp]),
        "mpm_renderer_execute_spheres": (i32, [vp, vp, i32, ctypes.POINTER(RenderUniforms), vp]),
        "mpm_renderer_download": (i32, [vp, i32, vp]),
        "mpm_renderer_color_device_ptr": (vp, [vp]),
        "mpm_sph_create": (i32, [i32, f32, vp, ctypes.c_size_t, ctypes.POINTER(vp)]),
        "mpm_sph_destroy": (i32, [vp]),
        "mpm_sph_reset_dambreak": (i32, [vp, i32, dp, ctypes.c_uint64]),
        "mpm_sph_upload": (i32, [vp, fp, i32, fp]),
        "mpm_sph_step": (i32, [vp, i32, vp]),
        "mpm_sph_set_graph": (i32, [vp, i32]),
        "mpm_sph_set_warp_per_particle": (i32, [vp, i32]),
        "mpm_sph_get_warp_per_particle": (i32, [vp]),
        "mpm_sph_set_real_box": (i32, [vp, fp]),
        "mpm_sph_num_particles": (i32, [vp]),
        "mpm_sph_grid_count": (i64, [vp]),
        "mpm_sph_posvel_device_ptr": (vp, [vp]),
        "mpm_sph_download_particles": (i32, [vp, fp]),
        "mpm_sph_download_posvel": (i32, [vp, fp]),
        "mpm_sph_scene_dambreak": (i32, [fp, i32, dp, ctypes.c_uint64]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L
