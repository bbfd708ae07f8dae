"""ctypes binding of ``libpbf103.so`` (the C ABI in include/pbf103.h).

Loading fails loudly when the library is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libpbf103.so")

c_f = ctypes.c_float
c_u32 = ctypes.c_uint32
c_i32 = ctypes.c_int32
c_u64 = ctypes.c_uint64
c_vp = ctypes.c_void_p
P = ctypes.POINTER

PBF_SUCCESS = 0
STATUS_NAMES = {
    0: "PBF_SUCCESS", 1: "PBF_ERROR_INVALID_ARGUMENT", 2: "PBF_ERROR_CUDA", 3: "PBF_ERROR_OUT_OF_MEMORY",
    4: "PBF_ERROR_CAPACITY", 5: "PBF_ERROR_GRID_TOO_LARGE", 6: "PBF_ERROR_BAD_PARAMETER",
    7: "PBF_ERROR_NOT_FOUND", 8: "PBF_ERROR_BUDGET", 9: "PBF_ERROR_NO_DEVICE", 10: "PBF_ERROR_NOT_READY",
}
PBF_FLAG_NONFINITE = 0x1
PBF_FLAG_COLLISION_LIMIT = 0x2
PBF_FLAG_CAPACITY = 0x4
PBF_ARRANGE_VOLUME, PBF_ARRANGE_RECTANGLE, PBF_ARRANGE_LINE, PBF_ARRANGE_CYLINDER = 0, 1, 2, 3
PBF_TENSILE_REFERENCE, PBF_TENSILE_TEXTBOOK, PBF_TENSILE_OFF = 0, 1, 2
PBF_VORTICITY_OFF, PBF_VORTICITY_REFERENCE, PBF_VORTICITY_TEXTBOOK = 0, 1, 2
PBF_XSPH_OFF, PBF_XSPH_WALK, PBF_XSPH_LIST = 0, 1, 2
PBF_SSF_SPLAT_QUAD, PBF_SSF_SPLAT_SPRITE = 0, 1
PBF_SSF_DEPTH, PBF_SSF_BLURRED, PBF_SSF_BLUR_INPUT, PBF_SSF_NORMAL, PBF_SSF_COLOR, PBF_SSF_RGBA8 = range(6)


class PbfParams(ctypes.Structure):
    _fields_ = [
        ("stable_density", c_f), ("stable_distance", c_f), ("particle_mass", c_f),
        ("smoothing_length", c_f), ("time_step", c_f), ("relaxation", c_f),
        ("xsph_parameter", c_f), ("vc_parameter", c_f), ("body_force", c_f * 3),
        ("max_pair_particle_num", c_u32), ("tensile_mode", c_i32), ("scorr_k", c_f),
        ("scorr_n", c_i32), ("scorr_dq", c_f), ("xsph_mode", c_i32), ("vorticity_mode", c_i32),
        ("max_collision_passes", c_u32), ("cell_width", c_f), ("grid_size", c_u32 * 3),
    ]


class PbfArrangement(ctypes.Structure):
    _fields_ = [
        ("kind", c_i32), ("axis", c_i32), ("origin", c_f * 3), ("end", c_f * 3), ("axis_value", c_f),
        ("radius", c_f), ("height", c_f), ("space", c_f),
    ]


class PbfSsfParams(ctypes.Structure):
    _fields_ = [
        ("width", c_u32), ("height", c_u32), ("projection", c_f * 16), ("view", c_f * 16),
        ("point_radius", c_f), ("point_scale", c_f), ("near_plane", c_f), ("far_plane", c_f),
        ("blur_radius", c_f), ("blur_scale", c_f), ("blur_passes", c_u32), ("splat_mode", c_u32),
        ("thickness", c_f), ("clear_color", c_f * 4),
    ]


class PbfServerConfig(ctypes.Structure):
    _fields_ = [
        ("hbm_budget_bytes", c_u64), ("max_scenes", c_u32), ("max_particles", c_u64),
        ("max_cells", c_u64), ("max_pair", c_u32), ("iters", c_i32), ("device", c_i32), ("tile", c_u32),
    ]


class PbfRequestDesc(ctypes.Structure):
    _fields_ = [
        ("params", PbfParams), ("domain_end", c_f * 3), ("area_min", c_f * 3), ("area_max", c_f * 3),
        ("n_planes", c_u32), ("plane_points", (c_f * 3) * 8), ("plane_normals", (c_f * 3) * 8),
        ("capacity", c_u32), ("horizon_steps", c_u32),
    ]


class PbfCompletion(ctypes.Structure):
    _fields_ = [
        ("request_id", c_u64), ("num", c_u32), ("steps", c_u32), ("flags", c_u32),
        ("arrival_s", ctypes.c_double), ("admit_s", ctypes.c_double), ("complete_s", ctypes.c_double),
    ]


class PbfServerStats(ctypes.Structure):
    _fields_ = [
        ("submitted", c_u64), ("admitted", c_u64), ("completed", c_u64), ("rejected", c_u64),
        ("substeps", c_u64), ("particle_steps", c_u64), ("resident_bytes", c_u64),
        ("peak_resident_bytes", c_u64), ("resident_scenes", c_u32), ("queued", c_u32),
        ("busy_s", ctypes.c_double), ("elapsed_s", ctypes.c_double),
    ]


# name -> (restype, argtypes); every function declared in include/pbf103.h
SIGNATURES = {
    "pbf_status_string": (ctypes.c_char_p, [c_i32]),
    "pbf_last_error": (ctypes.c_char_p, []),
    "pbf_abi_version": (ctypes.c_int, []),
    "pbf_params_init": (c_i32, [P(PbfParams)]),
    "pbf_calc_grid_size": (c_i32, [ctypes.c_double, P(c_f), P(c_u32)]),
    "pbf_boundary_create": (c_i32, [P(c_f), c_u32, P(c_f), c_u32, P(c_f), P(c_f), c_u32, P(c_vp)]),
    "pbf_boundary_destroy": (c_i32, [c_vp]),
    "pbf_create": (c_i32, [P(PbfParams), c_u32, P(c_f), ctypes.c_int, P(c_vp)]),
    "pbf_destroy": (c_i32, [c_vp]),
    "pbf_set_params": (c_i32, [c_vp, P(PbfParams)]),
    "pbf_get_params": (c_i32, [c_vp, P(PbfParams)]),
    "pbf_get_grid": (c_i32, [c_vp, P(c_u32), P(c_f)]),
    "pbf_set_particles": (c_i32, [c_vp, c_vp, c_vp, c_u32, ctypes.c_int, c_vp]),
    "pbf_add_particles": (c_i32, [c_vp, c_vp, c_vp, c_u32, ctypes.c_int, c_vp]),
    "pbf_one_step": (c_i32, [c_vp, c_vp, P(c_f), P(c_f), ctypes.c_int, c_vp]),
    "pbf_one_step_external": (c_i32, [c_vp, c_vp, c_vp, P(c_f), P(c_f), ctypes.c_int, c_vp]),
    "pbf_get_num": (c_i32, [c_vp, P(c_u32)]),
    "pbf_get_particles": (c_i32, [c_vp, c_vp, c_vp, ctypes.c_int, c_vp]),
    "pbf_get_flags": (c_i32, [c_vp, P(c_u32), ctypes.c_int]),
    "pbf_set_graph_mode": (c_i32, [c_vp, ctypes.c_int]),
    "pbf_get_neighbor_debug": (c_i32, [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, P(c_u32)]),
    "pbf_last_launches": (c_i32, [c_vp, P(c_u32)]),
    "pbf_profile_step": (c_i32, [c_vp, c_vp, P(c_f), P(c_f), ctypes.c_int, c_vp, P(c_f), c_vp, c_u32, P(c_u32)]),
    "pbf_batch_profile_step": (c_i32, [c_vp, ctypes.c_int, c_vp, P(c_f), c_vp, c_u32, P(c_u32)]),
    "pbf_cell_sort_noalloc": (c_i32, [c_vp, c_u32, c_f, P(c_u32), c_vp, c_vp, c_vp, c_vp]),
    "pbf_batch_create": (c_i32, [c_u32, c_u64, c_u64, c_u32, ctypes.c_int, P(c_vp)]),
    "pbf_batch_destroy": (c_i32, [c_vp]),
    "pbf_scene_bytes": (c_i32, [P(PbfParams), c_u32, P(c_f), P(c_u64)]),
    "pbf_batch_add_scene": (c_i32, [c_vp, P(PbfParams), c_u32, P(c_f), c_vp, P(c_f), P(c_f), c_vp, c_vp, c_u32,
                                    ctypes.c_int, c_vp, P(c_u32)]),
    "pbf_batch_remove_scene": (c_i32, [c_vp, c_u32]),
    "pbf_batch_num_scenes": (c_i32, [c_vp, P(c_u32)]),
    "pbf_batch_step": (c_i32, [c_vp, ctypes.c_int, c_vp]),
    "pbf_batch_get_scene": (c_i32, [c_vp, c_u32, c_vp, c_vp, P(c_u32), ctypes.c_int, c_vp]),
    "pbf_batch_get_flags": (c_i32, [c_vp, c_u32, P(c_u32), ctypes.c_int]),
    "pbf_batch_scene_ids": (c_i32, [c_vp, P(c_u32), c_u32, P(c_u32)]),
    "pbf_batch_set_all": (c_i32, [c_vp, c_vp, c_vp, c_vp, ctypes.c_int, c_vp]),
    "pbf_batch_get_all": (c_i32, [c_vp, c_vp, c_vp, c_vp, ctypes.c_int, c_vp]),
    "pbf_batch_step_packed": (c_i32, [c_vp, ctypes.c_int, c_vp, c_vp, c_vp, c_vp]),
    "pbf_batch_get_all_async": (c_i32, [c_vp, c_vp, c_vp, c_vp, c_vp]),
    "pbf_batch_autotune": (c_i32, [c_vp, ctypes.c_int, c_vp, P(c_u32)]),
    "pbf_batch_set_tile": (c_i32, [c_vp, c_u32]),
    "pbf_batch_set_chunk": (c_i32, [c_vp, c_u32]),
    "pbf_batch_set_cell_tile": (c_i32, [c_vp, c_u32]),
    "pbf_batch_get_cell_tile": (c_i32, [c_vp, P(c_u32)]),
    "pbf_batch_get_launch_shape": (c_i32, [c_vp, c_vp, c_vp]),
    "pbf_batch_set_graph_mode": (c_i32, [c_vp, ctypes.c_int]),
    "pbf_batch_last_launches": (c_i32, [c_vp, P(c_u32)]),
    "pbf_get_particle_ids": (c_i32, [c_vp, c_vp, ctypes.c_int, c_vp]),
    "pbf_restore_order": (c_i32, [c_vp, c_vp, c_vp, c_u32, ctypes.c_int, c_vp]),
    "pbf_get_particles_by_id": (c_i32, [c_vp, c_vp, c_vp, c_u32, ctypes.c_int, c_vp]),
    "pbf_arrangement_count": (c_i32, [P(PbfArrangement), P(c_u32)]),
    "pbf_generate": (c_i32, [c_vp, P(PbfArrangement), P(c_f), c_vp, P(c_u32)]),
    "pbf_emitter_create": (c_i32, [ctypes.c_int, c_vp, c_vp, c_u32, ctypes.c_int, P(c_vp)]),
    "pbf_emitter_create_arrangement": (c_i32, [ctypes.c_int, P(PbfArrangement), P(c_f), P(c_vp)]),
    "pbf_emitter_size": (c_i32, [c_vp, P(c_u32)]),
    "pbf_emitter_destroy": (c_i32, [c_vp]),
    "pbf_emit": (c_i32, [c_vp, c_vp, ctypes.c_double, c_vp]),
    "pbf_batch_get_particle_ids": (c_i32, [c_vp, c_u32, c_vp, P(c_u32), ctypes.c_int, c_vp]),
    "pbf_batch_restore_order": (c_i32, [c_vp, c_u32, c_vp, c_vp, c_u32, ctypes.c_int, c_vp]),
    "pbf_batch_get_particles_by_id": (c_i32, [c_vp, c_u32, c_vp, c_vp, c_u32, ctypes.c_int, c_vp]),
    "pbf_batch_generate": (c_i32, [c_vp, c_u32, P(PbfArrangement), P(c_f), c_vp, P(c_u32)]),
    "pbf_batch_emit": (c_i32, [c_vp, c_u32, c_vp, ctypes.c_double, c_vp]),
    "pbf_ssf_params_init": (c_i32, [P(PbfSsfParams)]),
    "pbf_ssf_create": (c_i32, [ctypes.c_int, P(PbfSsfParams), P(c_vp)]),
    "pbf_ssf_destroy": (c_i32, [c_vp]),
    "pbf_ssf_render": (c_i32, [c_vp, c_vp, c_u32, c_vp]),
    "pbf_ssf_render_particles": (c_i32, [c_vp, c_vp, c_vp]),
    "pbf_ssf_render_scene": (c_i32, [c_vp, c_vp, c_u32, c_vp]),
    "pbf_ssf_get_image": (c_i32, [c_vp, ctypes.c_int, c_vp, ctypes.c_int, c_vp]),
    "pbf_ssf_image_device": (c_i32, [c_vp, ctypes.c_int, P(c_vp), P(c_u64)]),
    "pbf_ssf_frame_constants": (c_i32, [c_vp, P(c_f), P(c_f)]),
    "pbf_ssf_last_launches": (c_i32, [c_vp, P(c_u32)]),
    "pbf_server_create": (c_i32, [P(PbfServerConfig), P(c_vp)]),
    "pbf_server_destroy": (c_i32, [c_vp]),
    "pbf_server_submit": (c_i32, [c_vp, P(PbfRequestDesc), c_vp, c_vp, c_u32, P(c_u64)]),
    "pbf_server_start": (c_i32, [c_vp]),
    "pbf_server_stop": (c_i32, [c_vp, ctypes.c_int]),
    "pbf_server_run_until_idle": (c_i32, [c_vp]),
    "pbf_server_poll": (c_i32, [c_vp, P(PbfCompletion), c_u32, P(c_u32)]),
    "pbf_server_result": (c_i32, [c_vp, c_u64, c_vp, c_vp, P(c_u32)]),
    "pbf_server_release": (c_i32, [c_vp, c_u64]),
    "pbf_server_get_stats": (c_i32, [c_vp, P(PbfServerStats)]),
    "pbf_server_clock": (ctypes.c_double, [c_vp]),
}


class PbfError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        msg = f"{where}: {STATUS_NAMES.get(status, status)}"
        if detail:
            msg += f" ({detail})"
        super().__init__(msg)


_lib = None


def load(path: str | None = None) -> ctypes.CDLL:
    """Load the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(f"{p} is missing: build it with `python -m ssf_pbf_cuda_gb300.build` "
                          "(the CUDA extension is required; there is no CPU fallback)")
    lib = ctypes.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(status: int, where: str) -> None:
    if status != PBF_SUCCESS:
        detail = ""
        if status == 2:
            try:
                detail = (load().pbf_last_error() or b"").decode()
            except Exception:  # pragma: no cover
                pass
        raise PbfError(status, where, detail)
