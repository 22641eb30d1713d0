"""ctypes binding of ``libmpm_gb300.so`` (C ABI declared in include/mpm_gb300.h).

There is no fallback: if the library is missing or a call fails, an
``MpmError`` is raised with the library's own message.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmpm_gb300.so")

ABI_VERSION = 6
MPM_OK = 0
STATUS_OUT_OF_GRID = 1
STATUS_NONFINITE = 2
STATUS_RENDER_BOX = 4

_c_p = ctypes.c_void_p
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_f64 = ctypes.c_double


class MpmError(RuntimeError):
    pass


class MpmParams(ctypes.Structure):
    _fields_ = [("abi_version", _i32), ("precision", _i32), ("n_grid", _i32), ("n_scenes", _i32),
                ("n_particles", _i64), ("ld", _i64),
                ("dx", _f64), ("inv_dx", _f64), ("dt", _f64), ("p_vol", _f64), ("p_mass", _f64),
                ("mu", _f64), ("lam", _f64), ("yield_stress", _f64),
                ("gravity", _f64 * 3), ("ground_friction", _f64), ("lower_bound", _f64)]


class MpmToolDesc(ctypes.Structure):
    _fields_ = [("type", _i32), ("action_dim", _i32), ("scene", _i32), ("collision_mask", _i32),
                ("friction", _f64), ("softness", _f64), ("radius", _f64), ("cap_h", _f64), ("cap_r", _f64),
                ("size", _f64 * 3), ("prism_h", _f64 * 2), ("prot", _f64 * 4),
                ("min_gap", _f64), ("max_gap", _f64), ("lower", _f64 * 3), ("upper", _f64 * 3),
                ("action_scale", _f64 * 7), ("torus", _f64 * 2)]


class MpmRenderVolume(ctypes.Structure):
    _fields_ = [("res", _i32 * 3), ("bake_size", _i32), ("dx", _f64), ("packed", _c_p), ("sdf", _c_p),
                ("sdf_copy", _c_p), ("color", _c_p), ("bbox", _c_p), ("kbox", _c_p)]


class MpmRenderView(ctypes.Structure):
    _fields_ = [("v2w", ctypes.c_float * 16), ("w2v", ctypes.c_float * 16), ("res", _i32 * 2),
                ("bias", ctypes.c_float * 2), ("sdf_threshold", ctypes.c_float), ("show_particles", _i32)]


class MpmTuning(ctypes.Structure):
    _fields_ = [("p2g_ctas", _i32), ("g2p_adj_ctas", _i32), ("p2g_adj_ctas", _i32), ("grid_ctas_per_sm", _i32),
                ("g2p_ctas", _i32), ("grid_op_adj_ctas", _i32)]


class MpmGridStore(ctypes.Structure):
    _fields_ = [("blocks", _c_p), ("block_ids", _c_p), ("slot_start", _c_p), ("slot_count", _c_p), ("bump", _c_p),
                ("capacity", _i64), ("n_slots", _i32), ("reserved", _i32)]


# every exported entry point and its ctypes signature
SIGNATURES = {
    "mpm_version": (ctypes.c_char_p, []),
    "mpm_create": (_i32, [ctypes.POINTER(MpmParams), ctypes.POINTER(_i64), ctypes.POINTER(_c_p)]),
    "mpm_destroy": (_i32, [_c_p]),
    "mpm_set_tools": (_i32, [_c_p, ctypes.POINTER(MpmToolDesc), _i32]),
    "mpm_set_collision_points": (_i32, [_c_p, _c_p, _i32]),
    "mpm_collision_pairs": (_i32, [_c_p]),
    "mpm_tools_action": (_i32, [_c_p, _c_p, _c_p, _c_p, _c_p, _i32, _c_p]),
    "mpm_tools_action_bwd": (_i32, [_c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _i32, _c_p]),
    "mpm_set_chained": (_i32, [_c_p, _i32]),
    "mpm_set_tuning": (_i32, [_c_p, ctypes.POINTER(MpmTuning)]),
    "mpm_get_tuning": (_i32, [_c_p, ctypes.POINTER(MpmTuning)]),
    "mpm_substep_fwd": (_i32, [_c_p, _c_p, _c_p, _c_p, _c_p, _c_p]),
    "mpm_substep_bwd": (_i32, [_c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p]),
    "mpm_substep_fwd_store": (_i32, [_c_p, _c_p, _c_p, _c_p, _c_p, ctypes.POINTER(MpmGridStore), _i32, _c_p]),
    "mpm_substep_bwd_store": (_i32, [_c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p,
                                     ctypes.POINTER(MpmGridStore), _i32, _c_p]),
    "mpm_grid_mass": (_i32, [_c_p, _c_p, _c_p, _c_p]),
    "mpm_grid_mass_bwd": (_i32, [_c_p, _c_p, _c_p, _c_p, _c_p]),
    "mpm_density_l1": (_i32, [_c_p, _c_p, _c_p, _f64, _c_p, _c_p, _c_p]),
    "mpm_soft_contact": (_i32, [_c_p, _c_p, _c_p, _c_p, _c_p, _c_p]),
    "mpm_soft_contact_bwd": (_i32, [_c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p]),
    "mpm_target_sdf": (_i32, [_c_p, _c_p, _c_p, _c_p, _c_p, _i32, _c_p]),
    "mpm_sdf_loss": (_i32, [_c_p, _c_p, _c_p, _f64, _c_p, _c_p, _c_p]),
    "mpm_iou": (_i32, [_c_p, _c_p, _c_p, _c_p, _c_p]),
    "mpm_contact_min_dist": (_i32, [_c_p, _c_p, _c_p, _c_p, _c_p, _c_p]),
    "mpm_contact_min_dist_bwd": (_i32, [_c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p]),
    "mpm_render_bake": (_i32, [_c_p, _c_p, _i32, _c_p, ctypes.POINTER(MpmRenderVolume), _c_p]),
    "mpm_render_trace": (_i32, [_c_p, ctypes.POINTER(MpmRenderVolume), ctypes.POINTER(MpmRenderView), _i32, _c_p,
                                _c_p, _c_p, _c_p, _c_p, _c_p, _c_p]),
    "mpm_tool_distance_cols": (_i32, [_c_p]),
    "mpm_tool_distance": (_i32, [_c_p, _c_p, _c_p, _c_p, _c_p]),
    "mpm_tool_distance_bwd": (_i32, [_c_p, _c_p, _c_p, _c_p, _c_p, _c_p, _c_p]),
    "mpm_substep_fwd_static": (_i32, [ctypes.POINTER(MpmParams), ctypes.POINTER(MpmToolDesc), _i32, _c_p, _c_p, _c_p,
                                      _c_p, _c_p, _c_p]),
    "mpm_status": (_i32, [_c_p, ctypes.POINTER(ctypes.c_uint32), _i32, _c_p]),
    "mpm_last_error": (_i32, [_c_p, ctypes.c_char_p, ctypes.c_size_t]),
    "mpm_launch_count": (_i64, [_c_p]),
    "mpm_profile_enable": (_i32, [_c_p, _i32]),
    "mpm_profile_read": (_i32, [_c_p, ctypes.POINTER(_f64), ctypes.POINTER(_i64)]),
    "mpm_sort_frame": (_i32, [_c_p, _c_p, _c_p, _c_p, _c_p]),
    "mpm_set_pipelined_adjoint": (_i32, [_c_p, _i32]),
    "mpm_unsort_frame": (_i32, [_c_p, _c_p, _c_p, _c_p, _c_p]),
}

# kernel kinds of mpm_profile_read (MPM_K_* in the header)
KERNEL_KINDS = ["p2g", "p2g_recompute", "grid_op", "g2p", "g2p_adj", "grid_op_adj", "p2g_adj", "clear", "other",
                "sort"]

_lib: Optional[ctypes.CDLL] = None


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise MpmError(f"{path} is missing: build it with diffskill_gb300.build.build() "
                       "(or __graft_entry__.build()); there is no CPU fallback")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error(handle=None) -> str:
    buf = ctypes.create_string_buffer(1024)
    load().mpm_last_error(handle, buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc: int, handle=None, what: str = "") -> None:
    if rc != MPM_OK:
        raise MpmError(f"{what} failed (code {rc}): {last_error(handle)}")
