"""ctypes binding of libvenusaur_gb300.so (the C ABI in include/venu.h).

There is no fallback: if the library is missing or does not load, every
entry point raises VenuError.  Build it with ``python -c "import
__graft_entry__ as g; g.build()"`` or ``python venusaur_gb300/build.py``.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libvenusaur_gb300.so")

SPHERE_DTYPE = np.dtype([
    ("center", "<f4", (3,)), ("radius", "<f4"), ("albedo", "<f4", (3,)),
    ("fuzz", "<f4"), ("ir", "<f4"), ("material", "<u4"), ("pad", "<u4", (2,)),
])
CAMERA_DTYPE = np.dtype([
    ("origin", "<f4", (3,)), ("u", "<f4", (3,)), ("v", "<f4", (3,)),
    ("w", "<f4", (3,)), ("lens_radius", "<f4"),
])
NODE_DTYPE = np.dtype([("lo", "<f4", (3,)), ("left", "<i4"), ("hi", "<f4", (3,)), ("right", "<i4")])

STATUS = {
    0: "VENU_OK", 1: "VENU_ERR_INVALID", 2: "VENU_ERR_CUDA", 3: "VENU_ERR_OOM",
    4: "VENU_ERR_NO_DEVICE", 5: "VENU_ERR_STACK", 6: "VENU_ERR_TIMEOUT",
    7: "VENU_ERR_CANCELLED", 8: "VENU_ERR_TOO_LARGE", 9: "VENU_ERR_NOT_READY",
}
FLAG_RESET_ACCUM = 1
RENDERER_COUNT = 1
RENDERER_PROFILE = 2
ACCUM_FLOATS = 8


class VenuError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class RenderOpts(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("samples_per_pixel", C.c_uint32),
                ("subframe_index", C.c_uint32), ("max_depth", C.c_uint32), ("flags", C.c_uint32)]


class SceneInfo(C.Structure):
    _fields_ = [("num_spheres", C.c_uint32), ("num_nodes", C.c_uint32), ("device_bytes", C.c_uint64),
                ("bounds", C.c_float * 6), ("build_ms", C.c_float), ("num_wide_nodes", C.c_uint32),
                ("wide_ms", C.c_float)]


class RenderStats(C.Structure):
    _fields_ = [("segments", C.c_uint64), ("paths", C.c_uint64), ("waves", C.c_uint32),
                ("kernel_launches", C.c_uint32), ("nodes_visited", C.c_uint64),
                ("spheres_tested", C.c_uint64), ("traverse_ms", C.c_float), ("shade_ms", C.c_float),
                ("traverse_launches", C.c_uint32), ("shade_launches", C.c_uint32),
                ("lane_steps", C.c_uint64), ("warp_steps", C.c_uint64)]


class Tuning(C.Structure):
    _fields_ = [("traverse_variant", C.c_uint32), ("refill_min", C.c_uint32), ("traverse_block", C.c_uint32),
                ("traverse_blocks_per_sm", C.c_uint32), ("shade_block", C.c_uint32),
                ("shade_blocks_per_sm", C.c_uint32), ("in_place_factor", C.c_uint32)]


class CameraC(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("u", C.c_float * 3), ("v", C.c_float * 3), ("w", C.c_float * 3),
                ("lens_radius", C.c_float)]


class JobDesc(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("camera", CameraC), ("opts", RenderOpts), ("accum", C.c_void_p),
                ("image_f", C.c_void_p), ("image8", C.c_void_p)]


class BatchStats(C.Structure):
    _fields_ = [("segments", C.c_uint64), ("paths_done", C.c_uint64), ("iterations", C.c_uint64),
                ("graph_launches", C.c_uint64), ("resident_bytes", C.c_uint64), ("active_jobs", C.c_uint32),
                ("reserved", C.c_uint32)]


class Request(C.Structure):
    _fields_ = [("spheres", C.c_void_p), ("num_spheres", C.c_uint32), ("reserved", C.c_uint32),
                ("scene_key", C.c_uint64), ("camera", CameraC), ("opts", RenderOpts), ("tag", C.c_uint64),
                ("session", C.c_uint64)]


class Result(C.Structure):
    _fields_ = [("request_id", C.c_uint64), ("tag", C.c_uint64), ("status", C.c_int32), ("width", C.c_uint32),
                ("height", C.c_uint32), ("reserved", C.c_uint32), ("image8", C.c_void_p), ("t_submit", C.c_double),
                ("t_admit", C.c_double), ("t_done", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("failed", C.c_uint64),
                ("resident_bytes", C.c_uint64), ("budget_bytes", C.c_uint64), ("segments", C.c_uint64),
                ("active", C.c_uint32), ("pending", C.c_uint32), ("p50_ms", C.c_double), ("p99_ms", C.c_double),
                ("busy_seconds", C.c_double), ("evictions", C.c_uint64), ("admission_waits", C.c_uint64),
                ("peak_resident_bytes", C.c_uint64)]


BATCH_NO_GRAPH = 1
RUN_STOP_ON_FINISH = 1
POLICY_FIFO = 0
POLICY_SHORTEST_FIRST = 1
POLICY_SEQUENTIAL = 2
POLICIES = {"fifo": POLICY_FIFO, "shortest_first": POLICY_SHORTEST_FIRST, "sequential": POLICY_SEQUENTIAL}
INJECT_ALLOC = 1
INJECT_SCENE = 2

_lib = None


def lib() -> C.CDLL:
    """Loads the library once; raises VenuError if it is not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise VenuError(4, f"{LIB_PATH} is missing: build the CUDA library first "
                           "(python venusaur_gb300/build.py)")
    L = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    u32 = C.c_uint32
    L.venu_last_error.restype = C.c_char_p
    L.venu_scene_generate_rtiow.restype = u32
    L.venu_scene_generate_rtiow.argtypes = [u32, vp, u32]
    L.venu_scene_generate_random.argtypes = [u32, u32, vp, vp, C.c_float, C.c_float, vp]
    L.venu_camera_look_at.restype = None
    L.venu_camera_look_at.argtypes = [vp, vp, C.c_float, C.c_float, C.c_float, C.c_float, vp]
    L.venu_camera_frame.restype = None
    L.venu_camera_frame.argtypes = [vp, vp, C.c_float, C.c_float, C.c_float, C.c_float, vp]
    L.venu_camera_rotate.restype = None
    L.venu_image_write_ppm.restype = C.c_int
    L.venu_image_write_ppm.argtypes = [C.c_char_p, vp, C.c_uint32, C.c_uint32]
    L.venu_image_write_pfm.restype = C.c_int
    L.venu_image_write_pfm.argtypes = [C.c_char_p, vp, C.c_uint32, C.c_uint32]
    L.venu_camera_rotate.argtypes = [vp, vp, C.c_float, vp]
    L.venu_device_check.argtypes = [vp, vp, vp]
    L.venu_scene_create.argtypes = [vp, u32, vp, C.POINTER(vp)]
    L.venu_scene_update.restype = C.c_int
    L.venu_scene_update.argtypes = [vp, vp, C.c_uint32, vp]
    L.venu_scene_update_device.restype = C.c_int
    L.venu_scene_update_device.argtypes = [vp, vp, C.c_uint32, vp]
    L.venu_scene_create_device.argtypes = [vp, u32, vp, C.POINTER(vp)]
    L.venu_scene_info_get.argtypes = [vp, C.POINTER(SceneInfo)]
    L.venu_scene_export_bvh.argtypes = [vp, vp, vp, vp]
    L.venu_scene_destroy.argtypes = [vp]
    L.venu_trace.argtypes = [vp, vp, u32, C.c_float, C.c_float, vp, vp, vp, vp]
    L.venu_renderer_create.argtypes = [u32, u32, C.POINTER(vp)]
    L.venu_render.argtypes = [vp, vp, vp, C.POINTER(RenderOpts), vp, vp, vp, vp]
    L.venu_renderer_stats.argtypes = [vp, C.POINTER(RenderStats)]
    L.venu_renderer_destroy.argtypes = [vp]
    L.venu_server_create.argtypes = [C.c_uint64, u32, u32, u32, C.POINTER(vp)]
    L.venu_server_submit.argtypes = [vp, C.POINTER(Request), C.POINTER(C.c_uint64)]
    L.venu_server_wait.argtypes = [vp, C.c_uint64, C.c_double, C.POINTER(Result)]
    L.venu_server_cancel.argtypes = [vp, C.c_uint64]
    L.venu_server_release.argtypes = [vp, C.c_uint64]
    L.venu_server_inject.argtypes = [vp, u32]
    L.venu_server_stats_get.argtypes = [vp, C.POINTER(ServerStats)]
    L.venu_server_destroy.argtypes = [vp]
    L.venu_batch_create.argtypes = [u32, u32, u32, C.POINTER(vp)]
    L.venu_batch_set_tuning.argtypes = [vp, C.POINTER(Tuning)]
    L.venu_batch_job_bytes.restype = C.c_uint64
    L.venu_batch_job_bytes.argtypes = [u32, u32, u32]
    L.venu_batch_submit.argtypes = [vp, C.POINTER(JobDesc), vp, C.POINTER(u32)]
    L.venu_batch_submit_many.argtypes = [vp, C.POINTER(JobDesc), u32, vp, C.POINTER(u32)]
    L.venu_batch_run.argtypes = [vp, u32, u32, vp]
    L.venu_batch_collect.argtypes = [vp, vp, vp, u32, C.POINTER(u32)]
    L.venu_batch_stats_get.argtypes = [vp, C.POINTER(BatchStats)]
    L.venu_batch_destroy.argtypes = [vp]
    L.venu_batch_set_policy.argtypes = [vp, u32]
    L.venu_batch_interrupt.argtypes = [vp, u32]
    L.venu_batch_set_chunk.argtypes = [vp, u32]
    L.venu_server_set_policy.argtypes = [vp, u32]
    L.venu_server_set_express.argtypes = [vp, C.c_uint64]
    L.venu_server_end_session.argtypes = [vp, C.c_uint64]
    L.venu_renderer_set_tuning.argtypes = [vp, C.POINTER(Tuning)]
    L.venu_renderer_get_tuning.argtypes = [vp, C.POINTER(Tuning)]
    L.venu_selftest_rng.argtypes = [vp, vp, u32, vp, u32, u32, vp, vp, vp]
    L.venu_selftest_srgb_pow.argtypes = [vp, C.c_uint64, u32, vp, vp]
    for name in ("venu_selftest_rng", "venu_selftest_srgb_pow","venu_device_check", "venu_scene_generate_random", "venu_scene_create",
                 "venu_scene_create_device", "venu_scene_update", "venu_scene_update_device",
                 "venu_scene_info_get", "venu_scene_export_bvh",
                 "venu_scene_destroy", "venu_trace", "venu_renderer_create", "venu_render",
                 "venu_renderer_stats", "venu_renderer_destroy", "venu_renderer_set_tuning",
                 "venu_renderer_get_tuning", "venu_batch_create", "venu_batch_set_tuning", "venu_batch_submit", "venu_batch_submit_many",
                 "venu_batch_run", "venu_batch_collect", "venu_batch_stats_get", "venu_batch_destroy",
                 "venu_batch_set_policy", "venu_batch_interrupt", "venu_batch_set_chunk", "venu_server_set_policy", "venu_server_set_express", "venu_server_end_session",
                 "venu_server_create", "venu_server_submit", "venu_server_wait", "venu_server_cancel",
                 "venu_server_release", "venu_server_inject", "venu_server_stats_get", "venu_server_destroy"):
        getattr(L, name).restype = C.c_int
    _lib = L
    return L


def check(status: int) -> None:
    if status != 0:
        msg = lib().venu_last_error()
        raise VenuError(status, msg.decode() if msg else "")


def ptr(a) -> C.c_void_p | None:
    """Address of a numpy array or torch tensor (None passes NULL)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return C.c_void_p(a.ctypes.data)
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    if isinstance(a, int):
        return C.c_void_p(a)
    raise TypeError(f"cannot take the address of {type(a)}")
