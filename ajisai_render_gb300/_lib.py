"""ctypes binding of libajisai_gpu.so (include/ajisai_gpu.h).

The library is loaded from the package's _build directory.  There is no CPU
fallback: if the shared library is missing, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libajisai_gpu.so"

AJG_OK = 0
STATUS = {0: "AJG_OK", 1: "AJG_ERR_INVALID", 2: "AJG_ERR_CUDA", 3: "AJG_ERR_OOM",
          4: "AJG_ERR_UNSUPPORTED", 5: "AJG_ERR_DEVICE", 6: "AJG_ERR_NOT_FOUND",
          7: "AJG_ERR_CANCELLED", 8: "AJG_ERR_TIMEOUT"}
AJG_ERR_CANCELLED = 7
AJG_ERR_TIMEOUT = 8
JOB_STATES = {0: "queued", 1: "running", 2: "done", 3: "cancelled", 4: "failed"}
SCHED_FAIR, SCHED_FIFO = 0, 1


class AjgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class Config(C.Structure):
    _fields_ = [("device", C.c_int32), ("wave_paths", C.c_uint32),
                ("hbm_budget_bytes", C.c_uint64)]


class MeshDesc(C.Structure):
    _fields_ = [("positions", C.c_void_p), ("normals", C.c_void_p),
                ("indices", C.c_void_p), ("num_vertices", C.c_uint32),
                ("num_triangles", C.c_uint32), ("material", C.c_uint32),
                ("flags", C.c_uint32)]


class Material(C.Structure):
    _fields_ = [("type", C.c_uint32), ("base_color", C.c_float * 3),
                ("params", C.c_float * 10), ("pad", C.c_float * 2)]


class Light(C.Structure):
    _fields_ = [("type", C.c_uint32), ("rgb", C.c_float * 3),
                ("direction", C.c_float * 3), ("cos_angle", C.c_float),
                ("scaler", C.c_float), ("rot_deg", C.c_float),
                ("pad", C.c_float * 2)]


class Emitter(C.Structure):
    _fields_ = [("radiance", C.c_float * 3), ("first_triangle", C.c_uint32),
                ("num_triangles", C.c_uint32), ("geometry", C.c_uint32),
                ("two_sided", C.c_uint32), ("reserved", C.c_uint32)]


class SppmParams(C.Structure):
    _fields_ = [("iterations", C.c_uint32), ("photons_per_iteration", C.c_uint32),
                ("forward_max_depth", C.c_int32), ("photon_min_depth", C.c_int32),
                ("photon_max_depth", C.c_int32), ("photon_cont_prob", C.c_float),
                ("init_radius", C.c_float), ("update_alpha", C.c_float),
                ("seed", C.c_uint64)]


class SceneOpts(C.Structure):
    _fields_ = [("search_radius", C.c_uint32), ("tri_test", C.c_uint32),
                ("radix_compat", C.c_uint32), ("bvh_width", C.c_uint32)]


class Camera(C.Structure):
    _fields_ = [("raster2camera", C.c_float * 16), ("camera2world", C.c_float * 16),
                ("lens_radius", C.c_float), ("focal_distance", C.c_float),
                ("width", C.c_uint32), ("height", C.c_uint32)]


class RenderParams(C.Structure):
    _fields_ = [("spp", C.c_uint32), ("min_bounces", C.c_int32),
                ("max_bounces", C.c_int32), ("cont_prob", C.c_float),
                ("use_mis", C.c_uint32), ("flags", C.c_uint32),
                ("seed", C.c_uint64)]


class SceneInfo(C.Structure):
    _fields_ = [("num_triangles", C.c_uint64), ("num_nodes", C.c_uint64),
                ("device_bytes", C.c_uint64), ("ploc_iterations", C.c_uint32),
                ("build_ms", C.c_float), ("bvh_width", C.c_uint32),
                ("bvh_node_bytes", C.c_uint32), ("bvh_nodes", C.c_uint64),
                ("closest_node_bytes", C.c_uint32), ("reserved", C.c_uint32)]


class Stats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in (
        "closest_rays", "any_rays", "nodes_visited", "tris_tested",
        "closest_nodes", "closest_tris", "any_nodes", "any_tris", "paths",
        "kernel_launches", "closest_launches", "any_launches",
        "shade_launches")] + [(n, C.c_double) for n in (
            "closest_ms", "any_ms", "shade_ms")]


class LaunchRecord(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("ms", C.c_float), ("rays", C.c_uint64),
                ("nodes", C.c_uint64), ("tris", C.c_uint64)]


class JobDesc(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("camera", Camera), ("params", RenderParams),
                ("window", C.c_uint32 * 4), ("progress_spp", C.c_uint32),
                ("reserved", C.c_uint32), ("out_rgbw", C.c_void_p),
                ("d_out_rgbw", C.c_void_p)]


class JobStatus(C.Structure):
    _fields_ = [("state", C.c_uint32), ("spp_done", C.c_uint32),
                ("spp_total", C.c_uint32), ("updates", C.c_uint32),
                ("error", C.c_int32), ("reserved", C.c_uint32),
                ("submit_ms", C.c_double), ("start_ms", C.c_double),
                ("first_result_ms", C.c_double), ("done_ms", C.c_double)]


class ServeOpts(C.Structure):
    _fields_ = [("policy", C.c_uint32), ("max_active_jobs", C.c_uint32),
                ("inflight_waves", C.c_uint32), ("wave_paths", C.c_uint32)]


class ServeStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in (
        "jobs_submitted", "jobs_done", "jobs_cancelled", "jobs_failed", "waves",
        "paths", "results_delivered", "graph_builds", "kernel_launches",
        "active_bytes")] + [("busy_ms", C.c_double)]


assert C.sizeof(Material) == 64 and C.sizeof(Light) == 48
assert C.sizeof(LaunchRecord) == 32
assert C.sizeof(Camera) == 144 and C.sizeof(RenderParams) == 32

_P = C.c_void_p
SIGNATURES = {
    "ajg_abi_version": ([], C.c_int),
    "ajg_create_context": ([C.POINTER(Config), C.POINTER(_P)], C.c_int),
    "ajg_destroy_context": ([_P], C.c_int),
    "ajg_last_error": ([_P], C.c_char_p),
    "ajg_get_stats": ([_P, C.POINTER(Stats), C.c_int], C.c_int),
    "ajg_set_profiling": ([_P, C.c_int], C.c_int),
    "ajg_get_launch_log": ([_P, C.POINTER(LaunchRecord), C.c_uint32,
                            C.POINTER(C.c_uint32), C.c_int], C.c_int),
    "ajg_scene_create": ([_P, C.POINTER(MeshDesc), C.c_uint32, C.POINTER(Material),
                          C.c_uint32, C.POINTER(Light), C.c_uint32,
                          C.POINTER(SceneOpts), C.POINTER(_P)], C.c_int),
    "ajg_scene_create_flat": ([_P, _P, _P, _P, _P, C.c_uint64, _P,
                               C.POINTER(Material), C.c_uint32, C.POINTER(Light),
                               C.c_uint32, C.POINTER(SceneOpts), C.POINTER(_P)],
                              C.c_int),
    "ajg_scene_create_ex": ([_P, C.POINTER(MeshDesc), C.c_uint32, C.POINTER(Material),
                             C.c_uint32, C.POINTER(Light), C.c_uint32,
                             C.POINTER(Emitter), C.c_uint32, C.POINTER(SceneOpts),
                             C.POINTER(_P)], C.c_int),
    "ajg_scene_create_flat_ex": ([_P, _P, _P, _P, _P, C.c_uint64, _P,
                                  C.POINTER(Material), C.c_uint32, C.POINTER(Light),
                                  C.c_uint32, C.POINTER(Emitter), C.c_uint32,
                                  C.POINTER(SceneOpts), C.POINTER(_P)], C.c_int),
    "ajg_scene_release": ([_P], C.c_int),
    "ajg_scene_get_info": ([_P, C.POINTER(SceneInfo)], C.c_int),
    "ajg_scene_download_bvh": ([_P, _P, _P, _P], C.c_int),
    "ajg_trace_closest": ([_P, _P, C.c_uint64, _P], C.c_int),
    "ajg_trace_any": ([_P, _P, C.c_uint64, _P], C.c_int),
    "ajg_trace_closest_device": ([_P, _P, C.c_uint64, _P, _P], C.c_int),
    "ajg_trace_any_device": ([_P, _P, C.c_uint64, _P, _P], C.c_int),
    "ajg_bsdf_query": ([_P, _P, _P, _P, _P, _P, _P, _P, C.c_uint64, _P], C.c_int),
    "ajg_camera_rays": ([_P, C.POINTER(Camera), _P, C.c_uint64, _P], C.c_int),
    "ajg_render": ([_P, C.POINTER(Camera), C.POINTER(RenderParams), _P], C.c_int),
    "ajg_render_sppm": ([_P, C.POINTER(Camera), C.POINTER(SppmParams), _P, _P],
                        C.c_int),
    "ajg_render_device": ([_P, C.POINTER(Camera), C.POINTER(RenderParams), _P, _P],
                          C.c_int),
    "ajg_render_static": ([_P, C.POINTER(Camera), C.POINTER(RenderParams), _P, _P],
                          C.c_int),
    "ajg_render_samples": ([_P, C.POINTER(Camera), C.POINTER(RenderParams),
                            C.c_uint64, C.c_uint64, _P], C.c_int),
    "ajg_serve_configure": ([_P, C.POINTER(ServeOpts)], C.c_int),
    "ajg_submit": ([_P, C.POINTER(JobDesc), C.POINTER(C.c_uint64)], C.c_int),
    "ajg_poll": ([_P, C.c_uint64, C.POINTER(JobStatus)], C.c_int),
    "ajg_wait": ([_P, C.c_uint64, C.c_int32, C.POINTER(JobStatus)], C.c_int),
    "ajg_job_read": ([_P, C.c_uint64, _P, C.POINTER(JobStatus)], C.c_int),
    "ajg_cancel": ([_P, C.c_uint64], C.c_int),
    "ajg_job_release": ([_P, C.c_uint64], C.c_int),
    "ajg_render_batch": ([_P, C.POINTER(JobDesc), C.c_uint32, C.POINTER(JobStatus)],
                         C.c_int),
    "ajg_serve_get_stats": ([_P, C.POINTER(ServeStats)], C.c_int),
    "ajg_image_rmse": ([_P, _P, C.c_uint32, _P, C.c_uint32, C.c_uint32, C.c_uint32,
                        C.POINTER(C.c_double), C.POINTER(C.c_uint64)], C.c_int),
}

class HostSceneView(C.Structure):
    _fields_ = [("num_triangles", C.c_uint64), ("tris", C.c_void_p),
                ("corner_normals", C.c_void_p), ("tri_material", C.c_void_p),
                ("tri_flags", C.c_void_p), ("world", C.c_float * 6),
                ("num_materials", C.c_uint32), ("num_lights", C.c_uint32),
                ("materials", C.c_void_p), ("lights", C.c_void_p),
                ("opts", SceneOpts), ("camera", Camera), ("params", RenderParams),
                ("num_outputs", C.c_uint32), ("num_emitters", C.c_uint32),
                ("outputs", C.POINTER(C.c_char_p)),
                ("emitters", C.POINTER(Emitter)),
                ("renderer", C.c_uint32), ("reserved", C.c_uint32),
                ("sppm", SppmParams)]


HOST_LIB_PATH = HERE / "_build" / "libajisai_host.so"
HOST_SIGNATURES = {
    "ajh_load_scene": ([C.c_char_p, C.POINTER(C.c_void_p), C.c_char_p, C.c_size_t],
                       C.c_int),
    "ajh_scene_view_get": ([C.c_void_p, C.POINTER(HostSceneView)], C.c_int),
    "ajh_scene_free": ([C.c_void_p], None),
    "ajh_write_image": ([C.c_char_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_char_p,
                         C.c_size_t], C.c_int),
}
_host = None


def load_host():
    """The host library (scene files, image output; no CUDA)."""
    global _host
    if _host is not None:
        return _host
    if not HOST_LIB_PATH.exists():
        raise RuntimeError(f"{HOST_LIB_PATH} is missing: build it with "
                           "`python -m ajisai_render_gb300.build`")
    lib = C.CDLL(str(HOST_LIB_PATH))
    for name, (args, res) in HOST_SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _host = lib
    return lib


_lib = None


def load(path: Path | None = None):
    """Load the shared library (raises if it was not built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else Path(os.environ.get("AJG_LIB", LIB_PATH))
    if not p.exists():
        raise RuntimeError(
            f"{p} is missing: build it with `python -m ajisai_render_gb300.build`"
            " (there is no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    if lib.ajg_abi_version() != 1:
        raise RuntimeError("libajisai_gpu ABI version mismatch")
    if path is None:
        _lib = lib
    return lib


def check(rc: int, ctx=None):
    if rc != AJG_OK:
        msg = load().ajg_last_error(ctx)
        raise AjgError(rc, msg.decode() if msg else "")
