"""ctypes binding of libdrgb.so (include/drgb.h).

The library is built in-tree (diffrender_tutorials_gb300/_build/libdrgb.so)
by build.py.  There is no fallback: every renderer call goes through the
CUDA library, and loading fails loudly when it is missing.
"""
import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libdrgb.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "drgb.h")

DRGB_OK = 0
# renderer / batch options (drgb_renderer_set_option, drgb_batch_set_option)
OPT_TRACE_BRUTEFORCE, OPT_TILE_W, OPT_TILE_H, OPT_USE_GRAPH, OPT_DETERMINISTIC, OPT_ADJOINT_HITS = 1, 2, 3, 4, 5, 6
OPT_PIXEL_GRID, OPT_EDGE_GRID, OPT_BVH_BUILDER, OPT_BVH_REBUILD = 7, 8, 9, 10
OPT_TRACE_STEP_LIMIT, OPT_EDGE_JACOBIAN, OPT_EDGE_SET, OPT_PRIMARY_RASTER = 11, 12, 13, 14
ERR_INVALID, ERR_CUDA, ERR_OOM, ERR_STATE, ERR_KERNEL, ERR_UNSUPPORTED, ERR_NO_DEVICE = -1, -2, -3, -4, -5, -6, -7
ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "out of device memory", -4: "bad call order",
          -5: "kernel error flag", -6: "unsupported", -7: "no CUDA device"}


class DrgbError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"drgb error {code} ({ERRORS.get(code, '?')}): {msg}")
        self.code = code


class Camera(C.Structure):
    _fields_ = [("world_view", C.c_float * 16), ("proj", C.c_float * 16), ("width", C.c_float), ("height", C.c_float)]


class MeshDesc(C.Structure):
    _fields_ = [("n_vertices", C.c_int32), ("n_indices", C.c_int32), ("vertices", C.c_void_p),
                ("colors", C.c_void_p), ("tc", C.c_void_p), ("normals", C.c_void_p), ("tangents", C.c_void_p),
                ("indices", C.c_void_p), ("n_instances", C.c_int32), ("transforms", C.c_void_p),
                ("tex_w", C.c_int32), ("tex_h", C.c_int32), ("tex_channels", C.c_int32), ("texture", C.c_void_p),
                ("restricted", C.c_void_p)]


class SceneDesc(C.Structure):
    _fields_ = [("n_meshes", C.c_int32), ("meshes", C.POINTER(MeshDesc))]


class ModelParams(C.Structure):
    _fields_ = [("light_pos", C.c_float * 3), ("light_intensity", C.c_float), ("ambient", C.c_float),
                ("path_depth", C.c_int32), ("seed", C.c_uint32)]


class OptParams(C.Structure):
    _fields_ = [("alg", C.c_int32), ("decay_period", C.c_int32), ("decay_mult", C.c_float),
                ("base_lr", C.c_float), ("position_lr", C.c_float), ("textures_lr", C.c_float),
                ("transforms_lr", C.c_float), ("flags", C.c_int32), ("n_dmesh_ids", C.c_int32),
                ("dmesh_ids", C.c_int32 * 16)]


class ServerConfig(C.Structure):
    _fields_ = [("device", C.c_int32), ("max_jobs", C.c_int32), ("hbm_budget_bytes", C.c_int64),
                ("start_worker", C.c_int32), ("deterministic", C.c_int32)]


class JobInfo(C.Structure):
    _fields_ = [("state", C.c_int32), ("error", C.c_int32), ("steps", C.c_int64), ("steps_done", C.c_int64),
                ("t_submit", C.c_double), ("t_admit", C.c_double), ("t_done", C.c_double),
                ("device_bytes", C.c_int64), ("final_loss", C.c_float)]


class ServerStats(C.Structure):
    _fields_ = [("queued", C.c_int32), ("running", C.c_int32), ("done", C.c_int32), ("failed", C.c_int32),
                ("bytes_in_use", C.c_int64), ("bytes_budget", C.c_int64), ("bytes_peak", C.c_int64),
                ("batch_steps", C.c_int64), ("job_iterations", C.c_int64), ("busy_seconds", C.c_double),
                ("now", C.c_double)]


VP = C.c_void_p
_SIGS = {
    "drgb_abi_version": (C.c_int, []),
    "drgb_last_error": (C.c_int, [C.c_char_p, C.c_size_t]),
    "drgb_kernel_launches": (C.c_int64, []),
    "drgb_debug_exclusive_scan": (C.c_int, [VP, C.c_int, VP]),
    "drgb_camera_look_at": (C.c_int, [VP, VP, VP, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float,
                                      C.POINTER(Camera)]),
    "drgb_renderer_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.POINTER(VP)]),
    "drgb_renderer_destroy": (C.c_int, [VP]),
    "drgb_renderer_set_option": (C.c_int, [VP, C.c_int, C.c_int64]),
    "drgb_renderer_set_model_params": (C.c_int, [VP, C.POINTER(ModelParams)]),
    "drgb_renderer_stream": (VP, [VP]),
    "drgb_commit": (C.c_int, [VP, C.POINTER(SceneDesc)]),
    "drgb_render": (C.c_int, [VP, C.POINTER(Camera), C.c_int, VP]),
    "drgb_dscene_layout": (C.c_int, [VP, VP, C.c_int, VP, C.POINTER(C.c_int64)]),
    "drgb_d_render": (C.c_int, [VP, C.POINTER(Camera), VP, C.c_int, C.c_int, VP, C.c_int, VP]),
    "drgb_d_render_and_compare": (C.c_int, [VP, C.POINTER(Camera), VP, C.c_int, C.c_int, VP, C.c_int, VP, VP, VP]),
    "drgb_d_render_and_compare_device": (C.c_int, [VP, C.POINTER(Camera), VP, C.c_int, C.c_int, VP, C.c_int, VP,
                                                   VP, VP]),
    "drgb_d_render_and_compare_noalloc": (C.c_int, [VP, C.POINTER(Camera), VP, C.c_int, C.c_int, VP, C.c_int, VP,
                                                    VP]),
    "drgb_cast_rays": (C.c_int, [VP, C.POINTER(Camera), VP, C.c_int64, VP, VP, VP, VP, VP, VP]),
    "drgb_opt_params_default": (C.c_int, [C.c_int, C.POINTER(OptParams)]),
    "drgb_optimizer_init": (C.c_int, [VP, C.POINTER(SceneDesc), C.POINTER(Camera), VP, C.c_int,
                                      C.POINTER(OptParams)]),
    "drgb_optimizer_run": (C.c_int, [VP, C.c_int64, VP, VP]),
    "drgb_optimizer_run_async": (C.c_int, [VP, C.c_int64]),
    "drgb_optimizer_get_mesh": (C.c_int, [VP, C.c_int, VP, VP, VP, VP]),
    "drgb_optimizer_get_restricted": (C.c_int, [VP, C.c_int, VP]),
    "drgb_batch_create": (C.c_int, [C.c_int, C.POINTER(VP)]),
    "drgb_batch_destroy": (C.c_int, [VP]),
    "drgb_batch_stream": (VP, [VP]),
    "drgb_batch_add_job": (C.c_int, [VP, C.c_int, C.c_int, C.POINTER(ModelParams), C.POINTER(SceneDesc),
                                     C.POINTER(Camera), VP, C.c_int, C.POINTER(OptParams), C.POINTER(C.c_int32)]),
    "drgb_batch_remove_job": (C.c_int, [VP, C.c_int32]),
    "drgb_batch_size": (C.c_int, [VP]),
    "drgb_batch_set_option": (C.c_int, [VP, C.c_int, C.c_int64]),
    "drgb_batch_run_async": (C.c_int, [VP, C.c_int64]),
    "drgb_batch_run": (C.c_int, [VP, C.c_int64]),
    "drgb_batch_sync": (C.c_int, [VP]),
    "drgb_batch_job_losses": (C.c_int, [VP, C.c_int32, C.c_int64, C.c_int64, VP, C.POINTER(C.c_int64)]),
    "drgb_batch_get_mesh": (C.c_int, [VP, C.c_int32, C.c_int, VP, VP, VP, VP]),
    "drgb_batch_get_restricted": (C.c_int, [VP, C.c_int32, C.c_int, VP]),
    "drgb_batch_job_device_bytes": (C.c_int64, [VP, C.c_int32]),
    "drgb_server_create": (C.c_int, [C.POINTER(ServerConfig), C.POINTER(VP)]),
    "drgb_server_destroy": (C.c_int, [VP]),
    "drgb_server_submit": (C.c_int, [VP, C.c_int, C.c_int, C.POINTER(ModelParams), C.POINTER(SceneDesc),
                                     C.POINTER(Camera), VP, C.c_int, C.POINTER(OptParams), C.c_int64,
                                     C.POINTER(C.c_int32)]),
    "drgb_server_step": (C.c_int, [VP, C.POINTER(C.c_int32)]),
    "drgb_server_wait": (C.c_int, [VP, C.c_int32, C.c_double]),
    "drgb_server_job_info": (C.c_int, [VP, C.c_int32, C.POINTER(JobInfo)]),
    "drgb_server_job_losses": (C.c_int, [VP, C.c_int32, C.c_int64, C.c_int64, VP]),
    "drgb_server_get_mesh": (C.c_int, [VP, C.c_int32, C.c_int, VP, VP, VP, VP]),
    "drgb_server_get_restricted": (C.c_int, [VP, C.c_int32, C.c_int, VP]),
    "drgb_server_release": (C.c_int, [VP, C.c_int32]),
    "drgb_server_get_stats": (C.c_int, [VP, C.POINTER(ServerStats)]),
    "drgb_server_step_times": (C.c_int, [VP, C.c_int64, C.c_int64, VP, VP]),
    "drgb_estimate_job_bytes": (C.c_int64, [C.c_int, C.c_int, C.POINTER(SceneDesc), C.POINTER(Camera), C.c_int]),
    "drgb_optimizer_profile": (C.c_int, [VP, C.c_int, VP]),
    "drgb_count_work": (C.c_int, [VP, VP]),
    "drgb_optimizer_autotune": (C.c_int, [VP, C.c_int, VP, C.POINTER(C.c_float)]),
    "drgb_batch_autotune": (C.c_int, [VP, C.c_int, VP, C.POINTER(C.c_float)]),
}

_lib = None


def header_functions():
    """Names of the functions declared in include/drgb.h."""
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(drgb_[a-z0-9_]+)\s*\(", text)))


def load(path=None):
    """Load libdrgb.so (building it first when it is absent) and set signatures."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or os.environ.get("DRGB_LIB") or LIB_PATH
    if not os.path.exists(path):
        from . import build as _build
        _build.build()
    if not os.path.exists(path):
        raise OSError(f"libdrgb.so not found at {path}; run diffrender_tutorials_gb300.build.build()")
    lib = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def last_error():
    buf = C.create_string_buffer(1024)
    load().drgb_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(code):
    if code != DRGB_OK:
        raise DrgbError(code, last_error())
    return code
