"""ctypes binding of libgs300.so (the C ABI in include/gs300.h).

Loading fails loudly when the library has not been built: there is no CPU fallback.
"""
import ctypes
import os

from . import records as R

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libgs300.so")

GS_OK = 0
GS_ERR_INVALID_ARG = 1
GS_ERR_OUT_OF_MEMORY = 2
GS_ERR_NOT_FOUND = 3
GS_ERR_CUDA = 4
GS_ERR_TIMEOUT = 5
GS_ERR_CAPACITY = 6
GS_ERR_ADMISSION = 7

STATUS_NAMES = {
    GS_OK: "GS_OK",
    GS_ERR_INVALID_ARG: "GS_ERR_INVALID_ARG",
    GS_ERR_OUT_OF_MEMORY: "GS_ERR_OUT_OF_MEMORY",
    GS_ERR_NOT_FOUND: "GS_ERR_NOT_FOUND",
    GS_ERR_CUDA: "GS_ERR_CUDA",
    GS_ERR_TIMEOUT: "GS_ERR_TIMEOUT",
    GS_ERR_CAPACITY: "GS_ERR_CAPACITY",
    GS_ERR_ADMISSION: "GS_ERR_ADMISSION",
}

# (name, restype, argtypes) of every exported symbol declared in include/gs300.h.
P = ctypes.c_void_p
U32 = ctypes.c_uint32
I32 = ctypes.c_int
F32 = ctypes.c_float
SZ = ctypes.c_size_t
ST = ctypes.c_int
CP = ctypes.c_char_p
PP = ctypes.POINTER(ctypes.c_void_p)

SIGNATURES = [
    ("gs_last_error", CP, []),
    ("gs_version", CP, []),
    ("gs_launch_count", ctypes.c_uint64, []),
    ("gs_profile_enable", ST, [I32]),
    ("gs_profile_read", ST, [P, P]),
    ("gs_profile_counters", ST, [P]),
    ("gs_camera_view", ST, [P, P]),
    ("gs_camera_projection", ST, [P, F32, P]),
    ("gs_camera_pod_new", ST, [P, U32, U32, P]),
    ("gs_gaussian_transform_pod_new", ST, [F32, U32, U32, I32, F32, P]),
    ("gs_model_transform_pod_new", ST, [P, P, P, P]),
    ("gs_gaussian_pack", ST, [P, SZ, P]),
    ("gs_ply_parse_header", ST, [P, SZ, P]),
    ("gs_ply_convert", ST, [P, P, U32, P, P]),
    ("gs_frame_uniforms_build", ST, [P, P, P, U32, U32, P]),
    ("gs_depth_capacity", U32, [U32]),
    ("gs_preprocess_scratch_bytes", SZ, [U32]),
    ("gs_preprocess", ST, [P, P, U32, U32, P, I32, P, P, P, P, U32, P, P, SZ, P]),
    ("gs_radix_sort_scratch_bytes", SZ, [U32]),
    ("gs_radix_sort", ST, [P, P, U32, P, U32, P, SZ, P]),
    ("gs_radix_sort_no_alloc", ST, [P, P, U32, P, U32, P]),
    ("gs_rasterize_scratch_bytes", SZ, [U32, U32, U32, U32]),
    ("gs_rasterize", ST, [P, P, P, P, U32, P, U32, U32, U32, U32, P, SZ, P]),
    ("gs_scratch_status", ST, [P, P, ctypes.POINTER(U32)]),
    ("gs_debug_set_wait_fault", ST, [U32, U32]),
    ("gs_viewer_create", ST, [P, U32, U32, PP]),
    ("gs_viewer_create_from_ply", ST, [P, SZ, U32, PP]),
    ("gs_viewer_destroy", None, [P]),
    ("gs_viewer_len", U32, [P]),
    ("gs_viewer_update_camera", ST, [P, P, U32, U32]),
    ("gs_viewer_update_camera_with_pod", ST, [P, P]),
    ("gs_viewer_update_model_transform", ST, [P, P, P, P]),
    ("gs_viewer_update_model_transform_with_pod", ST, [P, P]),
    ("gs_viewer_update_gaussian_transform", ST, [P, F32, U32, U32, I32, F32]),
    ("gs_viewer_update_gaussian_transform_with_pod", ST, [P, P]),
    ("gs_viewer_set_selection", ST, [P, P, I32]),
    ("gs_viewer_render", ST, [P, P, U32, U32, U32, P]),
    ("gs_viewer_synchronize", ST, [P, P]),
    ("gs_viewer_stats", ST, [P, P, ctypes.POINTER(U32), ctypes.POINTER(U32)]),
    ("gs_viewer_buffers", ST, [P, PP, PP, PP, PP]),
    ("gs_target_create", ST, [U32, U32, PP]),
    ("gs_target_destroy", None, [P]),
    ("gs_target_data", P, [P]),
    ("gs_target_pitch", U32, [P]),
    ("gs_target_download", ST, [P, P, P]),
    ("gs_target_download_async", ST, [P, P, P]),
    ("gs_multi_viewer_create", ST, [PP]),
    ("gs_multi_viewer_destroy", None, [P]),
    ("gs_multi_viewer_insert_model", ST, [P, CP, P, U32, U32]),
    ("gs_multi_viewer_insert_model_from_ply", ST, [P, CP, P, SZ, U32]),
    ("gs_multi_viewer_remove_model", ST, [P, CP]),
    ("gs_multi_viewer_model_count", U32, [P]),
    ("gs_multi_viewer_update_camera", ST, [P, P, U32, U32]),
    ("gs_multi_viewer_update_camera_with_pod", ST, [P, P]),
    ("gs_multi_viewer_update_model_transform", ST, [P, CP, P, P, P]),
    ("gs_multi_viewer_update_model_transform_with_pod", ST, [P, CP, P]),
    ("gs_multi_viewer_update_gaussian_transform", ST, [P, F32, U32, U32, I32, F32]),
    ("gs_multi_viewer_update_gaussian_transform_with_pod", ST, [P, P]),
    ("gs_multi_viewer_render", ST, [P, ctypes.POINTER(CP), U32, P, U32, U32, U32, P]),
    ("gs_multi_viewer_synchronize", ST, [P, P]),
    ("gs_batch_create", ST, [P, ctypes.POINTER(CP), U32, PP]),
    ("gs_batch_destroy", None, [P]),
    ("gs_batch_render", ST, [P, P, U32, P]),
    ("gs_batch_synchronize", ST, [P, P]),
    ("gs_tuning_default", ST, [P]),
    ("gs_batch_set_tuning", ST, [P, P]),
    ("gs_batch_get_tuning", ST, [P, P]),
    ("gs_batch_autotune", ST, [P, P, U32, U32, U32, P, P]),
    ("gs_server_create", ST, [P, SZ, U32, PP]),
    ("gs_server_destroy", None, [P]),
    ("gs_server_request_bytes", SZ, [U32, U32, U32]),
    ("gs_server_submit", ST, [P, CP, P, U32, U32, P, U32, I32, ctypes.POINTER(ctypes.c_uint64)]),
    ("gs_server_wait", ST, [P, ctypes.c_uint64, ctypes.c_double, ctypes.POINTER(ctypes.c_double)]),
    ("gs_server_stats", ST, [P, P]),
    ("gs_server_reset_stats", ST, [P]),
    ("gs_server_set_batching", ST, [P, U32, ctypes.c_double]),
]

_lib = None


class GsError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class ModelNotFound(GsError):
    """MultiModelViewerAccessError::ModelNotFound (src/error.rs:45-50)."""


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build the CUDA library first "
                "(python -c 'import __graft_entry__ as g; g.build()')"
            )
        L = ctypes.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status):
    if status != GS_OK:
        msg = lib().gs_last_error().decode(errors="replace")
        if status == GS_ERR_NOT_FOUND:
            raise ModelNotFound(status, msg)
        raise GsError(status, msg)


def ref(x):
    """Pointer to a ctypes structure / array."""
    return ctypes.cast(ctypes.byref(x), ctypes.c_void_p)


def FrameUniforms():
    return R.FrameUniforms()
