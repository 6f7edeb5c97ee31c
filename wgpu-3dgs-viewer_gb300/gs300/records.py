"""numpy views of the byte layouts in include/gs_record.h.

The structured dtypes below are byte-for-byte the C structs, so a numpy array of them can be
handed to the C ABI (or uploaded to the device) without conversion.
"""
import ctypes

import numpy as np

DISPLAY_SPLAT = 0
DISPLAY_ELLIPSE = 1
DISPLAY_POINT = 2

FORMAT_FP32 = 0
FORMAT_HALF_SH_FP16 = 1
FORMAT_HALF_SH_BF16 = 2

TILE = 16
SORT_BLOCK_KVS = 3840

# core::Gaussian (tests/e2e/viewer.rs:74-80)
GAUSSIAN_DTYPE = np.dtype(
    [("rot", "<f4", 4), ("pos", "<f4", 3), ("color", "u1", 4), ("sh", "<f4", 45), ("scale", "<f4", 3)]
)

# gs_gaussian_pod: 224 B
GAUSSIAN_POD_DTYPE = np.dtype(
    [("pos", "<f4", 3), ("color", "<u4"), ("sh", "<f4", 45), ("cov3d", "<f4", 6), ("_pad", "<u4")]
)
assert GAUSSIAN_POD_DTYPE.itemsize == 224

# gs_gaussian_pod_half: 128 B
GAUSSIAN_POD_HALF_DTYPE = np.dtype(
    [
        ("pos", "<f4", 3),
        ("color", "<u4"),
        ("rot", "<u2", 4),
        ("scale", "<u2", 3),
        ("sh", "<u2", 45),
        ("_pad", "<u2", 4),
    ]
)
assert GAUSSIAN_POD_HALF_DTYPE.itemsize == 128

# gs_splat: 48 B
SPLAT_DTYPE = np.dtype(
    [("cx", "<f4"), ("cy", "<f4"), ("ex", "<f4"), ("ey", "<f4"), ("q", "<f4", 4), ("s255", "<f4", 3), ("alpha", "<f4")]
)
assert SPLAT_DTYPE.itemsize == 48


class PlyLayout(ctypes.Structure):
    """gs_ply_layout: where the fields of one PLY vertex lie (byte offsets; -1 = absent)."""

    _fields_ = [
        ("data_offset", ctypes.c_uint64),
        ("count", ctypes.c_uint32),
        ("stride", ctypes.c_uint32),
        ("sh_rest", ctypes.c_uint32),
        ("pos", ctypes.c_int32 * 3),
        ("f_dc", ctypes.c_int32 * 3),
        ("opacity", ctypes.c_int32),
        ("scale", ctypes.c_int32 * 3),
        ("rot", ctypes.c_int32 * 4),
        ("f_rest", ctypes.c_int32 * 45),
    ]


class Camera(ctypes.Structure):
    """gs_camera (src/camera.rs:16-29)."""

    _fields_ = [
        ("pos", ctypes.c_float * 3),
        ("z_near", ctypes.c_float),
        ("z_far", ctypes.c_float),
        ("vertical_fov", ctypes.c_float),
        ("pitch", ctypes.c_float),
        ("yaw", ctypes.c_float),
    ]

    @staticmethod
    def new(z_near, z_far, vertical_fov, pos=(0.0, 0.0, 0.0), pitch=0.0, yaw=0.0):
        return Camera((ctypes.c_float * 3)(*pos), z_near, z_far, vertical_fov, pitch, yaw)


class CameraPod(ctypes.Structure):
    """gs_camera_pod = CameraPod (src/buffer/camera.rs:153-161), 144 B."""

    _fields_ = [
        ("view", ctypes.c_float * 16),
        ("proj", ctypes.c_float * 16),
        ("size", ctypes.c_float * 2),
        ("_padding", ctypes.c_uint32 * 2),
    ]

    def __eq__(self, other):
        return bytes(self) == bytes(other)


class ModelTransformPod(ctypes.Structure):
    _fields_ = [
        ("pos", ctypes.c_float * 3),
        ("_pad0", ctypes.c_float),
        ("rot", ctypes.c_float * 4),
        ("scale", ctypes.c_float * 3),
        ("_pad1", ctypes.c_float),
    ]

    @staticmethod
    def new(pos=(0.0, 0.0, 0.0), rot=(0.0, 0.0, 0.0, 1.0), scale=(1.0, 1.0, 1.0)):
        p = ModelTransformPod()
        p.pos[:] = list(pos)
        p.rot[:] = list(rot)
        p.scale[:] = list(scale)
        return p


class GaussianTransformPod(ctypes.Structure):
    _fields_ = [
        ("size", ctypes.c_float),
        ("display_mode", ctypes.c_uint32),
        ("sh_deg", ctypes.c_uint32),
        ("no_sh0", ctypes.c_uint32),
        ("max_std_dev", ctypes.c_float),
        ("_pad", ctypes.c_uint32 * 3),
    ]

    @staticmethod
    def new(size=1.0, display_mode=DISPLAY_SPLAT, sh_deg=3, no_sh0=False, max_std_dev=3.0):
        return GaussianTransformPod(size, display_mode, sh_deg, int(bool(no_sh0)), max_std_dev)


class FrameUniforms(ctypes.Structure):
    _fields_ = [
        ("pv", ctypes.c_float * 16),
        ("vm", ctypes.c_float * 16),
        ("model", ctypes.c_float * 16),
        ("wsr", ctypes.c_float * 9),
        ("inv_sr", ctypes.c_float * 9),
        ("cam_pos", ctypes.c_float * 3),
        ("size", ctypes.c_float * 2),
        ("focal", ctypes.c_float * 2),
        ("viewport", ctypes.c_float * 2),
        ("std_dev", ctypes.c_float),
        ("std_dev_scaled", ctypes.c_float),
        ("point_size", ctypes.c_float),
        ("display_mode", ctypes.c_uint32),
        ("sh_deg", ctypes.c_uint32),
        ("no_sh0", ctypes.c_uint32),
        ("_pad", ctypes.c_uint32 * 2),
    ]


def record_dtype(fmt):
    return GAUSSIAN_POD_DTYPE if fmt == FORMAT_FP32 else GAUSSIAN_POD_HALF_DTYPE


def sh_degree_checked(deg):
    """GaussianShDegree::new: 0..=3."""
    if not (0 <= int(deg) <= 3):
        raise ValueError(f"SH degree {deg} out of range 0..=3")
    return int(deg)


class BatchView(ctypes.Structure):
    """gs_batch_view: one view of a batch (model index, RGBA8 target, camera)."""

    _fields_ = [
        ("model", ctypes.c_uint32),
        ("width", ctypes.c_uint32),
        ("height", ctypes.c_uint32),
        ("pitch", ctypes.c_uint32),
        ("target", ctypes.c_void_p),
        ("camera", CameraPod),
    ]


class Tuning(ctypes.Structure):
    """gs_tuning: launch choices of a batch that change its speed, never its frames."""

    _fields_ = [
        ("suffix_min", ctypes.c_uint32),
        ("eps", ctypes.c_float),
        ("views_per_launch", ctypes.c_uint32),
        ("streams", ctypes.c_uint32),
        ("sort_match", ctypes.c_uint32),
        ("hist_blocks", ctypes.c_uint32),
        ("raster_grid", ctypes.c_uint32),
        ("sort_digit_bits", ctypes.c_uint32),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class ServerReport(ctypes.Structure):
    """gs_server_report: request counts and submit-to-completion latency percentiles."""

    _fields_ = [
        ("completed", ctypes.c_uint64),
        ("failed", ctypes.c_uint64),
        ("queued", ctypes.c_uint32),
        ("running", ctypes.c_uint32),
        ("reserved_bytes", ctypes.c_uint64),
        ("p50_ms", ctypes.c_double),
        ("p99_ms", ctypes.c_double),
        ("mean_ms", ctypes.c_double),
        ("max_ms", ctypes.c_double),
    ]
