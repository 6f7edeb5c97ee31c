"""gs300 — Python mirror of wgpu-3dgs-viewer's public API over the GB300 C ABI.

Names, argument meaning and error behaviour follow the crate (wgpu-3dgs-viewer 0.6.1):
  Camera / CameraPod              src/camera.rs, src/buffer/camera.rs
  Viewer                          src/lib.rs:64-275
  MultiModelViewer                src/multi_model.rs:289-531
  Preprocessor / RadixSorter /
  Renderer (stage level)          src/preprocessor.rs, src/radix_sorter.rs, src/renderer.rs
A wgpu TextureView becomes a RenderTarget (a headless RGBA8 device buffer).  Every call goes
through libgs300.so; nothing here computes a frame on the CPU.
"""
import ctypes
import math

import numpy as np

from . import records
from ._lib import GsError, ModelNotFound, check, lib, ref
from .records import (
    DISPLAY_ELLIPSE,
    DISPLAY_POINT,
    DISPLAY_SPLAT,
    FORMAT_FP32,
    FORMAT_HALF_SH_BF16,
    FORMAT_HALF_SH_FP16,
    GAUSSIAN_DTYPE,
    GAUSSIAN_POD_DTYPE,
    GAUSSIAN_POD_HALF_DTYPE,
    SPLAT_DTYPE,
    CameraPod,
    FrameUniforms,
    GaussianTransformPod,
    ModelTransformPod,
)

__all__ = [
    "Camera", "CameraPod", "GaussianTransformPod", "ModelTransformPod", "FrameUniforms", "Viewer",
    "MultiModelViewer", "RenderTarget", "Preprocessor", "RadixSorter", "Renderer", "GsError",
    "ModelNotFound", "GaussianDisplayMode", "pack_gaussians", "frame_uniforms", "Batch", "Server",
    "ply_parse_header", "ply_convert",
]


class GaussianDisplayMode:
    Splat = DISPLAY_SPLAT
    Ellipse = DISPLAY_ELLIPSE
    Point = DISPLAY_POINT


def launch_count():
    """Kernels launched by libgs300 so far."""
    return int(lib().gs_launch_count())


PROFILE_STAGES = ("preprocess", "depth_sort", "bin", "tile_sort", "ranges", "raster")


SPIN_LIMIT_DEFAULT = 1 << 22
NO_STALL = 0xFFFFFFFF


def debug_set_wait_fault(spin_limit=SPIN_LIMIT_DEFAULT, stall_tile=NO_STALL):
    """Test hook for the bounded device waits: look-backs enqueued afterwards poll at most
    `spin_limit` times, and look-back tile `stall_tile` (if any) never publishes its flags, so
    its successors' waits run out and report GS_ERR_TIMEOUT.  No arguments restore the defaults."""
    check(lib().gs_debug_set_wait_fault(int(spin_limit), int(stall_tile)))


def profile_enable(on=True, count=False):
    """Stage timers on or off; with count=True splat frames run the counting rasteriser."""
    check(lib().gs_profile_enable((2 if count else 1) if on else 0))


def profile_read():
    """{stage: (total ms, timed launches)} since profile_enable; synchronises the device."""
    ms = (ctypes.c_double * 6)()
    n = (ctypes.c_uint32 * 6)()
    check(lib().gs_profile_read(ref(ms), ref(n)))
    return {s: (ms[i], n[i]) for i, s in enumerate(PROFILE_STAGES)}


def profile_counters():
    """Counting-rasteriser work tallies since profile_enable(count=True): evaluations, alphas,
    blends, transmittance."""
    out = (ctypes.c_uint64 * 4)()
    check(lib().gs_profile_counters(ref(out)))
    return {"evaluations": out[0], "alphas": out[1], "blends": out[2], "transmittance": out[3]}


def _stream(stream):
    if stream is None:
        return None
    if isinstance(stream, int):
        return ctypes.c_void_p(stream)
    return ctypes.c_void_p(int(getattr(stream, "cuda_stream", stream)))


class Camera(records.Camera):
    """Camera (src/camera.rs:16-93): position, z range, vertical FOV, pitch, yaw."""

    UP = (0.0, 1.0, 0.0)
    PITCH_LIMIT = (-math.pi / 2 + 1e-6, math.pi / 2 - 1e-6)

    @classmethod
    def new(cls, z_near, z_far, vertical_fov, pos=(0.0, 0.0, 0.0), pitch=0.0, yaw=0.0):
        return cls((ctypes.c_float * 3)(*pos), z_near, z_far, vertical_fov, pitch, yaw)

    def get_forward(self):
        return (
            math.cos(self.pitch) * math.sin(self.yaw),
            math.sin(self.pitch),
            math.cos(self.pitch) * math.cos(self.yaw),
        )

    def pitch_by(self, delta):
        self.pitch = float(np.float32(min(max(np.float32(self.pitch) + np.float32(delta), self.PITCH_LIMIT[0]), self.PITCH_LIMIT[1])))

    def yaw_by(self, delta):
        self.yaw = float(np.float32(math.fmod(float(np.float32(self.yaw) + np.float32(delta)), 2 * math.pi) % (2 * math.pi)))

    def view(self):
        out = (ctypes.c_float * 16)()
        check(lib().gs_camera_view(ref(self), ref(out)))
        return np.array(out, dtype=np.float32).reshape(4, 4)  # [column][row]

    def projection(self, aspect_ratio):
        out = (ctypes.c_float * 16)()
        check(lib().gs_camera_projection(ref(self), float(aspect_ratio), ref(out)))
        return np.array(out, dtype=np.float32).reshape(4, 4)


def camera_pod(camera, size):
    """CameraPod::new(camera, size) (src/buffer/camera.rs:163-172)."""
    pod = CameraPod()
    check(lib().gs_camera_pod_new(ref(camera), int(size[0]), int(size[1]), ref(pod)))
    return pod


CameraPod.new = staticmethod(camera_pod)


def gaussian_transform_pod(size=1.0, display_mode=DISPLAY_SPLAT, sh_deg=3, no_sh0=False, max_std_dev=3.0):
    pod = GaussianTransformPod()
    check(lib().gs_gaussian_transform_pod_new(float(size), int(display_mode), int(sh_deg), int(bool(no_sh0)), float(max_std_dev), ref(pod)))
    return pod


def model_transform_pod(pos=(0.0, 0.0, 0.0), rot=(0.0, 0.0, 0.0, 1.0), scale=(1.0, 1.0, 1.0)):
    pod = ModelTransformPod()
    p, q, s = (ctypes.c_float * 3)(*pos), (ctypes.c_float * 4)(*rot), (ctypes.c_float * 3)(*scale)
    check(lib().gs_model_transform_pod_new(ref(p), ref(q), ref(s), ref(pod)))
    return pod


def pack_gaussians(gaussians):
    """core::Gaussian values (GAUSSIAN_DTYPE) -> default records via the library's packer."""
    g = np.ascontiguousarray(gaussians, dtype=GAUSSIAN_DTYPE).reshape(-1)
    out = np.zeros(len(g), dtype=GAUSSIAN_POD_DTYPE)
    check(lib().gs_gaussian_pack(g.ctypes.data_as(ctypes.c_void_p), len(g), out.ctypes.data_as(ctypes.c_void_p)))
    return out


def frame_uniforms(camera_pod, model_pod, gaussian_pod, viewport):
    u = FrameUniforms()
    check(lib().gs_frame_uniforms_build(ref(camera_pod), ref(model_pod), ref(gaussian_pod), int(viewport[0]), int(viewport[1]), ref(u)))
    return u


def _as_records(gaussians, fmt=None):
    """Accepts core::Gaussian values or device-format records; returns (records, format)."""
    a = np.asarray(gaussians)
    if a.dtype == GAUSSIAN_DTYPE:
        return pack_gaussians(a), FORMAT_FP32
    if a.dtype == GAUSSIAN_POD_DTYPE:
        return np.ascontiguousarray(a).reshape(-1), FORMAT_FP32
    if a.dtype == GAUSSIAN_POD_HALF_DTYPE:
        if fmt not in (FORMAT_HALF_SH_FP16, FORMAT_HALF_SH_BF16):
            raise GsError(1, "compressed records need fmt=FORMAT_HALF_SH_FP16 or FORMAT_HALF_SH_BF16")
        return np.ascontiguousarray(a).reshape(-1), fmt
    raise GsError(1, f"unsupported Gaussian array dtype {a.dtype}")


def _file_bytes(path_or_bytes):
    if isinstance(path_or_bytes, (bytes, bytearray)):
        return bytes(path_or_bytes)
    with open(path_or_bytes, "rb") as f:
        return f.read()


def tuning_default():
    """gs_tuning_default: the library's launch choices for batches."""
    t = records.Tuning()
    check(lib().gs_tuning_default(ctypes.byref(t)))
    return t.as_dict()


def ply_parse_header(path_or_bytes):
    """gs_ply_parse_header: the PlyLayout (field offsets, count, stride) of a PLY file."""
    data = _file_bytes(path_or_bytes)
    layout = records.PlyLayout()
    check(lib().gs_ply_parse_header(data, len(data), ctypes.byref(layout)))
    return layout


def ply_convert(vertices_ptr, layout, fmt, records_ptr, stream=None):
    """gs_ply_convert: device vertex block -> device records of `fmt` (asynchronous)."""
    check(lib().gs_ply_convert(ctypes.c_void_p(vertices_ptr), ctypes.byref(layout), int(fmt),
                               ctypes.c_void_p(records_ptr), _stream(stream)))


class RenderTarget:
    """Headless Rgba8Unorm render target (≙ wgpu::Texture + TextureView)."""

    def __init__(self, width, height):
        h = ctypes.c_void_p()
        check(lib().gs_target_create(int(width), int(height), ctypes.byref(h)))
        self._h = h
        self.width, self.height = int(width), int(height)

    @property
    def ptr(self):
        return lib().gs_target_data(self._h)

    @property
    def pitch(self):
        return lib().gs_target_pitch(self._h)

    def download(self, out=None, stream=None):
        if out is None:
            out = np.empty((self.height, self.width, 4), np.uint8)
        check(lib().gs_target_download(self._h, out.ctypes.data_as(ctypes.c_void_p), _stream(stream)))
        return out

    def download_async(self, out, stream=None):
        """Enqueue the copy into `out` (pinned host memory) on `stream` without waiting."""
        assert out.flags["C_CONTIGUOUS"] and out.nbytes >= self.width * self.height * 4
        check(lib().gs_target_download_async(self._h, out.ctypes.data_as(ctypes.c_void_p), _stream(stream)))
        return out

    def close(self):
        if getattr(self, "_h", None):
            lib().gs_target_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _target_args(target, size=None):
    if isinstance(target, RenderTarget):
        return target.ptr, target.width, target.height, target.pitch
    # A torch uint8 CUDA tensor of shape (H, W, 4)
    h, w = int(target.shape[0]), int(target.shape[1])
    return int(target.data_ptr()), w, h, int(target.stride(0))


class Viewer:
    """Viewer (src/lib.rs:64-275): owns the Gaussians and every per-frame buffer."""

    def __init__(self, gaussians, fmt=None):
        recs, f = _as_records(gaussians, fmt)
        h = ctypes.c_void_p()
        check(lib().gs_viewer_create(recs.ctypes.data_as(ctypes.c_void_p), len(recs), f, ctypes.byref(h)))
        self._h = h
        self.format = f

    @classmethod
    def from_ply(cls, path_or_bytes, fmt=FORMAT_FP32):
        """Viewer::new over Gaussians::read_from_file(path, GaussiansSource::Ply): the header is
        scanned on the host, the vertex block converted into `fmt` records on the GPU."""
        data = _file_bytes(path_or_bytes)
        self = cls.__new__(cls)
        h = ctypes.c_void_p()
        check(lib().gs_viewer_create_from_ply(data, len(data), int(fmt), ctypes.byref(h)))
        self._h = h
        self.format = int(fmt)
        return self

    def __len__(self):
        return lib().gs_viewer_len(self._h)

    def update_camera(self, camera, texture_size):
        check(lib().gs_viewer_update_camera(self._h, ref(camera), int(texture_size[0]), int(texture_size[1])))

    def update_camera_with_pod(self, pod):
        check(lib().gs_viewer_update_camera_with_pod(self._h, ref(pod)))

    def update_model_transform(self, pos, rot, scale):
        p, q, s = (ctypes.c_float * 3)(*pos), (ctypes.c_float * 4)(*rot), (ctypes.c_float * 3)(*scale)
        check(lib().gs_viewer_update_model_transform(self._h, ref(p), ref(q), ref(s)))

    def update_model_transform_with_pod(self, pod):
        check(lib().gs_viewer_update_model_transform_with_pod(self._h, ref(pod)))

    def update_gaussian_transform(self, size, display_mode, sh_deg, no_sh0, max_std_dev):
        check(lib().gs_viewer_update_gaussian_transform(self._h, float(size), int(display_mode), int(sh_deg), int(bool(no_sh0)), float(max_std_dev)))

    def update_gaussian_transform_with_pod(self, pod):
        check(lib().gs_viewer_update_gaussian_transform_with_pod(self._h, ref(pod)))

    def set_selection(self, bits, invert=False):
        if bits is None:
            check(lib().gs_viewer_set_selection(self._h, None, 0))
            return
        b = np.ascontiguousarray(bits, np.uint32)
        check(lib().gs_viewer_set_selection(self._h, b.ctypes.data_as(ctypes.c_void_p), int(bool(invert))))

    def render(self, target, stream=None):
        ptr, w, h, pitch = _target_args(target)
        check(lib().gs_viewer_render(self._h, ctypes.c_void_p(ptr), w, h, pitch, _stream(stream)))

    def synchronize(self, stream=None):
        check(lib().gs_viewer_synchronize(self._h, _stream(stream)))

    def stats(self, stream=None):
        """(visible splats, tile pairs) of the last render; synchronises the stream."""
        v, p = ctypes.c_uint32(), ctypes.c_uint32()
        check(lib().gs_viewer_stats(self._h, _stream(stream), ctypes.byref(v), ctypes.byref(p)))
        return v.value, p.value

    def buffers(self):
        """Device pointers of (IndirectIndicesBuffer, GaussiansDepthBuffer, IndirectArgsBuffer, splats)."""
        a, b, c, d = (ctypes.c_void_p() for _ in range(4))
        check(lib().gs_viewer_buffers(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), ctypes.byref(d)))
        return a.value, b.value, c.value, d.value

    def close(self):
        if getattr(self, "_h", None):
            lib().gs_viewer_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MultiModelViewer:
    """MultiModelViewer (src/multi_model.rs:289-531): models keyed by string."""

    def __init__(self):
        h = ctypes.c_void_p()
        check(lib().gs_multi_viewer_create(ctypes.byref(h)))
        self._h = h

    def insert_model(self, key, gaussians, fmt=None):
        recs, f = _as_records(gaussians, fmt)
        check(lib().gs_multi_viewer_insert_model(self._h, key.encode(), recs.ctypes.data_as(ctypes.c_void_p), len(recs), f))

    def insert_model_from_ply(self, key, path_or_bytes, fmt=FORMAT_FP32):
        data = _file_bytes(path_or_bytes)
        check(lib().gs_multi_viewer_insert_model_from_ply(self._h, key.encode(), data, len(data), int(fmt)))

    def remove_model(self, key):
        check(lib().gs_multi_viewer_remove_model(self._h, key.encode()))

    def __len__(self):
        return lib().gs_multi_viewer_model_count(self._h)

    def update_camera(self, camera, texture_size):
        check(lib().gs_multi_viewer_update_camera(self._h, ref(camera), int(texture_size[0]), int(texture_size[1])))

    def update_camera_with_pod(self, pod):
        check(lib().gs_multi_viewer_update_camera_with_pod(self._h, ref(pod)))

    def update_model_transform(self, key, pos, rot, scale):
        p, q, s = (ctypes.c_float * 3)(*pos), (ctypes.c_float * 4)(*rot), (ctypes.c_float * 3)(*scale)
        check(lib().gs_multi_viewer_update_model_transform(self._h, key.encode(), ref(p), ref(q), ref(s)))

    def update_model_transform_with_pod(self, key, pod):
        check(lib().gs_multi_viewer_update_model_transform_with_pod(self._h, key.encode(), ref(pod)))

    def update_gaussian_transform(self, size, display_mode, sh_deg, no_sh0, max_std_dev):
        check(lib().gs_multi_viewer_update_gaussian_transform(self._h, float(size), int(display_mode), int(sh_deg), int(bool(no_sh0)), float(max_std_dev)))

    def update_gaussian_transform_with_pod(self, pod):
        check(lib().gs_multi_viewer_update_gaussian_transform_with_pod(self._h, ref(pod)))

    def render(self, target, keys, stream=None):
        ptr, w, h, pitch = _target_args(target)
        arr = (ctypes.c_char_p * max(1, len(keys)))(*[k.encode() for k in keys])
        check(lib().gs_multi_viewer_render(self._h, arr, len(keys), ctypes.c_void_p(ptr), w, h, pitch, _stream(stream)))

    def synchronize(self, stream=None):
        check(lib().gs_multi_viewer_synchronize(self._h, _stream(stream)))

    def close(self):
        if getattr(self, "_h", None):
            lib().gs_multi_viewer_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many views (model key, camera, target) of a MultiModelViewer rendered by one CUDA graph per
    batch shape; no counterpart in the reference."""

    def __init__(self, viewer, keys):
        self.viewer = viewer  # keeps the models alive
        self.keys = list(keys)
        arr = (ctypes.c_char_p * max(1, len(self.keys)))(*[k.encode() for k in self.keys])
        h = ctypes.c_void_p()
        check(lib().gs_batch_create(viewer._h, arr, len(self.keys), ctypes.byref(h)))
        self._h = h

    def _views(self, views):
        views = list(views)
        arr = (records.BatchView * max(1, len(views)))()
        for i, (model, pod, target) in enumerate(views):
            idx = self.keys.index(model) if isinstance(model, str) else int(model)
            ptr, w, h, pitch = _target_args(target)
            arr[i].model, arr[i].width, arr[i].height, arr[i].pitch = idx, w, h, pitch
            arr[i].target = ptr
            arr[i].camera = pod
        return arr, len(views)

    def render(self, views, stream=None):
        """views: iterable of (key or model index, CameraPod, target)."""
        arr, n = self._views(views)
        check(lib().gs_batch_render(self._h, ctypes.cast(arr, ctypes.c_void_p), n, _stream(stream)))

    @property
    def tuning(self):
        t = records.Tuning()
        check(lib().gs_batch_get_tuning(self._h, ctypes.byref(t)))
        return t.as_dict()

    def set_tuning(self, **knobs):
        """Change launch choices (suffix_min, eps, views_per_launch, streams, sort_match, sort_digit_bits,
        hist_blocks); frames stay the same."""
        t = records.Tuning()
        check(lib().gs_batch_get_tuning(self._h, ctypes.byref(t)))
        for k, v in knobs.items():
            if k not in t.as_dict():
                raise GsError(1, f"unknown tuning knob {k}")
            setattr(t, k, v)
        check(lib().gs_batch_set_tuning(self._h, ctypes.byref(t)))

    def autotune(self, views, reps=3, rounds=1):
        """gs_batch_autotune: times these views under candidate tunings and keeps the fastest.
        Returns (tuning dict, ms per batch)."""
        arr, n = self._views(views)
        t = records.Tuning()
        ms = ctypes.c_double()
        check(lib().gs_batch_autotune(self._h, ctypes.cast(arr, ctypes.c_void_p), n, int(reps), int(rounds),
                                      ctypes.byref(t), ctypes.byref(ms)))
        return t.as_dict(), ms.value

    def synchronize(self, stream=None):
        check(lib().gs_batch_synchronize(self._h, _stream(stream)))

    def close(self):
        if getattr(self, "_h", None):
            lib().gs_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Request loop over resident scenes (the models of a MultiModelViewer): requests are admitted
    while their per-view memory fits `budget_bytes` and a slot is free, and overlap on the device."""

    def __init__(self, viewer, budget_bytes, max_inflight=8):
        self.viewer = viewer
        h = ctypes.c_void_p()
        check(lib().gs_server_create(viewer._h, int(budget_bytes), int(max_inflight), ctypes.byref(h)))
        self._h = h

    @staticmethod
    def request_bytes(n, width, height):
        return lib().gs_server_request_bytes(int(n), int(width), int(height))

    def submit(self, key, camera_pod, width, height, out=None):
        """Queue a request; `out` may be a host numpy (H, W, 4) uint8 array or a torch CUDA tensor."""
        ticket = ctypes.c_uint64()
        if out is None:
            ptr, pitch, host = None, 0, 0
        elif isinstance(out, np.ndarray):
            ptr, pitch, host = out.ctypes.data_as(ctypes.c_void_p), 0, 1
        else:
            ptr, pitch, host = ctypes.c_void_p(int(out.data_ptr())), int(out.stride(0)), 0
        check(lib().gs_server_submit(self._h, key.encode(), ref(camera_pod), int(width), int(height), ptr, pitch, host,
                                     ctypes.byref(ticket)))
        return ticket.value

    def wait(self, ticket, timeout_s=60.0):
        lat = ctypes.c_double()
        check(lib().gs_server_wait(self._h, ctypes.c_uint64(ticket), float(timeout_s), ctypes.byref(lat)))
        return lat.value

    def stats(self):
        r = records.ServerReport()
        check(lib().gs_server_stats(self._h, ref(r)))
        return {f: getattr(r, f) for f, _ in records.ServerReport._fields_}

    def reset_stats(self):
        check(lib().gs_server_reset_stats(self._h))

    def set_batching(self, max_views, max_wait_ms=0.0):
        """Dynamic batching: up to max_views (1..16) admitted requests of one scene share a
        preprocess launch (records read once); 1 runs every request alone.  max_wait_ms lets a
        request wait that long for busy slots to free up so that larger groups form."""
        check(lib().gs_server_set_batching(self._h, int(max_views), float(max_wait_ms)))

    def close(self):
        if getattr(self, "_h", None):
            lib().gs_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- stage level: caller-owned device buffers (torch CUDA tensors or raw device pointers) ----
def _ptr(x):
    if x is None:
        return None
    if isinstance(x, int):
        return ctypes.c_void_p(x)
    return ctypes.c_void_p(int(x.data_ptr()))


class Preprocessor:
    """Preprocessor::preprocess (src/preprocessor.rs:283-290) over caller buffers."""

    @staticmethod
    def scratch_bytes(n):
        return lib().gs_preprocess_scratch_bytes(int(n))

    @staticmethod
    def depth_capacity(n):
        return lib().gs_depth_capacity(int(n))

    @staticmethod
    def preprocess(uniforms, gaussians, fmt, n, indirect_args, sort_dispatch, indices, depths, depth_capacity,
                   splats, scratch, scratch_bytes, selection=None, invert_selection=False, stream=None):
        check(lib().gs_preprocess(ref(uniforms), _ptr(gaussians), int(fmt), int(n), _ptr(selection), int(bool(invert_selection)),
                                  _ptr(indirect_args), _ptr(sort_dispatch), _ptr(indices), _ptr(depths), int(depth_capacity),
                                  _ptr(splats), _ptr(scratch), int(scratch_bytes), _stream(stream)))


class RadixSorter:
    """RadixSorter::sort (src/radix_sorter.rs:56-96) over caller buffers."""

    @staticmethod
    def scratch_bytes(max_count):
        return lib().gs_radix_sort_scratch_bytes(int(max_count))

    @staticmethod
    def sort(keys, values, max_count, scratch, scratch_bytes, count=None, key_bits=32, stream=None):
        check(lib().gs_radix_sort(_ptr(keys), _ptr(values), int(max_count), _ptr(count), int(key_bits), _ptr(scratch), int(scratch_bytes), _stream(stream)))


class Renderer:
    """Renderer::render (src/renderer.rs:163-195) over caller buffers."""

    @staticmethod
    def scratch_bytes(max_splats, width, height, max_pairs):
        return lib().gs_rasterize_scratch_bytes(int(max_splats), int(width), int(height), int(max_pairs))

    @staticmethod
    def render(uniforms, splats, sorted_indices, count, max_splats, target, width, height, pitch, max_pairs, scratch,
               scratch_bytes, stream=None):
        check(lib().gs_rasterize(ref(uniforms), _ptr(splats), _ptr(sorted_indices), _ptr(count), int(max_splats), _ptr(target),
                                 int(width), int(height), int(pitch), int(max_pairs), _ptr(scratch), int(scratch_bytes), _stream(stream)))

    @staticmethod
    def status(scratch, stream=None):
        pairs = ctypes.c_uint32()
        st = lib().gs_scratch_status(_ptr(scratch), _stream(stream), ctypes.byref(pairs))
        return st, pairs.value
