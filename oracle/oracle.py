"""ctypes front end of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this module, and
only as the checker / the timed CPU restatement.  The product (gs300) never calls it.
"""
import ctypes
import os

import numpy as np

from . import build_oracle

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        _lib = ctypes.CDLL(path)
        _declare(_lib)
    return _lib


def _declare(L):
    P = ctypes.c_void_p
    U = ctypes.c_uint32
    I = ctypes.c_int
    L.oracle_camera_pod.argtypes = [P, U, U, P]
    L.oracle_frame_uniforms.argtypes = [P, P, P, U, U, P]
    L.oracle_preprocess.argtypes = [P, P, U, U, P, I, P, P, P, I]
    L.oracle_preprocess.restype = U
    L.oracle_stable_sort.argtypes = [P, P, U]
    L.oracle_radix_sort.argtypes = [P, P, U, I]
    L.oracle_clear.argtypes = [P, U, U]
    L.oracle_rasterize.argtypes = [P, P, P, U, P, U, U, I, I]
    L.oracle_exp_portable.argtypes = [ctypes.c_float]
    L.oracle_exp_portable.restype = ctypes.c_float
    L.oracle_render.argtypes = [P, P, U, U, P, P, P, P, U, U, I, I, I]
    L.oracle_render.restype = U
    L.oracle64_render.argtypes = [P, P, P, P, U, U, P, U, U, I]
    L.oracle64_render.restype = U
    L.oracle_ply_convert.argtypes = [P, P, U, P]
    L.oracle_render_quads.argtypes = [P, P, P, U, U, P, P, P, U, U, I]
    L.oracle_render_quads.restype = U
    L.oracle_wgpu_radix_sort.argtypes = [P, U, P, U, U, U, I]
    L.oracle_wgpu_radix_sort.restype = I


def _p(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        assert a.flags["C_CONTIGUOUS"]
        return a.ctypes.data_as(ctypes.c_void_p)
    return ctypes.cast(ctypes.byref(a), ctypes.c_void_p)


def camera_pod(camera, width, height):
    from gs300.records import CameraPod

    pod = CameraPod()
    lib().oracle_camera_pod(_p(camera), width, height, _p(pod))
    return pod


def frame_uniforms(camera_pod, model_pod, gt_pod, vw, vh):
    from gs300.records import FrameUniforms

    u = FrameUniforms()
    lib().oracle_frame_uniforms(_p(camera_pod), _p(model_pod), _p(gt_pod), vw, vh, _p(u))
    return u


def preprocess(u, records, fmt, selection=None, invert=False, threads=1, want_splats=True):
    """-> (indices[V] u32, depths[V] f32, splats[N] or None)."""
    from gs300.records import SPLAT_DTYPE

    n = len(records)
    idx = np.zeros(max(n, 1), np.uint32)
    dep = np.zeros(max(n, 1), np.float32)
    spl = np.zeros(max(n, 1), SPLAT_DTYPE) if want_splats else None
    sel = None if selection is None else np.ascontiguousarray(selection, np.uint32)
    v = lib().oracle_preprocess(_p(u), _p(records), fmt, n, _p(sel), int(bool(invert)), _p(idx), _p(dep), _p(spl), threads)
    return idx[:v].copy(), dep[:v].copy(), (spl[:n] if want_splats else None)


def stable_sort(keys, vals):
    k = np.ascontiguousarray(keys).view(np.uint32).copy()
    v = np.ascontiguousarray(vals, np.uint32).copy()
    lib().oracle_stable_sort(_p(k), _p(v), len(k))
    return k, v


def radix_sort(keys, vals, threads):
    k = np.ascontiguousarray(keys).view(np.uint32).copy()
    v = np.ascontiguousarray(vals, np.uint32).copy()
    lib().oracle_radix_sort(_p(k), _p(v), len(k), threads)
    return k, v


def new_target(w, h):
    t = np.empty((h, w, 4), np.uint8)
    lib().oracle_clear(_p(t), w, h)
    return t


def rasterize(u, splats, order, target, exp_mode=0, threads=0):
    h, w, _ = target.shape
    order = np.ascontiguousarray(order, np.uint32)
    lib().oracle_rasterize(_p(u), _p(splats), _p(order), len(order), _p(target), w, h, exp_mode, threads)
    return target


def render(u, records, fmt, w, h, exp_mode=0, threads=0, target=None):
    """Whole frame (preprocess -> stable sort -> clear -> blend).  Returns (rgba, indices, depths, splats)."""
    from gs300.records import SPLAT_DTYPE

    n = len(records)
    idx = np.zeros(max(n, 1), np.uint32)
    dep = np.zeros(max(n, 1), np.float32)
    spl = np.zeros(max(n, 1), SPLAT_DTYPE)
    clear = 1 if target is None else 0
    if target is None:
        target = np.empty((h, w, 4), np.uint8)
    v = lib().oracle_render(_p(u), _p(records), fmt, n, _p(idx), _p(dep), _p(spl), _p(target), w, h, exp_mode, threads, clear)
    return target, idx[:v].copy(), dep[:v].copy(), spl[:n]


def render64(camera_pod, model_pod, gt_pod, records, fmt, w, h, threads=0):
    """The same frame evaluated in FP64 from the same pods and records (precision reference)."""
    img = np.empty((h, w, 4), np.uint8)
    v = lib().oracle64_render(_p(camera_pod), _p(model_pod), _p(gt_pod), _p(records), fmt, len(records), _p(img), w, h,
                              threads or nproc())
    return img, v


def ply_convert(vertex_block, layout, fmt):
    """PLY vertex block (bytes from layout.data_offset on) -> records of `fmt` (numpy)."""
    from gs300.records import record_dtype

    v = np.frombuffer(bytes(vertex_block), dtype=np.uint8)
    assert len(v) >= layout.count * layout.stride
    out = np.zeros(layout.count, record_dtype(fmt))
    lib().oracle_ply_convert(_p(np.ascontiguousarray(v)), _p(layout), fmt, _p(out))
    return out


def exp_portable(x):
    return lib().oracle_exp_portable(float(x))


def nproc():
    return os.cpu_count() or 1


def wgpu_radix_sort(keys, payload, num_keys, dispatch_x, schedule=0):
    """The reference sorter (RadixSorter::sort_indirect, src/radix_sorter.rs:658-669) re-executed
    workgroup by workgroup on copies of `keys` (the depth buffer, u32) and `payload` (the index
    buffer, u32): num_keys = the sorter state's N, dispatch_x = ceil(V / 3840).  Returns the two
    buffers after the sort."""
    k = np.ascontiguousarray(keys, dtype=np.uint32).copy()
    p = np.ascontiguousarray(payload, dtype=np.uint32).copy()
    rc = lib().oracle_wgpu_radix_sort(_p(k), len(k), _p(p), len(p), int(num_keys), int(dispatch_x), int(schedule))
    if rc != 0:
        raise RuntimeError("reference sorter restatement: a look-back met an unpublished predecessor")
    return k, p


def render_quads(camera_pod, u, records, fmt, w, h, target=None):
    """The frame through the reference's own vertex stage taken literally (six clip-space
    vertices per instance, two triangles rasterised at pixel centres, interpolated quad offsets,
    frag_main): the check of the pixel -> quad map every other rasteriser here shares.
    Returns (rgba, V)."""
    n = len(records)
    idx = np.zeros(max(n, 1), np.uint32)
    dep = np.zeros(max(n, 1), np.float32)
    img = target if target is not None else np.empty((h, w, 4), np.uint8)
    v = lib().oracle_render_quads(_p(camera_pod), _p(u), _p(records), fmt, n, _p(idx), _p(dep), _p(img), w, h,
                                  0 if target is not None else 1)
    return img, v
