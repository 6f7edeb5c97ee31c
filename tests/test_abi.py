"""The C ABI library loads, exports every declared symbol, and its host-side math (camera pods,
frame uniforms, record packing, argument validation) agrees with the oracle.  No GPU needed."""
import ctypes
import math
import os
import re

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    text = open(os.path.join(REPO, "include", "gs300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gs_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(gs):
    from gs300 import _lib

    L = ctypes.CDLL(_lib.LIB_PATH)
    names = _declared_symbols()
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    bound = {s[0] for s in _lib.SIGNATURES}
    assert set(names) == bound


def test_version(gs):
    assert b"sm_103a" in gs.lib().gs_version()


def test_camera_pod_bit_identical_to_oracle(gs, oracle):
    from gs300 import scene as S

    for k in range(0, 120, 7):
        cam = S.orbit_camera(k)
        for w, h in ((1280, 720), (1920, 1080), (1024, 1024)):
            a = gs.CameraPod.new(cam, (w, h))
            b = oracle.camera_pod(cam, w, h)
            assert bytes(a) == bytes(b)


def test_camera_pod_new_should_return_correct_pod(gs):
    """tests/buffer/camera.rs:95-125."""
    cam = gs.Camera.new(0.1, 100.0, math.pi / 4)
    pod = gs.CameraPod.new(cam, (1280, 720))
    assert np.array_equal(np.array(pod.view, np.float32).reshape(4, 4), cam.view())
    assert np.array_equal(np.array(pod.proj, np.float32).reshape(4, 4), cam.projection(1280 / 720))
    assert tuple(pod.size) == (1280.0, 720.0)
    cam.pos[:] = [5.0, 10.0, 15.0]
    cam.pitch_by(math.pi / 6)
    cam.yaw_by(math.pi / 4)
    pod = gs.CameraPod.new(cam, (1024, 768))
    assert np.array_equal(np.array(pod.view, np.float32).reshape(4, 4), cam.view())
    assert tuple(pod.size) == (1024.0, 768.0)


def test_frame_uniforms_bit_identical_to_oracle(gs, oracle):
    from gs300 import records as R
    from gs300 import scene as S

    rng = np.random.default_rng(0)
    for trial in range(20):
        cam = S.orbit_camera(int(rng.integers(0, 120)), radius=float(rng.uniform(4, 12)))
        w, h = int(rng.integers(16, 4000)), int(rng.integers(16, 3000))
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        mt = gs.model_transform_pod(tuple(rng.normal(size=3)), tuple(q), tuple(rng.uniform(0.2, 3.0, size=3)))
        gt = gs.gaussian_transform_pod(float(rng.uniform(0.1, 2)), int(trial % 3), int(trial % 4), bool(trial % 2), float(rng.uniform(0, 3)))
        pod = gs.CameraPod.new(cam, (w, h))
        a = gs.frame_uniforms(pod, mt, gt, (w, h))
        b = oracle.frame_uniforms(pod, mt, gt, w, h)
        assert bytes(a) == bytes(b)


def test_gaussian_pack_matches_numpy(gs):
    from gs300 import scene as S

    rng = np.random.default_rng(2)
    g = np.zeros(64, dtype=gs.GAUSSIAN_DTYPE)
    q = rng.normal(size=(64, 4))
    g["rot"] = q / np.linalg.norm(q, axis=1, keepdims=True)
    g["pos"] = rng.normal(size=(64, 3))
    g["scale"] = np.exp(rng.normal(-2, 0.5, size=(64, 3)))
    g["color"] = rng.integers(0, 256, size=(64, 4))
    g["sh"] = rng.normal(size=(64, 45))
    a = gs.pack_gaussians(g)
    b = S.pack_gaussians(g)
    assert np.array_equal(a["pos"], b["pos"]) and np.array_equal(a["color"], b["color"])
    assert np.array_equal(a["sh"], b["sh"])
    assert np.allclose(a["cov3d"], b["cov3d"], rtol=1e-6, atol=1e-9)


@pytest.mark.parametrize(
    "args",
    [
        (1.0, 0, 4, False, 3.0),  # GaussianShDegree::new(4) fails
        (1.0, 0, 3, False, 3.5),  # GaussianMaxStdDev::new(3.5) fails
        (1.0, 0, 3, False, -0.1),
        (1.0, 3, 3, False, 3.0),  # no display mode 3
    ],
)
def test_gaussian_transform_validation(gs, args):
    with pytest.raises(gs.GsError) as e:
        gs.gaussian_transform_pod(*args)
    assert e.value.status == 1


def test_stage_calls_reject_bad_arguments_without_touching_the_gpu(gs):
    from gs300 import records as R

    u = R.FrameUniforms()
    L = gs.lib()
    # unknown record format
    st = L.gs_preprocess(ctypes.byref(u), None, 9, 0, None, 0, None, None, None, None, 0, None, None, 0, None)
    assert st == 1
    # key_bits out of range
    assert L.gs_radix_sort(None, None, 0, None, 33, None, 0, None) == 1
    # scratch too small
    assert L.gs_radix_sort(None, None, 10, None, 32, ctypes.c_void_p(256), 8, None) == 1
    # empty target
    assert L.gs_rasterize(ctypes.byref(u), None, None, None, 0, None, 0, 0, 0, 0, None, 0, None) == 1
    assert b"target" in L.gs_last_error()


def test_scratch_sizes_grow_with_problem(gs):
    L = gs.lib()
    assert L.gs_radix_sort_scratch_bytes(1 << 20) > L.gs_radix_sort_scratch_bytes(1 << 10)
    assert L.gs_preprocess_scratch_bytes(1 << 20) > L.gs_preprocess_scratch_bytes(1 << 10)
    assert L.gs_rasterize_scratch_bytes(1000, 1920, 1080, 8000) > L.gs_rasterize_scratch_bytes(1000, 64, 64, 8000)
    # keys_buffer_size(n) of the reference (src/radix_sorter.rs:931-934): rounded up to 3840
    assert L.gs_depth_capacity(1) == 3840 and L.gs_depth_capacity(3840) == 3840 and L.gs_depth_capacity(3841) == 7680


def test_tuning_default(gs):
    t = gs.tuning_default()
    assert t == {"suffix_min": 1024, "eps": pytest.approx(1e-6), "views_per_launch": 16, "streams": 16,
                 "sort_match": 0, "hist_blocks": 0, "raster_grid": 0, "sort_digit_bits": 8}


def test_wait_fault_hook_validates_and_restores(gs):
    """gs_debug_set_wait_fault: a zero poll limit is rejected; the defaults can be restored."""
    with pytest.raises(gs.GsError):
        gs.debug_set_wait_fault(0, 1)
    gs.debug_set_wait_fault(2000, 1)
    gs.debug_set_wait_fault()
