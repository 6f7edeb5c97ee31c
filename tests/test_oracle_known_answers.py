"""The reference's known-answer tests, restated against the CPU oracle.

The reference asserts per-channel counts of pixels with a channel > 0 over a 1024x1024
Rgba8Unorm target (tests/common/assert_render_target.rs:7-33, tests/common/given.rs:6-37).
These cases pin the oracle's cull/colour/blend semantics to the reference's expectations.
"""
import numpy as np
import pytest

from gs300 import records as R
from gs300 import scene as S

SIZE = 1024


def _channel_counts(img):
    return (img > 0).sum(axis=(0, 1))


def _render(oracle, gaussians, gt=None, mt=None, size=SIZE):
    pod = oracle.camera_pod(S.given_camera(), size, size)
    u = oracle.frame_uniforms(pod, mt or R.ModelTransformPod.new(), gt or R.GaussianTransformPod.new(), size, size)
    img, *_ = oracle.render(u, S.pack_gaussians(np.array(gaussians)), R.FORMAT_FP32, size, size)
    return img


def red():
    return S.gaussian(pos=(0.0, 0.0, 1.0), color=(255, 0, 0, 255))


def green():
    return S.gaussian(pos=(1.0, 0.0, 1.0), color=(0, 255, 0, 255))


# tests/e2e/viewer.rs:71-96
def test_viewer_render_should_render_correctly(oracle):
    c = _channel_counts(_render(oracle, [red()]))
    assert c[0] > 1 and c[1] < 1 and c[2] < 1 and c[3] > 1


# tests/e2e/viewer.rs:98-155
@pytest.mark.parametrize("with_pod", [False, True])
def test_viewer_no_sh0_renders_grayscale(oracle, with_pod):
    gt = R.GaussianTransformPod.new(1.0, R.DISPLAY_SPLAT, 3, True, 3.0)
    c = _channel_counts(_render(oracle, [red()], gt=gt))
    assert (c > 1).all()


# tests/e2e/viewer.rs:157-201: the model moved by -Z puts the Gaussian at the camera.
def test_viewer_model_behind_camera_renders_nothing(oracle):
    c = _channel_counts(_render(oracle, [red()], mt=R.ModelTransformPod.new(pos=(0.0, 0.0, -1.0))))
    assert c[0] == 0 and c[1] == 0 and c[2] == 0


# tests/e2e/multi_model.rs:114-156 — red then green, drawn in key order in one pass.
def test_multi_model_render_should_render_correctly(oracle):
    size = SIZE
    pod = oracle.camera_pod(S.given_camera(), size, size)
    gt = R.GaussianTransformPod.new()
    target = oracle.new_target(size, size)
    for g in (red(), green()):
        u = oracle.frame_uniforms(pod, R.ModelTransformPod.new(), gt, size, size)
        oracle.render(u, S.pack_gaussians(np.array([g])), R.FORMAT_FP32, size, size, target=target)
    c = _channel_counts(target)
    assert c[0] > 1 and c[1] > 1 and c[2] < 1 and c[3] > 1


def test_alpha_channel_stays_opaque(oracle):
    """Clear is Color::BLACK with alpha 1 and the alpha blend is OVER, so alpha stays 255."""
    img = _render(oracle, [red(), green()], size=128)
    assert (img[..., 3] == 255).all()


def test_camera_pod_matches_glam_definitions(oracle):
    """tests/buffer/camera.rs:95-125: view = look_to_rh, proj = perspective_rh (depth 0..1)."""
    import math

    cam = R.Camera.new(0.1, 100.0, math.pi / 4, pos=(5.0, 10.0, 15.0), pitch=math.pi / 6, yaw=math.pi / 4)
    pod = oracle.camera_pod(cam, 1024, 768)
    view = np.array(pod.view, np.float64).reshape(4, 4).T
    proj = np.array(pod.proj, np.float64).reshape(4, 4).T
    f = np.array([math.cos(cam.pitch) * math.sin(cam.yaw), math.sin(cam.pitch), math.cos(cam.pitch) * math.cos(cam.yaw)])
    eye = np.array([5.0, 10.0, 15.0])
    # the camera looks down -Z in view space and sits at the origin
    assert np.allclose(view @ np.append(eye, 1.0), [0, 0, 0, 1], atol=1e-4)
    assert np.allclose(view[:3, :3] @ f, [0, 0, -1], atol=1e-6)
    near_pt = view @ np.append(eye + 0.1 * f, 1.0)
    far_pt = view @ np.append(eye + 100.0 * f, 1.0)
    for p, z in ((near_pt, 0.0), (far_pt, 1.0)):
        c = proj @ p
        assert abs(c[2] / c[3] - z) < 1e-4
    assert abs(proj[1, 1] - 1.0 / math.tan(math.pi / 8)) < 1e-5
    assert abs(proj[0, 0] - proj[1, 1] / (1024 / 768)) < 1e-5
    assert tuple(pod.size) == (1024.0, 768.0)


def test_ellipse_and_point_modes_draw(oracle):
    for mode in (R.DISPLAY_ELLIPSE, R.DISPLAY_POINT):
        gt = R.GaussianTransformPod.new(display_mode=mode)
        c = _channel_counts(_render(oracle, [red()], gt=gt, size=256))
        assert c[0] > 1 and c[1] == 0 and c[2] == 0
