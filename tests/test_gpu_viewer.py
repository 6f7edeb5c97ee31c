"""The reference's e2e tests (tests/e2e/viewer.rs, tests/e2e/multi_model.rs) restated through the
Viewer / MultiModelViewer facades of the C ABI, plus frame parity of the facades with the oracle."""
import numpy as np
import pytest

from gpu_helpers import frame_psnr, within_one_fraction
from gs300 import records as R
from gs300 import scene as S

pytestmark = pytest.mark.gpu
SIZE = 1024


def _counts(img):
    return (img > 0).sum(axis=(0, 1))


def _red():
    return np.array([S.gaussian(pos=(0.0, 0.0, 1.0), color=(255, 0, 0, 255))])


def _green():
    return np.array([S.gaussian(pos=(1.0, 0.0, 1.0), color=(0, 255, 0, 255))])


def _viewer_frame(gs, viewer, target):
    viewer.render(target)
    viewer.synchronize()
    return target.download()


@pytest.fixture
def target(gs, cuda):
    t = gs.RenderTarget(SIZE, SIZE)
    yield t
    t.close()


def test_viewer_update_camera_when_with_or_without_pod_should_be_equal(gs, cuda):
    v1, v2 = gs.Viewer(_red()), gs.Viewer(_red())
    t1, t2 = gs.RenderTarget(SIZE, SIZE), gs.RenderTarget(SIZE, SIZE)
    cam = S.given_camera()
    v1.update_camera_with_pod(gs.CameraPod.new(cam, (SIZE, SIZE)))
    v2.update_camera(cam, (SIZE, SIZE))
    assert np.array_equal(_viewer_frame(gs, v1, t1), _viewer_frame(gs, v2, t2))


def test_viewer_render_should_render_correctly(gs, target):
    v = gs.Viewer(_red())
    v.update_camera_with_pod(gs.CameraPod.new(S.given_camera(), (SIZE, SIZE)))
    c = _counts(_viewer_frame(gs, v, target))
    assert c[0] > 1 and c[1] < 1 and c[2] < 1 and c[3] > 1


@pytest.mark.parametrize("with_pod", [False, True])
def test_viewer_no_sh0_renders_grayscale(gs, target, with_pod):
    v = gs.Viewer(_red())
    v.update_camera_with_pod(gs.CameraPod.new(S.given_camera(), (SIZE, SIZE)))
    if with_pod:
        v.update_gaussian_transform_with_pod(gs.gaussian_transform_pod(1.0, R.DISPLAY_SPLAT, 3, True, 3.0))
    else:
        v.update_gaussian_transform(1.0, R.DISPLAY_SPLAT, 3, True, 3.0)
    assert (_counts(_viewer_frame(gs, v, target)) > 1).all()


@pytest.mark.parametrize("with_pod", [False, True])
def test_viewer_model_pos_behind_camera_renders_nothing(gs, target, with_pod):
    v = gs.Viewer(_red())
    v.update_camera_with_pod(gs.CameraPod.new(S.given_camera(), (SIZE, SIZE)))
    if with_pod:
        v.update_model_transform_with_pod(gs.model_transform_pod((0.0, 0.0, -1.0)))
    else:
        v.update_model_transform((0.0, 0.0, -1.0), (0.0, 0.0, 0.0, 1.0), (1.0, 1.0, 1.0))
    c = _counts(_viewer_frame(gs, v, target))
    assert c[0] == 0 and c[1] == 0 and c[2] == 0


def test_viewer_invalid_gaussian_transform_is_rejected(gs, cuda):
    v = gs.Viewer(_red())
    with pytest.raises(gs.GsError):
        v.update_gaussian_transform(1.0, R.DISPLAY_SPLAT, 4, False, 3.0)


def _multi(gs):
    mv = gs.MultiModelViewer()
    mv.insert_model("red", _red())
    mv.insert_model("green", _green())
    mv.update_camera_with_pod(gs.CameraPod.new(S.given_camera(), (SIZE, SIZE)))
    return mv


def test_multi_model_viewer_render_should_render_correctly(gs, target):
    mv = _multi(gs)
    mv.render(target, ["red", "green"])
    mv.synchronize()
    c = _counts(target.download())
    assert c[0] > 1 and c[1] > 1 and c[2] < 1 and c[3] > 1


def test_multi_model_viewer_camera_with_or_without_pod_equal(gs, cuda):
    a, b = _multi(gs), _multi(gs)
    b.update_camera(S.given_camera(), (SIZE, SIZE))
    ta, tb = gs.RenderTarget(SIZE, SIZE), gs.RenderTarget(SIZE, SIZE)
    a.render(ta, ["red", "green"])
    b.render(tb, ["red", "green"])
    a.synchronize()
    b.synchronize()
    assert np.array_equal(ta.download(), tb.download())


def test_multi_model_viewer_no_sh0_grayscale(gs, target):
    mv = _multi(gs)
    mv.update_gaussian_transform(1.0, R.DISPLAY_SPLAT, 3, True, 3.0)
    mv.render(target, ["red", "green"])
    mv.synchronize()
    assert (_counts(target.download()) > 1).all()


def test_multi_model_viewer_model_behind_camera(gs, target):
    mv = _multi(gs)
    mv.update_model_transform("red", (0.0, 0.0, -1.0), (0.0, 0.0, 0.0, 1.0), (1.0, 1.0, 1.0))
    mv.update_model_transform_with_pod("green", gs.model_transform_pod((-1.0, 0.0, -1.0)))
    mv.render(target, ["red", "green"])
    mv.synchronize()
    c = _counts(target.download())
    assert c[0] == 0 and c[1] == 0 and c[2] == 0


def test_multi_model_viewer_remove_model(gs, target):
    """tests/e2e/multi_model.rs:331-375: after remove_model only red renders; the removed key errors."""
    mv = _multi(gs)
    mv.remove_model("green")
    assert len(mv) == 1
    mv.render(target, ["red"])
    mv.synchronize()
    c = _counts(target.download())
    assert c[0] > 1 and c[1] < 1 and c[2] < 1
    with pytest.raises(gs.ModelNotFound):
        mv.render(target, ["red", "green"])
    with pytest.raises(gs.ModelNotFound):
        mv.update_model_transform("green", (0, 0, 0), (0, 0, 0, 1), (1, 1, 1))
    with pytest.raises(gs.ModelNotFound):
        mv.remove_model("green")


def test_multi_model_draw_order_matches_oracle(gs, cuda, oracle, monkeypatch):
    """Models composite in key order (src/multi_model.rs:505-527), each over the previous ones."""
    monkeypatch.setenv("GS300_EXACT_EXP", "1")
    w, h = 256, 192
    scenes = [S.synth_scene(3000, seed=30 + i) for i in range(3)]
    mts = [gs.model_transform_pod((0.3 * i, 0.0, 0.0), (0.0, 0.0, 0.0, 1.0), (1.0, 1.0, 1.0)) for i in range(3)]
    mv = gs.MultiModelViewer()
    for i, sc in enumerate(scenes):
        mv.insert_model(f"m{i}", sc)
        mv.update_model_transform_with_pod(f"m{i}", mts[i])
    cam = S.orbit_camera(10, radius=5.0)
    pod = gs.CameraPod.new(cam, (w, h))
    mv.update_camera_with_pod(pod)
    t = gs.RenderTarget(w, h)
    for keys in (["m0", "m1", "m2"], ["m2", "m0"], ["m1"]):
        mv.render(t, keys)
        mv.synchronize()
        got = t.download()
        want = oracle.new_target(w, h)
        gt = gs.gaussian_transform_pod()
        for k in keys:
            i = int(k[1])
            u = oracle.frame_uniforms(pod, mts[i], gt, w, h)
            oracle.render(u, scenes[i], R.FORMAT_FP32, w, h, exp_mode=0, threads=4, target=want)
        assert np.array_equal(got, want)


def test_viewer_matches_oracle_and_recovers_from_pair_overflow(gs, cuda, oracle):
    """The facade grows its tile-pair list when a frame overflows it and renders again."""
    sc = S.synth_scene(200_000, seed=31)
    v = gs.Viewer(sc)
    w, h = 800, 600
    cam = S.orbit_camera(33, radius=4.0)  # close orbit: large splats, many pairs
    v.update_camera(cam, (w, h))
    t = gs.RenderTarget(w, h)
    v.render(t)
    v.synchronize()
    got = t.download()
    pod = gs.CameraPod.new(cam, (w, h))
    u = oracle.frame_uniforms(pod, gs.model_transform_pod(), gs.gaussian_transform_pod(), w, h)
    want, *_ = oracle.render(u, sc, R.FORMAT_FP32, w, h, exp_mode=1, threads=16)
    assert within_one_fraction(got, want) >= 0.999 and frame_psnr(got, want) >= 45.0


@pytest.mark.parametrize("fmt", [R.FORMAT_HALF_SH_FP16, R.FORMAT_HALF_SH_BF16])
def test_viewer_half_records(gs, cuda, oracle, fmt):
    sc = S.synth_scene(100_000, seed=32, fmt=fmt)
    v = gs.Viewer(sc, fmt=fmt)
    w, h = 640, 360
    cam = S.orbit_camera(5)
    v.update_camera(cam, (w, h))
    t = gs.RenderTarget(w, h)
    v.render(t)
    v.synchronize()
    pod = gs.CameraPod.new(cam, (w, h))
    u = oracle.frame_uniforms(pod, gs.model_transform_pod(), gs.gaussian_transform_pod(), w, h)
    want, *_ = oracle.render(u, sc, fmt, w, h, exp_mode=1, threads=16)
    got = t.download()
    assert within_one_fraction(got, want) >= 0.999 and frame_psnr(got, want) >= 45.0


def test_download_async_matches_download(gs, cuda):
    sc = S.synth_scene(30_000, seed=77)
    v = gs.Viewer(sc)
    v.update_camera(S.orbit_camera(5), (320, 180))
    t = gs.RenderTarget(320, 180)
    s = cuda.cuda.Stream()
    v.render(t, stream=s.cuda_stream)
    pinned = cuda.empty((180, 320, 4), dtype=cuda.uint8, pin_memory=True).numpy()
    t.download_async(pinned, stream=s.cuda_stream)
    s.synchronize()
    assert np.array_equal(pinned, t.download())
