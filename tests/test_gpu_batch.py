"""Batching tier: many views (model, camera, resolution) rendered by one graph-captured launch
must give, view by view, the frames the Viewer path gives for the same model and camera — the
batch changes scheduling, not results — including across calls that reuse the captured graph
with new cameras."""
import numpy as np
import pytest

from gs300 import records as R
from gs300 import scene as S

pytestmark = pytest.mark.gpu

SIZES = [(640, 360), (1280, 720), (333, 197), (1920, 1080)]


def _single(gs, records, mt, cam, w, h, fmt=None):
    v = gs.Viewer(records, fmt)
    v.update_model_transform_with_pod(mt)
    v.update_camera(cam, (w, h))
    t = gs.RenderTarget(w, h)
    v.render(t)
    v.synchronize()
    return t.download()


def test_batch_matches_single_views(gs, cuda, monkeypatch):
    monkeypatch.setenv("GS300_EXACT_EXP", "1")
    scenes = {f"m{i}": S.synth_scene(n, seed=40 + i) for i, n in enumerate((30_000, 60_000, 90_000))}
    mts = {k: gs.model_transform_pod((0.2 * i, -0.1 * i, 0.0), (0.0, 0.0, 0.0, 1.0), (1.0, 1.0, 1.0))
           for i, k in enumerate(scenes)}
    mv = gs.MultiModelViewer()
    for k, sc in scenes.items():
        mv.insert_model(k, sc)
        mv.update_model_transform_with_pod(k, mts[k])
    keys = list(scenes)
    batch = gs.Batch(mv, keys)
    rng = np.random.default_rng(0)
    n_views = 12
    plan = [(keys[i % 3], SIZES[i % 4]) for i in range(n_views)]
    targets = [gs.RenderTarget(w, h) for _, (w, h) in plan]
    for call in range(3):  # the second and third calls replay the captured graph with new cameras
        cams = [S.orbit_camera(int(rng.integers(0, 120)), radius=float(rng.uniform(5, 9))) for _ in range(n_views)]
        batch.render([(k, gs.CameraPod.new(c, wh), t) for (k, wh), c, t in zip(plan, cams, targets)])
        batch.synchronize()
        for (k, (w, h)), cam, t in zip(plan, cams, targets):
            want = _single(gs, scenes[k], mts[k], cam, w, h)
            assert np.array_equal(t.download(), want)


def test_batch_reports_missing_model(gs, cuda):
    mv = gs.MultiModelViewer()
    mv.insert_model("a", S.synth_scene(1000, seed=1))
    batch = gs.Batch(mv, ["a", "b"])
    t = gs.RenderTarget(64, 64)
    pod = gs.CameraPod.new(S.orbit_camera(0), (64, 64))
    with pytest.raises(gs.ModelNotFound):
        batch.render([("b", pod, t)])
    batch.render([("a", pod, t)])
    batch.synchronize()


def test_batch_shared_record_reads(gs, cuda, monkeypatch):
    """Views of one model share one preprocess launch (records read once, up to 16 views per
    launch): 20 views of a half-record model make two launches (16 + 4), interleaved with views
    of an FP32 model and of an empty model; every view equals its single-view render."""
    monkeypatch.setenv("GS300_EXACT_EXP", "1")
    scenes = {"half": (S.synth_scene(50_000, seed=7, fmt=R.FORMAT_HALF_SH_BF16), R.FORMAT_HALF_SH_BF16),
              "fp32": (S.synth_scene(20_000, seed=8), None),
              "empty": (S.synth_scene(0, seed=9), None)}
    mv = gs.MultiModelViewer()
    for k, (sc, fmt) in scenes.items():
        mv.insert_model(k, sc, fmt)
    keys = list(scenes)
    batch = gs.Batch(mv, keys)
    plan = []
    for i in range(20):
        plan.append(("half", (320 + 16 * (i % 3), 180)))
        if i % 7 == 3:
            plan.append(("fp32", (256, 144)))
    plan.insert(5, ("empty", (64, 48)))
    targets = [gs.RenderTarget(w, h) for _, (w, h) in plan]
    mt = gs.model_transform_pod()
    for call in range(2):
        cams = [S.orbit_camera(3 * j + 17 * call, radius=6.0 + 0.1 * j) for j in range(len(plan))]
        batch.render([(k, gs.CameraPod.new(c, wh), t) for (k, wh), c, t in zip(plan, cams, targets)])
        batch.synchronize()
        for (k, (w, h)), cam, t in zip(plan, cams, targets):
            sc, fmt = scenes[k]
            got = t.download()
            if k == "empty":
                assert (got[..., :3] == 0).all() and (got[..., 3] == 255).all()
                continue
            assert np.array_equal(got, _single(gs, sc, mt, cam, w, h, fmt))


TUNINGS = [
    dict(views_per_launch=1, streams=1),
    dict(suffix_min=1, eps=0.3),            # every tile takes the early-out, with frequent restarts
    dict(sort_match=0, hist_blocks=7, views_per_launch=3, streams=5),
    dict(raster_grid=1),                    # one rasteriser grid over all views
    dict(raster_grid=1, views_per_launch=2, streams=3, suffix_min=1),
    dict(sort_digit_bits=6),                # six depth-sort passes of 5 and 6 bits
    dict(sort_digit_bits=7, sort_match=0),  # five passes of 6 bits, ballot ranking
]


@pytest.mark.parametrize("knobs", TUNINGS, ids=["serial", "early_out_everywhere", "ballot_sort", "one_grid",
                                                "one_grid_early_out", "digits_6", "digits_7_ballot"])
def test_batch_tuning_changes_no_frame(gs, cuda, monkeypatch, knobs):
    monkeypatch.setenv("GS300_EXACT_EXP", "1")
    sc = S.synth_scene(40_000, seed=12)
    mv = gs.MultiModelViewer()
    mv.insert_model("m", sc)
    batch = gs.Batch(mv, ["m"])
    batch.set_tuning(**knobs)
    assert all(batch.tuning[k] == pytest.approx(v) for k, v in knobs.items())
    plan = [(320, 180), (256, 256), (640, 360), (200, 120), (320, 180)]
    targets = [gs.RenderTarget(w, h) for w, h in plan]
    cams = [S.orbit_camera(9 * j + 2, radius=5.5) for j in range(len(plan))]
    batch.render([("m", gs.CameraPod.new(c, wh), t) for wh, c, t in zip(plan, cams, targets)])
    batch.synchronize()
    mt = gs.model_transform_pod()
    for (w, h), cam, t in zip(plan, cams, targets):
        assert np.array_equal(t.download(), _single(gs, sc, mt, cam, w, h))


def test_batch_tuning_rejects_bad_values(gs, cuda):
    mv = gs.MultiModelViewer()
    mv.insert_model("m", S.synth_scene(100, seed=1))
    batch = gs.Batch(mv, ["m"])
    for bad in (dict(views_per_launch=0), dict(views_per_launch=17), dict(streams=0), dict(streams=17),
                dict(sort_match=2), dict(eps=0.0), dict(eps=0.7), dict(suffix_min=0), dict(hist_blocks=5000),
                dict(raster_grid=2), dict(sort_digit_bits=5), dict(sort_digit_bits=9)):
        with pytest.raises(gs.GsError):
            batch.set_tuning(**bad)
    assert batch.tuning == gs.tuning_default()


def test_batch_autotune(gs, cuda, monkeypatch):
    """The autotuner returns a valid tuning, leaves it set, and the frames stay the single-view ones."""
    monkeypatch.setenv("GS300_EXACT_EXP", "1")
    sc = S.synth_scene(60_000, seed=13)
    mv = gs.MultiModelViewer()
    mv.insert_model("m", sc)
    batch = gs.Batch(mv, ["m"])
    plan = [(480, 270)] * 4
    targets = [gs.RenderTarget(w, h) for w, h in plan]
    cams = [S.orbit_camera(30 * j, radius=6.0) for j in range(len(plan))]
    views = [("m", gs.CameraPod.new(c, wh), t) for wh, c, t in zip(plan, cams, targets)]
    best, ms = batch.autotune(views, reps=2)
    assert ms > 0 and batch.tuning == best
    assert 1 <= best["views_per_launch"] <= 16 and 1 <= best["streams"] <= 16
    batch.render(views)
    batch.synchronize()
    mt = gs.model_transform_pod()
    for (w, h), cam, t in zip(plan, cams, targets):
        assert np.array_equal(t.download(), _single(gs, sc, mt, cam, w, h))


def test_batching_config_shape(gs, cuda, monkeypatch):
    """The batching configuration's shape at reduced size: 4 models with random rigid model
    transforms and 10% of Gaussians carrying a per-Gaussian translation, 16 views of
    resolutions drawn from {640x360, 1280x720, 1920x1080, 3840x2160} on random orbits of radius
    6-12, in one batch call; every view equals the Viewer's frame for its model and camera."""
    monkeypatch.setenv("GS300_EXACT_EXP", "1")
    rng = np.random.default_rng(8)
    sizes = (25_000, 50_000, 75_000, 150_000)
    scenes, mts = {}, {}
    for i, n in enumerate(sizes):
        k = f"m{i}"
        scenes[k] = S.synth_scene(n, seed=70 + i, translate_fraction=0.1)
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        mts[k] = gs.model_transform_pod(tuple(rng.normal(0.0, 0.5, 3)), tuple(q), (1.0, 1.0, 1.0))
    mv = gs.MultiModelViewer()
    for k, sc in scenes.items():
        mv.insert_model(k, sc)
        mv.update_model_transform_with_pod(k, mts[k])
    keys = list(scenes)
    res = [(640, 360), (1280, 720), (1920, 1080), (3840, 2160)]
    plan = [(keys[int(rng.integers(0, 4))], res[int(rng.integers(0, 4))]) for _ in range(16)]
    cams = [S.orbit_camera(int(rng.integers(0, 120)), radius=float(rng.uniform(6, 12))) for _ in plan]
    targets = [gs.RenderTarget(w, h) for _, (w, h) in plan]
    batch = gs.Batch(mv, keys)
    want = [_single(gs, scenes[k], mts[k], cam, w, h) for (k, (w, h)), cam in zip(plan, cams)]
    for grid in (0, 1):  # views rasterised one by one, then one grid over all views' tiles
        batch.set_tuning(raster_grid=grid)
        batch.render([(k, gs.CameraPod.new(c, wh), t) for (k, wh), c, t in zip(plan, cams, targets)])
        batch.synchronize()
        for t, w_ in zip(targets, want):
            assert np.array_equal(t.download(), w_)


def test_batch_renders_back_to_back(gs, cuda, monkeypatch):
    """Two batch renders with different cameras enqueued without a sync between them (each read
    back asynchronously): each read-back holds its own cameras' frames."""
    monkeypatch.setenv("GS300_EXACT_EXP", "1")
    sc = S.synth_scene(40_000, seed=14)
    mv = gs.MultiModelViewer()
    mv.insert_model("m", sc)
    batch = gs.Batch(mv, ["m"])
    plan = [(320, 180), (256, 144), (400, 200)]
    targets = [gs.RenderTarget(w, h) for w, h in plan]
    s = cuda.cuda.Stream()
    rounds = []
    for r in range(3):
        cams = [S.orbit_camera(20 * r + 3 * j, radius=6.0) for j in range(len(plan))]
        batch.render([("m", gs.CameraPod.new(c, wh), t) for wh, c, t in zip(plan, cams, targets)], stream=s.cuda_stream)
        hosts = [cuda.empty((h, w, 4), dtype=cuda.uint8, pin_memory=True).numpy() for w, h in plan]
        for t, hbuf in zip(targets, hosts):
            t.download_async(hbuf, stream=s.cuda_stream)
        rounds.append((cams, hosts))
    s.synchronize()
    batch.synchronize(stream=s.cuda_stream)
    mt = gs.model_transform_pod()
    for cams, hosts in rounds:
        for (w, h), cam, hbuf in zip(plan, cams, hosts):
            assert np.array_equal(hbuf, _single(gs, sc, mt, cam, w, h))
