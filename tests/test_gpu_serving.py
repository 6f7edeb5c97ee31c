"""Serving tier: requests over resident scenes, admitted by memory budget, overlapping on the
device.  Each result must be the same alone and in the mix (bit-identical frames)."""
import numpy as np
import pytest

from gs300 import scene as S

pytestmark = pytest.mark.gpu

RES = [(320, 180), (640, 360), (1280, 720)]


def _requests(rng, keys, count):
    out = []
    for _ in range(count):
        k = keys[int(rng.integers(0, len(keys)))]
        w, h = RES[int(rng.integers(0, len(RES)))]
        cam = S.orbit_camera(int(rng.integers(0, 120)), radius=float(rng.uniform(6, 12)))
        out.append((k, w, h, cam))
    return out


def test_results_same_alone_and_in_the_mix(gs, cuda):
    mv = gs.MultiModelViewer()
    scenes = {"s0": 20_000, "s1": 60_000, "s2": 150_000}
    for i, (k, n) in enumerate(scenes.items()):
        mv.insert_model(k, S.synth_scene(n, seed=50 + i))
    reqs = _requests(np.random.default_rng(3), list(scenes), 24)
    sv = gs.Server(mv, budget_bytes=8 << 30, max_inflight=8)
    alone = []
    for k, w, h, cam in reqs:
        out = np.zeros((h, w, 4), np.uint8)
        sv.wait(sv.submit(k, gs.CameraPod.new(cam, (w, h)), w, h, out))
        alone.append(out)
    mixed = [np.zeros((h, w, 4), np.uint8) for _, w, h, _ in reqs]
    tickets = [sv.submit(k, gs.CameraPod.new(cam, (w, h)), w, h, o) for (k, w, h, cam), o in zip(reqs, mixed)]
    lat = [sv.wait(t) for t in tickets]
    for a, b in zip(alone, mixed):
        assert np.array_equal(a, b)
    st = sv.stats()
    assert st["completed"] == 48 and st["failed"] == 0 and st["p99_ms"] >= st["p50_ms"] > 0
    assert min(lat) > 0


def test_admission_by_memory_budget(gs, cuda):
    mv = gs.MultiModelViewer()
    mv.insert_model("s", S.synth_scene(100_000, seed=60))
    need = gs.Server.request_bytes(100_000, 640, 360)
    sv = gs.Server(mv, budget_bytes=int(need * 1.5), max_inflight=8)  # one request at a time fits
    cam = gs.CameraPod.new(S.orbit_camera(0), (640, 360))
    tickets = [sv.submit("s", cam, 640, 360) for _ in range(6)]
    seen = 0
    while True:
        st = sv.stats()
        seen = max(seen, st["running"])
        assert st["reserved_bytes"] <= int(need * 1.5)
        if st["completed"] == 6:
            break
    assert seen <= 1
    for t in tickets:
        sv.wait(t)
    with pytest.raises(gs.GsError) as e:
        sv.submit("s", gs.CameraPod.new(S.orbit_camera(0), (3840, 2160)), 3840, 2160)
    assert e.value.status == 7  # GS_ERR_ADMISSION
    with pytest.raises(gs.ModelNotFound):
        sv.submit("missing", cam, 640, 360)


def test_dynamic_batching_matches_viewer(gs, cuda, monkeypatch):
    """A burst of requests for one scene is admitted as groups sharing one preprocess launch
    (up to 16, here limited by 12 slots); every frame equals the Viewer's for that camera."""
    monkeypatch.setenv("GS300_EXACT_EXP", "1")
    sc = S.synth_scene(80_000, seed=61)
    mv = gs.MultiModelViewer()
    mv.insert_model("s", sc)
    sv = gs.Server(mv, budget_bytes=16 << 30, max_inflight=12)
    reqs = [(RES[i % 3], S.orbit_camera(7 * i, radius=6.0 + 0.2 * i)) for i in range(20)]
    outs = [np.zeros((h, w, 4), np.uint8) for (w, h), _ in reqs]
    tickets = [sv.submit("s", gs.CameraPod.new(cam, (w, h)), w, h, o) for ((w, h), cam), o in zip(reqs, outs)]
    for t in tickets:
        sv.wait(t)
    v = gs.Viewer(sc)
    for ((w, h), cam), o in zip(reqs, outs):
        v.update_camera(cam, (w, h))
        tgt = gs.RenderTarget(w, h)
        v.render(tgt)
        v.synchronize()
        assert np.array_equal(o, tgt.download())
    sv.set_batching(1)  # every request alone
    again = [np.zeros((h, w, 4), np.uint8) for (w, h), _ in reqs]
    tickets = [sv.submit("s", gs.CameraPod.new(cam, (w, h)), w, h, o) for ((w, h), cam), o in zip(reqs, again)]
    for t in tickets:
        sv.wait(t)
    for a, b in zip(outs, again):
        assert np.array_equal(a, b)
    sv.set_batching(16, max_wait_ms=2.0)  # batching window
    third = [np.zeros((h, w, 4), np.uint8) for (w, h), _ in reqs]
    tickets = [sv.submit("s", gs.CameraPod.new(cam, (w, h)), w, h, o) for ((w, h), cam), o in zip(reqs, third)]
    for t in tickets:
        sv.wait(t)
    for a, b in zip(outs, third):
        assert np.array_equal(a, b)
    for bad in ((0, 0.0), (17, 0.0), (4, -1.0), (4, 5000.0)):
        with pytest.raises(gs.GsError):
            sv.set_batching(*bad)
