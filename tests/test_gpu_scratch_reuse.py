"""Scratch areas reused across calls of different sizes.

Look-back flags of a scratch area sit at a fixed offset (its flag arena) and carry the epoch of
the call that wrote them; a call whose arena is longer than the previous call's clears the
difference before reading any flag.  These tests drive every facade and stage through shrinking
and growing layouts, with payload planted where a stale layout would have put flags."""
import numpy as np
import pytest

from gs300 import records as R
from gs300 import scene as S

from gpu_helpers import uniforms

pytestmark = pytest.mark.gpu

SERIAL_WORD = 14  # Ctrl::serial (the area's epoch counter), in 32-bit words from the area's start


def _keys(n, seed, bits=32):
    rng = np.random.default_rng(seed)
    keys = rng.integers(0, 1 << bits, size=n, dtype=np.uint64).astype(np.uint32)
    keys[rng.integers(0, n, size=n // 5)] = keys[0]  # ties
    return keys


def _sort_in(gs, torch, scratch, nbytes, keys, vals, key_bits=32):
    dk = torch.from_numpy(keys.view(np.int32).copy()).cuda()
    dv = torch.from_numpy(vals.view(np.int32).copy()).cuda()
    gs.RadixSorter.sort(dk, dv, len(keys), scratch, nbytes, key_bits=key_bits)
    st, _ = gs.Renderer.status(scratch)
    assert st == 0
    return dk.cpu().numpy().view(np.uint32), dv.cpu().numpy().view(np.uint32)


def _check_sorted(keys, vals, got, key_bits=32):
    m = np.uint64((1 << key_bits) - 1)
    order = np.argsort(keys.astype(np.uint64) & m, kind="stable")
    assert np.array_equal(got[1], vals[order])
    assert np.array_equal(got[0], keys[order])


def test_sort_scratch_sizes_alternate_with_planted_flags(gs, cuda):
    """Each sort leaves (key, value) pairs in its ping-pong buffers whose values make every pair
    read as an 'aggregate' look-back flag of the next call's epoch; the next call, smaller or
    larger, must not take any of them for a published flag."""
    torch = cuda
    big = 1 << 20
    nbytes = gs.RadixSorter.scratch_bytes(big)
    scratch = torch.zeros(nbytes, dtype=torch.uint8, device="cuda")
    for n, seed in ((5_000, 1), (100_000, 2), (big, 3), (300_001, 4), (big, 5), (7_681, 6), (big, 7)):
        serial = int(scratch[: 4 * (SERIAL_WORD + 1)].cpu().numpy().view(np.uint32)[SERIAL_WORD])
        e_next = serial + 2  # this call takes epoch serial + 1, the next one serial + 2
        k = _keys(n, seed)
        v = np.full(n, 4 * e_next + 1, np.uint32)  # flag word: epoch e_next, status 'aggregate'
        _check_sorted(k, v, _sort_in(gs, torch, scratch, nbytes, k, v))


def test_sort_scratch_sizes_and_key_bits_in_any_order(gs, cuda):
    torch = cuda
    nbytes = gs.RadixSorter.scratch_bytes(600_000)
    scratch = torch.zeros(nbytes, dtype=torch.uint8, device="cuda")
    for n, bits, seed in ((600_000, 32, 5), (50_000, 12, 6), (400_000, 20, 7), (3_840, 7, 8), (600_000, 32, 9),
                          (123_457, 32, 10), (600_000, 17, 11)):
        k = _keys(n, seed, bits)
        v = np.random.default_rng(seed).permutation(n).astype(np.uint32)
        _check_sorted(k, v, _sort_in(gs, torch, scratch, nbytes, k, v, key_bits=bits), key_bits=bits)


def test_rasterize_scratch_reused_across_sizes(gs, cuda):
    """gs_rasterize on one scratch with max_splats / target / max_pairs changing between calls
    gives the frame a fresh zeroed scratch gives."""
    torch = cuda
    from gpu_helpers import StagePipeline

    cap_splats, cap_pairs, cap_w, cap_h = 80_000, 8 * 80_000 + 4096, 640, 480
    nbytes = gs.Renderer.scratch_bytes(cap_splats, cap_w, cap_h, cap_pairs)
    shared = torch.zeros(nbytes, dtype=torch.uint8, device="cuda")
    for n, w, h, seed in ((80_000, 640, 480, 12), (20_000, 320, 240, 13), (60_000, 640, 360, 14), (5_000, 200, 120, 15),
                          (80_000, 640, 480, 16)):
        p = StagePipeline(gs, torch, S.synth_scene(n, seed=seed), R.FORMAT_FP32, w, h)
        u = uniforms(gs, w, h, k=seed, radius=6.0)
        want = p.render(u)
        p.target.zero_()
        mp = 8 * n + 4096
        assert gs.Renderer.scratch_bytes(n, w, h, mp) <= nbytes
        gs.Renderer.render(u, p.splats, p.indices, p.control.data_ptr() + 4, n, p.target, w, h, w * 4, mp, shared, nbytes)
        st, _ = gs.Renderer.status(shared)
        assert st == 0
        assert np.array_equal(p.frame(), want)


def test_server_slot_moves_to_a_smaller_scene(gs, cuda):
    """One slot serves a 150k scene, then a 120k scene at the same resolution (its raster scratch
    is kept and laid out for fewer splats); every frame equals the Viewer's."""
    mv = gs.MultiModelViewer()
    scenes = {"a": S.synth_scene(150_000, seed=20), "b": S.synth_scene(120_000, seed=21), "c": S.synth_scene(40_000, seed=22)}
    for k, sc in scenes.items():
        mv.insert_model(k, sc)
    sv = gs.Server(mv, budget_bytes=8 << 30, max_inflight=1)
    w, h = 640, 360
    for step, key in enumerate(["a", "b", "c", "b", "a", "c"]):
        cam = S.orbit_camera(3 * step + 1, radius=7.0)
        pod = gs.CameraPod.new(cam, (w, h))
        out = np.zeros((h, w, 4), np.uint8)
        sv.wait(sv.submit(key, pod, w, h, out))
        v = gs.Viewer(scenes[key])
        v.update_camera_with_pod(pod)
        t = gs.RenderTarget(w, h)
        v.render(t)
        v.synchronize()
        assert np.array_equal(out, t.download()), (step, key)
    assert sv.stats()["failed"] == 0


def test_multi_viewer_after_remove_model_matches_oracle(gs, cuda, oracle, monkeypatch):
    """The shared raster scratch keeps its size when the models' total shrinks (remove_model);
    frames stay equal to the oracle's key-order composite."""
    monkeypatch.setenv("GS300_EXACT_EXP", "1")
    w, h = 320, 240
    sizes = {"m0": 20_000, "m1": 30_000, "m2": 10_000}
    scenes = {k: S.synth_scene(n, seed=40 + i) for i, (k, n) in enumerate(sizes.items())}
    mts = {k: gs.model_transform_pod((0.25 * i, 0.0, 0.0), (0.0, 0.0, 0.0, 1.0), (1.0, 1.0, 1.0))
           for i, k in enumerate(sizes)}
    mv = gs.MultiModelViewer()
    for k, sc in scenes.items():
        mv.insert_model(k, sc)
        mv.update_model_transform_with_pod(k, mts[k])
    t = gs.RenderTarget(w, h)

    def check(keys, cam_k):
        pod = gs.CameraPod.new(S.orbit_camera(cam_k, radius=5.0), (w, h))
        mv.update_camera_with_pod(pod)
        mv.render(t, keys)
        mv.synchronize()
        want = oracle.new_target(w, h)
        for k in keys:
            u = oracle.frame_uniforms(pod, mts[k], gs.gaussian_transform_pod(), w, h)
            oracle.render(u, scenes[k], R.FORMAT_FP32, w, h, exp_mode=0, threads=8, target=want)
        assert np.array_equal(t.download(), want), keys

    check(["m0", "m1", "m2"], 4)
    mv.remove_model("m1")
    check(["m0", "m2"], 9)
    check(["m2"], 17)
    mv.insert_model("m1", scenes["m1"])
    mv.update_model_transform_with_pod("m1", mts["m1"])
    check(["m2", "m1", "m0"], 25)
