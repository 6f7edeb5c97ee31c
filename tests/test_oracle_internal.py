"""Self-consistency of the CPU oracle: literal vs tiled rasteriser, sorts, exp, compaction."""
import math

import numpy as np
import pytest

from gs300 import records as R
from gs300 import scene as S


def _uniforms(oracle, w, h, k=0, mode=R.DISPLAY_SPLAT, radius=8.0, mt=None, sh_deg=3, no_sh0=False, std=3.0):
    pod = oracle.camera_pod(S.orbit_camera(k, radius=radius), w, h)
    gt = R.GaussianTransformPod.new(display_mode=mode, sh_deg=sh_deg, no_sh0=no_sh0, max_std_dev=std)
    return oracle.frame_uniforms(pod, mt or R.ModelTransformPod.new(), gt, w, h)


@pytest.mark.parametrize("mode", [R.DISPLAY_SPLAT, R.DISPLAY_ELLIPSE, R.DISPLAY_POINT])
@pytest.mark.parametrize("exp_mode", [0, 1])
def test_tiled_rasteriser_equals_literal_quads(oracle, mode, exp_mode):
    sc = S.synth_scene(4000, seed=3)
    u = _uniforms(oracle, 200, 120, k=5, mode=mode, radius=6.0)
    a, idx, dep, spl = oracle.render(u, sc, R.FORMAT_FP32, 200, 120, exp_mode=exp_mode, threads=0)
    b, idx2, dep2, spl2 = oracle.render(u, sc, R.FORMAT_FP32, 200, 120, exp_mode=exp_mode, threads=4)
    assert np.array_equal(idx, idx2) and np.array_equal(dep.view(np.uint32), dep2.view(np.uint32))
    assert np.array_equal(a, b)
    assert a[..., :3].max() > 0


def test_exp_portable_accuracy(oracle):
    xs = np.linspace(-10.0, 0.0, 20001, dtype=np.float32)
    got = np.array([oracle.exp_portable(float(x)) for x in xs], np.float64)
    want = np.exp(xs.astype(np.float64))
    rel = np.abs(got - want) / want
    assert rel.max() < 3.0 * 2.0 ** -23


def test_stable_sort_matches_numpy(oracle):
    rng = np.random.default_rng(1)
    keys = rng.integers(0, 50, size=5000).astype(np.uint32)
    vals = np.arange(5000, dtype=np.uint32)
    k, v = oracle.stable_sort(keys, vals)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(k, keys[order]) and np.array_equal(v, vals[order])


@pytest.mark.parametrize("threads", [1, 3, 8])
def test_parallel_radix_sort_equals_stable_sort(oracle, threads):
    rng = np.random.default_rng(threads)
    keys = rng.random(30011).astype(np.float32)
    keys[::7] = keys[3]  # many ties
    vals = rng.integers(0, 1 << 31, size=keys.size).astype(np.uint32)
    a = oracle.stable_sort(keys, vals)
    b = oracle.radix_sort(keys, vals, threads)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_preprocess_compaction_is_ordered_and_keys_in_range(oracle):
    sc = S.synth_scene(20000, seed=4)
    u = _uniforms(oracle, 320, 180, k=17)
    idx, dep, spl = oracle.preprocess(u, sc, R.FORMAT_FP32)
    assert len(idx) > 0.5 * len(sc)
    assert np.all(np.diff(idx.astype(np.int64)) > 0)
    assert np.all((dep >= 0.0) & (dep <= 1.0))
    # Gaussians behind the camera are culled
    cam = S.orbit_camera(17)
    fwd = -np.array(cam.pos, np.float64) / np.linalg.norm(cam.pos)
    behind = (sc["pos"].astype(np.float64) - np.array(cam.pos)) @ fwd < 0
    assert not np.isin(np.nonzero(behind)[0], idx).any()


def test_preprocess_threads_agree(oracle):
    sc = S.synth_scene(10000, seed=5)
    u = _uniforms(oracle, 320, 180, k=3)
    a = oracle.preprocess(u, sc, R.FORMAT_FP32, threads=1)
    b = oracle.preprocess(u, sc, R.FORMAT_FP32, threads=6)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert a[2].tobytes() == b[2].tobytes()


def test_selection_mask(oracle):
    sc = S.synth_scene(3000, seed=6)
    u = _uniforms(oracle, 160, 90)
    all_idx, *_ = oracle.preprocess(u, sc, R.FORMAT_FP32)
    bits = np.zeros((3000 + 31) // 32, np.uint32)
    chosen = np.arange(0, 3000, 3)
    np.bitwise_or.at(bits, chosen // 32, (1 << (chosen % 32)).astype(np.uint32))
    # preprocess.wesl:68-78 — skipped when (invert != 0) == bit
    sel, *_ = oracle.preprocess(u, sc, R.FORMAT_FP32, selection=bits, invert=False)
    inv, *_ = oracle.preprocess(u, sc, R.FORMAT_FP32, selection=bits, invert=True)
    assert np.array_equal(sel, np.intersect1d(all_idx, chosen))
    assert np.array_equal(inv, np.setdiff1d(all_idx, chosen))


@pytest.mark.parametrize("fmt", [R.FORMAT_HALF_SH_FP16, R.FORMAT_HALF_SH_BF16])
def test_half_records_close_to_fp32(oracle, fmt):
    n, w, h = 20000, 320, 180
    full = S.synth_scene(n, seed=7)
    half = S.synth_scene(n, seed=7, fmt=fmt)
    u = _uniforms(oracle, w, h, k=9)
    a, *_ = oracle.render(u, full, R.FORMAT_FP32, w, h, threads=4)
    b, *_ = oracle.render(u, half, fmt, w, h, threads=4)
    d = np.abs(a.astype(np.int32) - b.astype(np.int32))[..., :3]
    mse = (d.astype(np.float64) ** 2).mean()
    psnr = 10 * math.log10(255.0 ** 2 / max(mse, 1e-12))
    assert psnr > 35.0


def test_fp64_twin_agrees_with_fp32_oracle(oracle):
    """The FP64 twin (precision reference) and the FP32 oracle differ by rounding only."""
    n, w, h = 30000, 320, 180
    sc = S.synth_scene(n, seed=8)
    pod = oracle.camera_pod(S.orbit_camera(4), w, h)
    mt, gt = R.ModelTransformPod.new(), R.GaussianTransformPod.new()
    u = oracle.frame_uniforms(pod, mt, gt, w, h)
    a, *_ = oracle.render(u, sc, R.FORMAT_FP32, w, h, exp_mode=1, threads=4)
    b, v = oracle.render64(pod, mt, gt, sc, R.FORMAT_FP32, w, h, threads=4)
    d = np.abs(a.astype(np.int32) - b.astype(np.int32))[..., :3]
    mse = (d.astype(np.float64) ** 2).mean()
    assert v > n // 2 and d.max() <= 2 and 10 * math.log10(255.0 ** 2 / max(mse, 1e-12)) > 60.0
