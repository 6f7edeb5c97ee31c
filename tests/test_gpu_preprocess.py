"""K1 preprocess on the GPU against the CPU oracle.

Keys, indices, counts and pads are compared bit for bit; so are the splat records (2D axes ->
pixel-to-quad map, SH colour): both sides evaluate the same FP32 operations in the same order
with no contraction, so the stated ulp bound for keys, conics and colours is 0."""
import numpy as np
import pytest

from gpu_helpers import StagePipeline, uniforms
from gs300 import records as R
from gs300 import scene as S

pytestmark = pytest.mark.gpu


def _compare(oracle, pipe, u, records, fmt, selection=None, invert=False):
    pipe.preprocess(u, selection=selection, invert=invert)
    pipe.torch.cuda.synchronize()
    idx, dep, spl = oracle.preprocess(u, records, fmt, selection=selection, invert=invert, threads=8)
    v = len(idx)
    ctl = pipe.control.cpu().numpy().view(np.uint32)
    assert ctl[0] == 6 and ctl[1] == v and ctl[2] == 0 and ctl[3] == 0  # DrawIndirectArgs
    assert ctl[4] == (v + 3839) // 3840 and ctl[5] == 1 and ctl[6] == 1  # sort dispatch
    got_idx = pipe.indices.cpu().numpy().view(np.uint32)[:v]
    got_dep = pipe.depths.cpu().numpy()
    assert np.array_equal(got_idx, idx)
    assert np.array_equal(got_dep[:v].view(np.uint32), dep.view(np.uint32))
    pad_end = min(((v + 3839) // 3840) * 3840, pipe.depth_cap)
    assert np.all(got_dep[v:pad_end] == 2.0)
    got_spl = pipe.splat_records()
    if v:
        assert got_spl[idx].tobytes() == spl[idx].tobytes()
    return v


@pytest.mark.parametrize("n", [1, 127, 128, 129, 5000, 100_000])
@pytest.mark.parametrize("mode", [R.DISPLAY_SPLAT, R.DISPLAY_POINT])
def test_preprocess_bit_exact_fp32(gs, cuda, oracle, n, mode):
    sc = S.synth_scene(n, seed=n)
    pipe = StagePipeline(gs, cuda, sc, R.FORMAT_FP32, 320, 180)
    for k in (0, 31):
        u = uniforms(gs, 320, 180, k=k, mode=mode, radius=6.0)
        _compare(oracle, pipe, u, sc, R.FORMAT_FP32)


@pytest.mark.parametrize("fmt", [R.FORMAT_HALF_SH_FP16, R.FORMAT_HALF_SH_BF16])
def test_preprocess_bit_exact_half(gs, cuda, oracle, fmt):
    sc = S.synth_scene(50_000, seed=11, fmt=fmt)
    pipe = StagePipeline(gs, cuda, sc, fmt, 640, 360)
    u = uniforms(gs, 640, 360, k=44)
    assert _compare(oracle, pipe, u, sc, fmt) > 1000


def test_preprocess_model_transform_and_sh_degrees(gs, cuda, oracle):
    sc = S.synth_scene(20_000, seed=12)
    pipe = StagePipeline(gs, cuda, sc, R.FORMAT_FP32, 400, 300)
    mt = gs.model_transform_pod((0.5, -0.2, 1.0), (0.1, 0.2, 0.3, 0.927361849549570), (1.5, 0.7, 1.1))
    for deg in range(4):
        for no_sh0 in (False, True):
            u = uniforms(gs, 400, 300, k=7, mt=mt, sh_deg=deg, no_sh0=no_sh0, std=2.0, size=0.8)
            _compare(oracle, pipe, u, sc, R.FORMAT_FP32)


def test_preprocess_selection_mask(gs, cuda, oracle):
    n = 30_000
    sc = S.synth_scene(n, seed=13)
    pipe = StagePipeline(gs, cuda, sc, R.FORMAT_FP32, 320, 180)
    u = uniforms(gs, 320, 180, k=2)
    bits = np.random.default_rng(0).integers(0, 1 << 32, size=(n + 31) // 32, dtype=np.uint64).astype(np.uint32)
    for invert in (False, True):
        _compare(oracle, pipe, u, sc, R.FORMAT_FP32, selection=bits, invert=invert)


def test_preprocess_large_scene(gs, cuda, oracle):
    """1M Gaussians (the full-scale plain configuration) at 1920x1080."""
    sc = S.synth_scene(1_000_000, seed=1)
    pipe = StagePipeline(gs, cuda, sc, R.FORMAT_FP32, 1920, 1080, max_pairs=16)
    u = uniforms(gs, 1920, 1080, k=60)
    assert _compare(oracle, pipe, u, sc, R.FORMAT_FP32) > 800_000


def test_preprocess_everything_culled(gs, cuda, oracle):
    """All Gaussians moved far behind the camera: V = 0, dispatch 0, no pads."""
    sc = S.synth_scene(1000, seed=14)
    pipe = StagePipeline(gs, cuda, sc, R.FORMAT_FP32, 64, 64)
    cam = S.orbit_camera(0)
    pos = np.array(cam.pos, np.float64)
    fwd = -pos / np.linalg.norm(pos)
    mt = gs.model_transform_pod(tuple(pos - 100.0 * fwd))
    u = uniforms(gs, 64, 64, camera=cam, mt=mt)
    assert _compare(oracle, pipe, u, sc, R.FORMAT_FP32) == 0
