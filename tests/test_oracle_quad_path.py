"""The pixel -> quad-offset map every rasteriser here shares, checked against the reference's own
vertex stage taken literally.

oracle.render_quads builds each visible instance's six clip-space vertices as vert_main does
(proj·(view·world) plus the quad corners scaled by w, src/shader/render.wesl:75-130), rasterises
its two triangles at pixel centres under the top-left rule with the interpolated quad offset,
and runs frag_main and the blend (render.wesl:143-181, src/renderer.rs:296-300).  Its frames
must match the oracle's (which the CUDA path matches bit for bit) within the path's tolerance:
at least 99.9 % of pixels within 1/255 and PSNR >= 45 dB, in all three display modes."""
import math

import numpy as np
import pytest

from gs300 import records as R
from gs300 import scene as S


def _cmp(a, b):
    d = np.abs(a.astype(np.int32) - b.astype(np.int32))[..., :3]
    mse = (d.astype(np.float64) ** 2).mean()
    psnr = math.inf if mse == 0 else 10.0 * math.log10(255.0 ** 2 / mse)
    return float((d.max(axis=-1) <= 1).mean()), psnr


CASES = [(30_000, 320, 240, R.DISPLAY_SPLAT, 3, 6.0), (30_000, 320, 240, R.DISPLAY_ELLIPSE, 5, 6.0),
         (30_000, 320, 240, R.DISPLAY_POINT, 7, 6.0), (100_000, 640, 360, R.DISPLAY_SPLAT, 9, 8.0),
         (50_000, 300, 200, R.DISPLAY_SPLAT, 11, 4.0)]


@pytest.mark.parametrize("n,w,h,mode,k,radius", CASES)
def test_quad_map_matches_the_reference_vertex_stage(oracle, n, w, h, mode, k, radius):
    sc = S.synth_scene(n, seed=n + k)
    pod = oracle.camera_pod(S.orbit_camera(k, radius=radius), w, h)
    gt = R.GaussianTransformPod.new(display_mode=mode)
    u = oracle.frame_uniforms(pod, R.ModelTransformPod.new(), gt, w, h)
    mapped, *_ = oracle.render(u, sc, R.FORMAT_FP32, w, h, exp_mode=1, threads=4)
    literal, v = oracle.render_quads(pod, u, sc, R.FORMAT_FP32, w, h)
    assert v > 0 and literal[..., :3].max() > 0
    within, psnr = _cmp(mapped, literal)
    assert within >= 0.999 and psnr >= 45.0
    assert np.all(literal[..., 3] == 255)


def test_quad_path_known_answer_red_gaussian(oracle):
    """tests/e2e/viewer.rs:72-96 through the literal vertex stage: one red Gaussian at (0,0,1)
    renders red only."""
    g = np.zeros(1, dtype=R.GAUSSIAN_DTYPE)
    g["rot"] = (0.0, 0.0, 0.0, 1.0)
    g["pos"] = (0.0, 0.0, 1.0)
    g["color"] = (255, 0, 0, 255)
    g["scale"] = (1.0, 1.0, 1.0)
    recs = S.pack_gaussians(g)
    pod = oracle.camera_pod(S.given_camera(), 1024, 1024)
    u = oracle.frame_uniforms(pod, R.ModelTransformPod.new(), R.GaussianTransformPod.new(), 1024, 1024)
    img, v = oracle.render_quads(pod, u, recs, R.FORMAT_FP32, 1024, 1024)
    assert v == 1
    counts = (img > 0).sum(axis=(0, 1))
    assert counts[0] > 1 and counts[1] == 0 and counts[2] == 0 and counts[3] > 1
