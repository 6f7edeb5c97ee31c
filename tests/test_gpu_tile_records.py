"""Tile records stored by the preprocess of a one-model view.

The Viewer's preprocess writes each visible splat's tiles (rectangle, kept-corner mask, count) and
its binning gathers those 16-byte records; the stage-level path gathers the 48-byte splat and
works the tiles out in the count kernel.  Both must give the same tile lists: the same frame and
the same number of (tile, splat) pairs, in every display mode and record format, at targets
whose tile grid is ragged and at 4K."""
import numpy as np
import pytest

from gpu_helpers import StagePipeline, uniforms
from gs300 import records as R
from gs300 import scene as S

pytestmark = pytest.mark.gpu

MODES = [R.DISPLAY_SPLAT, R.DISPLAY_ELLIPSE, R.DISPLAY_POINT]


def _viewer_frame(gs, sc, fmt, w, h, k, mode, radius):
    v = gs.Viewer(sc, fmt=None if fmt == R.FORMAT_FP32 else fmt)
    try:
        v.update_gaussian_transform(1.0, mode, 3, False, 3.0)
        v.update_camera(S.orbit_camera(k, radius=radius), (w, h))
        t = gs.RenderTarget(w, h)
        v.render(t)
        v.synchronize()
        _, pairs = v.stats()
        return t.download(), pairs
    finally:
        v.close()


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("fmt", [R.FORMAT_FP32, R.FORMAT_HALF_SH_BF16])
@pytest.mark.parametrize("w,h", [(1280, 720), (1000, 563)])
def test_viewer_tile_records_match_stage_binning(gs, cuda, mode, fmt, w, h):
    sc = S.synth_scene(150_000, seed=31, fmt=fmt)
    pipe = StagePipeline(gs, cuda, sc, fmt, w, h)
    for k in (3, 47):
        got, pairs = _viewer_frame(gs, sc, fmt, w, h, k, mode, 6.0)
        want = pipe.render(uniforms(gs, w, h, k=k, mode=mode, radius=6.0))
        st, stage_pairs = gs.Renderer.status(pipe.r_scratch)
        assert st == 0
        assert pairs == stage_pairs > 0
        assert np.array_equal(got, want), f"{(got != want).any(axis=-1).sum()} pixels differ"


def test_viewer_tile_records_follow_target_size(gs, cuda):
    """One viewer rendering a sequence of target sizes: each frame's records are for its own
    tile grid (the stage path recomputes the tiles every time)."""
    sc = S.synth_scene(100_000, seed=32)
    v = gs.Viewer(sc)
    try:
        for k, (w, h) in enumerate([(640, 360), (1920, 1080), (333, 197), (3840, 2160), (640, 360)]):
            v.update_camera(S.orbit_camera(k, radius=6.0), (w, h))
            t = gs.RenderTarget(w, h)
            v.render(t)
            v.synchronize()
            _, pairs = v.stats()
            pipe = StagePipeline(gs, cuda, sc, R.FORMAT_FP32, w, h, max_pairs=64 * len(sc))
            want = pipe.render(uniforms(gs, w, h, k=k, radius=6.0))
            st, stage_pairs = gs.Renderer.status(pipe.r_scratch)
            assert st == 0 and pairs == stage_pairs
            assert np.array_equal(t.download(), want)
    finally:
        v.close()
