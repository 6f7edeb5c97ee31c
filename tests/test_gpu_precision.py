"""Precision tier: FP16 rotation/scale with FP16 or BF16 SH records rendered on the GPU (FP32
projection, conic and blending) against the host FP64 oracle of the same pipeline: PSNR >= 45 dB
and at most a few 8-bit levels of per-channel error, next to the FP32 records."""
import math

import numpy as np
import pytest

from gs300 import records as R
from gs300 import scene as S

pytestmark = pytest.mark.gpu


def _psnr(a, b):
    d = a[..., :3].astype(np.float64) - b[..., :3].astype(np.float64)
    mse = (d ** 2).mean()
    return math.inf if mse == 0 else 10.0 * math.log10(255.0 ** 2 / mse)


@pytest.mark.parametrize("fmt", [R.FORMAT_FP32, R.FORMAT_HALF_SH_FP16, R.FORMAT_HALF_SH_BF16])
def test_frames_against_fp64_oracle(gs, cuda, oracle, fmt):
    n, w, h = 1_000_000, 1920, 1080
    sc = S.synth_scene(n, seed=6, fmt=fmt)
    v = gs.Viewer(sc, fmt=None if fmt == R.FORMAT_FP32 else fmt)
    t = gs.RenderTarget(w, h)
    for k in (0, 45):
        cam = S.orbit_camera(k)
        v.update_camera(cam, (w, h))
        v.render(t)
        v.synchronize()
        got = t.download()
        ref, _ = oracle.render64(gs.CameraPod.new(cam, (w, h)), gs.model_transform_pod(), gs.gaussian_transform_pod(),
                                 sc, fmt, w, h, threads=16)
        err = np.abs(got.astype(np.int32) - ref.astype(np.int32))[..., :3]
        assert _psnr(got, ref) >= 45.0
        assert err.max() <= 8
