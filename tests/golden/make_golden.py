"""Regenerates the golden fixtures in this folder (run in a container that has the reference
checkout; nothing at test time reads the reference).

model_ply.npz — from the reference's own 9-Gaussian PLY fixture (coverage/model.ply):
  * vertices:  the decoded PLY vertex block (62 FP32 fields per vertex, this file's own copy);
  * gaussians: core::Gaussian values after this library's PLY conversion;
  * records:   the packed 224-byte device records;
  * sorted_indices/sorted_depths/frame: the CPU oracle's depth-sorted draw order and keys and
    its 128x128 RGBA8 frame for one
    camera looking at the model's centre (splat mode, std 3, SH degree 3).
synthetic_small.npz — a 600-Gaussian seeded scene rendered by the oracle at 96x64 in all
three display modes (portable exp), to catch drift of the oracle itself.

Usage: python tests/golden/make_golden.py PATH/TO/coverage/model.ply
(the reference checkout's 9-Gaussian PLY fixture; the path is required).
"""
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "wgpu-3dgs-viewer_gb300"))

from gs300 import ply  # noqa: E402
from gs300 import records as R  # noqa: E402
from gs300 import scene as S  # noqa: E402
from oracle import oracle as O  # noqa: E402

MODEL_CENTRE = (4.0, 4.0, 4.0)


def model_camera():
    yaw, pitch, dist = 0.1, 0.1, 18.0
    f = np.array([math.cos(pitch) * math.sin(yaw), math.sin(pitch), math.cos(pitch) * math.cos(yaw)])
    pos = np.array(MODEL_CENTRE) - dist * f
    return R.Camera.new(0.1, 1e4, math.radians(60.0), pos=tuple(float(x) for x in pos), pitch=pitch, yaw=yaw)


def render_model(records, w=128, h=128):
    pod = O.camera_pod(model_camera(), w, h)
    u = O.frame_uniforms(pod, R.ModelTransformPod.new(), R.GaussianTransformPod.new(), w, h)
    return O.render(u, records, R.FORMAT_FP32, w, h, exp_mode=0, threads=0)


def synthetic_frames():
    sc = S.synth_scene(600, seed=0)
    out = {"records": sc}
    for mode, name in ((R.DISPLAY_SPLAT, "splat"), (R.DISPLAY_ELLIPSE, "ellipse"), (R.DISPLAY_POINT, "point")):
        pod = O.camera_pod(S.orbit_camera(3, radius=6.0), 96, 64)
        u = O.frame_uniforms(pod, R.ModelTransformPod.new(), R.GaussianTransformPod.new(display_mode=mode), 96, 64)
        img, idx, dep, _ = O.render(u, sc, R.FORMAT_FP32, 96, 64, exp_mode=0, threads=0)
        out[f"{name}_frame"] = img
        out[f"{name}_sorted_indices"] = idx
        out[f"{name}_sorted_depths"] = dep
    return out


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py PATH/TO/coverage/model.ply (the reference's PLY fixture)")
    src = sys.argv[1]
    verts = ply.read_vertices(src)
    g = ply.vertices_to_gaussians(verts)
    recs = S.pack_gaussians(g)
    frame, idx, dep, spl = render_model(recs)
    np.savez_compressed(
        os.path.join(HERE, "model_ply.npz"),
        vertices=np.asarray(verts.tolist(), dtype=np.float32),
        field_names=np.array(verts.dtype.names),
        gaussians=g, records=recs, sorted_indices=idx, sorted_depths=dep, frame=frame,
    )
    np.savez_compressed(os.path.join(HERE, "synthetic_small.npz"), **synthetic_frames())
    print("wrote", os.listdir(HERE))


if __name__ == "__main__":
    main()
