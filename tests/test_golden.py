"""Golden fixtures (tests/golden/, made by make_golden.py from the reference's coverage/model.ply
and a seeded scene): the PLY conversion, the oracle, and on the GPU the CUDA path, against them."""
import os

import numpy as np
import pytest

from gs300 import ply
from gs300 import records as R
from gs300 import scene as S

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


def _ply_bytes(names, verts):
    head = ["ply", "format binary_little_endian 1.0", f"element vertex {len(verts)}"]
    head += [f"property float {n}" for n in names]
    head.append("end_header")
    return ("\n".join(head) + "\n").encode() + np.ascontiguousarray(verts, dtype="<f4").tobytes()


def test_model_ply_decodes_to_pure_colours():
    """The fixture's f_dc / opacity decode to exact 8-bit primaries under rgb = 0.5 + SH_C0·dc,
    alpha = sigmoid(opacity): evidence that this is the crate's convention."""
    d = _load("model_ply.npz")
    g = ply.load_ply(_ply_bytes([str(n) for n in d["field_names"]], d["vertices"]))
    assert np.array_equal(g, d["gaussians"])
    colours = {tuple(c) for c in g["color"].tolist()}
    assert (255, 0, 0, 255) in colours and (0, 0, 255, 255) in colours and (0, 0, 0, 255) in colours
    assert np.allclose(np.linalg.norm(g["rot"], axis=1), 1.0, atol=1e-6)


def test_model_ply_oracle_matches_golden(oracle):
    d = _load("model_ply.npz")
    recs = S.pack_gaussians(d["gaussians"])
    assert recs.tobytes() == d["records"].tobytes()
    from golden.make_golden import render_model  # noqa: E402

    frame, idx, dep, _ = render_model(recs)
    assert np.array_equal(idx, d["sorted_indices"])
    assert np.array_equal(dep.view(np.uint32), d["sorted_depths"].view(np.uint32))
    assert np.array_equal(frame, d["frame"])
    assert (frame[..., :3] > 0).any(axis=-1).sum() > 1000


@pytest.mark.parametrize("mode", ["splat", "ellipse", "point"])
def test_synthetic_oracle_matches_golden(oracle, mode):
    from golden.make_golden import synthetic_frames

    d = _load("synthetic_small.npz")
    assert d["records"].tobytes() == S.synth_scene(600, seed=0).tobytes()
    now = synthetic_frames()
    assert np.array_equal(now[f"{mode}_frame"], d[f"{mode}_frame"])
    assert np.array_equal(now[f"{mode}_sorted_indices"], d[f"{mode}_sorted_indices"])


@pytest.mark.gpu
def test_model_ply_cuda_matches_golden(gs, cuda, monkeypatch):
    """The CUDA path (portable exp) renders the golden frame bit for bit through the Viewer."""
    from golden.make_golden import model_camera

    monkeypatch.setenv("GS300_EXACT_EXP", "1")
    d = _load("model_ply.npz")
    v = gs.Viewer(d["records"])
    v.update_camera(model_camera(), (128, 128))
    t = gs.RenderTarget(128, 128)
    v.render(t)
    v.synchronize()
    assert np.array_equal(t.download(), d["frame"])


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [R.DISPLAY_SPLAT, R.DISPLAY_ELLIPSE, R.DISPLAY_POINT])
def test_synthetic_cuda_matches_golden(gs, cuda, monkeypatch, mode):
    monkeypatch.setenv("GS300_EXACT_EXP", "1")
    d = _load("synthetic_small.npz")
    name = {R.DISPLAY_SPLAT: "splat", R.DISPLAY_ELLIPSE: "ellipse", R.DISPLAY_POINT: "point"}[mode]
    v = gs.Viewer(d["records"])
    v.update_camera(S.orbit_camera(3, radius=6.0), (96, 64))
    v.update_gaussian_transform(1.0, mode, 3, False, 3.0)
    t = gs.RenderTarget(96, 64)
    v.render(t)
    v.synchronize()
    assert np.array_equal(t.download(), d[f"{name}_frame"])
