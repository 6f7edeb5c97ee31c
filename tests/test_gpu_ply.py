"""PLY ingest on the GPU: gs_ply_convert against the oracle's conversion (bit-exact), and the
Viewer / MultiModelViewer facades that build their records from a PLY file on the device."""
import ctypes

import numpy as np
import pytest

from gs300 import records as R
from gs300 import scene as S
from ply_helpers import CASES, gaussian_fields, ply_bytes, random_vertices

FORMATS = [R.FORMAT_FP32, R.FORMAT_HALF_SH_FP16, R.FORMAT_HALF_SH_BF16]


def _device_convert(gs, cuda, data, fmt, offset=0):
    L = gs.ply_parse_header(data)
    block = np.frombuffer(data[L.data_offset:L.data_offset + L.count * L.stride], dtype=np.uint8)
    dev = cuda.zeros(len(block) + 64, dtype=cuda.uint8, device="cuda")
    dev[offset:offset + len(block)] = cuda.from_numpy(block.copy()).cuda()
    rb = R.record_dtype(fmt).itemsize
    out = cuda.full((max(L.count, 1) * rb,), 0xAB, dtype=cuda.uint8, device="cuda")
    s = cuda.cuda.current_stream()
    gs.ply_convert(dev.data_ptr() + offset, L, fmt, out.data_ptr(), stream=s.cuda_stream)
    s.synchronize()
    return L, out.cpu().numpy()[:L.count * rb].view(R.record_dtype(fmt))


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("fmt", FORMATS)
def test_convert_matches_oracle(gs, oracle, cuda, case, fmt):
    _, fields, before = case
    data = ply_bytes(random_vertices(100_003, fields, seed=21), fields, before=before)
    L, got = _device_convert(gs, cuda, data, fmt)
    want = oracle.ply_convert(data[L.data_offset:], L, fmt)
    assert got.tobytes() == want.tobytes()


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 2, 127, 128, 129, 4097])
def test_convert_sizes_and_unaligned_base(gs, oracle, cuda, n):
    """Ragged CTA tails, and a vertex block starting 4 bytes into its allocation."""
    fields = gaussian_fields(extra=[("flag", "uchar")])  # stride 249: fields at every byte phase
    data = ply_bytes(random_vertices(n, fields, seed=n), fields)
    for fmt in FORMATS:
        L, got = _device_convert(gs, cuda, data, fmt, offset=4)
        assert got.tobytes() == oracle.ply_convert(data[L.data_offset:], L, fmt).tobytes()


@pytest.mark.gpu
def test_convert_rejects_bad_arguments(gs, cuda):
    fields = gaussian_fields()
    data = ply_bytes(random_vertices(10, fields, seed=1), fields)
    L = gs.ply_parse_header(data)
    dev = cuda.zeros(4096, dtype=cuda.uint8, device="cuda")
    out = cuda.zeros(4096, dtype=cuda.uint8, device="cuda")
    with pytest.raises(gs.GsError):  # vertices not 4-byte aligned
        gs.ply_convert(dev.data_ptr() + 2, L, R.FORMAT_FP32, out.data_ptr())
    with pytest.raises(gs.GsError):  # records not 16-byte aligned
        gs.ply_convert(dev.data_ptr(), L, R.FORMAT_FP32, out.data_ptr() + 8)
    with pytest.raises(gs.GsError):  # unknown format
        gs.ply_convert(dev.data_ptr(), L, 7, out.data_ptr())
    bad = R.PlyLayout.from_buffer_copy(bytes(L))
    bad.rot[2] = bad.stride - 2  # a field reaching past the vertex
    with pytest.raises(gs.GsError):
        gs.ply_convert(dev.data_ptr(), bad, R.FORMAT_FP32, out.data_ptr())


def _frame(viewer, gs, w=320, h=180):
    viewer.update_camera(S.orbit_camera(3, radius=6.0), (w, h))
    t = gs.RenderTarget(w, h)
    viewer.render(t)
    viewer.synchronize()
    return t.download()


@pytest.mark.gpu
@pytest.mark.parametrize("fmt", FORMATS)
def test_viewer_from_ply(gs, oracle, cuda, fmt):
    fields = gaussian_fields(extra=[("red", "uchar")])
    data = ply_bytes(random_vertices(30_000, fields, seed=4), fields)
    L = gs.ply_parse_header(data)
    recs = oracle.ply_convert(data[L.data_offset:], L, fmt)
    a = gs.Viewer.from_ply(data, fmt)
    b = gs.Viewer(recs, fmt)
    assert len(a) == 30_000
    fa, fb = _frame(a, gs), _frame(b, gs)
    assert (fa[..., :3] > 0).any()
    assert np.array_equal(fa, fb)


@pytest.mark.gpu
def test_multi_viewer_from_ply(gs, oracle, cuda):
    fields = gaussian_fields(sh_rest=8)
    data = ply_bytes(random_vertices(20_000, fields, seed=8), fields)
    L = gs.ply_parse_header(data)
    recs = oracle.ply_convert(data[L.data_offset:], L, R.FORMAT_FP32)
    mv_a, mv_b = gs.MultiModelViewer(), gs.MultiModelViewer()
    mv_a.insert_model_from_ply("m", data)
    mv_b.insert_model("m", recs)
    frames = []
    for mv in (mv_a, mv_b):
        mv.update_camera(S.orbit_camera(5, radius=6.0), (256, 256))
        t = gs.RenderTarget(256, 256)
        mv.render(t, ["m"])
        frames.append(t.download())
    assert np.array_equal(frames[0], frames[1])


@pytest.mark.gpu
def test_viewer_from_ply_edge_cases(gs, cuda):
    fields = gaussian_fields()
    data = ply_bytes(random_vertices(100, fields, seed=9), fields)
    with pytest.raises(gs.GsError) as e:  # shorter than the header says
        gs.Viewer.from_ply(data[:-1])
    assert e.value.status == 1
    empty = ply_bytes(random_vertices(0, fields, seed=9), fields)
    v = gs.Viewer.from_ply(empty)
    assert len(v) == 0
    frame = _frame(v, gs, 64, 32)
    assert (frame[..., :3] == 0).all() and (frame[..., 3] == 255).all()
