"""PLY ingest on the CPU: the library's header scan (gs_ply_parse_header, host only) against the
Python reader, its error cases, and the oracle's vertex -> record conversion against the Python
reader + packers (gs300/ply.py, gs300/scene.py) and the coverage/model.ply golden fixture."""
import os

import numpy as np
import pytest

from gs300 import ply
from gs300 import records as R
from gs300 import scene as S
from ply_helpers import CASES, gaussian_fields, ply_bytes, random_vertices

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FORMATS = [R.FORMAT_FP32, R.FORMAT_HALF_SH_FP16, R.FORMAT_HALF_SH_BF16]


def _python_records(data, fmt):
    g = ply.load_ply(data)
    return S.pack_gaussians(g) if fmt == R.FORMAT_FP32 else S.pack_gaussians_half(g, fmt)


def _assert_same_records(got, want, fmt):
    """Bit-exact, except that the FP32 record's cov3d may differ by 1 ulp from numpy's: its 3x3
    double products may round a sum differently in the last bit (the library and the oracle
    use one fixed order without contraction)."""
    if fmt != R.FORMAT_FP32:
        assert got.tobytes() == want.tobytes()
        return
    for f in ("pos", "color", "sh", "_pad"):
        assert np.array_equal(got[f].view(np.uint32), want[f].view(np.uint32)), f
    a = got["cov3d"].view(np.int32).astype(np.int64)
    b = want["cov3d"].view(np.int32).astype(np.int64)
    ulps = np.abs(a - b)
    assert ulps.max() <= 1
    if ulps.size >= 1000:
        assert (ulps == 0).mean() > 0.99


def _model_ply():
    d = np.load(os.path.join(GOLDEN, "model_ply.npz"), allow_pickle=False)
    names = [str(n) for n in d["field_names"]]
    verts = np.ascontiguousarray(d["vertices"], dtype="<f4")
    data = ply_bytes(verts.reshape(-1).view(np.dtype([(n, "<f4") for n in names])), [(n, "float") for n in names])
    return d, data


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_native_header_matches_python(gs, case):
    _, fields, before = case
    v = random_vertices(37, fields, seed=1)
    data = ply_bytes(v, fields, before=before, after=("face", 3, [("vertex_indices", "int")]))
    L = gs.ply_parse_header(data)
    count, dt, off = ply.parse_header(data)
    assert (L.count, L.stride, L.data_offset) == (count, dt.itemsize, off)
    name_off = {n: dt.fields[n][1] for n in dt.names}
    assert list(L.pos) == [name_off[n] for n in "xyz"]
    assert list(L.f_dc) == [name_off[f"f_dc_{c}"] for c in range(3)]
    assert L.opacity == name_off["opacity"]
    assert list(L.scale) == [name_off[f"scale_{i}"] for i in range(3)]
    assert list(L.rot) == [name_off[f"rot_{i}"] for i in range(4)]
    m = sum(1 for n in dt.names if n.startswith("f_rest_"))
    assert L.sh_rest == m // 3
    assert list(L.f_rest)[:m] == [name_off[f"f_rest_{i}"] for i in range(m)]
    assert all(x == -1 for x in list(L.f_rest)[m:])


def test_native_header_model_ply(gs):
    d, data = _model_ply()
    L = gs.ply_parse_header(data)
    assert L.count == 9 and L.stride == 4 * len(d["field_names"]) and L.sh_rest == 15


def _bad(fields=None, fmt="binary_little_endian", before=None, mutate=None):
    fields = fields or gaussian_fields()
    data = ply_bytes(random_vertices(4, fields, seed=2), fields, before=before, fmt=fmt)
    return mutate(data) if mutate else data


BAD = [
    ("ascii", lambda: _bad(fmt="ascii")),
    ("big_endian", lambda: _bad(fmt="binary_big_endian")),
    ("not_ply", lambda: b"plx\n" + _bad()[4:]),
    ("no_end_header", lambda: _bad().replace(b"end_header\n", b"end_headr\n")),
    ("missing_rot_3", lambda: _bad(fields=[f for f in gaussian_fields() if f[0] != "rot_3"])),
    ("double_x", lambda: _bad(fields=[("x", "double") if f[0] == "x" else f for f in gaussian_fields()])),
    ("f_rest_10", lambda: _bad(fields=[f for f in gaussian_fields() if f[0] not in
                                       {f"f_rest_{i}" for i in range(10, 45)}])),
    ("f_rest_gap", lambda: _bad(fields=[f for f in gaussian_fields(sh_rest=3) if f[0] != "f_rest_4"]
                                + [("f_rest_9", "float")])),
    ("stride_over_1024", lambda: _bad(fields=gaussian_fields(extra=[(f"e{i}", "double") for i in range(100)]))),
    ("list_before_vertex", lambda: _bad().replace(b"element vertex", b"element face 1\nproperty list uchar int idx\n"
                                                                    b"element vertex")),
    ("unknown_type", lambda: _bad().replace(b"property float x\n", b"property quad q\nproperty float x\n")),
    ("count_not_a_number", lambda: _bad().replace(b"element vertex 4", b"element vertex 4x")),
]


@pytest.mark.parametrize("make", [b[1] for b in BAD], ids=[b[0] for b in BAD])
def test_native_header_rejects(gs, make):
    with pytest.raises(gs.GsError) as e:
        gs.ply_parse_header(make())
    assert e.value.status == 1


def test_native_header_list_in_vertex(gs):
    fields = gaussian_fields()
    data = ply_bytes(random_vertices(2, fields, seed=3), fields).replace(
        b"property float x\n", b"property list uchar int idx\nproperty float x\n")
    with pytest.raises(gs.GsError):
        gs.ply_parse_header(data)
    with pytest.raises(ValueError):
        ply.parse_header(data)


def test_oracle_model_ply_matches_python_and_golden(oracle):
    d, data = _model_ply()
    import gs300

    L = gs300.ply_parse_header(data)
    block = data[L.data_offset:]
    for fmt in FORMATS:
        _assert_same_records(oracle.ply_convert(block, L, fmt), _python_records(data, fmt), fmt)
    _assert_same_records(oracle.ply_convert(block, L, R.FORMAT_FP32), d["records"], R.FORMAT_FP32)


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("fmt", FORMATS)
def test_oracle_convert_matches_python(gs, oracle, case, fmt):
    """The oracle's restatement and the Python reader + packers agree bit for bit."""
    _, fields, before = case
    v = random_vertices(20_000, fields, seed=11)
    data = ply_bytes(v, fields, before=before)
    L = gs.ply_parse_header(data)
    _assert_same_records(oracle.ply_convert(data[L.data_offset:], L, fmt), _python_records(data, fmt), fmt)


def test_pack_matches_oracle_cov3d(gs, oracle):
    """gs_gaussian_pack (the library's host packer, same cov3d routine as the device
    converter) equals the oracle's FP32 records built from the same core::Gaussian values."""
    fields = gaussian_fields()
    data = ply_bytes(random_vertices(5000, fields, seed=5), fields)
    L = gs.ply_parse_header(data)
    want = oracle.ply_convert(data[L.data_offset:], L, R.FORMAT_FP32)
    got = gs.pack_gaussians(ply.load_ply(data))
    assert got.tobytes() == want.tobytes()
