"""Reader for the standard 3D Gaussian splatting PLY layout (binary little-endian vertices with
x, y, z, nx, ny, nz, f_dc_0..2, f_rest_0..44, opacity, scale_0..2, rot_0..3).

The reference loads scenes through the un-vendored wgpu-3dgs-core 0.6.0 PLY reader
(examples/simple.rs:156-160); its fixture is coverage/model.ply.  This module follows the
published convention of that format:
  * colour rgb = 0.5 + SH_C0 · f_dc (clamped, rounded to 8 bits), alpha = sigmoid(opacity);
  * f_rest is stored channel-major (K coefficients of R, then G, then B; K = 3, 8 or 15 for SH
    degree 1, 2 or 3, the missing bands zero);
  * scale = exp(scale_i); rotation is stored (w, x, y, z) and normalised.
The conversion constants are this library's own choice where the crate is unpinned.
"""
import numpy as np

from .records import GAUSSIAN_DTYPE
from .scene import SH_C0

_TYPES = {
    "float": "<f4", "float32": "<f4", "double": "<f8", "float64": "<f8",
    "uchar": "u1", "uint8": "u1", "char": "i1", "int8": "i1",
    "ushort": "<u2", "uint16": "<u2", "short": "<i2", "int16": "<i2",
    "uint": "<u4", "uint32": "<u4", "int": "<i4", "int32": "<i4",
}


def parse_header(data):
    """-> (vertex count, numpy dtype of one vertex, byte offset of the vertex block)."""
    end = data.find(b"end_header\n")
    if not data.startswith(b"ply") or end < 0:
        raise ValueError("not a PLY file")
    lines = data[:end].decode("ascii").splitlines()
    fmt = None
    elements = []  # [name, count, [(field, type)], has_list]
    for ln in lines[1:]:
        parts = ln.split()
        if not parts or parts[0] in ("comment", "obj_info"):
            continue
        if parts[0] == "format":
            fmt = parts[1]
        elif parts[0] == "element":
            elements.append([parts[1], int(parts[2]), [], False])
        elif parts[0] == "property":
            if parts[1] == "list":
                if elements[-1][0] == "vertex":
                    raise ValueError("list properties are not supported in the vertex element")
                elements[-1][3] = True
            else:
                elements[-1][2].append((parts[2], _TYPES[parts[1]]))
    if fmt != "binary_little_endian":
        raise ValueError(f"unsupported PLY format {fmt}")
    offset = end + len(b"end_header\n")
    for name, count, fields, has_list in elements:
        if name == "vertex":
            return count, np.dtype(fields), offset
        if has_list:
            raise ValueError(f"element {name} before the vertex element has a list property")
        offset += count * np.dtype(fields).itemsize
    raise ValueError("PLY has no vertex element")


def read_vertices(path_or_bytes):
    data = path_or_bytes if isinstance(path_or_bytes, (bytes, bytearray)) else open(path_or_bytes, "rb").read()
    count, dt, off = parse_header(data)
    return np.frombuffer(data, dtype=dt, count=count, offset=off)


def vertices_to_gaussians(v):
    """Structured PLY vertices -> core::Gaussian values (GAUSSIAN_DTYPE)."""
    n = len(v)
    out = np.zeros(n, dtype=GAUSSIAN_DTYPE)
    out["pos"] = np.stack([v["x"], v["y"], v["z"]], axis=1)
    dc = np.stack([v[f"f_dc_{c}"] for c in range(3)], axis=1).astype(np.float64)
    rgb = np.clip(0.5 + SH_C0 * dc, 0.0, 1.0)
    op = 1.0 / (1.0 + np.exp(-v["opacity"].astype(np.float64)))
    out["color"][:, :3] = np.rint(rgb * 255.0).astype(np.uint8)
    out["color"][:, 3] = np.rint(op * 255.0).astype(np.uint8)
    names = v.dtype.names
    m = sum(1 for r in names if r.startswith("f_rest_"))
    if m not in (0, 9, 24, 45):
        raise ValueError(f"PLY f_rest count must be 0, 9, 24 or 45, not {m}")
    if m:
        k = m // 3  # coefficients per channel; bands above the file's degree stay zero
        fr = np.stack([v[f"f_rest_{i}"] for i in range(m)], axis=1).reshape(n, 3, k)  # [channel][coefficient]
        sh = np.zeros((n, 15, 3), dtype=np.float32)
        sh[:, :k, :] = np.transpose(fr, (0, 2, 1))
        out["sh"] = sh.reshape(n, 45)
    out["scale"] = np.exp(np.stack([v[f"scale_{i}"] for i in range(3)], axis=1).astype(np.float64))
    q = np.stack([v["rot_1"], v["rot_2"], v["rot_3"], v["rot_0"]], axis=1).astype(np.float64)
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    out["rot"] = q
    return out


def load_ply(path_or_bytes):
    """A PLY file (path or bytes) -> core::Gaussian values ready for Viewer / pack_gaussians."""
    return vertices_to_gaussians(read_vertices(path_or_bytes))


def vertex_block(path_or_bytes):
    """(raw vertex bytes, count, stride, {field: byte offset}) for the device-side converter."""
    data = path_or_bytes if isinstance(path_or_bytes, (bytes, bytearray)) else open(path_or_bytes, "rb").read()
    count, dt, off = parse_header(data)
    offsets = {name: dt.fields[name][1] for name in dt.names}
    return data[off:off + count * dt.itemsize], count, dt.itemsize, offsets
