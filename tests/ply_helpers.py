"""Seeded PLY files for the ingest tests: the standard 3D Gaussian splatting vertex, with
optional extra properties (any PLY type, so strides need not be multiples of 4), fewer SH bands,
and elements declared before the vertex element."""
import numpy as np

_NP = {"float": "<f4", "double": "<f8", "uchar": "u1", "char": "i1", "ushort": "<u2", "short": "<i2",
       "uint": "<u4", "int": "<i4"}


def gaussian_fields(sh_rest=15, normals=True, extra=()):
    """[(name, ply type)] of a vertex: x y z [nx ny nz] f_dc_0..2 f_rest_0..3K-1 opacity scale rot,
    with `extra` (name, type) pairs inserted after the normals."""
    f = [("x", "float"), ("y", "float"), ("z", "float")]
    if normals:
        f += [("nx", "float"), ("ny", "float"), ("nz", "float")]
    f += list(extra)
    f += [(f"f_dc_{c}", "float") for c in range(3)]
    f += [(f"f_rest_{i}", "float") for i in range(3 * sh_rest)]
    f += [("opacity", "float")]
    f += [(f"scale_{i}", "float") for i in range(3)]
    f += [(f"rot_{i}", "float") for i in range(4)]
    return f


def random_vertices(n, fields, seed):
    rng = np.random.default_rng(seed)
    dt = np.dtype([(name, _NP[t]) for name, t in fields])
    v = np.zeros(n, dt)
    for name, t in fields:
        if t != "float" and t != "double":
            info = np.iinfo(_NP[t])
            v[name] = rng.integers(info.min, info.max, size=n, endpoint=True)
        elif name in ("x", "y", "z"):
            v[name] = rng.normal(0.0, 2.0, n)
        elif name.startswith("f_dc_"):
            v[name] = rng.normal(0.0, 0.8, n)
        elif name.startswith("f_rest_"):
            v[name] = rng.normal(0.0, 0.05, n)
        elif name == "opacity":
            v[name] = rng.normal(0.0, 2.0, n)
        elif name.startswith("scale_"):
            v[name] = rng.normal(-4.0, 0.5, n)
        elif name.startswith("rot_"):
            v[name] = rng.normal(0.0, 1.0, n)
        else:
            v[name] = rng.normal(0.0, 1.0, n)
    return v


def ply_bytes(vertices, fields, before=None, after=None, fmt="binary_little_endian"):
    """PLY file bytes.  `before` / `after`: (element name, count, [(name, type)]) declared before
    or after the vertex element, with zero-filled data."""
    head = ["ply", f"format {fmt} 1.0", "comment seeded test file"]
    body = b""
    if before:
        name, cnt, props = before
        head.append(f"element {name} {cnt}")
        head += [f"property {t} {p}" for p, t in props]
        body += np.zeros(cnt, np.dtype([(p, _NP[t]) for p, t in props])).tobytes()
    head.append(f"element vertex {len(vertices)}")
    head += [f"property {t} {name}" for name, t in fields]
    body += np.ascontiguousarray(vertices).tobytes()
    if after:
        name, cnt, props = after
        head.append(f"element {name} {cnt}")
        head += [f"property {t} {p}" for p, t in props]
        body += b"\0" * 64
    head.append("end_header")
    return ("\n".join(head) + "\n").encode() + body


# Layout cases shared by the CPU and GPU tests: (id, fields, before-element)
CASES = [
    ("standard", gaussian_fields(), None),
    ("odd_stride", gaussian_fields(extra=[("red", "uchar"), ("t", "short")]), None),
    ("sh_deg1_no_normals", gaussian_fields(sh_rest=3, normals=False), None),
    ("sh_deg2", gaussian_fields(sh_rest=8, extra=[("w8", "uchar")]), None),
    ("sh_deg0", gaussian_fields(sh_rest=0), ("camera", 2, [("cx", "double"), ("id", "uchar")])),
]
