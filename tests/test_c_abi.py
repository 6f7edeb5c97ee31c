"""The public header is C: a C99 program includes include/gs300.h (gcc -std=c99 -Wall -Wextra
-Werror -pedantic), links libgs300.so and calls it.  Host-side results must equal the Python
binding's; on a GPU the C program's Viewer frame must equal the Python Viewer's."""
import os
import shutil
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(REPO, "tests", "c_abi", "gs_abi_smoke.c")


@pytest.fixture(scope="module")
def c_program(gs, tmp_path_factory):
    from gs300 import _lib

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    out = str(tmp_path_factory.mktemp("c_abi") / "gs_abi_smoke")
    libdir = os.path.dirname(_lib.LIB_PATH)
    cmd = [cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", os.path.join(REPO, "include"), SRC,
           "-o", out, "-L", libdir, "-l:libgs300.so", f"-Wl,-rpath,{libdir}", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def _camera(gs):
    import math

    from gs300 import records as R

    c = R.Camera()
    c.z_near, c.z_far = 0.1, 1e4
    c.vertical_fov = np.float32(60.0 * math.pi / 180.0)
    c.pitch, c.yaw = 0.1, 0.1
    return c


def test_header_compiles_as_c99_and_host_calls_match(gs, c_program):
    r = subprocess.run([c_program, "host"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = dict(line.split(" ", 1) for line in r.stdout.strip().splitlines())
    assert lines["version"] == gs.lib().gs_version().decode()
    caps = [int(x) for x in lines["depth_capacity"].split()]
    assert caps == [gs.Preprocessor.depth_capacity(n) for n in (0, 1_000_000, 3840)]
    assert int(lines["bad_sh_degree"]) == 1
    import ctypes

    from gs300 import records as R

    sizes = [int(x) for x in lines["sizeof"].split()]
    assert sizes == [224, 144, ctypes.sizeof(R.FrameUniforms)]
    c = _camera(gs)
    c.pos[:] = [np.uint32(int(x, 16)).view(np.float32) for x in lines["camera"].split()]
    pod = gs.CameraPod.new(c, (1920, 1080))

    def bits(a):
        return " ".join(f"{int(x):08x}" for x in np.asarray(a, np.float32).view(np.uint32))

    assert lines["view"] == bits(pod.view)
    assert lines["proj"] == bits(pod.proj)
    assert lines["size"] == bits(pod.size)


@pytest.mark.gpu
def test_c_program_renders_the_python_viewers_frame(gs, cuda, c_program, tmp_path):
    from gs300 import scene as S

    sc = S.synth_scene(50_000, seed=9)
    recs = tmp_path / "records.bin"
    recs.write_bytes(np.ascontiguousarray(sc).tobytes())
    w, h = 320, 240
    out = tmp_path / "frame.rgba"
    r = subprocess.run([c_program, "render", str(recs), str(out), str(w), str(h)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = np.frombuffer(out.read_bytes(), np.uint8).reshape(h, w, 4)
    # the same camera through the Python binding: position as the C program computed it
    host = subprocess.run([c_program, "host"], capture_output=True, text=True).stdout
    pos = [np.uint32(int(x, 16)).view(np.float32) for x in dict(l.split(" ", 1) for l in host.splitlines())["camera"].split()]
    c = _camera(gs)
    c.pos[:] = pos
    v = gs.Viewer(sc)
    v.update_camera(c, (w, h))
    t = gs.RenderTarget(w, h)
    v.render(t)
    v.synchronize()
    want = t.download()
    assert got[..., :3].max() > 0
    assert np.array_equal(got, want)
