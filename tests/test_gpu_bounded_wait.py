"""Bounded device waits: a look-back whose predecessor never publishes gives up after its poll
limit, the stage reports GS_ERR_TIMEOUT through its scratch status (or the facade's
synchronize), the call returns, and the next calls on the same buffers are correct again.

The failure is made on purpose without faulting anything: with gs_debug_set_wait_fault, one
look-back tile of each launch publishes nothing (a flag that nothing sets), and the poll limit is
lowered so that the waits end within milliseconds."""
import numpy as np
import pytest

from gs300 import records as R
from gs300 import scene as S

from gpu_helpers import StagePipeline, uniforms

pytestmark = pytest.mark.gpu

TIMEOUT = 5  # GS_ERR_TIMEOUT


@pytest.fixture
def wait_fault(gs):
    gs.debug_set_wait_fault(2000, 1)  # tile 1 of every look-back launch never publishes
    try:
        yield
    finally:
        gs.debug_set_wait_fault()


def test_sort_wait_runs_out_then_recovers(gs, cuda):
    torch = cuda
    n = 50_000  # 7 sort blocks of 7680 keys: tiles 2.. wait on tile 1
    rng = np.random.default_rng(1)
    keys = rng.integers(0, 1 << 32, size=n, dtype=np.uint64).astype(np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    nbytes = gs.RadixSorter.scratch_bytes(n)
    scratch = torch.zeros(nbytes, dtype=torch.uint8, device="cuda")
    # every buffer of the call has a guard zone after it that must stay untouched
    pad = 4096
    dk = torch.zeros(n + pad, dtype=torch.int32, device="cuda")
    dv = torch.zeros(n + pad, dtype=torch.int32, device="cuda")
    dk[n:] = -7
    dv[n:] = -7
    dk[:n] = torch.from_numpy(keys.view(np.int32).copy()).cuda()
    dv[:n] = torch.from_numpy(vals.view(np.int32).copy()).cuda()
    gs.debug_set_wait_fault(2000, 1)
    try:
        gs.RadixSorter.sort(dk, dv, n, scratch, nbytes)
        st, _ = gs.Renderer.status(scratch)
    finally:
        gs.debug_set_wait_fault()
    assert st == TIMEOUT
    assert bool((dk[n:] == -7).all()) and bool((dv[n:] == -7).all())
    dk[:n] = torch.from_numpy(keys.view(np.int32).copy()).cuda()
    dv[:n] = torch.from_numpy(vals.view(np.int32).copy()).cuda()
    gs.RadixSorter.sort(dk, dv, n, scratch, nbytes)
    st, _ = gs.Renderer.status(scratch)
    assert st == 0
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(dk[:n].cpu().numpy().view(np.uint32), keys[order])
    assert np.array_equal(dv[:n].cpu().numpy().view(np.uint32), vals[order])


def test_preprocess_wait_runs_out_then_recovers(gs, cuda):
    torch = cuda
    sc = S.synth_scene(40_000, seed=2)  # 313 preprocess tiles
    w, h = 320, 240
    p = StagePipeline(gs, torch, sc, R.FORMAT_FP32, w, h)
    u = uniforms(gs, w, h, k=3, radius=6.0)
    gs.debug_set_wait_fault(2000, 1)
    try:
        p.preprocess(u)
        st, _ = gs.Renderer.status(p.pre_scratch)
    finally:
        gs.debug_set_wait_fault()
    assert st == TIMEOUT
    assert p.count() <= p.n
    p.preprocess(u)
    st, _ = gs.Renderer.status(p.pre_scratch)
    assert st == 0
    idx = p.indices[: p.count()].cpu().numpy()
    assert np.all(np.diff(idx) > 0)  # compaction in ascending Gaussian order again


def test_viewer_frame_reports_timeout_then_renders_again(gs, cuda, wait_fault):
    sc = S.synth_scene(60_000, seed=4)
    w, h = 320, 240
    v = gs.Viewer(sc)
    v.update_camera(S.orbit_camera(7, radius=6.0), (w, h))
    t = gs.RenderTarget(w, h)
    v.render(t)
    with pytest.raises(gs.GsError) as err:
        v.synchronize()
    assert err.value.status == TIMEOUT
    gs.debug_set_wait_fault()
    v.render(t)
    v.synchronize()
    got = t.download()
    ref = gs.Viewer(sc)
    ref.update_camera(S.orbit_camera(7, radius=6.0), (w, h))
    t2 = gs.RenderTarget(w, h)
    ref.render(t2)
    ref.synchronize()
    assert np.array_equal(got, t2.download())

