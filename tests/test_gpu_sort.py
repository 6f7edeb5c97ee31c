"""K2 radix sort on the GPU: bit-exact against a stable sort of the same (key, value) pairs.

The reference RadixSorter is a stable LSD sort (src/radix_sorter.rs:73 builds it with
subgroup size 1, so its in-block ranking is index-ordered), hence a stable sort by u32 key is
its exact restatement; tests/test_oracle_wgpu_sort.py pins that by re-executing the reference
sorter workgroup by workgroup, and the last test here holds the CUDA depth sort of a real
preprocess output to that re-execution directly."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(gs, torch, keys, vals, count=None, key_bits=32, max_count=None):
    n = len(keys) if max_count is None else max_count
    dk = torch.from_numpy(keys.view(np.int32).copy()).cuda()
    dv = torch.from_numpy(vals.view(np.int32).copy()).cuda()
    if n == 0:
        dk = torch.zeros(1, dtype=torch.int32, device="cuda")
        dv = torch.zeros(1, dtype=torch.int32, device="cuda")
    nb = gs.RadixSorter.scratch_bytes(n)
    scratch = torch.zeros(max(nb, 1), dtype=torch.uint8, device="cuda")
    cnt = None
    if count is not None:
        cnt = torch.tensor([count], dtype=torch.int32, device="cuda")
    gs.RadixSorter.sort(dk, dv, n, scratch, nb, count=cnt, key_bits=key_bits)
    torch.cuda.synchronize()
    st, _ = gs.Renderer.status(scratch)
    assert st == 0
    return dk.cpu().numpy().view(np.uint32), dv.cpu().numpy().view(np.uint32)


def _expect(keys, vals, key_bits=32):
    mask = np.uint32(0xFFFFFFFF) if key_bits == 32 else np.uint32((1 << key_bits) - 1)
    order = np.argsort(keys & mask, kind="stable")
    return keys[order], vals[order]


@pytest.mark.parametrize("n", [0, 1, 2, 31, 255, 3839, 3840, 3841, 7681, 100003, 1 << 20])
def test_sort_bit_exact(gs, cuda, n):
    rng = np.random.default_rng(n)
    keys = rng.random(n).astype(np.float32).view(np.uint32)
    if n > 10:
        keys[rng.integers(0, n, size=n // 3)] = keys[0]  # heavy ties
    vals = rng.permutation(n).astype(np.uint32)
    k, v = _run(gs, cuda, keys, vals)
    ek, ev = _expect(keys, vals)
    assert np.array_equal(k[:n], ek) and np.array_equal(v[:n], ev)


def test_sort_all_equal_keys_is_identity(gs, cuda):
    n = 50000
    keys = np.full(n, 0x3F000000, np.uint32)
    vals = np.arange(n, dtype=np.uint32)[::-1].copy()
    k, v = _run(gs, cuda, keys, vals)
    assert np.array_equal(v, vals) and np.array_equal(k, keys)


def test_sort_extreme_keys_and_pads(gs, cuda):
    """Keys 0, 0xFFFFFFFF and the 2.0 pad of preprocess.wesl:118-125 sort like any other."""
    rng = np.random.default_rng(7)
    n = 20000
    keys = rng.integers(0, 1 << 32, size=n, dtype=np.uint64).astype(np.uint32)
    keys[::5] = 0xFFFFFFFF
    keys[1::5] = 0
    keys[2::11] = np.float32(2.0).view(np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    k, v = _run(gs, cuda, keys, vals)
    ek, ev = _expect(keys, vals)
    assert np.array_equal(k, ek) and np.array_equal(v, ev)


@pytest.mark.parametrize("count", [0, 1, 3840, 12345])
def test_sort_device_count_leaves_tail_untouched(gs, cuda, count):
    """sort_indirect semantics: only the first `count` pairs (read on the device) are sorted."""
    rng = np.random.default_rng(count + 1)
    n = 20000
    keys = rng.random(n).astype(np.float32).view(np.uint32)
    vals = rng.permutation(n).astype(np.uint32)
    k, v = _run(gs, cuda, keys, vals, count=count)
    ek, ev = _expect(keys[:count], vals[:count])
    assert np.array_equal(k[:count], ek) and np.array_equal(v[:count], ev)
    assert np.array_equal(k[count:], keys[count:]) and np.array_equal(v[count:], vals[count:])


@pytest.mark.parametrize("bits", [1, 7, 13, 16, 20, 30])  # 30: depth keys, match.any in the last pass
def test_sort_partial_key_bits(gs, cuda, bits):
    rng = np.random.default_rng(bits)
    n = 70000
    keys = rng.integers(0, 1 << bits, size=n).astype(np.uint32)
    keys[::3] |= rng.integers(0, 1 << 32, size=keys[::3].size, dtype=np.uint64).astype(np.uint32) & ~np.uint32((1 << bits) - 1)
    vals = np.arange(n, dtype=np.uint32)
    k, v = _run(gs, cuda, keys, vals, key_bits=bits)  # bits above key_bits are ignored
    ek, ev = _expect(keys, vals, bits)
    assert np.array_equal(k, ek) and np.array_equal(v, ev)


def test_sort_repeated_calls_reuse_scratch(gs, cuda):
    """Look-back flags are epoch-tagged, so one scratch area serves many sorts without clearing."""
    torch = cuda
    n = 30000
    nb = gs.RadixSorter.scratch_bytes(n)
    scratch = torch.zeros(nb, dtype=torch.uint8, device="cuda")
    for it in range(6):
        rng = np.random.default_rng(100 + it)
        keys = rng.random(n).astype(np.float32).view(np.uint32)
        vals = rng.permutation(n).astype(np.uint32)
        dk = torch.from_numpy(keys.view(np.int32).copy()).cuda()
        dv = torch.from_numpy(vals.view(np.int32).copy()).cuda()
        gs.RadixSorter.sort(dk, dv, n, scratch, nb)
        torch.cuda.synchronize()
        ek, ev = _expect(keys, vals)
        assert np.array_equal(dk.cpu().numpy().view(np.uint32), ek)
        assert np.array_equal(dv.cpu().numpy().view(np.uint32), ev)


def test_sort_full_size_properties(gs, cuda):
    """6M depth keys (the largest plain scene): sorted, a permutation, stable on ties."""
    torch = cuda
    n = 6_000_000
    g = torch.Generator(device="cuda").manual_seed(5)
    keys = torch.rand(n, generator=g, device="cuda")
    keys = torch.floor(keys * 1e5) / 1e5  # ~1e5 distinct keys -> many ties
    dk = keys.view(torch.int32).clone()
    vals = torch.arange(n, dtype=torch.int32, device="cuda")
    nb = gs.RadixSorter.scratch_bytes(n)
    scratch = torch.zeros(nb, dtype=torch.uint8, device="cuda")
    gs.RadixSorter.sort(dk, vals, n, scratch, nb)
    torch.cuda.synchronize()
    sk = dk.view(torch.float32)
    assert bool((sk[1:] >= sk[:-1]).all())
    assert bool((torch.sort(vals.long())[0] == torch.arange(n, device="cuda")).all())
    same = sk[1:] == sk[:-1]
    assert bool((vals[1:][same] > vals[:-1][same]).all())
    assert bool((keys[vals.long()] == sk).all())


def test_depth_sort_equals_reference_sorter_reexecution(gs, cuda, oracle):
    """Preprocess -> sort through the stage entry points; the depth buffer and index buffer as the
    preprocess left them (V keys, 2.0 pads up to the dispatch) go through the literal re-execution
    of the reference sorter (num_keys = N, dispatch ceil(V / 3840)); the first V entries of both
    must be identical."""
    from gs300 import records as R
    from gs300 import scene as S

    from gpu_helpers import StagePipeline, uniforms

    torch = cuda
    for n, seed, radius in ((150_000, 3, 8.0), (20_000, 4, 5.0)):
        p = StagePipeline(gs, torch, S.synth_scene(n, seed=seed), R.FORMAT_FP32, 640, 360)
        p.preprocess(uniforms(gs, 640, 360, k=seed, radius=radius))
        torch.cuda.synchronize()
        v = p.count()
        x = int(p.control[4].item())  # the sort dispatch {ceil(V/3840), 1, 1}
        assert x == (v + 3839) // 3840
        keys = p.depths.cpu().numpy().view(np.uint32).copy()
        idx = p.indices.cpu().numpy().view(np.uint32).copy()
        depth = np.zeros(4 * p.depth_cap, np.uint32)  # GaussiansDepthBuffer is 4 x keys_buffer_size
        depth[: len(keys)] = keys
        rk, rp = oracle.wgpu_radix_sort(depth, idx, n, x, 1)
        p.sort()
        torch.cuda.synchronize()
        gk = p.depths.cpu().numpy().view(np.uint32)
        gi = p.indices.cpu().numpy().view(np.uint32)
        assert np.array_equal(gk[:v], rk[:v]) and np.array_equal(gi[:v], rp[:v])
