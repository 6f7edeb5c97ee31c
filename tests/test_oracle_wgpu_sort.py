"""The stable-sort oracle of the depth sort, pinned to the reference's own algorithm.

oracle/gs_oracle_wgpusort.cpp re-executes the reference sorter workgroup by workgroup
(src/shader/radix_sort.wgsl:78-529 as src/radix_sorter.rs builds it: subgroup size 1, 4 x 8-bit
passes, 3840-key blocks, state num_keys = N, indirect dispatch ceil(V / 3840)), on buffers laid
out as the reference's preprocess leaves them (keys [0, V) then 2.0 pads up to the dispatch,
src/shader/preprocess.wesl:108-126).  Its first V outputs must equal a stable sort of the V
(key, index) pairs — the oracle the CUDA sort is held to — under two workgroup schedules."""
import numpy as np
import pytest

BLOCK = 3840
TWO = np.float32(2.0).view(np.uint32)


def keys_buffer_size(n):
    return (n + BLOCK - 1) // BLOCK * BLOCK


def depth_buffers(rng, n, v, kind):
    """Depth buffer (4 x keys_buffer_size(N) u32, as GaussiansDepthBuffer allocates) and index
    buffer (N u32) after a preprocess that found v visible Gaussians."""
    keys = rng.integers(0, 1 << 32, size=4 * keys_buffer_size(n), dtype=np.uint64).astype(np.uint32)  # stale
    if kind == "uniform":
        real = rng.random(v, dtype=np.float32)
    elif kind == "near_far":  # 1 - ndc.z near 0.01: few distinct keys, many ties
        real = (np.float32(1.0) - (np.float32(0.99) + rng.integers(0, 2000, v).astype(np.float32) * np.float32(6e-8)))
    elif kind == "all_equal":
        real = np.full(v, np.float32(0.25))
    else:
        raise ValueError(kind)
    keys[:v] = np.asarray(real, np.float32).view(np.uint32)
    x = (v + BLOCK - 1) // BLOCK
    keys[v:min(x * BLOCK, len(keys))] = TWO  # `post` pads the dispatch's last block with 2.0
    idx = rng.integers(0, 1 << 32, size=n, dtype=np.uint64).astype(np.uint32)  # stale entries
    idx[:v] = np.sort(rng.choice(n, size=v, replace=False)).astype(np.uint32)  # ascending compaction
    return keys, idx, x


CASES = [(1, 1, "uniform"), (5000, 3839, "uniform"), (5000, 3840, "uniform"), (8000, 3841, "near_far"),
         (60_000, 50_000, "uniform"), (60_000, 57_599, "near_far"), (20_000, 20_000, "all_equal"),
         (120_000, 100_003, "near_far"), (7681, 7681, "uniform")]


@pytest.mark.parametrize("n,v,kind", CASES)
def test_reference_sorter_equals_stable_sort(oracle, n, v, kind):
    rng = np.random.default_rng(n + v)
    keys, idx, x = depth_buffers(rng, n, v, kind)
    order = np.argsort(keys[:v], kind="stable")
    for schedule in (0, 1):
        k, p = oracle.wgpu_radix_sort(keys, idx, n, x, schedule)
        assert np.array_equal(k[:v], keys[:v][order])
        assert np.array_equal(p[:v], idx[:v][order])
    # the std::stable_sort oracle the CUDA tests use, on the same pairs
    sk, sv = keys[:v].copy(), idx[:v].copy()
    oracle.lib().oracle_stable_sort(oracle._p(sk), oracle._p(sv), v)
    assert np.array_equal(sk, k[:v]) and np.array_equal(sv, p[:v])


def test_reference_sorter_full_range_keys(oracle):
    """Arbitrary u32 keys (not only depths): over the processed slots [0, x·3840) the result is the
    stable sort of those slots, padding keys included."""
    rng = np.random.default_rng(7)
    n = 3 * BLOCK
    keys = rng.integers(0, 1 << 32, size=4 * keys_buffer_size(n), dtype=np.uint64).astype(np.uint32)
    keys[: n // 3] = keys[0]
    idx = np.arange(n, dtype=np.uint32)
    k, p = oracle.wgpu_radix_sort(keys, idx, n, 3, 1)
    order = np.argsort(keys[:n], kind="stable")
    assert np.array_equal(k[:n], keys[:n][order]) and np.array_equal(p, idx[order])


def test_reference_sorter_empty_dispatch_leaves_buffers(oracle):
    rng = np.random.default_rng(8)
    keys, idx, x = depth_buffers(rng, 1000, 0, "uniform")
    assert x == 0
    k, p = oracle.wgpu_radix_sort(keys, idx, 1000, x, 0)
    assert np.array_equal(k, keys) and np.array_equal(p, idx)
