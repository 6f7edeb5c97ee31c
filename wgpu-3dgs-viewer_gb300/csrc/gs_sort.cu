// gs_sort.cu — K2: stable LSD onesweep radix sort of u32 keys carrying u32 values.
//
// Same contract as the reference RadixSorter (src/radix_sorter.rs:56-96,658-669; kernels
// src/shader/radix_sort.wgsl:78-529): 8-bit digits, least significant first, 3840 keys per
// block, stable.  The GB300 design differs: one global-histogram kernel reads the keys once
// for all passes; each pass is a single kernel that ranks its block with warp ballots (so
// equal digits keep input order), publishes per-digit counts and resolves the block's global
// offsets by decoupled look-back (virtual block ids from an atomic ticket, every wait bounded),
// then scatters through shared memory so that each digit's run is written contiguously.
// The key count may live in device memory (the preprocess instance count), so a whole frame
// can be enqueued (or graph-captured) without a host round trip.
#include "gs_internal.h"

namespace gs {

constexpr uint32_t kSortThreads = 256;
constexpr uint32_t kSortRows = 15;
constexpr uint32_t kTileKeys = kSortThreads * kSortRows;  // 3840
constexpr uint32_t kSortWarps = kSortThreads / 32;
static_assert(kTileKeys == GS_SORT_BLOCK_KVS, "block size must match the reference's");

__global__ void ctrl_init_kernel(Ctrl *ctrl, int mode) {
    const uint32_t t = threadIdx.x;
    if (t == 0) {
        uint32_t e = ctrl->epoch + 1u;
        if (e >= (1u << 30) || e == 0u) e = 1u;
        ctrl->epoch = e;
        ctrl->ticket[0] = 0u;
        if (mode == 1) {
            ctrl->status = 0u;
            for (int k = 1; k < 8; ++k) ctrl->ticket[k] = 0u;
            ctrl->count = 0u;
            ctrl->total = 0u;
            ctrl->pair_base = 0u;
        }
    }
    if (mode == 1)
        for (uint32_t k = t; k < 4 * 256; k += blockDim.x) (&ctrl->hist[0][0])[k] = 0u;
}

__device__ __forceinline__ uint32_t load_count(const uint32_t *count, uint32_t max_count) {
    return count ? min(*count, max_count) : max_count;
}

// Global digit histograms of all passes in one read of the keys.  Per pass, the warp counts
// the digit of lane 0 with one ballot (the high digits of float depth keys are nearly
// constant, and same-address shared atomics would serialise) and the other keys with plain
// shared atomics.
__global__ void __launch_bounds__(256) sort_hist_kernel(const uint32_t *__restrict__ keys,
                                                        const uint32_t *count, uint32_t max_count,
                                                        uint32_t npasses, Ctrl *ctrl) {
    __shared__ uint32_t h[4][256];
    for (uint32_t k = threadIdx.x; k < 4 * 256; k += blockDim.x) (&h[0][0])[k] = 0u;
    __syncthreads();
    const uint32_t n = load_count(count, max_count);
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t lane = threadIdx.x & 31u;
    // Whole warps iterate together (bounds padded to the warp) so the ballots see 32 lanes.
    const uint32_t nr = (n + 31u) & ~31u;
    for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < nr; idx += stride) {
        const bool valid = idx < n;
        const uint32_t k = valid ? keys[idx] : 0u;
        for (uint32_t p = 0; p < npasses; ++p) {
            const uint32_t d = (k >> (8u * p)) & 255u;
            const uint32_t d0 = __shfl_sync(0xFFFFFFFFu, d, 0);
            const uint32_t same = __ballot_sync(0xFFFFFFFFu, valid && d == d0);
            if (lane == 0 && same) atomicAdd(&h[p][d0], (uint32_t)__popc(same));
            if (valid && d != d0) atomicAdd(&h[p][d], 1u);
        }
    }
    __syncthreads();
    for (uint32_t p = 0; p < npasses; ++p) {
        const uint32_t v = h[p][threadIdx.x];
        if (v) atomicAdd(&ctrl->hist[p][threadIdx.x], v);
    }
}

// Exclusive block scan of one value per thread (256 threads).  `tmp` holds 8 words.
__device__ __forceinline__ uint32_t block_scan_excl(uint32_t v, uint32_t *tmp, uint32_t *total) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) tmp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t t = lane < kSortWarps ? tmp[lane] : 0u;
#pragma unroll
        for (uint32_t o = 1; o < kSortWarps; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < kSortWarps) tmp[lane] = t;
    }
    __syncthreads();
    const uint32_t before = warp ? tmp[warp - 1] : 0u;
    *total = tmp[kSortWarps - 1];
    __syncthreads();
    return before + x - v;
}

__global__ void __launch_bounds__(kSortThreads) sort_pass_kernel(
    const uint32_t *__restrict__ kin, const uint32_t *__restrict__ vin, uint32_t *__restrict__ kout,
    uint32_t *__restrict__ vout, const uint32_t *count, uint32_t max_count, uint32_t pass, Ctrl *ctrl,
    uint64_t *flags) {
    __shared__ uint32_t s_keys[kTileKeys];
    __shared__ uint32_t s_vals[kTileKeys];
    __shared__ uint32_t s_whist[kSortWarps][256];
    __shared__ uint32_t s_start[256];
    __shared__ uint32_t s_gbase[256];
    __shared__ uint32_t s_tmp[kSortWarps];
    __shared__ uint32_t s_tile, s_epoch;

    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    if (tid == 0) {
        s_epoch = *(volatile uint32_t *)&ctrl->epoch;
        s_tile = atomicAdd(&ctrl->ticket[1 + pass], 1u);
    }
    for (uint32_t k = tid; k < kSortWarps * 256; k += kSortThreads) (&s_whist[0][0])[k] = 0u;
    __syncthreads();
    const uint32_t n = load_count(count, max_count);
    const uint32_t ntiles = (n + kTileKeys - 1) / kTileKeys;
    const uint32_t tile = s_tile, epoch = s_epoch;
    if (tile >= ntiles) return;
    const uint32_t shift = 8u * pass;
    const uint32_t base = tile * kTileKeys + warp * (32u * kSortRows);

    uint32_t k[kSortRows], v[kSortRows], r[kSortRows];
#pragma unroll
    for (uint32_t i = 0; i < kSortRows; ++i) {
        const uint32_t pos = base + i * 32u + lane;
        const bool ok = pos < n;
        k[i] = ok ? kin[pos] : 0xFFFFFFFFu;
        v[i] = ok ? vin[pos] : 0u;
    }
    // Warp-local stable ranking: lanes that share a digit form a peer mask from 8 ballots.
    const uint32_t lt = lanemask_lt();
#pragma unroll
    for (uint32_t i = 0; i < kSortRows; ++i) {
        const uint32_t d = (k[i] >> shift) & 255u;
        uint32_t peers = 0xFFFFFFFFu;
#pragma unroll
        for (uint32_t b = 0; b < 8; ++b) {
            const uint32_t bit = (d >> b) & 1u;
            const uint32_t bal = __ballot_sync(0xFFFFFFFFu, bit);
            peers &= bit ? bal : ~bal;
        }
        const uint32_t rank = __popc(peers & lt);
        const uint32_t pre = s_whist[warp][d];
        __syncwarp();
        if (rank == 0) s_whist[warp][d] = pre + __popc(peers);
        __syncwarp();
        r[i] = pre + rank;
    }
    __syncthreads();

    // Thread d owns digit d: per-warp exclusive offsets, block count, publication.
    const uint32_t d = tid;
    uint32_t run = 0;
#pragma unroll
    for (uint32_t w = 0; w < kSortWarps; ++w) {
        const uint32_t c = s_whist[w][d];
        s_whist[w][d] = run;
        run += c;
    }
    const uint32_t total = run;
    const uint32_t invalid = (tile == ntiles - 1) ? ntiles * kTileKeys - n : 0u;
    const uint32_t pub = (d == 255u) ? total - invalid : total;
    uint64_t *f = flags + (size_t)tile * 256u + d;
    if (tile == 0)
        st_release(f, pack_flag(epoch, kFlagPrefix, pub));
    else
        st_release(f, pack_flag(epoch, kFlagAggregate, pub));

    uint32_t blk_total, hist_total;
    const uint32_t start = block_scan_excl(total, s_tmp, &blk_total);
    const uint32_t goff = block_scan_excl(ctrl->hist[pass][d], s_tmp, &hist_total);
    uint32_t prefix = 0;
    if (tile > 0) {
        prefix = look_back(flags + d, 256u, tile, epoch, &ctrl->status);
        st_release(f, pack_flag(epoch, kFlagPrefix, prefix + pub));
    }
    s_start[d] = start;
    s_gbase[d] = goff + prefix;
    __syncthreads();

#pragma unroll
    for (uint32_t i = 0; i < kSortRows; ++i) {
        const uint32_t dd = (k[i] >> shift) & 255u;
        const uint32_t p = s_start[dd] + s_whist[warp][dd] + r[i];
        s_keys[p] = k[i];
        s_vals[p] = v[i];
    }
    __syncthreads();
    const uint32_t valid = min(kTileKeys, n - tile * kTileKeys);
    for (uint32_t j = tid; j < valid; j += kSortThreads) {
        const uint32_t key = s_keys[j];
        const uint32_t dd = (key >> shift) & 255u;
        const uint32_t o = s_gbase[dd] + (j - s_start[dd]);
        if (o < n) {  // always true unless a look-back timed out (status already set)
            kout[o] = key;
            vout[o] = s_vals[j];
        }
    }
}

__global__ void copy_pairs_kernel(const uint32_t *ks, const uint32_t *vs, uint32_t *kd, uint32_t *vd,
                                  const uint32_t *count, uint32_t max_count) {
    const uint32_t n = load_count(count, max_count);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        kd[i] = ks[i];
        vd[i] = vs[i];
    }
}

static inline uint32_t sort_passes(uint32_t key_bits) { return (key_bits + 7u) / 8u; }

struct SortLayout {
    Ctrl *ctrl;
    uint32_t *kalt, *valt;
    uint64_t *flags;
    uint32_t ntiles;
};

static SortLayout sort_layout(void *scratch, uint32_t max_count) {
    SortLayout L;
    uint8_t *p = reinterpret_cast<uint8_t *>(scratch);
    L.ntiles = (max_count + kTileKeys - 1) / kTileKeys;
    if (L.ntiles == 0) L.ntiles = 1;
    L.ctrl = reinterpret_cast<Ctrl *>(p);
    p += align_up(sizeof(Ctrl), 256);
    L.kalt = reinterpret_cast<uint32_t *>(p);
    p += align_up((size_t)max_count * 4, 256);
    L.valt = reinterpret_cast<uint32_t *>(p);
    p += align_up((size_t)max_count * 4, 256);
    L.flags = reinterpret_cast<uint64_t *>(p);
    return L;
}

size_t sort_scratch_bytes(uint32_t max_count, uint32_t key_bits) {
    size_t ntiles = (max_count + kTileKeys - 1) / kTileKeys;
    if (ntiles == 0) ntiles = 1;
    return align_up(sizeof(Ctrl), 256) + 2 * align_up((size_t)max_count * 4, 256) +
           (size_t)sort_passes(key_bits) * ntiles * 256 * sizeof(uint64_t);
}

cudaError_t launch_sort(uint32_t *keys, uint32_t *vals, uint32_t max_count, const uint32_t *count,
                        uint32_t key_bits, void *scratch, cudaStream_t st, int prof_stage) {
    const SortLayout L = sort_layout(scratch, max_count);
    const uint32_t npasses = sort_passes(key_bits);
    ctrl_init_kernel<<<1, 256, 0, st>>>(L.ctrl, 1);
    count_launches(1);
    if (max_count == 0) return cudaGetLastError();
    prof_mark(prof_stage, true, st);
    uint32_t hist_blocks = (max_count + 256 * 16 - 1) / (256 * 16);
    if (hist_blocks > 152 * 8) hist_blocks = 152 * 8;
    sort_hist_kernel<<<hist_blocks, 256, 0, st>>>(keys, count, max_count, npasses, L.ctrl);
    uint32_t *ka = keys, *va = vals, *kb = L.kalt, *vb = L.valt;
    for (uint32_t p = 0; p < npasses; ++p) {
        sort_pass_kernel<<<L.ntiles, kSortThreads, 0, st>>>(ka, va, kb, vb, count, max_count, p, L.ctrl,
                                                           L.flags + (size_t)p * L.ntiles * 256);
        uint32_t *t = ka;
        ka = kb;
        kb = t;
        t = va;
        va = vb;
        vb = t;
    }
    if (npasses & 1u) {
        uint32_t blocks = (max_count + 255) / 256;
        if (blocks > 152 * 8) blocks = 152 * 8;
        copy_pairs_kernel<<<blocks, 256, 0, st>>>(ka, va, keys, vals, count, max_count);
        count_launches(1);
    }
    count_launches(1 + npasses);
    prof_mark(prof_stage, false, st);
    return cudaGetLastError();
}

}  // namespace gs
