// gs_sort.cu — K2: stable LSD onesweep radix sort of u32 keys carrying u32 values.
//
// Same contract as the reference RadixSorter (src/radix_sorter.rs:56-96,658-669; kernels
// src/shader/radix_sort.wgsl:78-529): 8-bit digits, least significant first, stable; the
// reference's 3840-key block stays the unit of the depth buffer's padding.  The GB300 design
// differs: 7680-key pass blocks; one global-histogram kernel reads the keys once
// for all passes (its last CTA turns the histograms into exclusive digit offsets); each pass is
// a single kernel that ranks its block warp by warp (match.any, or one ballot per digit bit, so
// equal digits keep input order), publishes per-digit counts and resolves the block's global
// offsets by decoupled look-back (block = CTA index: CTAs are dispatched in index order, so a
// block waits only for blocks already resident or finished; every wait is bounded all the same),
// then scatters through shared memory so that each digit's run is written contiguously.
// The key count may live in device memory (the preprocess instance count), so a whole frame
// can be enqueued (or graph-captured) without a host round trip.
#include <atomic>
#include <mutex>

#include "gs300.h"
#include "gs_internal.h"

namespace gs {

// A pass block is 512 threads x 15 keys = 7680 keys, two of the reference's 3840-key blocks:
// longer digit runs in the scatter, and two CTAs (32 warps) per SM.  Threads 0..255 own the
// digits in the per-digit phases.  The reordered block (60 KB) lives in dynamic shared memory.
constexpr uint32_t kSortThreads = 512;
constexpr uint32_t kSortRows = 15;
constexpr uint32_t kTileKeys = kSortThreads * kSortRows;  // 7680
constexpr uint32_t kSortWarps = kSortThreads / 32;
constexpr uint32_t kSortCtasPerSm = 2;
constexpr size_t kSortDynSmem = (size_t)kTileKeys * sizeof(uint2);
static_assert(kTileKeys % GS_SORT_BLOCK_KVS == 0, "a pass block covers whole blocks of the reference");

__global__ void ctrl_init_kernel(Ctrl *ctrl, int mode, Ctrl *owner, uint32_t arena_words, WaitCfg cfg) {
    ctrl_reset(ctrl, mode, owner ? owner : ctrl, arena_words, cfg);
}

__device__ __forceinline__ uint32_t load_count(const uint32_t *count, uint32_t max_count) {
    return count ? min(*count, max_count) : max_count;
}

// Exclusive block scan of one value per thread (WARPS warps).  `tmp` holds WARPS words.
template <uint32_t WARPS>
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
        uint32_t t = lane < WARPS ? tmp[lane] : 0u;
#pragma unroll
        for (uint32_t o = 1; o < WARPS; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < WARPS) tmp[lane] = t;
    }
    __syncthreads();
    const uint32_t before = warp ? tmp[warp - 1] : 0u;
    *total = tmp[WARPS - 1];
    __syncthreads();
    return before + x - v;
}

// Global digit histograms of all passes in one read of the keys (four keys per thread and
// iteration, 16-byte loads when the keys are 16-byte aligned).  Low digits are counted with plain
// shared atomics; for the top digit the warp counts the digit of lane 0 with one ballot (the high
// digits of float depth keys are nearly constant, and same-address shared atomics would
// serialise) and the other keys with plain shared atomics.
__device__ __forceinline__ void hist_add(uint32_t *h, uint32_t k, bool valid, const PassSplit &sp, uint32_t hs,
                                         uint32_t lane) {
    // unrolled over the fixed maximum so every field of the split is read at a constant offset
#pragma unroll
    for (uint32_t p = 0; p < kMaxPasses; ++p) {
        if (p >= sp.n) break;
        const uint32_t d = (k >> sp.shift[p]) & ((1u << sp.bits[p]) - 1u);
        if (p + 1 < sp.n) {  // low digits: spread over the bins, rarely equal within a warp
            if (valid) atomicAdd(&h[p * hs + d], 1u);
            continue;
        }
        const uint32_t d0 = __shfl_sync(0xFFFFFFFFu, d, 0);
        const uint32_t same = __ballot_sync(0xFFFFFFFFu, valid && d == d0);
        if (lane == 0 && same) atomicAdd(&h[p * hs + d0], (uint32_t)__popc(same));
        if (valid && d != d0) atomicAdd(&h[p * hs + d], 1u);
    }
}

// Every CTA first clears its share of the flag-arena words this call must clear (the passes,
// which are the arena's only readers, run after this kernel).
// With `vals`, each CTA also asks L2 for the values of the keys it reads, which the first pass
// reads next (the keys themselves arrive in L2 through this kernel's reads).
__global__ void __launch_bounds__(256) sort_hist_kernel(const uint32_t *__restrict__ keys,
                                                        const uint32_t *__restrict__ vals, const uint32_t *count,
                                                        uint32_t max_count, const PassSplit sp, Ctrl *ctrl,
                                                        uint64_t *arena) {
    __shared__ uint32_t h[1024];
    const uint32_t npasses = sp.n, hs = hist_stride(sp.n);
    uint32_t *gh = &ctrl->hist[0][0];
    arena_clear(ctrl, arena);
    for (uint32_t k = threadIdx.x; k < 1024; k += blockDim.x) h[k] = 0u;
    __syncthreads();
    const uint32_t n = load_count(count, max_count);
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t lane = threadIdx.x & 31u;
    const bool vec = ((uintptr_t)keys & 15u) == 0;
    // Whole warps iterate together (bounds padded to the warp) so the ballots see 32 lanes.
    const uint32_t n4 = (n + 3u) / 4u;
    const uint32_t nr = (n4 + 31u) & ~31u;
    const bool pf = vals && ((uintptr_t)vals & 15u) == 0;
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nr; q += stride) {
        const uint32_t i0 = q * 4u;
        if (pf && threadIdx.x == 0 && i0 < n) {
            // this CTA's 4 x blockDim keys of the iteration start at i0 (a multiple of 16 bytes)
            const uint32_t bytes = min(4u * 4u * blockDim.x, (n - i0) * 4u) & ~15u;
            if (bytes) prefetch_l2_bulk(vals + i0, bytes);
        }
        uint32_t k[4];
        if (vec && i0 + 4u <= n) {
            const uint4 v = *reinterpret_cast<const uint4 *>(keys + i0);
            k[0] = v.x;
            k[1] = v.y;
            k[2] = v.z;
            k[3] = v.w;
        } else {
#pragma unroll
            for (uint32_t j = 0; j < 4; ++j) k[j] = i0 + j < n ? keys[i0 + j] : 0u;
        }
#pragma unroll
        for (uint32_t j = 0; j < 4; ++j) hist_add(h, k[j], i0 + j < n, sp, hs, lane);
    }
    __syncthreads();
    for (uint32_t p = 0; p < npasses; ++p) {
        const uint32_t v = threadIdx.x < (1u << sp.bits[p]) ? h[p * hs + threadIdx.x] : 0u;
        if (v) atomicAdd(&gh[p * hs + threadIdx.x], v);
    }
    // The last CTA to finish turns the histograms into exclusive digit offsets, once for every
    // block of every pass.
    __shared__ uint32_t s_last, s_tmp[8];
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(&ctrl->ticket[7], 1u) == gridDim.x - 1 ? 1u : 0u;
    __syncthreads();
    if (s_last) {
        __threadfence();
        for (uint32_t p = 0; p < npasses; ++p) {
            uint32_t total;
            const bool live = threadIdx.x < (1u << sp.bits[p]);
            const uint32_t off = block_scan_excl<8>(live ? __ldcg(&gh[p * hs + threadIdx.x]) : 0u, s_tmp, &total);
            if (live) gh[p * hs + threadIdx.x] = off;
        }
    }
}

// Look-back of one digit counter (flags[j * stride], j < tile) that polls up to four
// predecessors per round trip.  The flag word carries everything the reader uses, so relaxed
// loads suffice.  Returns the exclusive prefix; after `limit` polls that find an unpublished
// predecessor it sets the status bit and returns what it has summed.
__device__ __forceinline__ uint32_t look_back_digit(const uint64_t *flags, uint32_t tile, uint32_t epoch,
                                                    uint32_t *status, uint32_t stride, uint32_t limit) {
    uint32_t prefix = 0;
    int64_t j = (int64_t)tile - 1;
    uint32_t spins = 0;
    while (j >= 0) {
        uint64_t w[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) w[q] = (j - q >= 0) ? ld_relaxed(flags + (uint64_t)(j - q) * stride) : 0ull;
        bool stalled = false, done = false;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            if (stalled || done || j < 0) continue;
            const uint32_t st = (uint32_t)(w[q] >> 32) & 3u;
            if ((uint32_t)(w[q] >> 34) != epoch || st == 0u) {
                stalled = true;
                continue;
            }
            prefix += (uint32_t)w[q];
            if (st == kFlagPrefix) done = true;
            else --j;
        }
        if (done) break;
        if (stalled) {
            if (++spins > limit) {
                atomicOr(status, kStatusTimeout);
                break;
            }
            if (spins > 64) __nanosleep(32);
        }
    }
    return prefix;
}

// One LSD pass over the digit at `shift`.  Input and output are either split (keys[],
// values[]) or packed (uint2 {key, value}); packed ping-pong buffers keep each digit's run of
// 8-byte pairs contiguous in the scatter.
// MATCH: peers from one match.any instead of a ballot per digit bit.  Measured on GB300 with
// 512-thread blocks, the ballots are the cheaper of the two for both depth keys (0.224 against
// 0.247 ms for a 6M-key sort) and tile keys (0.29 against 0.40 ms).  match.any is a tuning choice
// of the depth sort, and the last pass of float depth keys, whose top digit takes a few values
// per warp, ranks by it.
// The pass of one block (`block`: the look-back tile; lower blocks are lower, earlier-dispatched
// CTAs of the same launch).
template <bool IN_PACKED, bool OUT_PACKED, bool MATCH>
__device__ __forceinline__ void sort_pass_block(
    const uint32_t *__restrict__ kin, const uint32_t *__restrict__ vin, const uint2 *__restrict__ pin,
    uint32_t *__restrict__ kout, uint32_t *__restrict__ vout, uint2 *__restrict__ pout, const uint32_t *count,
    uint32_t max_count, uint32_t hoff, uint32_t shift, uint32_t digit_bits, Ctrl *ctrl, uint64_t *flags,
    uint32_t hist_scanned, uint32_t block) {
    extern __shared__ uint2 s_kv[];  // kTileKeys pairs (dynamic)
    __shared__ uint32_t s_whist[kSortWarps][256];
    __shared__ uint32_t s_start[256];
    __shared__ uint32_t s_gbase[256];
    __shared__ uint32_t s_tmp[kSortWarps];
    __shared__ uint32_t s_tile, s_epoch, s_limit, s_stall;

    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    if (tid == 0) {
        s_epoch = *(volatile uint32_t *)&ctrl->epoch;
        s_limit = ctrl->spin_limit;
        s_stall = ctrl->stall_tile;
        s_tile = block;
    }
    for (uint32_t k = tid; k < kSortWarps * 256; k += kSortThreads) (&s_whist[0][0])[k] = 0u;
    __syncthreads();
    const uint32_t n = load_count(count, max_count);
    const uint32_t ntiles = (n + kTileKeys - 1) / kTileKeys;
    const uint32_t tile = s_tile, epoch = s_epoch;
    if (tile >= ntiles) return;
    const uint32_t dmask = (1u << digit_bits) - 1u;  // bits above the key width are ignored
    const uint32_t base = tile * kTileKeys + warp * (32u * kSortRows);

    uint32_t k[kSortRows], r[kSortRows];
    uint32_t v[IN_PACKED ? kSortRows : 1];
#pragma unroll
    for (uint32_t i = 0; i < kSortRows; ++i) {
        const uint32_t pos = base + i * 32u + lane;
        const bool ok = pos < n;
        if constexpr (IN_PACKED) {
            const uint2 kv = ok ? pin[pos] : make_uint2(0xFFFFFFFFu, 0u);
            k[i] = kv.x;
            v[i] = kv.y;
        } else {
            k[i] = ok ? kin[pos] : 0xFFFFFFFFu;
        }
    }
    // Warp-local stable ranking: lanes that share a digit form a peer mask (match.any, or one
    // ballot per live digit bit).
    const uint32_t lt = lanemask_lt();
#pragma unroll
    for (uint32_t i = 0; i < kSortRows; ++i) {
        const uint32_t d = (k[i] >> shift) & dmask;
        uint32_t peers = 0xFFFFFFFFu;
        if constexpr (MATCH) {
            peers = __match_any_sync(0xFFFFFFFFu, d);
        } else {
#pragma unroll
            for (uint32_t b = 0; b < 8; ++b) {
                if (b >= digit_bits) break;  // bits above the key width are zero in every key
                const uint32_t bit = (d >> b) & 1u;
                const uint32_t bal = __ballot_sync(0xFFFFFFFFu, bit);
                peers &= bit ? bal : ~bal;
            }
        }
        const uint32_t rank = __popc(peers & lt);
        const uint32_t pre = s_whist[warp][d];
        __syncwarp();
        if (rank == 0) s_whist[warp][d] = pre + __popc(peers);
        __syncwarp();
        r[i] = pre + rank;
    }
    __syncthreads();

    // Thread d < 256 owns digit d: per-warp exclusive offsets, block count, publication.
    const uint32_t d = tid;
    const bool owner = d < 256u;
    uint32_t run = 0;
    if (owner) {
#pragma unroll
        for (uint32_t w = 0; w < kSortWarps; ++w) {
            const uint32_t c = s_whist[w][d];
            s_whist[w][d] = run;
            run += c;
        }
    }
    const uint32_t total = run;
    const uint32_t invalid = (tile == ntiles - 1) ? ntiles * kTileKeys - n : 0u;
    // Padding keys (all ones) rank last, in the largest digit.
    const uint32_t pub = (d == dmask) ? total - invalid : total;
    // Digits above dmask hold no key (padding keys sit in digit dmask), so only live digits
    // publish and look back: a pass over 5 live bits keeps 32 flags per block, not 256.
    const bool live = d <= dmask;
    const uint32_t fstride = dmask + 1u;
    uint64_t *f = flags + (size_t)tile * fstride + d;
    if (live) publish_flag(f, tile, s_stall, pack_flag(epoch, tile == 0 ? kFlagPrefix : kFlagAggregate, pub));

    uint32_t blk_total, hist_total;
    const uint32_t start = block_scan_excl<kSortWarps>(total, s_tmp, &blk_total);
    // the digit's first place in the output: the histograms hold exclusive offsets already
    // when their producer scanned them (hist_scanned is uniform over the grid)
    // (pass histogram at flat offset hoff; digits above dmask hold no key)
    const uint32_t hv = live ? (&ctrl->hist[0][0])[hoff + d] : 0u;
    const uint32_t goff = hist_scanned ? hv : block_scan_excl<kSortWarps>(hv, s_tmp, &hist_total);
    uint32_t prefix = 0;
    if (tile > 0 && live) {
        prefix = look_back_digit(flags + d, tile, epoch, &ctrl->status, fstride, s_limit);
        publish_flag(f, tile, s_stall, pack_flag(epoch, kFlagPrefix, prefix + pub));
    }
    if (owner) {
        s_start[d] = start;
        // key j of the reordered block (j >= start for digit d) goes to goff + prefix + (j - start)
        s_gbase[d] = goff + prefix - start;
    }
    __syncthreads();

    if constexpr (IN_PACKED) {
#pragma unroll
        for (uint32_t i = 0; i < kSortRows; ++i) {
            const uint32_t dd = (k[i] >> shift) & dmask;
            const uint32_t at = s_start[dd] + s_whist[warp][dd] + r[i];
            if (at < kTileKeys) s_kv[at] = make_uint2(k[i], v[i]);
            else atomicOr(&ctrl->status, kStatusBounds);
        }
    } else {
        // Values are read only now, after ranking, which keeps them out of registers above.
#pragma unroll
        for (uint32_t i = 0; i < kSortRows; ++i) {
            const uint32_t pos = base + i * 32u + lane;
            const uint32_t vv = pos < n ? vin[pos] : 0u;
            const uint32_t dd = (k[i] >> shift) & dmask;
            const uint32_t at = s_start[dd] + s_whist[warp][dd] + r[i];
            if (at < kTileKeys) s_kv[at] = make_uint2(k[i], vv);
            else atomicOr(&ctrl->status, kStatusBounds);
        }
    }
    __syncthreads();
    const uint32_t valid = min(kTileKeys, n - tile * kTileKeys);
    for (uint32_t j = tid; j < valid; j += kSortThreads) {
        const uint2 kv = s_kv[j];
        const uint32_t dd = (kv.x >> shift) & dmask;
        const uint32_t o = s_gbase[dd] + j;
        if (o < n) {  // always true unless a look-back timed out (status already set)
            if constexpr (OUT_PACKED) {
                pout[o] = kv;
            } else {
                kout[o] = kv.x;
                vout[o] = kv.y;
            }
        }
    }
}

template <bool IN_PACKED, bool OUT_PACKED, bool MATCH>
__global__ void __launch_bounds__(kSortThreads, kSortCtasPerSm) sort_pass_kernel(
    const uint32_t *__restrict__ kin, const uint32_t *__restrict__ vin, const uint2 *__restrict__ pin,
    uint32_t *__restrict__ kout, uint32_t *__restrict__ vout, uint2 *__restrict__ pout, const uint32_t *count,
    uint32_t max_count, uint32_t hoff, uint32_t shift, uint32_t digit_bits, Ctrl *ctrl, uint64_t *flags,
    uint32_t hist_scanned) {
    // look-back predecessors are lower, earlier-dispatched CTAs
    sort_pass_block<IN_PACKED, OUT_PACKED, MATCH>(kin, vin, pin, kout, vout, pout, count, max_count, hoff, shift,
                                                  digit_bits, ctrl, flags, hist_scanned, blockIdx.x);
}

// One pass of many independent packed pair sorts in a single launch (a segmented sort): segment v
// owns the CTAs [block_base[v], block_base[v + 1]) and each of them runs the pass on a block of
// that segment's pairs with the segment's own control block, digit offsets and look-back flags.
// Pass 0 reads `data` and writes `alt`, pass 1 the reverse, so two passes leave the pairs in place.
__global__ void __launch_bounds__(kSortThreads, kSortCtasPerSm)
    sort_segments_kernel(const SortSegment *__restrict__ segs, const uint32_t *__restrict__ block_base, uint32_t nseg,
                         uint32_t pass) {
    uint32_t lo = 0, hi = nseg - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (block_base[mid] <= blockIdx.x) lo = mid;
        else hi = mid - 1;
    }
    const SortSegment &S = segs[lo];
    const uint2 *in = pass ? S.alt : S.data;
    uint2 *out = pass ? S.data : S.alt;
    sort_pass_block<true, true, false>(nullptr, nullptr, in, nullptr, nullptr, out, S.count, S.max_count,
                                       pass * hist_stride(2), S.shift[pass], S.bits[pass], S.ctrl, S.flags[pass],
                                       S.hist_scanned, blockIdx.x - block_base[lo]);
}

// Each segment's sort status into the control block of the area it belongs to.
__global__ void merge_segments_status_kernel(const SortSegment *segs, uint32_t nseg) {
    for (uint32_t v = threadIdx.x; v < nseg; v += blockDim.x) atomicOr(&segs[v].owner->status, segs[v].ctrl->status);
}

__global__ void unpack_pairs_kernel(const uint2 *src, uint32_t *kd, uint32_t *vd, const uint32_t *count,
                                    uint32_t max_count) {
    const uint32_t n = load_count(count, max_count);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint2 kv = src[i];
        kd[i] = kv.x;
        vd[i] = kv.y;
    }
}

__global__ void copy_packed_kernel(const uint2 *src, uint2 *dst, const uint32_t *count, uint32_t max_count) {
    const uint32_t n = load_count(count, max_count);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = src[i];
}

static inline uint32_t sort_passes(uint32_t key_bits) { return (key_bits + 7u) / 8u; }
// Live bits of pass p's digit: keys are below 2^key_bits.  Invalid (padding) keys are all ones
// but sort last either way, because they hold the largest value in every live bit.
PassSplit even_split(uint32_t key_bits) {
    PassSplit sp{};
    sp.n = sort_passes(key_bits);
    const uint32_t base = sp.n ? key_bits / sp.n : 0u, extra = sp.n ? key_bits % sp.n : 0u;
    uint32_t at = 0;
    for (uint32_t p = 0; p < sp.n; ++p) {
        sp.shift[p] = at;
        sp.bits[p] = base + (p < extra ? 1u : 0u);
        at += sp.bits[p];
    }
    return sp;
}

// Passes of a tile-pair sort: two passes up to 16 key bits (a target of up to 65536 tiles), so the
// pairs of every such view end where they started and views can share one segmented launch.
PassSplit tile_split(uint32_t key_bits) {
    if (key_bits > 16) return even_split(key_bits);
    PassSplit sp{};
    sp.n = 2;
    sp.bits[0] = (key_bits + 1) / 2;
    sp.bits[1] = key_bits / 2;
    sp.shift[0] = 0;
    sp.shift[1] = sp.bits[0];
    return sp;
}

// Passes of `key_bits` in digits of at most max_digit bits, spread evenly.
PassSplit even_split_max(uint32_t key_bits, uint32_t max_digit) {
    PassSplit sp{};
    sp.n = (key_bits + max_digit - 1) / max_digit;
    if (sp.n > kMaxPasses) sp.n = kMaxPasses;
    const uint32_t base = sp.n ? key_bits / sp.n : 0u, extra = sp.n ? key_bits % sp.n : 0u;
    uint32_t at = 0;
    for (uint32_t p = 0; p < sp.n; ++p) {
        sp.shift[p] = at;
        sp.bits[p] = base + (p < extra ? 1u : 0u);
        at += sp.bits[p];
    }
    return sp;
}

// Digit widths the split-array sort can be run with (Tuning::sort_digit_bits).
constexpr uint32_t kMinDigitBits = 6, kMaxDigitBits = 8;

static size_t sort_tiles(uint32_t max_count) {
    size_t t = (max_count + kTileKeys - 1) / kTileKeys;
    return t ? t : 1;
}

// Look-back flags of a sort: per pass, one word per block and live digit ([tiles][2^bits]).
size_t sort_flag_words(uint32_t max_count, const PassSplit &sp) {
    size_t w = 0;
    for (uint32_t p = 0; p < sp.n; ++p) w += sort_tiles(max_count) << sp.bits[p];
    return w;
}

struct SortLayout {
    Ctrl *ctrl;
    uint64_t *flags;  // the area's flag arena
    uint2 *alt_a, *alt_b;
    uint32_t ntiles;
    size_t flag_words;
};

// Scratch: control block | flag arena (look-back flags of every pass) | packed buffer A | packed
// buffer B (split sorts of 3+ passes only).  The control block and the arena start at offsets no
// call size moves; the buffers after the arena follow its size.
static SortLayout sort_layout(void *scratch, uint32_t max_count, const PassSplit &sp) {
    SortLayout L;
    uint8_t *p = reinterpret_cast<uint8_t *>(scratch);
    L.ntiles = (uint32_t)sort_tiles(max_count);
    L.ctrl = reinterpret_cast<Ctrl *>(p);
    p += align_up(sizeof(Ctrl), 256);
    L.flags = reinterpret_cast<uint64_t *>(p);
    L.flag_words = sort_flag_words(max_count, sp);
    p += align_up(L.flag_words * sizeof(uint64_t), 256);
    L.alt_a = reinterpret_cast<uint2 *>(p);
    p += align_up((size_t)max_count * 8, 256);
    L.alt_b = reinterpret_cast<uint2 *>(p);
    return L;
}

// Sized for the widest layout over every digit width a call may use, so a caller's scratch fits
// whatever width the tuning picks.
size_t sort_scratch_bytes(uint32_t max_count, uint32_t key_bits) {
    size_t flags = 0;
    uint32_t np = 0;
    for (uint32_t db = kMinDigitBits; db <= kMaxDigitBits; ++db) {
        const PassSplit sp = even_split_max(key_bits, db);
        const size_t f = sort_flag_words(max_count, sp);
        if (f > flags) flags = f;
        if (sp.n > np) np = sp.n;
    }
    return align_up(sizeof(Ctrl), 256) + align_up(flags * sizeof(uint64_t), 256) +
           (np >= 3 ? 2 : 1) * align_up((size_t)max_count * 8, 256);
}

static uint32_t grid_for(uint32_t max_count) {
    uint32_t blocks = (max_count + 255) / 256;
    if (blocks > 152 * 8) blocks = 152 * 8;
    return blocks ? blocks : 1;
}

// MATCH_LAST: the last pass ranks by match.any whatever MATCH says (the top digit of float depth
// keys takes a few values per warp, where one match.any is cheaper than a ballot per bit).
template <bool MATCH, bool MATCH_LAST>
static void launch_sort_passes(uint32_t *keys, uint32_t *vals, uint32_t max_count, const uint32_t *count,
                               const PassSplit &sp, const SortLayout &L, cudaStream_t st) {
    const uint32_t npasses = sp.n, hs = hist_stride(sp.n);
    uint64_t *f = L.flags;
    if (npasses == 1) {
        sort_pass_kernel<false, true, MATCH><<<L.ntiles, kSortThreads, kSortDynSmem, st>>>(
            keys, vals, nullptr, nullptr, nullptr, L.alt_a, count, max_count, 0, sp.shift[0], sp.bits[0], L.ctrl, f, 1u);
        unpack_pairs_kernel<<<grid_for(max_count), 256, 0, st>>>(L.alt_a, keys, vals, count, max_count);
        count_launches(2);
        return;
    }
    uint2 *src = L.alt_a, *dst = L.alt_b;
    sort_pass_kernel<false, true, MATCH><<<L.ntiles, kSortThreads, kSortDynSmem, st>>>(
        keys, vals, nullptr, nullptr, nullptr, src, count, max_count, 0, sp.shift[0], sp.bits[0], L.ctrl, f, 1u);
    f += (size_t)L.ntiles << sp.bits[0];
    for (uint32_t p = 1; p + 1 < npasses; ++p) {
        sort_pass_kernel<true, true, MATCH><<<L.ntiles, kSortThreads, kSortDynSmem, st>>>(
            nullptr, nullptr, src, nullptr, nullptr, dst, count, max_count, p * hs, sp.shift[p], sp.bits[p], L.ctrl, f,
            1u);
        f += (size_t)L.ntiles << sp.bits[p];
        uint2 *t = src;
        src = dst;
        dst = t;
    }
    sort_pass_kernel<true, false, MATCH || MATCH_LAST><<<L.ntiles, kSortThreads, kSortDynSmem, st>>>(
        nullptr, nullptr, src, keys, vals, nullptr, count, max_count, (npasses - 1) * hs, sp.shift[npasses - 1],
        sp.bits[npasses - 1], L.ctrl, f, 1u);
    count_launches(npasses);
}

// The pass kernels take kSortDynSmem of dynamic shared memory, above the default 48 KB a launch
// may ask for: allow it once per device, before the first launch there.
static cudaError_t ensure_sort_smem() {
    static std::atomic<uint64_t> ready{0};  // bit d: device d's pass kernels allow kSortDynSmem
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const uint64_t bit = dev < 64 ? (1ull << dev) : 0ull;
    if (bit && (ready.load(std::memory_order_acquire) & bit)) return cudaSuccess;
    const void *fns[] = {
        (const void *)sort_pass_kernel<false, true, false>, (const void *)sort_pass_kernel<true, true, false>,
        (const void *)sort_pass_kernel<true, false, false>, (const void *)sort_pass_kernel<false, true, true>,
        (const void *)sort_pass_kernel<true, true, true>,   (const void *)sort_pass_kernel<true, false, true>,
        (const void *)sort_segments_kernel,
    };
    for (const void *f : fns) {
        e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSortDynSmem);
        if (e != cudaSuccess) return e;
    }
    ready.fetch_or(bit, std::memory_order_acq_rel);
    return cudaSuccess;
}

cudaError_t launch_sort(uint32_t *keys, uint32_t *vals, uint32_t max_count, const uint32_t *count,
                        uint32_t key_bits, void *scratch, cudaStream_t st, int prof_stage, const Tuning *tuning) {
    if (cudaError_t e = ensure_sort_smem(); e != cudaSuccess) return e;
    const Tuning tn = tuning ? *tuning : default_tuning();
    const uint32_t db = tn.sort_digit_bits < kMinDigitBits   ? kMinDigitBits
                        : tn.sort_digit_bits > kMaxDigitBits ? kMaxDigitBits
                                                             : tn.sort_digit_bits;
    const PassSplit sp = even_split_max(key_bits, db);
    const SortLayout L = sort_layout(scratch, max_count, sp);
    // With no pairs no kernel reads the flags, and none clears them: the arena mark stays.
    ctrl_init_kernel<<<1, 256, 0, st>>>(L.ctrl, 1, nullptr, max_count ? (uint32_t)L.flag_words : kKeepArena,
                                        wait_config());
    count_launches(1);
    if (max_count == 0) return cudaGetLastError();
    prof_mark(prof_stage, true, st);
    uint32_t hist_blocks = (max_count + 256 * 4 * 4 - 1) / (256 * 4 * 4);
    if (hist_blocks > 152 * 8) hist_blocks = 152 * 8;
    if (tn.hist_blocks) hist_blocks = tn.hist_blocks < 152 * 8 ? tn.hist_blocks : 152 * 8;
    sort_hist_kernel<<<hist_blocks, 256, 0, st>>>(keys, vals, count, max_count, sp, L.ctrl, L.flags);
    count_launches(1);
    // Keys of kDepthKeyBits are the render path's float depth keys (1 - ndc.z).
    if (tn.sort_match)
        launch_sort_passes<true, true>(keys, vals, max_count, count, sp, L, st);
    else if (key_bits == kDepthKeyBits)
        launch_sort_passes<false, true>(keys, vals, max_count, count, sp, L, st);
    else
        launch_sort_passes<false, false>(keys, vals, max_count, count, sp, L, st);
    prof_mark(prof_stage, false, st);
    return cudaGetLastError();
}

size_t sort_pairs_flag_words(uint32_t max_count, uint32_t key_bits) {
    return sort_flag_words(max_count, tile_split(key_bits));
}

uint32_t sort_pairs_blocks(uint32_t max_count) { return (uint32_t)sort_tiles(max_count); }

cudaError_t launch_sort_segments(const SortSegment *segs_dev, const uint32_t *block_base_dev, uint32_t nseg,
                                 uint32_t total_blocks, cudaStream_t st) {
    if (nseg == 0 || total_blocks == 0) return cudaSuccess;
    if (cudaError_t e = ensure_sort_smem(); e != cudaSuccess) return e;
    for (uint32_t pass = 0; pass < 2; ++pass)
        sort_segments_kernel<<<total_blocks, kSortThreads, kSortDynSmem, st>>>(segs_dev, block_base_dev, nseg, pass);
    merge_segments_status_kernel<<<1, 256, 0, st>>>(segs_dev, nseg);
    count_launches(3);
    return cudaGetLastError();
}

cudaError_t sort_pairs_begin(Ctrl *ctrl, Ctrl *owner, cudaStream_t st) {
    ctrl_init_kernel<<<1, 256, 0, st>>>(ctrl, 1, owner, kKeepArena, wait_config());
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_sort_pairs(uint2 *data, uint32_t max_count, const uint32_t *count, uint32_t key_bits, Ctrl *ctrl,
                              uint64_t *flags, uint2 *alt, cudaStream_t st, bool hist_scanned) {
    const PassSplit split = tile_split(key_bits);
    if (max_count == 0) return cudaSuccess;
    if (cudaError_t e = ensure_sort_smem(); e != cudaSuccess) return e;
    const uint32_t ntiles = (uint32_t)sort_tiles(max_count);
    uint2 *src = data, *dst = alt;
    uint64_t *f = flags;
    for (uint32_t p = 0; p < split.n; ++p) {
        sort_pass_kernel<true, true, false><<<ntiles, kSortThreads, kSortDynSmem, st>>>(nullptr, nullptr, src, nullptr, nullptr, dst,
                                                                            count, max_count, p * hist_stride(split.n),
                                                                            split.shift[p],
                                                                            split.bits[p], ctrl, f,
                                                                            hist_scanned ? 1u : 0u);
        f += (size_t)ntiles << split.bits[p];
        uint2 *t = src;
        src = dst;
        dst = t;
    }
    count_launches(split.n);
    if (split.n & 1u) {
        copy_packed_kernel<<<grid_for(max_count), 256, 0, st>>>(src, data, count, max_count);
        count_launches(1);
    }
    return cudaGetLastError();
}

// ---- allocation-free sort entry point -------------------------------------------------------
// Scratch for gs_radix_sort_no_alloc lives in this file-scope device array instead of memory the
// caller provides, so that entry point never allocates.  It holds the largest layout the entry
// point accepts (kNoAllocMaxPairs pairs of 32-bit keys, four passes) and every device that loads
// the library holds it until the process exits.  A __device__ array without an initialiser is
// zero when the module loads, which is the state a fresh scratch area needs; after that, calls of
// any size and key width reuse it as any caller scratch is reused (the flag arena sits at a fixed
// offset and is cleared where a call's layout grows past the previous one).
constexpr uint32_t kNoAllocMaxPairs = 1u << 20;
constexpr size_t kNoAllocTiles = (kNoAllocMaxPairs + kTileKeys - 1) / kTileKeys;
constexpr size_t kNoAllocBytes = ((sizeof(Ctrl) + 255) / 256) * 256 +
                                 ((4 * kNoAllocTiles * 256 * sizeof(uint64_t) + 255) / 256) * 256 +
                                 2 * (((size_t)kNoAllocMaxPairs * 8 + 255) / 256) * 256;
static __device__ __align__(256) unsigned char g_no_alloc_scratch[kNoAllocBytes];

namespace {
std::mutex g_no_alloc_mu;
constexpr int kNoAllocDevices = 64;
void *g_no_alloc_ptr[kNoAllocDevices] = {};
}  // namespace

// Device address of the array on the current device.  In host code the array's name is only a
// stand-in, not a device address: the first call on a device looks the address up with that
// device current and caches it; later calls reuse it.
static cudaError_t no_alloc_scratch(void **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kNoAllocDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> g(g_no_alloc_mu);
    if (!g_no_alloc_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_no_alloc_scratch);
        if (e != cudaSuccess) return e;
        g_no_alloc_ptr[dev] = p;
    }
    *out = g_no_alloc_ptr[dev];
    return cudaSuccess;
}

}  // namespace gs

extern "C" gs_status gs_radix_sort_no_alloc(uint32_t *keys, uint32_t *values, uint32_t max_count,
                                            const uint32_t *count, uint32_t key_bits, gs_stream stream) {
    using namespace gs;
    if (key_bits < 1 || key_bits > 32) return set_error(GS_ERR_INVALID_ARG, "gs_radix_sort_no_alloc: key_bits not in 1..=32");
    if (max_count > kNoAllocMaxPairs)
        return set_error(GS_ERR_INVALID_ARG,
                         "gs_radix_sort_no_alloc: max_count exceeds the static scratch limit of 1048576 pairs "
                         "(use gs_radix_sort with caller scratch)");
    if (max_count && (!keys || !values)) return set_error(GS_ERR_INVALID_ARG, "gs_radix_sort_no_alloc: NULL buffer");
    if (sort_scratch_bytes(max_count, key_bits) > kNoAllocBytes)
        return set_error(GS_ERR_INVALID_ARG, "gs_radix_sort_no_alloc: layout exceeds the static scratch");
    cudaStream_t st = (cudaStream_t)stream;
    void *scratch = nullptr;
    cudaError_t e = no_alloc_scratch(&scratch);
    if (e == cudaSuccess) e = launch_sort(keys, values, max_count, count, key_bits, scratch, st);
    if (e != cudaSuccess) return set_error(GS_ERR_CUDA, cudaGetErrorString(e));
    return GS_OK;
}
