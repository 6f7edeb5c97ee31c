// gs_raster.cu — K3 tile binning + K4 tile rasteriser.
//
// The reference draws one instanced quad per visible splat with fixed-function
// BlendState::ALPHA_BLENDING onto a Rgba8Unorm target cleared to opaque black
// (src/renderer.rs:162-195, 284-308; src/shader/render.wesl:46-56, 75-181).  This file
// restates that per pixel:
//   * K3 walks the depth-sorted splats, gathers each splat record into draw order, counts the
//     16x16 tiles its fragment box touches, scans the counts (block scan + decoupled
//     look-back) and emits (tile, draw-rank) pairs; a stable 8-bit-digit radix sort by tile
//     then groups the pairs per tile with draw order kept inside each tile.
//   * K4 runs one CTA per tile; each thread owns one pixel and walks the tile's splats in
//     draw order (far to near), staged 256 at a time in shared memory.  For every fragment
//     it evaluates the interpolated quad offset q, the discard test, the alpha of the display
//     mode, and blends with the 8-bit re-quantisation a Rgba8Unorm attachment performs after
//     every fragment: d' = round(d·(1-α) + s·α) in units of 1/255.
// Fragments whose alpha cannot move an 8-bit channel (see splat_r2_bound) lie outside the splat's
// fragment box and are never visited; skipping them leaves every pixel bit-identical.
#include <cstdlib>

#include "gs_internal.h"

namespace gs {

constexpr uint32_t kBinThreads = 256;
constexpr uint32_t kRasterThreads = 256;
// A warp's pixel block is 8x4 pixels: its pixel centres span 7 x 3 pixels.
constexpr float kBlockSpanX = 7.0f, kBlockSpanY = 3.0f;

struct RasterLayout {
    Ctrl *ctrl;          // raster control block: owns the area's epoch counter and flag arena
    Ctrl *sort_ctrl;     // tile sort control block
    uint64_t *flags;     // flag arena, first part: scan look-back flags
    uint64_t *sort_flags;  // flag arena, second part: tile-sort look-back flags
    uint32_t arena_words;  // words of the flag arena (both parts)
    gs_splat *sorted;    // draw-ordered splats (several models), capacity max_splats
    uint4 *info;         // per draw rank: tile rectangle, kept-tile mask, pair value
    uint32_t *offsets;   // per draw rank: tile count, then its exclusive scan
    uint2 *pairs;        // (tile, value), capacity max_pairs
    uint2 *ranges;       // per tile [start, end)
    uint32_t *counts;    // per tile pair count (counting path; null above kCountTiles tiles)
    uint32_t *blockcounts;  // per emit CTA and tile pair count (counting path)
    uint32_t *order;     // tiles by descending pair count: the rasteriser's launch order (counting path)
    uint2 *sort_alt;     // the tile sort's ping-pong buffer, capacity max_pairs
    uint32_t tiles_x, tiles_y, ntiles, key_bits;
};

// Up to kCountTiles tiles (1080p has 8160), the emit kernel counts pairs per tile in shared
// memory; the per-tile counts give the tile-sort histograms and, scanned, the tile ranges.
// Larger targets count per digit instead and find the ranges in the sorted pairs.
constexpr uint32_t kCountTiles = 8192;
constexpr uint32_t kEmitBlocks = 152 * 8;

constexpr uint32_t kScanItems = 16;
constexpr uint32_t kScanTile = 256 * kScanItems;

static uint32_t bits_for(uint32_t v) {
    uint32_t b = 1;
    while (b < 32 && (v >> b) != 0) ++b;
    return b;
}

// Scan flags: one per 4096-count tile (plus one), padded to 256 bytes so the tile-sort flags
// after them stay 256-byte aligned.
static size_t scan_flag_words(uint32_t max_splats) {
    return align_up(((size_t)max_splats + kScanTile - 1) / kScanTile + 1, 32);
}

// Scratch: raster control block | tile-sort control block | flag arena (scan flags, tile-sort
// flags) | buffers.  The two control blocks and the arena's start sit at offsets no call size
// moves; the arena's length and everything after it follow (max_splats, width, height, max_pairs).
static RasterLayout raster_layout(void *scratch, uint32_t max_splats, uint32_t w, uint32_t h,
                                  uint32_t max_pairs) {
    RasterLayout L;
    L.tiles_x = (w + GS_TILE - 1) / GS_TILE;
    L.tiles_y = (h + GS_TILE - 1) / GS_TILE;
    L.ntiles = L.tiles_x * L.tiles_y;
    L.key_bits = bits_for(L.ntiles > 0 ? L.ntiles - 1 : 0);
    uint8_t *p = reinterpret_cast<uint8_t *>(scratch);
    L.ctrl = reinterpret_cast<Ctrl *>(p);
    p += align_up(sizeof(Ctrl), 256);
    L.sort_ctrl = reinterpret_cast<Ctrl *>(p);
    p += align_up(sizeof(Ctrl), 256);
    const size_t scan_words = scan_flag_words(max_splats);
    const size_t arena = scan_words + sort_pairs_flag_words(max_pairs, L.key_bits);
    L.flags = reinterpret_cast<uint64_t *>(p);
    L.sort_flags = L.flags + scan_words;
    L.arena_words = (uint32_t)arena;
    p += align_up(arena * sizeof(uint64_t), 256);
    L.sorted = reinterpret_cast<gs_splat *>(p);
    p += align_up((size_t)max_splats * sizeof(gs_splat), 256);
    L.info = reinterpret_cast<uint4 *>(p);
    p += align_up((size_t)max_splats * 16, 256);
    L.offsets = reinterpret_cast<uint32_t *>(p);
    p += align_up((size_t)max_splats * 4 + 16, 256);
    L.pairs = reinterpret_cast<uint2 *>(p);
    p += align_up((size_t)max_pairs * 8, 256);
    L.ranges = reinterpret_cast<uint2 *>(p);
    p += align_up((size_t)L.ntiles * sizeof(uint2), 256);
    L.counts = L.blockcounts = L.order = nullptr;
    if (L.ntiles <= kCountTiles) {
        L.counts = reinterpret_cast<uint32_t *>(p);
        p += align_up((size_t)L.ntiles * 4, 256);
        L.order = reinterpret_cast<uint32_t *>(p);
        p += align_up((size_t)L.ntiles * 4, 256);
        L.blockcounts = reinterpret_cast<uint32_t *>(p);
        p += align_up((size_t)kEmitBlocks * L.ntiles * 4, 256);
    }
    L.sort_alt = reinterpret_cast<uint2 *>(p);
    return L;
}

size_t raster_scratch_bytes(uint32_t max_splats, uint32_t w, uint32_t h, uint32_t max_pairs) {
    const uint32_t tiles = ((w + GS_TILE - 1) / GS_TILE) * ((h + GS_TILE - 1) / GS_TILE);
    const uint32_t key_bits = bits_for(tiles > 0 ? tiles - 1 : 0);
    const size_t arena = scan_flag_words(max_splats) + sort_pairs_flag_words(max_pairs, key_bits);
    return 2 * align_up(sizeof(Ctrl), 256) + align_up(arena * sizeof(uint64_t), 256) +
           align_up((size_t)max_splats * sizeof(gs_splat), 256) + align_up((size_t)max_splats * 16, 256) +
           align_up((size_t)max_splats * 4 + 16, 256) + align_up((size_t)max_pairs * 8, 256) +
           align_up((size_t)tiles * sizeof(uint2), 256) +
           (tiles <= kCountTiles ? 2 * align_up((size_t)tiles * 4, 256) +
                                       align_up((size_t)kEmitBlocks * tiles * 4, 256)
                                 : 0) +
           align_up((size_t)max_pairs * 8, 256);
}

const Ctrl *raster_ctrl(const void *scratch) { return reinterpret_cast<const Ctrl *>(scratch); }

Tuning default_tuning() {
    Tuning t;
    if (const char *v = getenv("GS300_SUFFIX_MIN")) t.suffix_min = (uint32_t)strtoul(v, nullptr, 10);
    if (const char *v = getenv("GS300_SUFFIX_EPS")) t.eps = strtof(v, nullptr);
    if (const char *v = getenv("GS300_SORT_DIGIT_BITS")) t.sort_digit_bits = (uint32_t)strtoul(v, nullptr, 10);
    if (const char *v = getenv("GS300_HIST_BLOCKS")) t.hist_blocks = (uint32_t)strtoul(v, nullptr, 10);
    if (const char *v = getenv("GS300_SORT_MATCH")) t.sort_match = (uint32_t)strtoul(v, nullptr, 10) ? 1u : 0u;
    return t;
}

// K3a: per draw rank, the splat's tile rectangle, the corner tiles its footprint misses, and
// its tile count.  With `binfo` (one view of one model, its preprocess having stored each
// visible splat's tiles) the rank gathers that 16-byte record; otherwise it gathers the 48-byte
// splat and works the tiles out here.  Several models first copy their splats into draw order.
// The first segment's launch (arena non-null) also clears the flag-arena words the call must
// clear, before the scan and the tile sort read any flag.
__global__ void __launch_bounds__(kBinThreads) bin_count_kernel(
    const gs_splat *__restrict__ splats, const uint4 *__restrict__ binfo, const uint32_t *__restrict__ sorted_index,
    const uint32_t *count, uint32_t max_count, uint32_t rank_offset, gs_splat *__restrict__ sorted_out, int direct,
    uint32_t tiles_x, uint32_t tiles_y, uint32_t mode, float std2, uint4 *__restrict__ info,
    uint32_t *__restrict__ counts, const Ctrl *owner, uint64_t *arena) {
    if (arena) arena_clear(owner, arena);
    const uint32_t n = count ? min(*count, max_count) : max_count;
    const uint32_t k = blockIdx.x * kBinThreads + threadIdx.x;
    if (k >= n) return;
    // Indices come from the depth sort; the bound check only matters if that sort timed out.
    const uint32_t gi = sorted_index[k];
    uint4 t = make_uint4(0u, 0u, 0u, 0u);  // x0 | y0 << 16, w | h << 16, mask, count
    if (gi < max_count) {
        if (binfo) {
            t = binfo[gi];
        } else {
            // all three 16-byte parts in one round trip (the colour bounds the corner-tile test)
            const float4 *src = reinterpret_cast<const float4 *>(splats + gi);
            const float4 a = __ldg(src);
            const float4 q = __ldg(src + 1);
            const float4 c = __ldg(src + 2);
            if (!direct) {
                float4 *dst = reinterpret_cast<float4 *>(sorted_out + rank_offset + k);
                dst[0] = a;
                dst[1] = q;
                dst[2] = c;
            }
            t = splat_tile_info(a, q, c, tiles_x, tiles_y, mode, std2);
        }
    }
    info[k] = make_uint4(t.x, t.y, t.z, direct ? gi : rank_offset + k);
    counts[k] = t.w;
}

// K3b: exclusive scan of the tile counts in place (decoupled look-back over 4096-count tiles);
// the last tile records the segment's total.
__global__ void __launch_bounds__(256) bin_scan_kernel(uint32_t *__restrict__ data, const uint32_t *count,
                                                       uint32_t max_count, Ctrl *ctrl, uint64_t *flags) {
    __shared__ uint32_t s_warp[8];
    __shared__ uint32_t s_tile, s_epoch, s_prefix, s_limit, s_stall;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    if (tid == 0) {
        s_epoch = *(volatile uint32_t *)&ctrl->epoch;
        s_limit = ctrl->spin_limit;
        s_stall = ctrl->stall_tile;
        s_tile = blockIdx.x;  // look-back predecessors are lower, earlier-dispatched CTAs
    }
    __syncthreads();
    const uint32_t n = count ? min(*count, max_count) : max_count;
    const uint32_t ntiles = (n + kScanTile - 1) / kScanTile;
    const uint32_t tile = s_tile, epoch = s_epoch;
    if (tile >= ntiles) return;
    const uint32_t base = tile * kScanTile + tid * kScanItems;
    uint32_t v[kScanItems];
    if (base + kScanItems <= n) {
#pragma unroll
        for (uint32_t i = 0; i < kScanItems; i += 4) {
            const uint4 x = *reinterpret_cast<const uint4 *>(data + base + i);
            v[i] = x.x;
            v[i + 1] = x.y;
            v[i + 2] = x.z;
            v[i + 3] = x.w;
        }
    } else {
#pragma unroll
        for (uint32_t i = 0; i < kScanItems; ++i) v[i] = base + i < n ? data[base + i] : 0u;
    }
    uint32_t sum = 0;
#pragma unroll
    for (uint32_t i = 0; i < kScanItems; ++i) sum += v[i];
    uint32_t x = sum;
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t wv = lane < 8 ? s_warp[lane] : 0u;
        uint32_t wi = wv;
#pragma unroll
        for (uint32_t o = 1; o < 8; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, wi, o);
            if (lane >= o) wi += y;
        }
        const uint32_t total = __shfl_sync(0xFFFFFFFFu, wi, 7);
        if (lane == 0)
            publish_flag(flags + tile, tile, s_stall, pack_flag(epoch, tile == 0 ? kFlagPrefix : kFlagAggregate, total));
        const uint32_t prefix = tile == 0 ? 0u : look_back_warp(flags, tile, epoch, &ctrl->status, s_limit);
        if (lane < 8) s_warp[lane] = wi - wv;  // exclusive per-warp offsets
        if (lane == 0) {
            const uint64_t incl = (uint64_t)prefix + total;
            const uint32_t sat = incl > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)incl;
            if (tile > 0) publish_flag(flags + tile, tile, s_stall, pack_flag(epoch, kFlagPrefix, sat));
            s_prefix = prefix;
            if (tile == ntiles - 1) ctrl->seg_total = sat;
        }
    }
    __syncthreads();
    uint32_t run = s_prefix + s_warp[warp] + x - sum;
    if (base + kScanItems <= n) {
#pragma unroll
        for (uint32_t i = 0; i < kScanItems; i += 4) {
            uint4 o;
            o.x = run;
            run += v[i];
            o.y = run;
            run += v[i + 1];
            o.z = run;
            run += v[i + 2];
            o.w = run;
            run += v[i + 3];
            *reinterpret_cast<uint4 *>(data + base + i) = o;
        }
    } else {
#pragma unroll
        for (uint32_t i = 0; i < kScanItems; ++i) {
            if (base + i < n) data[base + i] = run;
            run += v[i];
        }
    }
}

// Place, in its w x h rectangle, of the n-th kept tile of a splat (n < its tile count).  The
// kept-tile mask (splat_tile_info) only ever drops corner tiles, at places 0, w-1, (h-1)w and
// hw-1, so the place is n moved past each dropped corner at or before it, in increasing order
// (the last corner has no place after it): cheaper than a general n-th-set-bit search.
__device__ __forceinline__ uint32_t kept_tile_place(uint32_t m, uint32_t w, uint32_t h, uint32_t n) {
    uint32_t pos = n;
    if (!(m & 1u)) ++pos;
    if (w > 1u && !((m >> (w - 1u)) & 1u) && pos >= w - 1u) ++pos;
    const uint32_t c2 = (h - 1u) * w;
    if (h > 1u && !((m >> c2) & 1u) && pos >= c2) ++pos;
    return pos;
}

// K3c: every splat writes its (tile, value) pairs at its scanned offset, its kept tiles in
// row-major order.  The 32 ranks of a warp own one contiguous run of pairs, and the warp writes
// that run together: pair r of the run goes to lane r mod 32, which finds its splat by binary
// search over the warp's exclusive count prefix and its tile from the pair's place in the
// splat's rectangle (its kept tiles skip the dropped corners).  Stores are consecutive, every
// lane has a pair in every round but the last, and one large splat is spread over the warp like
// any other.  Also accumulates the tile counts (or the tile-key digit histograms of the tile
// sort) in shared memory: each CTA loops over chunks of 256 ranks (grid-stride) and hands its
// shared bins on once.
template <bool COUNTS>
__global__ void __launch_bounds__(kBinThreads) bin_emit_kernel(
    const uint4 *__restrict__ info, const uint32_t *__restrict__ offsets, const uint32_t *count, uint32_t max_count,
    uint2 *__restrict__ pairs, uint32_t max_pairs, uint32_t tiles_x, uint32_t ntiles, const Ctrl *ctrl,
    Ctrl *sort_ctrl, const PassSplit split, uint32_t *__restrict__ blockcounts) {
    // COUNTS: one counter per tile; else the tile-key digit histograms of the tile sort
    extern __shared__ uint32_t s_bins[];
    const uint32_t nbins = COUNTS ? ntiles : 4u * 256u;
    const uint32_t tid = threadIdx.x, lane = tid & 31u;
    const uint32_t n = count ? min(*count, max_count) : max_count;
    for (uint32_t i = tid; i < nbins; i += kBinThreads) s_bins[i] = 0u;
    __syncthreads();
    const uint32_t seg_total = ctrl->seg_total;
    const uint64_t pair_base = ctrl->pair_base;
    auto emit = [&](uint32_t t, uint32_t value, uint64_t at) {
        if (at < max_pairs) {
            pairs[at] = make_uint2(t, value);
            if constexpr (COUNTS) {
                if (t < ntiles) atomicAdd(&s_bins[t], 1u);
                else atomicOr(&const_cast<Ctrl *>(ctrl)->status, kStatusBounds);
            } else {
                for (uint32_t p = 0; p < split.n; ++p)
                    atomicAdd(&s_bins[p * 256u + ((t >> split.shift[p]) & ((1u << split.bits[p]) - 1u))], 1u);
            }
        }
    };
    for (uint32_t k0 = blockIdx.x * kBinThreads; k0 < n; k0 += gridDim.x * kBinThreads) {
        const uint32_t k = k0 + tid;
        uint4 in = make_uint4(0u, 0u, 0u, 0u);
        uint32_t cnt = 0;
        uint64_t o = 0;
        if (k < n) {
            in = info[k];
            const uint32_t off = offsets[k];
            const uint32_t next = (k + 1 < n) ? offsets[k + 1] : seg_total;
            cnt = next - off;
            o = pair_base + off;
            // A count beyond the splat's tile rectangle can only come from a scan whose
            // look-back gave up (status already set): emit nothing for it.
            if (next < off || cnt > (in.y & 0xFFFFu) * (in.y >> 16)) {
                if (cnt) atomicOr(&const_cast<Ctrl *>(ctrl)->status, kStatusBounds);
                cnt = 0;
            }
        }
        // warp-exclusive prefix of the counts: this lane's pairs are [excl, excl + cnt) of the run
        uint32_t incl = cnt;
#pragma unroll
        for (uint32_t d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, d);
            if (lane >= d) incl += y;
        }
        const uint32_t excl = incl - cnt, run = __shfl_sync(0xFFFFFFFFu, incl, 31);
        // a lane's rectangle: x0 | y0 << 16, width, kept-tile mask, value, 1 / width
        const uint32_t w = in.y & 0xFFFFu;
        const float inv_w = w ? 1.0f / (float)w : 0.0f;
        for (uint32_t r0 = 0; r0 < run; r0 += 32) {
            const uint32_t r = r0 + lane;
            // the largest lane whose run starts at or before r (a lane with no pairs shares its
            // start with the next lane, so the search lands on a lane that has pairs)
            uint32_t src = 0;
#pragma unroll
            for (uint32_t step = 16; step >= 1; step >>= 1) {
                const uint32_t e = __shfl_sync(0xFFFFFFFFu, excl, src + step);
                if (e <= r) src += step;
            }
            const uint32_t sx = __shfl_sync(0xFFFFFFFFu, in.x, src), swh = __shfl_sync(0xFFFFFFFFu, in.y, src);
            const uint32_t sw = swh & 0xFFFFu;  // in.y: w | h << 16
            const uint32_t smask = __shfl_sync(0xFFFFFFFFu, in.z, src), sval = __shfl_sync(0xFFFFFFFFu, in.w, src);
            const float sinv = __shfl_sync(0xFFFFFFFFu, inv_w, src);
            const uint32_t sex = __shfl_sync(0xFFFFFFFFu, excl, src);
            const uint32_t olo = __shfl_sync(0xFFFFFFFFu, (uint32_t)o, src);
            const uint32_t ohi = __shfl_sync(0xFFFFFFFFu, (uint32_t)(o >> 32), src);
            if (r < run) {
                const uint32_t local = r - sex;
                // in.z: tiles kept of a rectangle of at most 16 (bit ty·w + tx); 0 = all of it
                const uint32_t pos = smask ? kept_tile_place(smask, sw, swh >> 16, local) : local;
                // row = floor(pos / w), exact in float: pos < 2^24 and the error of 1/w is
                // far below the 1/w gap between pos/w and the next integer
                const uint32_t ty = (uint32_t)(((float)pos + 0.5f) * sinv), tx = pos - ty * sw;
                const uint64_t at = (((uint64_t)ohi << 32) | olo) + local;
                emit(((sx >> 16) + ty) * tiles_x + (sx & 0xFFFFu) + tx, sval, at);
            }
        }
    }
    __syncthreads();
    if constexpr (COUNTS) {
        // every CTA of the grid writes its slice (zeros when it had no ranks): plain stores,
        // summed per tile by tile_count_kernel
        uint32_t *dst = blockcounts + (size_t)blockIdx.x * ntiles;
        for (uint32_t t = tid; t < ntiles; t += kBinThreads) dst[t] = s_bins[t];
    } else {
        for (uint32_t p = 0; p < split.n; ++p) {
            const uint32_t v = s_bins[p * 256u + tid];
            if (v) atomicAdd(&sort_ctrl->hist[p][tid], v);
        }
    }
}

// Per-tile pair counts of one segment (the sum over the emit CTAs), added to the running
// counts.  blockIdx.y takes a slice of the emit CTAs, so the sum runs wide, not long.
constexpr uint32_t kCountSlices = 16;

__global__ void __launch_bounds__(256) tile_count_kernel(const uint32_t *__restrict__ blockcounts, uint32_t nblocks,
                                                         uint32_t ntiles, uint32_t *__restrict__ counts) {
    const uint32_t t = blockIdx.x * 256u + threadIdx.x;
    if (t >= ntiles) return;
    const uint32_t per = (nblocks + kCountSlices - 1) / kCountSlices;
    const uint32_t b0 = blockIdx.y * per, b1 = min(nblocks, b0 + per);
    uint32_t part[4] = {0, 0, 0, 0};
    uint32_t b = b0;
    for (; b + 4 <= b1; b += 4)
#pragma unroll
        for (uint32_t q = 0; q < 4; ++q) part[q] += blockcounts[(size_t)(b + q) * ntiles + t];
    for (; b < b1; ++b) part[0] += blockcounts[(size_t)b * ntiles + t];
    const uint32_t c = (part[0] + part[1]) + (part[2] + part[3]);
    if (c) atomicAdd(&counts[t], c);
}

// Size class of a tile list for the launch order: two classes per power of two, 0 = empty.
constexpr uint32_t kOrderClasses = 66;
__device__ __forceinline__ uint32_t order_class(uint32_t c) {
    if (c == 0) return 0u;
    const uint32_t lg = 31u - __clz(c);
    return 1u + 2u * lg + (lg > 0 ? (c >> (lg - 1u)) & 1u : 0u);
}

// [start, end) of every tile from the per-tile counts (exclusive scan; one CTA, 8 tiles a
// thread), the tile sort's digit offsets (exclusive scans of the digit histograms, which are sums
// of those counts), and the rasteriser's
// launch order: tiles by descending size class (a counting sort), so the longest lists start
// first and the grid does not end on a few long tiles that started late.  The order inside a
// class is whatever the shared atomics give; it only schedules CTAs, every tile's pixels are
// the same in any order.
__global__ void __launch_bounds__(1024) tile_scan_kernel(const uint32_t *__restrict__ counts, uint32_t ntiles,
                                                         uint2 *__restrict__ ranges, uint32_t *__restrict__ order,
                                                         Ctrl *sort_ctrl, const PassSplit split) {
    __shared__ uint32_t s_w[32];
    __shared__ uint32_t s_h[4][256];
    __shared__ uint32_t s_cls[kOrderClasses];
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    (&s_h[0][0])[tid] = 0u;
    if (tid < kOrderClasses) s_cls[tid] = 0u;
    __syncthreads();
    const uint32_t base = tid * 8u;
    uint32_t v[8], sum = 0;
#pragma unroll
    for (uint32_t j = 0; j < 8; ++j) {
        v[j] = base + j < ntiles ? counts[base + j] : 0u;
        sum += v[j];
        if (base + j < ntiles) atomicAdd(&s_cls[order_class(v[j])], 1u);
        if (v[j])
            for (uint32_t p = 0; p < split.n; ++p)
                atomicAdd(&s_h[p][((base + j) >> split.shift[p]) & ((1u << split.bits[p]) - 1u)], v[j]);
    }
    uint32_t inc = sum;
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
        const uint32_t x = __shfl_up_sync(0xFFFFFFFFu, inc, o);
        if (lane >= o) inc += x;
    }
    if (lane == 31) s_w[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint32_t x = s_w[lane], xi = x;
#pragma unroll
        for (uint32_t o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, xi, o);
            if (lane >= o) xi += y;
        }
        s_w[lane] = xi - x;  // exclusive over warps
    }
    if (tid == 32) {  // first position of each size class, largest class first
        uint32_t at = 0;
        for (int c = (int)kOrderClasses - 1; c >= 0; --c) {
            const uint32_t k = s_cls[c];
            s_cls[c] = at;
            at += k;
        }
    }
    __syncthreads();
    uint32_t run = s_w[warp] + inc - sum;
#pragma unroll
    for (uint32_t j = 0; j < 8; ++j) {
        if (base + j < ntiles) {
            ranges[base + j] = make_uint2(run, run + v[j]);
            order[atomicAdd(&s_cls[order_class(v[j])], 1u)] = base + j;
        }
        run += v[j];
    }
    // the tile sort's digit offsets: per pass (256 threads each), the exclusive scan of its counts
    __shared__ uint32_t s_hw[32];
    const uint32_t p = tid >> 8, d = tid & 255u;
    const uint32_t hv = s_h[p][d];
    uint32_t hx = hv;
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, hx, o);
        if (lane >= o) hx += y;
    }
    if (lane == 31) s_hw[warp] = hx;
    __syncthreads();
    uint32_t hpre = 0;
    for (uint32_t w = p * 8u; w < warp; ++w) hpre += s_hw[w];
    if (p < split.n) sort_ctrl->hist[p][d] = hpre + hx - hv;
}

// K3d: advance the running pair base past a segment; flags a tile-pair list overflow.
__global__ void bin_advance_kernel(Ctrl *ctrl, const uint32_t *count, uint32_t max_count, uint32_t max_pairs) {
    const uint32_t n = count ? min(*count, max_count) : max_count;
    const uint64_t seg = n ? ctrl->seg_total : 0u;
    const uint64_t want = (uint64_t)ctrl->total + seg;
    const uint32_t sat = want > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)want;
    const uint32_t kept = sat > max_pairs ? max_pairs : sat;
    if (sat > max_pairs) ctrl->status |= kStatusCapacity;
    ctrl->total = sat;
    ctrl->count = kept;
    ctrl->pair_base = kept;
}

// [start, end) of every tile's run in the tile-sorted pairs; each thread checks four
// consecutive pairs with two 16-byte loads.
__global__ void tile_ranges_kernel(const uint2 *__restrict__ pairs, const Ctrl *ctrl, uint2 *ranges,
                                   uint32_t ntiles) {
    const uint32_t n = ctrl->count;
    const uint32_t stride = gridDim.x * blockDim.x * 4u;
    for (uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) * 4u; base < n; base += stride) {
        uint32_t t[6];  // t[0] = previous pair, t[1..4] = this thread's pairs, t[5] = next pair
        if (base + 4u <= n) {
            const uint4 a = *reinterpret_cast<const uint4 *>(pairs + base);
            const uint4 b = *reinterpret_cast<const uint4 *>(pairs + base + 2);
            t[1] = a.x;
            t[2] = a.z;
            t[3] = b.x;
            t[4] = b.z;
        } else {
            for (uint32_t i = 0; i < 4; ++i) t[1 + i] = base + i < n ? pairs[base + i].x : 0xFFFFFFFFu;
        }
        t[0] = base > 0 ? pairs[base - 1].x : 0xFFFFFFFFu;
        t[5] = base + 4u < n ? pairs[base + 4].x : 0xFFFFFFFFu;
#pragma unroll
        for (uint32_t i = 1; i <= 4; ++i) {
            const uint32_t p = base + i - 1;
            const uint32_t k = t[i];
            if (p >= n || k >= ntiles) continue;
            if (t[i - 1] != k) ranges[k].x = p;
            if (t[i + 1] != k) ranges[k].y = p + 1;
        }
    }
}

// The tile sort keeps its own control block; fold its status bits into the raster's.
__global__ void merge_status_kernel(Ctrl *dst, const Ctrl *src) { dst->status |= src->status; }

// One fragment of a staged splat at the pixel centre (pxc, pyc) (render.wesl:143-181):
// false when discarded or when it cannot change the pixel, else its alpha.
template <uint32_t MODE, bool PORTABLE_EXP>
__device__ __forceinline__ bool fragment(const float4 a, const float4 b, float pxc, float pyc, float outline2,
                                         float *alpha) {
    const float dx = __fsub_rn(pxc, a.x), dy = __fsub_rn(pyc, a.y);
    if constexpr (MODE == GS_DISPLAY_POINT) {
        if (!(dx >= -b.x && dx < b.x && dy >= -b.y && dy < b.y)) return false;
        *alpha = 1.0f;
        return true;
    } else {
        const float qx = fmaf(b.x, dx, __fmul_rn(b.y, dy));
        const float qy = fmaf(b.z, dx, __fmul_rn(b.w, dy));
        const float r2 = fmaf(qx, qx, __fmul_rn(qy, qy));
        if (!(r2 <= a.z)) return false;
        if constexpr (MODE == GS_DISPLAY_SPLAT) {
            const float e = PORTABLE_EXP ? exp_portable(-r2) : __expf(-r2);
            *alpha = __fmul_rn(a.w, e);
        } else {
            *alpha = (r2 > outline2) ? 1.0f : a.w;
        }
        return true;
    }
}

// BlendState::ALPHA_BLENDING onto an 8-bit channel, in units of 1/255: round(d·(1-α) + s·α).
__device__ __forceinline__ float blend8(float d, float om, float s_alpha) { return rintf(fmaf(d, om, s_alpha)); }

struct RasterShared {
    float4 a[kRasterThreads];    // cx, cy, r² limit, alpha
    float4 b[kRasterThreads];    // q (or the point half sides)
    float4 c[kRasterThreads];    // s255.rgb
    float4 box[kRasterThreads];  // fragment box in pixel-centre coordinates
    float2 inv[kRasterThreads];  // 1 / |Q·(7, 0)|², 1 / |Q·(0, 3)|² (the block edges in quad space)
    uint8_t list[kRasterThreads / 32][kRasterThreads];
    uint32_t kmin;
};

// Stage list entries [rel0, rel0 + cnt) of the tile (cnt <= 256), one per thread.
template <uint32_t MODE>
__device__ __forceinline__ void stage_chunk(RasterShared &S, const gs_splat *__restrict__ sorted,
                                            const uint2 *__restrict__ pairs, uint32_t first, uint32_t cnt,
                                            float std2, uint32_t max_splats) {
    const uint32_t tid = threadIdx.x;
    if (tid < cnt) {
        const uint32_t k = pairs[first + tid].y;
        float4 a = make_float4(0.0f, 0.0f, -1.0f, -1.0f), b = make_float4(0.0f, 0.0f, 0.0f, 0.0f), c = b;
        if (k < max_splats) {  // ranks come from the tile sort; false only after a timeout
            const float4 *src = reinterpret_cast<const float4 *>(sorted + k);
            a = __ldg(src);
            b = __ldg(src + 1);
            c = __ldg(src + 2);
        }
        // Fragments beyond the r² limit cannot change the pixel (see splat_r2_bound).
        const float lim =
            (MODE == GS_DISPLAY_SPLAT) ? splat_r2_bound(c.w, splat_colour_reach(c.x, c.y, c.z), std2) : std2;
        S.a[tid] = make_float4(a.x, a.y, lim, c.w);
        S.b[tid] = b;
        S.c[tid] = c;
        S.box[tid] = make_float4(a.x - a.z, a.x + a.z, a.y - a.w, a.y + a.w);
        if constexpr (MODE != GS_DISPLAY_POINT) {
            const float e1x = b.x * kBlockSpanX, e1y = b.z * kBlockSpanX;
            const float e2x = b.y * kBlockSpanY, e2y = b.w * kBlockSpanY;
            S.inv[tid] = make_float2(__frcp_rn(e1x * e1x + e1y * e1y), __frcp_rn(e2x * e2x + e2y * e2y));
        }
    }
}

// Whether the fragment ellipse {p : |Q·(p - c)|² <= lim} of a staged splat meets the rectangle
// of pixel centres [bx0, bx0 + 7] x [by0, by0 + 3] of a warp's block.  With c outside the
// rectangle, the nearest point of the rectangle in the quadratic norm lies on an edge whose
// half-plane c violates (moving from it toward c must leave the rectangle); Q maps each edge
// to a segment in quad space, where the distance from the origin is minimised in closed form.
// The limit carries a margin (0.2 % + 1e-4) above the rounding of either side, so a block
// holding a pixel centre the fragment test accepts is never dropped; dropping the others
// leaves every pixel unchanged.
__device__ __forceinline__ bool seg_within(float ux, float uy, float ex, float ey, float inv, float lim) {
    float t = -(ux * ex + uy * ey) * inv;
    t = fminf(fmaxf(t, 0.0f), 1.0f);
    const float px = ux + t * ex, py = uy + t * ey;
    return px * px + py * py <= lim;
}

__device__ __forceinline__ bool ellipse_meets_block(const float4 a, const float4 q, const float2 inv, float bx0,
                                                    float bx1, float by0, float by1) {
    const bool inx = a.x >= bx0 && a.x <= bx1, iny = a.y >= by0 && a.y <= by1;
    if (inx && iny) return true;
    const float lim = a.z * 1.002f + 1e-4f;
    const float dx = bx0 - a.x, dy = by0 - a.y;
    const float ux = q.x * dx + q.y * dy, uy = q.z * dx + q.w * dy;  // corner (bx0, by0)
    const float e1x = q.x * kBlockSpanX, e1y = q.z * kBlockSpanX;   // along x, 7 px
    const float e2x = q.y * kBlockSpanY, e2y = q.w * kBlockSpanY;   // along y, 3 px
    bool m = false;
    if (!inx) {  // left edge (c left of the block) or right edge
        const bool left = a.x < bx0;
        m = seg_within(left ? ux : ux + e1x, left ? uy : uy + e1y, e2x, e2y, inv.y, lim);
    }
    if (!iny && !m) {  // top edge (c above) or bottom edge
        const bool top = a.y < by0;
        m = seg_within(top ? ux : ux + e2x, top ? uy : uy + e2y, e1x, e1y, inv.x, lim);
    }
    return m;
}

// The calling warp's list of staged entries whose fragments can reach its pixel block, in draw
// order: the fragment box, then (splat and ellipse modes) the ellipse itself must meet the block.
template <uint32_t MODE>
__device__ __forceinline__ uint32_t compact_chunk(RasterShared &S, uint32_t cnt, float bx0, float bx1, float by0,
                                                  float by1) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t lt = lanemask_lt();
    uint32_t nl = 0;
    for (uint32_t j0 = 0; j0 < cnt; j0 += 32) {
        const uint32_t j = j0 + lane;
        bool hit = false;
        if (j < cnt) {
            const float4 box = S.box[j];
            hit = !(box.y < bx0 || box.x > bx1 || box.w < by0 || box.z > by1);
            if (MODE != GS_DISPLAY_POINT && hit) hit = ellipse_meets_block(S.a[j], S.b[j], S.inv[j], bx0, bx1, by0, by1);
        }
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, hit);
        if (hit) S.list[warp][nl + __popc(m & lt)] = (uint8_t)j;
        nl += __popc(m);
    }
    __syncwarp();
    return nl;
}

// K4.  One CTA per 16x16 tile; each warp owns an 8x4 pixel block, each thread one pixel.
// Short tile lists are blended back to front in one pass.  Long ones use an exact early-out:
//   A. walk the list front to back (nearest first) until the pixel's transmittance drops
//      below `eps`, at list position k;
//   B. blend positions k.. back to front twice, from destination 0 and from 255.  The blend
//      with 8-bit rounding is monotone in the destination, so the two results bound the
//      result of every history before k; when they meet, that is the exact pixel.  A pixel
//      whose bounds do not meet restarts B from k - (n - k) (k = 0 starts from the cleared
//      value, which is exact).
// Every pixel therefore ends bit-identical to the full back-to-front pass.
template <uint32_t MODE, bool PORTABLE_EXP, bool COUNT>
__device__ __forceinline__ void raster_tile(
    RasterShared &S, const gs_splat *__restrict__ sorted, const uint2 *__restrict__ pairs,
    const uint2 *__restrict__ ranges, uint8_t *__restrict__ target, uint32_t W, uint32_t H, uint32_t pitch,
    uint32_t tiles_x, float std2, float outline2, uint32_t max_splats, uint32_t suffix_min, float eps,
    unsigned long long *counters, Ctrl *pctrl, uint32_t tile) {
    // Work tallies of the counting variant (profiling only): fragment evaluations, alphas,
    // channel-triple blends and transmittance updates.
    uint32_t n_eval = 0, n_alpha = 0, n_blend = 0, n_trans = 0;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t tx = tile % tiles_x, ty = tile / tiles_x;
    uint2 range = ranges[tile];
    if (range.y < range.x || range.y > pctrl->count) {
        if (threadIdx.x == 0) atomicOr(&pctrl->status, kStatusBounds);
        range = make_uint2(0u, 0u);
    }
    const uint32_t s0 = range.x, n = range.y - range.x;
    const uint32_t wx0 = tx * GS_TILE + (warp & 1u) * 8u, wy0 = ty * GS_TILE + (warp >> 1) * 4u;
    const uint32_t px = wx0 + (lane & 7u), py = wy0 + (lane >> 3);
    const float pxc = (float)px + 0.5f, pyc = (float)py + 0.5f;
    const float bx0 = (float)wx0 + 0.5f, bx1 = (float)wx0 + 7.5f;
    const float by0 = (float)wy0 + 0.5f, by1 = (float)wy0 + 3.5f;
    float d0 = 0.0f, d1 = 0.0f, d2 = 0.0f;

    if (n < suffix_min) {
        for (uint32_t base = 0; base < n; base += kRasterThreads) {
            const uint32_t cnt = min(kRasterThreads, n - base);
            stage_chunk<MODE>(S, sorted, pairs, s0 + base, cnt, std2, max_splats);
            __syncthreads();
            const uint32_t nl = compact_chunk<MODE>(S, cnt, bx0, bx1, by0, by1);
            for (uint32_t i = 0; i < nl; ++i) {
                const uint32_t j = S.list[warp][i];
                float al;
                if (COUNT) ++n_eval;
                if (!fragment<MODE, PORTABLE_EXP>(S.a[j], S.b[j], pxc, pyc, outline2, &al)) continue;
                if (COUNT) ++n_alpha, ++n_blend;
                const float4 c = S.c[j];
                const float om = __fsub_rn(1.0f, al);
                d0 = blend8(d0, om, __fmul_rn(c.x, al));
                d1 = blend8(d1, om, __fmul_rn(c.y, al));
                d2 = blend8(d2, om, __fmul_rn(c.z, al));
            }
            __syncthreads();
        }
    } else {
        // ---- A: front-to-back transmittance to find the start position k ----
        float T = 1.0f;
        uint32_t k = 0;
        bool found = false;
        for (uint32_t end = n; end > 0;) {
            const uint32_t base = end > kRasterThreads ? end - kRasterThreads : 0u;
            const uint32_t cnt = end - base;
            stage_chunk<MODE>(S, sorted, pairs, s0 + base, cnt, std2, max_splats);
            __syncthreads();
            if (__any_sync(0xFFFFFFFFu, !found)) {
                const uint32_t nl = compact_chunk<MODE>(S, cnt, bx0, bx1, by0, by1);
                for (int i = (int)nl - 1; i >= 0; --i) {
                    if (__all_sync(0xFFFFFFFFu, found)) break;
                    const uint32_t j = S.list[warp][i];
                    float al;
                    if (COUNT && !found) ++n_eval;
                    if (!found && fragment<MODE, PORTABLE_EXP>(S.a[j], S.b[j], pxc, pyc, outline2, &al)) {
                        if (COUNT) ++n_alpha, ++n_trans;
                        T = __fmul_rn(T, __fsub_rn(1.0f, al));
                        if (T < eps) {
                            found = true;
                            k = base + j;
                        }
                    }
                }
            }
            if (__syncthreads_and(found)) break;
            end = base;
        }
        if (!found) k = 0;
        // The bounds argument holds from any start position, so a warp starts all its pixels at
        // the smallest k among them: lanes share issue slots, the earlier start costs the warp
        // nothing, and it makes the bounds more likely to meet on the first pass.
        k = __reduce_min_sync(0xFFFFFFFFu, k);
        // ---- B: bounded back-to-front passes from k ----
        bool active = true;
        float h0 = 0.0f, h1 = 0.0f, h2 = 0.0f;
        for (;;) {
            if (tid == 0) S.kmin = 0xFFFFFFFFu;
            __syncthreads();
            const uint32_t wmin = __reduce_min_sync(0xFFFFFFFFu, active ? k : 0xFFFFFFFFu);
            if (lane == 0 && wmin != 0xFFFFFFFFu) atomicMin(&S.kmin, wmin);
            __syncthreads();
            const uint32_t kmin = S.kmin;
            if (kmin == 0xFFFFFFFFu) break;
            if (active) {
                const float top = (k == 0) ? 0.0f : 255.0f;
                d0 = d1 = d2 = 0.0f;
                h0 = h1 = h2 = top;
            }
            for (uint32_t base = kmin / kRasterThreads * kRasterThreads; base < n; base += kRasterThreads) {
                const uint32_t cnt = min(kRasterThreads, n - base);
                __syncthreads();
                stage_chunk<MODE>(S, sorted, pairs, s0 + base, cnt, std2, max_splats);
                __syncthreads();
                // k is uniform across the warp: a warp whose suffix starts past this chunk skips it
                const bool inside = active && k < base + kRasterThreads;  // chunk holds suffix entries
                if (__any_sync(0xFFFFFFFFu, inside)) {
                    const uint32_t nl = compact_chunk<MODE>(S, cnt, bx0, bx1, by0, by1);
                    // Bounds that have met stay equal (same inputs, same operations), so once
                    // every started lane of the warp has met, one chain per channel suffices.
                    const bool met = d0 == h0 && d1 == h1 && d2 == h2;
                    if (__all_sync(0xFFFFFFFFu, !inside || (met && base >= k))) {
                        for (uint32_t i = 0; i < nl; ++i) {
                            const uint32_t j = S.list[warp][i];
                            float al;
                            if (!inside) continue;
                            if (COUNT) ++n_eval;
                            if (!fragment<MODE, PORTABLE_EXP>(S.a[j], S.b[j], pxc, pyc, outline2, &al)) continue;
                            if (COUNT) ++n_alpha, ++n_blend;
                            const float4 c = S.c[j];
                            const float om = __fsub_rn(1.0f, al);
                            d0 = blend8(d0, om, __fmul_rn(c.x, al));
                            d1 = blend8(d1, om, __fmul_rn(c.y, al));
                            d2 = blend8(d2, om, __fmul_rn(c.z, al));
                        }
                        if (inside) {
                            h0 = d0;
                            h1 = d1;
                            h2 = d2;
                        }
                    } else {
                        for (uint32_t i = 0; i < nl; ++i) {
                            const uint32_t j = S.list[warp][i];
                            float al;
                            if (!active || base + j < k) continue;
                            if (COUNT) ++n_eval;
                            if (!fragment<MODE, PORTABLE_EXP>(S.a[j], S.b[j], pxc, pyc, outline2, &al)) continue;
                            if (COUNT) ++n_alpha, n_blend += 2;
                            const float4 c = S.c[j];
                            const float om = __fsub_rn(1.0f, al);
                            const float s0a = __fmul_rn(c.x, al), s1a = __fmul_rn(c.y, al), s2a = __fmul_rn(c.z, al);
                            d0 = blend8(d0, om, s0a);
                            d1 = blend8(d1, om, s1a);
                            d2 = blend8(d2, om, s2a);
                            h0 = blend8(h0, om, s0a);
                            h1 = blend8(h1, om, s1a);
                            h2 = blend8(h2, om, s2a);
                        }
                    }
                }
            }
            __syncthreads();
            if (active) {
                if (d0 == h0 && d1 == h1 && d2 == h2) {
                    active = false;
                } else {
                    const uint32_t suffix = n - k;
                    k = k > suffix ? k - suffix : 0u;
                }
            }
        }
    }
    if (px < W && py < H) {
        const uint32_t rgba = (uint32_t)d0 | ((uint32_t)d1 << 8) | ((uint32_t)d2 << 16) | 0xFF000000u;
        *reinterpret_cast<uint32_t *>(target + (size_t)py * pitch + (size_t)px * 4u) = rgba;
    }
    if constexpr (COUNT) {
        const uint32_t v[4] = {n_eval, n_alpha, n_blend, n_trans};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint32_t w = __reduce_add_sync(0xFFFFFFFFu, v[q]);
            if (lane == 0 && w) atomicAdd(counters + q, (unsigned long long)w);
        }
    }
}


template <uint32_t MODE, bool PORTABLE_EXP, bool COUNT>
__global__ void __launch_bounds__(kRasterThreads, 6) raster_kernel(const RasterJob J, float std2, float outline2,
                                                                uint32_t suffix_min, float eps,
                                                                unsigned long long *counters) {
    __shared__ RasterShared S;
    raster_tile<MODE, PORTABLE_EXP, COUNT>(S, J.splats, J.pairs, J.ranges, J.target, J.W, J.H, J.pitch, J.tiles_x,
                                           std2, outline2, J.max_splats, suffix_min, eps, counters, J.ctrl,
                                           J.order ? J.order[blockIdx.x] : blockIdx.x);
}

// One grid over the tiles of several views (a batch): CTA b rasterises tile b - tile_base[v] of
// the view v with tile_base[v] <= b < tile_base[v + 1].
template <uint32_t MODE, bool PORTABLE_EXP>
__global__ void __launch_bounds__(kRasterThreads, 6) raster_views_kernel(const RasterJob *__restrict__ jobs,
                                                                      const uint32_t *__restrict__ tile_base,
                                                                      uint32_t nviews, float std2, float outline2,
                                                                      uint32_t suffix_min, float eps) {
    __shared__ RasterShared S;
    uint32_t lo = 0, hi = nviews - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (tile_base[mid] <= blockIdx.x) lo = mid;
        else hi = mid - 1;
    }
    const RasterJob &J = jobs[lo];
    const uint32_t b = blockIdx.x - tile_base[lo];
    raster_tile<MODE, PORTABLE_EXP, false>(S, J.splats, J.pairs, J.ranges, J.target, J.W, J.H, J.pitch, J.tiles_x,
                                           std2, outline2, J.max_splats, suffix_min, eps, nullptr, J.ctrl,
                                           J.order ? J.order[b] : b);
}

// Work tallies of the counting raster variant (profiling only).
static __device__ unsigned long long g_raster_counts[4];

cudaError_t raster_counters(unsigned long long out[4], bool reset) {
    cudaError_t e = cudaMemcpyFromSymbol(out, g_raster_counts, sizeof(g_raster_counts));
    if (e == cudaSuccess && reset) {
        const unsigned long long zero[4] = {0, 0, 0, 0};
        e = cudaMemcpyToSymbol(g_raster_counts, zero, sizeof(zero));
    }
    return e;
}

template <uint32_t MODE>
static void launch_raster_mode(const RasterJob &J, uint32_t ntiles, float std2, float outline2, int exact,
                               cudaStream_t st, const Tuning &t) {
    if (exact) {
        raster_kernel<MODE, true, false><<<ntiles, kRasterThreads, 0, st>>>(J, std2, outline2, t.suffix_min, t.eps,
                                                                            nullptr);
    } else if (MODE == GS_DISPLAY_SPLAT && prof_counting()) {
        unsigned long long *counts = nullptr;
        cudaGetSymbolAddress((void **)&counts, g_raster_counts);
        raster_kernel<GS_DISPLAY_SPLAT, false, true><<<ntiles, kRasterThreads, 0, st>>>(J, std2, outline2,
                                                                                       t.suffix_min, t.eps, counts);
    } else {
        raster_kernel<MODE, false, false><<<ntiles, kRasterThreads, 0, st>>>(J, std2, outline2, t.suffix_min, t.eps,
                                                                             nullptr);
    }
}

template <uint32_t MODE>
static void launch_raster_views_mode(const RasterJob *jobs, const uint32_t *tile_base, uint32_t nviews,
                                     uint32_t total_tiles, float std2, float outline2, int exact, cudaStream_t st,
                                     const Tuning &t) {
    if (exact)
        raster_views_kernel<MODE, true><<<total_tiles, kRasterThreads, 0, st>>>(jobs, tile_base, nviews, std2,
                                                                                 outline2, t.suffix_min, t.eps);
    else
        raster_views_kernel<MODE, false><<<total_tiles, kRasterThreads, 0, st>>>(jobs, tile_base, nviews, std2,
                                                                                  outline2, t.suffix_min, t.eps);
}

RasterJob raster_job(const RasterSegment *segs, uint32_t nseg, uint8_t *target, uint32_t W, uint32_t H,
                     uint32_t pitch, uint32_t max_pairs, void *scratch) {
    uint32_t max_splats = 0;
    for (uint32_t s = 0; s < nseg; ++s) max_splats += segs[s].max_count;
    const RasterLayout L = raster_layout(scratch, max_splats, W, H, max_pairs);
    RasterJob J;
    // Pair values index the model's own splat array (one segment) or the draw-ordered copy.
    J.splats = nseg == 1 ? segs[0].splats : L.sorted;
    J.max_splats = nseg == 1 ? segs[0].max_count : max_splats;
    J.pairs = L.pairs;
    J.ranges = L.ranges;
    J.order = L.order;
    J.target = target;
    J.W = W;
    J.H = H;
    J.pitch = pitch;
    J.tiles_x = L.tiles_x;
    J.ntiles = L.ntiles;
    J.ctrl = L.ctrl;
    return J;
}

cudaError_t launch_raster_views(const RasterJob *jobs_dev, const uint32_t *tile_base_dev, uint32_t nviews,
                                uint32_t total_tiles, const RasterMode &u, int exact_exp, cudaStream_t st,
                                const Tuning *tuning) {
    if (nviews == 0 || total_tiles == 0) return cudaSuccess;
    const Tuning tn = tuning ? *tuning : default_tuning();
    const float std2 = u.std_dev * u.std_dev;
    const float o = u.std_dev - 0.1f;
    const float outline2 = o * o;
    prof_mark(kProfRaster, true, st);
    count_launches(1);
    switch (u.display_mode) {
        case GS_DISPLAY_SPLAT:
            launch_raster_views_mode<GS_DISPLAY_SPLAT>(jobs_dev, tile_base_dev, nviews, total_tiles, std2, outline2,
                                                       exact_exp, st, tn);
            break;
        case GS_DISPLAY_ELLIPSE:
            launch_raster_views_mode<GS_DISPLAY_ELLIPSE>(jobs_dev, tile_base_dev, nviews, total_tiles, std2, outline2,
                                                         exact_exp, st, tn);
            break;
        default:
            launch_raster_views_mode<GS_DISPLAY_POINT>(jobs_dev, tile_base_dev, nviews, total_tiles, std2, outline2,
                                                       exact_exp, st, tn);
            break;
    }
    prof_mark(kProfRaster, false, st);
    return cudaGetLastError();
}

cudaError_t launch_binning_front(const RasterSegment *segs, uint32_t nseg, const RasterMode &u, uint32_t W,
                           uint32_t H, uint32_t max_pairs, void *scratch, cudaStream_t st) {
    uint32_t max_splats = 0;
    for (uint32_t s = 0; s < nseg; ++s) max_splats += segs[s].max_count;
    const RasterLayout L = raster_layout(scratch, max_splats, W, H, max_pairs);
    if (L.ntiles == 0) return cudaSuccess;
    // The first segment with splats clears the arena in its bin_count launch; with none, no kernel
    // reads a flag and the arena mark stays.
    bool any = false;
    for (uint32_t s = 0; s < nseg; ++s) any = any || segs[s].max_count > 0;
    const WaitCfg cfg = wait_config();
    ctrl_init_kernel<<<1, 256, 0, st>>>(L.ctrl, 1, nullptr, any ? L.arena_words : kKeepArena, cfg);
    count_launches(1);
    cudaError_t e = sort_pairs_begin(L.sort_ctrl, L.ctrl, st);
    if (e != cudaSuccess) return e;
    Ctrl *sort_ctrl = L.sort_ctrl;
    if (L.counts) {
        e = cudaMemsetAsync(L.counts, 0, (size_t)L.ntiles * 4, st);
        if (e != cudaSuccess) return e;
    }
    const PassSplit split = tile_split(L.key_bits);
    // The emit kernel loops over its ranks grid-stride with equal shares per CTA: one resident
    // wave (at most kEmitBlocks, the per-CTA count area) keeps a second, late wave from
    // doubling the kernel's span.
    const size_t emit_smem = L.counts ? (size_t)L.ntiles * 4u : 4u * 256u * 4u;
    uint32_t emit_wave = kEmitBlocks;
    {
        int dev = 0, sms = 0, per_sm = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
            (L.counts ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bin_emit_kernel<true>, kBinThreads, emit_smem)
                      : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bin_emit_kernel<false>, kBinThreads,
                                                                       emit_smem)) == cudaSuccess &&
            sms > 0 && per_sm > 0) {
            const uint32_t wave = (uint32_t)sms * (uint32_t)per_sm;
            if (wave < emit_wave) emit_wave = wave;
        }
    }
    uint32_t rank_offset = 0;
    bool cleared = false;
    prof_mark(kProfBin, true, st);
    const int direct = nseg == 1 ? 1 : 0;
    for (uint32_t s = 0; s < nseg; ++s) {
        const RasterSegment &g = segs[s];
        const uint32_t blocks = (g.max_count + kBinThreads - 1) / kBinThreads;
        if (blocks == 0) continue;
        if (s > 0) {
            ctrl_init_kernel<<<1, 32, 0, st>>>(L.ctrl, 0, nullptr, kKeepArena, cfg);
            count_launches(1);
        }
        // a stored tile record is only for the target the preprocess was given (one model)
        const uint4 *binfo = direct && g.binfo && g.binfo_w == W && g.binfo_h == H ? g.binfo : nullptr;
        bin_count_kernel<<<blocks, kBinThreads, 0, st>>>(g.splats, binfo, g.sorted_index, g.count, g.max_count,
                                                         rank_offset, L.sorted, direct, L.tiles_x, L.tiles_y,
                                                         u.display_mode, u.std_dev * u.std_dev, L.info, L.offsets,
                                                         L.ctrl, cleared ? nullptr : L.flags);
        cleared = true;
        const uint32_t scan_blocks = (g.max_count + kScanTile - 1) / kScanTile;
        bin_scan_kernel<<<scan_blocks, 256, 0, st>>>(L.offsets, g.count, g.max_count, L.ctrl, L.flags);
        const uint32_t eblocks = blocks < emit_wave ? blocks : emit_wave;
        if (L.counts) {
            bin_emit_kernel<true><<<eblocks, kBinThreads, emit_smem, st>>>(
                L.info, L.offsets, g.count, g.max_count, L.pairs, max_pairs, L.tiles_x, L.ntiles, L.ctrl, sort_ctrl,
                split, L.blockcounts);
            tile_count_kernel<<<dim3((L.ntiles + 255) / 256, kCountSlices), 256, 0, st>>>(L.blockcounts, eblocks,
                                                                                         L.ntiles, L.counts);
            count_launches(1);
        } else {
            bin_emit_kernel<false><<<eblocks, kBinThreads, emit_smem, st>>>(
                L.info, L.offsets, g.count, g.max_count, L.pairs, max_pairs, L.tiles_x, L.ntiles, L.ctrl, sort_ctrl,
                split, nullptr);
        }
        bin_advance_kernel<<<1, 1, 0, st>>>(L.ctrl, g.count, g.max_count, max_pairs);
        count_launches(4);
        rank_offset += g.max_count;
    }
    if (L.counts) {
        tile_scan_kernel<<<1, 1024, 0, st>>>(L.counts, L.ntiles, L.ranges, L.order, sort_ctrl, split);
        count_launches(1);
    }
    prof_mark(kProfBin, false, st);
    return cudaGetLastError();
}

SortSegment tile_sort_segment(const RasterSegment *segs, uint32_t nseg, uint32_t W, uint32_t H, uint32_t max_pairs,
                              void *scratch) {
    uint32_t max_splats = 0;
    for (uint32_t s = 0; s < nseg; ++s) max_splats += segs[s].max_count;
    const RasterLayout L = raster_layout(scratch, max_splats, W, H, max_pairs);
    const PassSplit split = tile_split(L.key_bits);
    const uint32_t blocks = sort_pairs_blocks(max_pairs);
    SortSegment S;
    S.data = L.pairs;
    S.alt = L.sort_alt;
    S.count = &L.ctrl->count;
    S.max_count = max_pairs;
    for (int p = 0; p < 2; ++p) {
        S.shift[p] = split.shift[p];
        S.bits[p] = split.bits[p];
    }
    S.hist_scanned = L.counts ? 1u : 0u;
    S.ctrl = L.sort_ctrl;
    S.owner = L.ctrl;
    S.flags[0] = L.sort_flags;
    S.flags[1] = L.sort_flags + ((size_t)blocks << split.bits[0]);
    return S;
}

bool tile_sort_segmentable(uint32_t W, uint32_t H) {
    const uint32_t tiles = ((W + GS_TILE - 1) / GS_TILE) * ((H + GS_TILE - 1) / GS_TILE);
    return tile_split(bits_for(tiles > 0 ? tiles - 1 : 0)).n == 2;
}

cudaError_t launch_binning_ranges(const RasterSegment *segs, uint32_t nseg, uint32_t W, uint32_t H, uint32_t max_pairs,
                                  void *scratch, cudaStream_t st) {
    uint32_t max_splats = 0;
    for (uint32_t s = 0; s < nseg; ++s) max_splats += segs[s].max_count;
    const RasterLayout L = raster_layout(scratch, max_splats, W, H, max_pairs);
    cudaError_t e = cudaSuccess;
    if (L.ntiles > 0 && !L.counts) {  // more tiles than the counting path covers: ranges from the sorted pairs
        prof_mark(kProfRanges, true, st);
        e = cudaMemsetAsync(L.ranges, 0, (size_t)L.ntiles * sizeof(uint2), st);
        if (e != cudaSuccess) return e;
        uint32_t rblocks = (max_pairs + 255) / 256;
        if (rblocks > 152 * 8) rblocks = 152 * 8;
        if (rblocks == 0) rblocks = 1;
        tile_ranges_kernel<<<rblocks, 256, 0, st>>>(L.pairs, L.ctrl, L.ranges, L.ntiles);
        prof_mark(kProfRanges, false, st);
        count_launches(1);
    }
    return cudaGetLastError();
}

cudaError_t launch_binning(const RasterSegment *segs, uint32_t nseg, const RasterMode &u, uint32_t W, uint32_t H,
                           uint32_t max_pairs, void *scratch, cudaStream_t st) {
    uint32_t max_splats = 0;
    for (uint32_t s = 0; s < nseg; ++s) max_splats += segs[s].max_count;
    const RasterLayout L = raster_layout(scratch, max_splats, W, H, max_pairs);
    if (L.ntiles == 0) return cudaSuccess;
    cudaError_t e = launch_binning_front(segs, nseg, u, W, H, max_pairs, scratch, st);
    if (e != cudaSuccess) return e;
    prof_mark(kProfTileSort, true, st);
    // counting path: tile_scan wrote the digit offsets already scanned; else the emit's counts
    e = launch_sort_pairs(L.pairs, max_pairs, &L.ctrl->count, L.key_bits, L.sort_ctrl, L.sort_flags, L.sort_alt, st,
                          L.counts != nullptr);
    prof_mark(kProfTileSort, false, st);
    if (e != cudaSuccess) return e;
    merge_status_kernel<<<1, 1, 0, st>>>(L.ctrl, L.sort_ctrl);
    count_launches(1);
    return launch_binning_ranges(segs, nseg, W, H, max_pairs, scratch, st);
}

cudaError_t launch_raster(const RasterSegment *segs, uint32_t nseg, const RasterMode &u, uint8_t *target,
                          uint32_t W, uint32_t H, uint32_t pitch, uint32_t max_pairs, void *scratch, int exact_exp,
                          cudaStream_t st, const Tuning *tuning) {
    const Tuning tn = tuning ? *tuning : default_tuning();
    cudaError_t e = launch_binning(segs, nseg, u, W, H, max_pairs, scratch, st);
    if (e != cudaSuccess) return e;
    const RasterJob J = raster_job(segs, nseg, target, W, H, pitch, max_pairs, scratch);
    if (J.ntiles == 0) return cudaSuccess;
    const float std2 = u.std_dev * u.std_dev;
    const float o = u.std_dev - 0.1f;
    const float outline2 = o * o;
    prof_mark(kProfRaster, true, st);
    count_launches(1);
    switch (u.display_mode) {
        case GS_DISPLAY_SPLAT:
            launch_raster_mode<GS_DISPLAY_SPLAT>(J, J.ntiles, std2, outline2, exact_exp, st, tn);
            break;
        case GS_DISPLAY_ELLIPSE:
            launch_raster_mode<GS_DISPLAY_ELLIPSE>(J, J.ntiles, std2, outline2, exact_exp, st, tn);
            break;
        default:
            launch_raster_mode<GS_DISPLAY_POINT>(J, J.ntiles, std2, outline2, exact_exp, st, tn);
            break;
    }
    prof_mark(kProfRaster, false, st);
    return cudaGetLastError();
}

}  // namespace gs
