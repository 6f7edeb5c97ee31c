// gs_common.cuh — device-side helpers shared by the preprocess, sort and raster kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gs_record.h"

namespace gs {

// Sticky error bits of a scratch area's control block.
constexpr uint32_t kStatusTimeout = 1u;
constexpr uint32_t kStatusCapacity = 2u;
constexpr uint32_t kStatusBounds = 4u;  // an index check failed; the access was skipped

// Default upper bound on polls of a look-back flag before a kernel gives up, records
// kStatusTimeout and carries on with a garbage value (so that waiting successors also end).
// The bound a launch uses is carried in its control block (Ctrl::spin_limit); mbarrier waits
// use this constant.
constexpr uint32_t kSpinLimit = 1u << 22;

// Look-back configuration of the launches a stage enqueues: the poll bound, and for testing the
// bounded-wait path a look-back tile that never publishes its flags (kNoStall: none), so that
// its successors' waits run out on a flag nothing sets.
constexpr uint32_t kNoStall = 0xFFFFFFFFu;
struct WaitCfg {
    uint32_t spin_limit = kSpinLimit;
    uint32_t stall_tile = kNoStall;
};

// Argument of ctrl_reset for a call that runs no arena-clearing kernel: leave the mark alone.
constexpr uint32_t kKeepArena = 0xFFFFFFFFu;
// Serial numbers above this restart at 0 with the whole arena cleared, so no epoch of a call
// (at most a few per segment) ever wraps inside it.
constexpr uint32_t kSerialRestart = (1u << 30) - (1u << 20);

// Control block at a fixed offset of every scratch area.  Look-back flags live in the area's
// flag arena, which starts right after the area's control blocks at an offset that no call size
// moves; each flag word carries the epoch it was written under.  One counter per area (`serial`,
// in the block that owns the area) hands out every epoch of that area, so a flag word left by an
// earlier call, segment or stage of the area never carries the epoch a reader expects.  The
// arena grows and shrinks with the call sizes, and the area's other buffers follow it: `clean`
// counts the arena words known to hold only zeros or flag words; a call whose arena is larger
// clears the words beyond it (clear_lo..clear_hi) in its first multi-CTA kernel, before any flag
// is read, so stale payload of a larger earlier layout is never read as a published flag.
struct Ctrl {
    uint32_t epoch;       // epoch of this block's flags for the current call or segment
    uint32_t status;
    uint32_t ticket[8];
    uint32_t count;       // preprocess: V; raster: tile pairs kept
    uint32_t total;       // raster: tile pairs wanted (saturating)
    uint32_t pair_base;   // raster: running pair offset across segments
    uint32_t seg_total;   // raster: pairs of the segment being binned
    uint32_t serial;      // area owner: last epoch handed out in the area
    uint32_t clean;       // area owner: leading arena words holding only zeros or flag words
    uint32_t clear_lo;    // area owner: arena words [clear_lo, clear_hi) to clear in this call
    uint32_t clear_hi;
    uint32_t spin_limit;  // look-back poll bound of this call
    uint32_t stall_tile;  // testing: look-back tile that never publishes (kNoStall: none)
    uint32_t pad[4];
    uint32_t hist[4][256];  // sort: global digit histograms
};
static_assert(sizeof(Ctrl) % 16 == 0, "Ctrl must keep 16-byte alignment of what follows");

// Resets a control block (one CTA): mode 1 = a new stage call (epoch, status, tickets, counters,
// histograms, wait configuration); mode 0 = a new segment inside a call (epoch and tickets 0..1
// only).  The epoch comes from `owner`, the block holding the area's serial counter (the block
// itself for a single-stage area).  `arena_words` (owner, mode 1 only): words of the flag arena
// this call uses, or kKeepArena when this call runs no clearing kernel.
__device__ __forceinline__ void ctrl_reset(Ctrl *ctrl, int mode, Ctrl *owner, uint32_t arena_words, WaitCfg cfg) {
    const uint32_t t = threadIdx.x;
    if (t == 0) {
        if (ctrl == owner && mode == 1) {
            if (owner->serial >= kSerialRestart) {
                owner->serial = 0u;
                owner->clean = 0u;  // flags of the old serial range may match new epochs
            }
            if (arena_words != kKeepArena) {
                const uint32_t c = owner->clean;
                owner->clear_lo = c < arena_words ? c : arena_words;
                owner->clear_hi = arena_words;
                // Past `arena_words` the area's other buffers begin, so only this call's arena
                // is known clean once the clearing kernel has run.
                owner->clean = arena_words;
            } else {
                owner->clear_lo = owner->clear_hi = 0u;
            }
        }
        const uint32_t e = owner->serial + 1u;
        owner->serial = e;
        ctrl->epoch = e;
        ctrl->ticket[0] = 0u;
        ctrl->ticket[1] = 0u;
        if (mode == 1) {
            ctrl->status = 0u;
            for (int k = 1; k < 8; ++k) ctrl->ticket[k] = 0u;
            ctrl->count = 0u;
            ctrl->total = 0u;
            ctrl->pair_base = 0u;
            ctrl->seg_total = 0u;
            ctrl->spin_limit = cfg.spin_limit;
            ctrl->stall_tile = cfg.stall_tile;
        }
    }
    if (mode == 1)
        for (uint32_t k = t; k < 4 * 256; k += blockDim.x) (&ctrl->hist[0][0])[k] = 0u;
}

// The arena words this call must clear (set by the owner's mode-1 reset), cleared by every CTA
// of a grid that runs before any look-back of the call (grid-stride, 16-byte stores).
__device__ __forceinline__ void arena_clear(const Ctrl *owner, uint64_t *arena) {
    const uint32_t lo = owner->clear_lo, hi = owner->clear_hi;
    if (lo >= hi) return;
    const uint32_t stride = gridDim.x * blockDim.x;
    uint32_t a = (lo + 1u) & ~1u;  // first even word
    if (a > hi) a = hi;
    if (lo < a && blockIdx.x == 0 && threadIdx.x == 0) arena[lo] = 0ull;
    const uint32_t b = a + ((hi - a) & ~1u);
    for (uint32_t w = a + 2u * (blockIdx.x * blockDim.x + threadIdx.x); w < b; w += 2u * stride)
        *reinterpret_cast<ulonglong2 *>(arena + w) = make_ulonglong2(0ull, 0ull);
    if (b < hi && blockIdx.x == 0 && threadIdx.x == 0) arena[b] = 0ull;
}

// L2 prefetch hint for a byte range (no data returned): 16-byte aligned address, size a
// nonzero multiple of 16.
__device__ __forceinline__ void prefetch_l2_bulk(const void *src, uint32_t bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

// Look-back flag word: epoch (30 bits) | status (2 bits) | value (32 bits).
constexpr uint32_t kFlagAggregate = 1u;
constexpr uint32_t kFlagPrefix = 2u;

__device__ __forceinline__ uint64_t pack_flag(uint32_t epoch, uint32_t status, uint32_t value) {
    return ((uint64_t)epoch << 34) | ((uint64_t)status << 32) | (uint64_t)value;
}

__device__ __forceinline__ void st_relaxed(uint64_t *p, uint64_t v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Publishes a look-back flag unless `tile` is the stalled tile of a bounded-wait test.
__device__ __forceinline__ void publish_flag(uint64_t *p, uint32_t tile, uint32_t stall_tile, uint64_t v) {
    if (tile != stall_tile) st_relaxed(p, v);
}

__device__ __forceinline__ uint64_t ld_relaxed(const uint64_t *p) {
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// Look-back flags are published and read with relaxed atomics: a flag word carries everything
// its reader uses (epoch, status and the count itself), and no other memory is read on the
// strength of a flag, so no release/acquire ordering (and no fence) is needed.

// Warp-cooperative look-back of one counter (flags[j], j < tile), called by all 32 lanes of a
// warp: each round reads 32 predecessors at once, adds every aggregate down to the nearest
// inclusive prefix and stops there.  Returns the exclusive prefix in every lane.  After
// `limit` polls that find an unpublished predecessor it sets kStatusTimeout and returns what
// it has summed.
__device__ __forceinline__ uint32_t look_back_warp(const uint64_t *flags, uint32_t tile, uint32_t epoch,
                                                   uint32_t *status, uint32_t limit) {
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t prefix = 0;
    int64_t hi = (int64_t)tile;  // window is [hi - 32, hi)
    uint32_t spins = 0;
    while (hi > 0) {
        const int64_t j = hi - 1 - (int64_t)lane;
        uint64_t w;
        if (j >= 0) {
            w = ld_relaxed(flags + j);
        } else {
            w = pack_flag(epoch, kFlagPrefix, 0u);  // before the first tile: an empty prefix
        }
        const bool ok = (uint32_t)(w >> 34) == epoch && ((uint32_t)(w >> 32) & 3u) != 0u;
        const bool pre = ok && ((uint32_t)(w >> 32) & 3u) == kFlagPrefix;
        const uint32_t pmask = __ballot_sync(0xFFFFFFFFu, pre);
        const uint32_t bad = __ballot_sync(0xFFFFFFFFu, !ok);
        const uint32_t upto = pmask ? (uint32_t)(__ffs(pmask) - 1) : 31u;  // lanes 0..upto needed
        const uint32_t need = upto == 31u ? 0xFFFFFFFFu : ((2u << upto) - 1u);
        if (bad & need) {
            if (++spins > limit) {
                if (lane == 0) atomicOr(status, kStatusTimeout);
                break;
            }
            if (spins > 64) __nanosleep(32);
            continue;
        }
        uint32_t v = (lane <= upto) ? (uint32_t)w : 0u;
#pragma unroll
        for (uint32_t o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
        prefix += v;
        if (pmask) break;
        hi -= 32;
    }
    return prefix;
}

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Round to nearest even for |x| < 2^22 with two IEEE adds (no conversion instruction).
__device__ __forceinline__ float rint_small(float x) {
    const float m = 12582912.0f;
    return __fsub_rn(__fadd_rn(x, m), m);
}

// exp(x) on [-10, 0]: Cody–Waite reduction with the classic two-part ln2, degree-7 Taylor
// polynomial in Horner form with FMAs, scale by 2^k through the exponent field.  The CPU
// oracle evaluates the identical sequence, so the two agree bit for bit.
__device__ __forceinline__ float exp_portable(float x) {
    const float k = rint_small(__fmul_rn(x, 1.44269504088896341f));
    float r = fmaf(-k, 0.693359375f, x);
    r = fmaf(-k, -2.12194440e-4f, r);
    float p = 1.0f / 5040.0f;
    p = fmaf(p, r, 1.0f / 720.0f);
    p = fmaf(p, r, 1.0f / 120.0f);
    p = fmaf(p, r, 1.0f / 24.0f);
    p = fmaf(p, r, 1.0f / 6.0f);
    p = fmaf(p, r, 0.5f);
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    const int ki = (int)k;
    return __fmul_rn(p, __uint_as_float((uint32_t)(ki + 127) << 23));
}

// Fragment-bearing r² bound of a splat (see gs_splat.ex).  A fragment of alpha a moves a channel
// of destination d in [0, 255] by a·(s - d), |s - d| <= m = max over the colour channels of
// max(s, 255 - s); with a·m <= 0.499 (plus FP32 rounding far below 1e-3) the rounded blend gives
// d back, so the fragment cannot change the pixel.  a = alpha·exp(-r²) <= 0.499/m whenever
// r² >= ln(alpha·m/0.499); ln x <= ln2·(e + mant - 1 + 0.0861) for x = mant·2^e, plus margins.
__host__ __device__ __forceinline__ float splat_colour_reach(float s0, float s1, float s2) {
    const float t0 = s0 > 255.0f - s0 ? s0 : 255.0f - s0;
    const float t1 = s1 > 255.0f - s1 ? s1 : 255.0f - s1;
    const float t2 = s2 > 255.0f - s2 ? s2 : 255.0f - s2;
    const float t01 = t0 > t1 ? t0 : t1;
    return t01 > t2 ? t01 : t2;
}

__device__ __forceinline__ float splat_r2_bound(float alpha, float reach, float std2) {
    const float x = (alpha * reach) * 2.0041f;  // >= alpha·reach / 0.499
    if (!(x > 0.0f)) return -1.0f;
    const uint32_t bits = __float_as_uint(x);
    const float e = (float)((int)((bits >> 23) & 0xFFu) - 127);
    const float mant = __uint_as_float((bits & 0x7FFFFFu) | 0x3F800000u);
    const float r2 = 0.693147182f * (e + (mant - 1.0f) + 0.0862f) + 0.01f;
    return (r2 < std2) ? r2 : std2;
}

// Tile rectangle of a splat's fragment box; false when it touches no tile.
__device__ __forceinline__ bool tile_rect(const float4 a, uint32_t tiles_x, uint32_t tiles_y, uint32_t *x0,
                                          uint32_t *y0, uint32_t *w, uint32_t *h) {
    const float cx = a.x, cy = a.y, ex = a.z, ey = a.w;
    if (!(ex >= 0.0f && ey >= 0.0f) || !isfinite(cx) || !isfinite(cy) || !isfinite(ex) || !isfinite(ey))
        return false;
    const float inv = 1.0f / (float)GS_TILE;
    const float fx0 = floorf((cx - ex) * inv), fx1 = floorf((cx + ex) * inv);
    const float fy0 = floorf((cy - ey) * inv), fy1 = floorf((cy + ey) * inv);
    const float lx = fmaxf(fx0, 0.0f), hx = fminf(fx1, (float)tiles_x - 1.0f);
    const float ly = fmaxf(fy0, 0.0f), hy = fminf(fy1, (float)tiles_y - 1.0f);
    if (lx > hx || ly > hy) return false;
    *x0 = (uint32_t)lx;
    *y0 = (uint32_t)ly;
    *w = (uint32_t)hx - *x0 + 1u;
    *h = (uint32_t)hy - *y0 + 1u;
    return true;
}

// Conservative test whether a splat's fragment ellipse {p : |Q·(p - c)|² <= r2} meets the 16x16
// tiles of a rectangle.  A tile's box of pixel centres maps to a parallelogram in quad-offset
// space with the same two edge vectors for every tile; the ellipse becomes the disc of radius
// sqrt(r2) about the origin, which lies outside the parallelogram when c lies outside the box,
// so the two meet iff an edge comes within the radius.  The limit carries a small margin, so
// rounding can only keep a tile, never drop one.
struct TileCull {
    float cx, cy, q0, q1, q2, q3, e1x, e1y, e2x, e2y, i1, i2, lim;

    __device__ __forceinline__ TileCull(const float4 a, const float4 q, float r2) {
        cx = a.x;
        cy = a.y;
        q0 = q.x;
        q1 = q.y;
        q2 = q.z;
        q3 = q.w;
        const float side = (float)(GS_TILE - 1);
        e1x = q.x * side;
        e1y = q.z * side;
        e2x = q.y * side;
        e2y = q.w * side;
        i1 = __frcp_rn(e1x * e1x + e1y * e1y);
        i2 = __frcp_rn(e2x * e2x + e2y * e2y);
        lim = r2 * 1.002f + 1e-4f;
    }

    __device__ __forceinline__ bool edge(float ux, float uy, float ex, float ey, float inv) const {
        float t = -(ux * ex + uy * ey) * inv;
        t = fminf(fmaxf(t, 0.0f), 1.0f);
        const float px = ux + t * ex, py = uy + t * ey;
        return px * px + py * py <= lim;
    }

    // Tile whose first pixel centre is (x0, y0).  Only box edges facing the centre can hold
    // the point nearest to it, and a linear map keeps which side of an edge a point lies on.
    __device__ __forceinline__ bool meets(float x0, float y0) const {
        const float x1 = x0 + (float)(GS_TILE - 1), y1 = y0 + (float)(GS_TILE - 1);
        const float dx = x0 - cx, dy = y0 - cy;
        const float ux = q0 * dx + q1 * dy, uy = q2 * dx + q3 * dy;  // corner (x0, y0)
        if (cx < x0 && edge(ux, uy, e2x, e2y, i2)) return true;                  // left edge
        if (cx > x1 && edge(ux + e1x, uy + e1y, e2x, e2y, i2)) return true;      // right edge
        if (cy < y0 && edge(ux, uy, e1x, e1y, i1)) return true;                  // top edge
        if (cy > y1 && edge(ux + e2x, uy + e2y, e1x, e1y, i1)) return true;      // bottom edge
        return cx >= x0 && cx <= x1 && cy >= y0 && cy <= y1;                     // centre inside
    }
};

// A splat's tiles as the binning stores them: {x0 | y0 << 16, w | h << 16, kept-tile mask,
// count}.  The footprint is convex and its box meets every tile of the rectangle, so only the
// corner tiles of a rectangle (up to 16 tiles) can miss it; the mask (bit ty·w + tx) drops those
// that do, and is 0 when the whole rectangle is kept.
__device__ __forceinline__ uint4 splat_tile_info(const float4 a, const float4 q, const float4 c, uint32_t tiles_x,
                                                 uint32_t tiles_y, uint32_t mode, float std2) {
    uint32_t x0 = 0, y0 = 0, w = 0, h = 0, mask = 0, cnt = 0;
    if (tile_rect(a, tiles_x, tiles_y, &x0, &y0, &w, &h)) {
        cnt = w * h;
        if (mode != GS_DISPLAY_POINT && cnt > 1 && cnt <= 16) {
            const float r2 =
                (mode == GS_DISPLAY_SPLAT) ? splat_r2_bound(c.w, splat_colour_reach(c.x, c.y, c.z), std2) : std2;
            const TileCull cull(a, q, r2);
            mask = cnt == 16 ? 0xFFFFu : (1u << cnt) - 1u;
#pragma unroll
            for (uint32_t corner = 0; corner < 4; ++corner) {
                const uint32_t tx = (corner & 1u) ? w - 1 : 0u, ty = (corner & 2u) ? h - 1 : 0u;
                if (((corner & 1u) && w == 1) || ((corner & 2u) && h == 1)) continue;  // same tile again
                if (!cull.meets((float)((x0 + tx) * GS_TILE) + 0.5f, (float)((y0 + ty) * GS_TILE) + 0.5f))
                    mask &= ~(1u << (ty * w + tx));
            }
            cnt = __popc(mask);
        }
    }
    return make_uint4(x0 | (y0 << 16), w | (h << 16), mask, cnt);
}

// Scratch carving: 256-byte aligned sub-allocations.
__host__ __device__ __forceinline__ size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

}  // namespace gs
