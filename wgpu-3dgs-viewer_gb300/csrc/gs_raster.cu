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
// Fragments whose alpha cannot move an 8-bit channel (alpha <= 1/512) lie outside the splat's
// fragment box and are never visited; skipping them leaves every pixel bit-identical.
#include <cstdlib>

#include "gs_internal.h"

namespace gs {

constexpr uint32_t kBinThreads = 256;
constexpr uint32_t kRasterThreads = 256;

struct RasterLayout {
    Ctrl *ctrl;
    gs_splat *sorted;    // draw-ordered splats, capacity max_splats
    uint64_t *flags;     // bin look-back flags, ceil(max_splats / 256)
    uint2 *pairs;        // (tile, draw rank), capacity max_pairs
    uint2 *ranges;       // per tile [start, end)
    void *sort_scratch;
    uint32_t tiles_x, tiles_y, ntiles, key_bits;
};

static uint32_t bits_for(uint32_t v) {
    uint32_t b = 1;
    while (b < 32 && (v >> b) != 0) ++b;
    return b;
}

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
    L.sorted = reinterpret_cast<gs_splat *>(p);
    p += align_up((size_t)max_splats * sizeof(gs_splat), 256);
    L.flags = reinterpret_cast<uint64_t *>(p);
    p += align_up(((size_t)max_splats + kBinThreads - 1) / kBinThreads * 8 + 8, 256);
    L.pairs = reinterpret_cast<uint2 *>(p);
    p += align_up((size_t)max_pairs * 8, 256);
    L.ranges = reinterpret_cast<uint2 *>(p);
    p += align_up((size_t)L.ntiles * sizeof(uint2), 256);
    L.sort_scratch = p;
    return L;
}

size_t raster_scratch_bytes(uint32_t max_splats, uint32_t w, uint32_t h, uint32_t max_pairs) {
    const uint32_t tiles = ((w + GS_TILE - 1) / GS_TILE) * ((h + GS_TILE - 1) / GS_TILE);
    const uint32_t key_bits = bits_for(tiles > 0 ? tiles - 1 : 0);
    return align_up(sizeof(Ctrl), 256) + align_up((size_t)max_splats * sizeof(gs_splat), 256) +
           align_up(((size_t)max_splats + kBinThreads - 1) / kBinThreads * 8 + 8, 256) +
           align_up((size_t)max_pairs * 8, 256) + align_up((size_t)tiles * sizeof(uint2), 256) +
           sort_pairs_scratch_bytes(max_pairs, key_bits);
}

const Ctrl *raster_ctrl(const void *scratch) { return reinterpret_cast<const Ctrl *>(scratch); }

// Early-out knobs of the rasteriser (results are identical for any values): tiles with fewer
// list entries than `suffix_min` take the single pass; `eps` is the transmittance that ends the
// front-to-back walk.  Overridable for tuning by GS300_SUFFIX_MIN / GS300_SUFFIX_EPS.
struct RasterTuning {
    uint32_t suffix_min;
    float eps;
};

static RasterTuning raster_tuning() {
    RasterTuning r{2048u, 1e-6f};
    if (const char *v = getenv("GS300_SUFFIX_MIN")) r.suffix_min = (uint32_t)strtoul(v, nullptr, 10);
    if (const char *v = getenv("GS300_SUFFIX_EPS")) r.eps = strtof(v, nullptr);
    return r;
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

// K3: gather into draw order + count tiles + scan + emit (tile, rank) pairs.
__global__ void __launch_bounds__(kBinThreads) bin_kernel(
    const gs_splat *__restrict__ splats, const uint32_t *__restrict__ sorted_index, const uint32_t *count,
    uint32_t max_count, uint32_t rank_offset, gs_splat *__restrict__ sorted_out, uint2 *__restrict__ pairs,
    uint32_t max_pairs, uint32_t tiles_x, uint32_t tiles_y, Ctrl *ctrl, uint64_t *flags, Ctrl *sort_ctrl,
    uint32_t key_passes) {
    __shared__ uint32_t s_incl[kBinThreads];
    __shared__ uint32_t s_x0[kBinThreads], s_y0[kBinThreads], s_w[kBinThreads];
    __shared__ uint32_t s_tmp[kBinThreads / 32];
    __shared__ uint32_t s_tile, s_epoch, s_base, s_seg_base, s_seg_want;
    __shared__ uint32_t s_hist[4][256];  // digit histograms of the emitted tile ids (tile sort)
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    for (uint32_t i = tid; i < 4 * 256; i += kBinThreads) (&s_hist[0][0])[i] = 0u;
    if (tid == 0) {
        s_epoch = *(volatile uint32_t *)&ctrl->epoch;
        s_seg_base = *(volatile uint32_t *)&ctrl->pair_base;
        s_seg_want = *(volatile uint32_t *)&ctrl->total;
        s_tile = atomicAdd(&ctrl->ticket[0], 1u);
    }
    __syncthreads();
    const uint32_t n = count ? min(*count, max_count) : max_count;
    const uint32_t ntiles = (n + kBinThreads - 1) / kBinThreads;
    const uint32_t tile = s_tile, epoch = s_epoch;
    if (tile >= ntiles) return;
    const uint32_t k = tile * kBinThreads + tid;
    uint32_t cnt = 0, x0 = 0, y0 = 0, w = 0, h = 0;
    // Indices come from the depth sort; the bound check only matters if that sort timed out.
    const uint32_t gi = k < n ? sorted_index[k] : 0xFFFFFFFFu;
    if (gi < max_count) {
        const float4 *src = reinterpret_cast<const float4 *>(splats + gi);
        const float4 a = __ldg(src), b = __ldg(src + 1), c = __ldg(src + 2);
        float4 *dst = reinterpret_cast<float4 *>(sorted_out + rank_offset + k);
        dst[0] = a;
        dst[1] = b;
        dst[2] = c;
        if (tile_rect(a, tiles_x, tiles_y, &x0, &y0, &w, &h)) cnt = w * h;
    }
    // Block inclusive scan of the tile counts.
    uint32_t x = cnt;
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_tmp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t run = 0, mine = 0;
        for (uint32_t i = 0; i < kBinThreads / 32; ++i) {
            const uint32_t c = s_tmp[i];
            if (lane == i) mine = run;
            run += c;
        }
        const uint32_t total = run;
        if (lane == 0)
            st_release(flags + tile, pack_flag(epoch, tile == 0 ? kFlagPrefix : kFlagAggregate, total));
        const uint32_t prefix = tile == 0 ? 0u : look_back_warp(flags, tile, epoch, &ctrl->status);
        __syncwarp();
        if (lane < kBinThreads / 32) s_tmp[lane] = mine;
        if (lane == 0) {
            if (tile > 0) {
                const uint64_t incl = (uint64_t)prefix + total;
                st_release(flags + tile,
                           pack_flag(epoch, kFlagPrefix, incl > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)incl));
            }
            s_base = prefix;
            if (tile == ntiles - 1) {
                const uint64_t want = (uint64_t)s_seg_want + prefix + total;
                const uint32_t kept = want > max_pairs ? max_pairs : (uint32_t)want;
                if (want > max_pairs) atomicOr(&ctrl->status, kStatusCapacity);
                ctrl->total = want > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)want;
                ctrl->count = kept;
                ctrl->pair_base = kept;
            }
        }
    }
    __syncthreads();
    const uint32_t incl = s_tmp[warp] + x;
    s_incl[tid] = incl;
    s_x0[tid] = x0;
    s_y0[tid] = y0;
    s_w[tid] = w;
    __syncthreads();
    const uint32_t block_pairs = s_incl[kBinThreads - 1];
    const uint64_t out0 = (uint64_t)s_seg_base + s_base;
    // Load-balanced emission: pair j of the block belongs to the first thread whose
    // inclusive count exceeds j.
    for (uint32_t j = tid; j < block_pairs; j += kBinThreads) {
        uint32_t lo = 0, hi = kBinThreads - 1;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (s_incl[mid] > j) hi = mid; else lo = mid + 1;
        }
        const uint32_t owner = lo;
        const uint32_t excl = owner ? s_incl[owner - 1] : 0u;
        const uint32_t r = j - excl;
        const uint32_t ww = s_w[owner];
        const uint32_t tyy = s_y0[owner] + r / ww, txx = s_x0[owner] + r % ww;
        const uint64_t o = out0 + j;
        if (o < max_pairs) {
            const uint32_t t = tyy * tiles_x + txx;
            pairs[o] = make_uint2(t, rank_offset + tile * kBinThreads + owner);
            for (uint32_t p = 0; p < key_passes; ++p) atomicAdd(&s_hist[p][(t >> (8u * p)) & 255u], 1u);
        }
    }
    __syncthreads();
    for (uint32_t p = 0; p < key_passes; ++p) {
        const uint32_t v = s_hist[p][tid];
        if (v) atomicAdd(&sort_ctrl->hist[p][tid], v);
    }
}

__global__ void tile_ranges_kernel(const uint2 *__restrict__ pairs, const Ctrl *ctrl, uint2 *ranges,
                                   uint32_t ntiles) {
    const uint32_t n = ctrl->count;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const uint32_t t = pairs[p].x;
        if (t >= ntiles) continue;
        if (p == 0 || pairs[p - 1].x != t) ranges[t].x = p;
        if (p == n - 1 || pairs[p + 1].x != t) ranges[t].y = p + 1;
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
__device__ __forceinline__ float blend8(float d, float om, float s_alpha) { return rint_small(fmaf(d, om, s_alpha)); }

struct RasterShared {
    float4 a[kRasterThreads];    // cx, cy, r² limit, alpha
    float4 b[kRasterThreads];    // q (or the point half sides)
    float4 c[kRasterThreads];    // s255.rgb
    float4 box[kRasterThreads];  // fragment box in pixel-centre coordinates
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
        const float lim = (MODE == GS_DISPLAY_SPLAT) ? splat_r2_bound(c.w, std2) : std2;
        S.a[tid] = make_float4(a.x, a.y, lim, c.w);
        S.b[tid] = b;
        S.c[tid] = c;
        S.box[tid] = make_float4(a.x - a.z, a.x + a.z, a.y - a.w, a.y + a.w);
    }
}

// The calling warp's list of staged entries whose box meets its pixel block, in draw order.
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
template <uint32_t MODE, bool PORTABLE_EXP>
__global__ void __launch_bounds__(kRasterThreads) raster_kernel(
    const gs_splat *__restrict__ sorted, const uint2 *__restrict__ pairs, const uint2 *__restrict__ ranges,
    uint8_t *__restrict__ target, uint32_t W, uint32_t H, uint32_t pitch, uint32_t tiles_x, float std2,
    float outline2, uint32_t max_splats, uint32_t suffix_min, float eps) {
    __shared__ RasterShared S;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
    const uint2 range = ranges[blockIdx.x];
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
            const uint32_t nl = compact_chunk(S, cnt, bx0, bx1, by0, by1);
            for (uint32_t i = 0; i < nl; ++i) {
                const uint32_t j = S.list[warp][i];
                float al;
                if (!fragment<MODE, PORTABLE_EXP>(S.a[j], S.b[j], pxc, pyc, outline2, &al)) continue;
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
                const uint32_t nl = compact_chunk(S, cnt, bx0, bx1, by0, by1);
                for (int i = (int)nl - 1; i >= 0; --i) {
                    if (__all_sync(0xFFFFFFFFu, found)) break;
                    const uint32_t j = S.list[warp][i];
                    float al;
                    if (!found && fragment<MODE, PORTABLE_EXP>(S.a[j], S.b[j], pxc, pyc, outline2, &al)) {
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
                if (__any_sync(0xFFFFFFFFu, active)) {
                    const uint32_t nl = compact_chunk(S, cnt, bx0, bx1, by0, by1);
                    for (uint32_t i = 0; i < nl; ++i) {
                        const uint32_t j = S.list[warp][i];
                        float al;
                        if (!active || base + j < k) continue;
                        if (!fragment<MODE, PORTABLE_EXP>(S.a[j], S.b[j], pxc, pyc, outline2, &al)) continue;
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
}

template <uint32_t MODE>
static void launch_raster_mode(const RasterLayout &L, uint8_t *target, uint32_t W, uint32_t H, uint32_t pitch,
                               float std2, float outline2, int exact, uint32_t max_splats, cudaStream_t st) {
    const RasterTuning t = raster_tuning();
    if (exact)
        raster_kernel<MODE, true><<<L.ntiles, kRasterThreads, 0, st>>>(
            L.sorted, L.pairs, L.ranges, target, W, H, pitch, L.tiles_x, std2, outline2, max_splats, t.suffix_min, t.eps);
    else
        raster_kernel<MODE, false><<<L.ntiles, kRasterThreads, 0, st>>>(
            L.sorted, L.pairs, L.ranges, target, W, H, pitch, L.tiles_x, std2, outline2, max_splats, t.suffix_min, t.eps);
}

cudaError_t launch_raster(const RasterSegment *segs, uint32_t nseg, const gs_frame_uniforms &u, uint8_t *target,
                          uint32_t W, uint32_t H, uint32_t pitch, uint32_t max_pairs, void *scratch, int exact_exp,
                          cudaStream_t st) {
    uint32_t max_splats = 0;
    for (uint32_t s = 0; s < nseg; ++s) max_splats += segs[s].max_count;
    const RasterLayout L = raster_layout(scratch, max_splats, W, H, max_pairs);
    if (L.ntiles == 0) return cudaSuccess;
    ctrl_init_kernel<<<1, 256, 0, st>>>(L.ctrl, 1);
    count_launches(1);
    cudaError_t e = sort_pairs_begin(L.sort_scratch, st);
    if (e != cudaSuccess) return e;
    Ctrl *sort_ctrl = sort_pairs_ctrl(L.sort_scratch);
    const uint32_t key_passes = (L.key_bits + 7u) / 8u;
    uint32_t rank_offset = 0;
    prof_mark(kProfBin, true, st);
    for (uint32_t s = 0; s < nseg; ++s) {
        if (s > 0) {
            ctrl_init_kernel<<<1, 32, 0, st>>>(L.ctrl, 0);
            count_launches(1);
        }
        const uint32_t blocks = (segs[s].max_count + kBinThreads - 1) / kBinThreads;
        if (blocks > 0) {
            bin_kernel<<<blocks, kBinThreads, 0, st>>>(segs[s].splats, segs[s].sorted_index, segs[s].count,
                                                       segs[s].max_count, rank_offset, L.sorted, L.pairs, max_pairs,
                                                       L.tiles_x, L.tiles_y, L.ctrl, L.flags, sort_ctrl, key_passes);
            count_launches(1);
        }
        rank_offset += segs[s].max_count;
    }
    prof_mark(kProfBin, false, st);
    prof_mark(kProfTileSort, true, st);
    e = launch_sort_pairs(L.pairs, max_pairs, &L.ctrl->count, L.key_bits, L.sort_scratch, st);
    prof_mark(kProfTileSort, false, st);
    if (e != cudaSuccess) return e;
    merge_status_kernel<<<1, 1, 0, st>>>(L.ctrl, sort_ctrl);
    count_launches(1);
    e = cudaMemsetAsync(L.ranges, 0, (size_t)L.ntiles * sizeof(uint2), st);
    if (e != cudaSuccess) return e;
    uint32_t rblocks = (max_pairs + 255) / 256;
    if (rblocks > 152 * 8) rblocks = 152 * 8;
    if (rblocks == 0) rblocks = 1;
    prof_mark(kProfRanges, true, st);
    tile_ranges_kernel<<<rblocks, 256, 0, st>>>(L.pairs, L.ctrl, L.ranges, L.ntiles);
    prof_mark(kProfRanges, false, st);
    count_launches(1);
    const float std2 = u.std_dev * u.std_dev;
    const float o = u.std_dev - 0.1f;
    const float outline2 = o * o;
    prof_mark(kProfRaster, true, st);
    count_launches(1);
    switch (u.display_mode) {
        case GS_DISPLAY_SPLAT:
            launch_raster_mode<GS_DISPLAY_SPLAT>(L, target, W, H, pitch, std2, outline2, exact_exp, max_splats, st);
            break;
        case GS_DISPLAY_ELLIPSE:
            launch_raster_mode<GS_DISPLAY_ELLIPSE>(L, target, W, H, pitch, std2, outline2, exact_exp, max_splats, st);
            break;
        default:
            launch_raster_mode<GS_DISPLAY_POINT>(L, target, W, H, pitch, std2, outline2, exact_exp, max_splats, st);
            break;
    }
    prof_mark(kProfRaster, false, st);
    return cudaGetLastError();
}

}  // namespace gs
