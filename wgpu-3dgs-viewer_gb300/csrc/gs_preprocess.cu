// gs_preprocess.cu — K1: fused preprocess (cull, depth key, order-preserving compaction,
// screen-space splat: 2D axes -> pixel-to-quad map, SH colour).
//
// Restates src/shader/preprocess.wesl:52-126 (pre / main / post) and moves the per-instance
// vertex work of src/shader/render.wesl:75-130 (cov2d_axes, view colour, quad geometry) here,
// once per Gaussian instead of six times per splat.  Compiled with -fmad=false: every FP32
// multiply and add rounds on its own, in the order of the CPU oracle (oracle/gs_oracle.cpp).
//
// Layout: a CTA owns 128 consecutive Gaussians and stages their records in shared memory, one
// record per row: FP32 records (224 B) with a single cp.async.bulk copy completing on an
// mbarrier; half records (128 B) with coalesced 16-byte cp.async copies into rows padded to
// 144 B.  Every thread reads its own row with 128-bit shared loads, so the 8 rows a quarter-warp
// touches meet at most 2 to a bank (224-byte rows) or not at all (144-byte rows); dense
// 128-byte rows would put a whole quarter-warp on one bank.  Visible Gaussians are compacted in ascending index
// order with a warp ballot, a block scan and a decoupled look-back across CTAs (tile = CTA
// index: CTAs are dispatched in index order, so a CTA only ever waits for CTAs already resident
// or finished; every wait is bounded all the same).
#include "gs_internal.h"

namespace gs {

constexpr uint32_t kPreThreads = 128;

struct PreParams {
    gs_frame_uniforms u;
    const gs_frame_uniforms *u_dev;  // when set (graph-captured batches), uniforms are read here
    const uint8_t *records;
    uint32_t n;
    uint32_t ntiles;
    const uint32_t *selection;
    uint32_t invert;
    uint32_t *indirect;
    uint32_t *dispatch;
    uint32_t *indices;
    float *depths;
    uint32_t depth_cap;
    gs_splat *splats;
    uint4 *binfo;  // optional: each visible splat's tiles (splat_tile_info) for the viewport's tiles
    uint32_t tiles_x, tiles_y;
    Ctrl *ctrl;
    uint64_t *flags;
};

struct PreViewsParams {
    const uint8_t *records;
    uint32_t n;
    uint32_t ntiles;
    const uint32_t *selection;
    uint32_t invert;
    const PreView *views;  // device array of nviews
    uint32_t nviews;
    Ctrl *group;           // status of the record staging
};

// ---- FP32 math in the oracle's evaluation order ------------------------------------------
__device__ __forceinline__ void mat4_vec(const float *m, const float *v, float *o) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        float s = m[0 * 4 + r] * v[0];
        s = s + m[1 * 4 + r] * v[1];
        s = s + m[2 * 4 + r] * v[2];
        s = s + m[3 * 4 + r] * v[3];
        o[r] = s;
    }
}

__device__ __forceinline__ void mat3_vec(const float *m, const float *v, float *o) {
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        float s = m[0 * 3 + r] * v[0];
        s = s + m[1 * 3 + r] * v[1];
        s = s + m[2 * 3 + r] * v[2];
        o[r] = s;
    }
}

__device__ __forceinline__ float minf_wgsl(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float clamp01(float v) { return v > 0.0f ? (v < 1.0f ? v : 1.0f) : 0.0f; }
__device__ __forceinline__ float len2(float x, float y) { return sqrtf(x * x + y * y); }
__device__ __forceinline__ bool cull(float x, float y, float z) {
    return !(x >= -1.0f && y >= -1.0f && z >= 0.0f && x <= 1.0f && y <= 1.0f && z <= 1.0f);
}

// Record staged in a padded shared-memory row (16-byte chunks), with the fields every visible
// Gaussian needs unpacked to FP32.  SH coefficients stay in the row until the colour pass.
struct Rec {
    float pos[3];
    uint32_t color;
    const uint4 *row;
    float cov3d[6];
};

template <uint32_t FMT>
__device__ __forceinline__ float sh_decode(uint32_t bits) {
    if constexpr (FMT == GS_FORMAT_FP32) {
        return __uint_as_float(bits);
    } else if constexpr (FMT == GS_FORMAT_HALF_SH_FP16) {
        return __half2float(__ushort_as_half((unsigned short)bits));
    } else {
        return __uint_as_float(bits << 16);
    }
}

// SH coefficients [K0, K1) of the row into out[0 .. K1-K0), read as the few 16-byte chunks
// that hold them.  Coefficient k sits at byte 16 + 4k (FP32 record) or 30 + 2k (half record).
template <uint32_t FMT, int K0, int K1>
__device__ __forceinline__ void sh_load(const uint4 *row, float *out) {
    constexpr int B = (FMT == GS_FORMAT_FP32) ? 4 : 2;
    constexpr int OFF = (FMT == GS_FORMAT_FP32) ? 16 : 30;
    constexpr int C0 = (OFF + K0 * B) / 16, C1 = (OFF + K1 * B - 1) / 16;
    uint32_t w[(C1 - C0 + 1) * 4];
#pragma unroll
    for (int c = C0; c <= C1; ++c) {
        const uint4 v = row[c];
        w[(c - C0) * 4 + 0] = v.x;
        w[(c - C0) * 4 + 1] = v.y;
        w[(c - C0) * 4 + 2] = v.z;
        w[(c - C0) * 4 + 3] = v.w;
    }
#pragma unroll
    for (int k = K0; k < K1; ++k) {
        const int byte = OFF + k * B - C0 * 16;
        uint32_t bits = w[byte >> 2];
        if (B == 2) bits = (byte & 2) ? (bits >> 16) : (bits & 0xFFFFu);
        out[k - K0] = sh_decode<FMT>(bits);
    }
}

__device__ __forceinline__ void quat_to_mat3(const float *q, float *m) {
    const float x = q[0], y = q[1], z = q[2], w = q[3];
    const float x2 = x + x, y2 = y + y, z2 = z + z;
    const float xx = x * x2, xy = x * y2, xz = x * z2;
    const float yy = y * y2, yz = y * z2, zz = z * z2;
    const float wx = w * x2, wy = w * y2, wz = w * z2;
    m[0] = 1.0f - (yy + zz);
    m[1] = xy + wz;
    m[2] = xz - wy;
    m[3] = xy - wz;
    m[4] = 1.0f - (xx + zz);
    m[5] = yz + wx;
    m[6] = xz + wy;
    m[7] = yz - wx;
    m[8] = 1.0f - (xx + yy);
}

template <uint32_t FMT>
__device__ __forceinline__ Rec load_rec(const uint4 *row) {
    Rec g;
    const uint4 head = row[0];
    g.pos[0] = __uint_as_float(head.x);
    g.pos[1] = __uint_as_float(head.y);
    g.pos[2] = __uint_as_float(head.z);
    g.color = head.w;
    g.row = row;
    if constexpr (FMT == GS_FORMAT_FP32) {
        // cov3d occupies bytes 196..219: chunk 12 (.y .z .w) and chunk 13 (.x .y .z)
        const uint4 c12 = row[12], c13 = row[13];
        g.cov3d[0] = __uint_as_float(c12.y);
        g.cov3d[1] = __uint_as_float(c12.z);
        g.cov3d[2] = __uint_as_float(c12.w);
        g.cov3d[3] = __uint_as_float(c13.x);
        g.cov3d[4] = __uint_as_float(c13.y);
        g.cov3d[5] = __uint_as_float(c13.z);
    } else {
        // rot[4] at bytes 16..23, scale[3] at bytes 24..29 (chunk 1)
        const uint4 c1 = row[1];
        const uint16_t rot[4] = {(uint16_t)(c1.x & 0xFFFFu), (uint16_t)(c1.x >> 16), (uint16_t)(c1.y & 0xFFFFu),
                                 (uint16_t)(c1.y >> 16)};
        const uint16_t scale[3] = {(uint16_t)(c1.z & 0xFFFFu), (uint16_t)(c1.z >> 16), (uint16_t)(c1.w & 0xFFFFu)};
        float q[4], sc[3];
#pragma unroll
        for (int k = 0; k < 4; ++k) q[k] = __half2float(__ushort_as_half(rot[k]));
#pragma unroll
        for (int k = 0; k < 3; ++k) sc[k] = __half2float(__ushort_as_half(scale[k]));
        const float nrm = sqrtf(((q[0] * q[0] + q[1] * q[1]) + q[2] * q[2]) + q[3] * q[3]);
#pragma unroll
        for (int k = 0; k < 4; ++k) q[k] = q[k] / nrm;
        float R[9], M[9];
        quat_to_mat3(q, R);
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int r = 0; r < 3; ++r) M[c * 3 + r] = R[c * 3 + r] * sc[c];
        auto cv = [&](int a, int b) {
            float acc = M[0 * 3 + a] * M[0 * 3 + b];
            acc = acc + M[1 * 3 + a] * M[1 * 3 + b];
            acc = acc + M[2 * 3 + a] * M[2 * 3 + b];
            return acc;
        };
        g.cov3d[0] = cv(0, 0);
        g.cov3d[1] = cv(0, 1);
        g.cov3d[2] = cv(0, 2);
        g.cov3d[3] = cv(1, 1);
        g.cov3d[4] = cv(1, 2);
        g.cov3d[5] = cv(2, 2);
    }
    return g;
}

// cov2d (utils.wesl:25-48) + cov2d_axes (utils.wesl:54-79): (major.xy, minor.xy).
__device__ __forceinline__ void cov2d_axes(const gs_frame_uniforms &u, const float *c,
                                           const float *p4, float std_dev, float *axes) {
    float t[4];
    mat4_vec(u.vm, p4, t);
    const float fx = u.focal[0], fy = u.focal[1];
    const float tz2 = t[2] * t[2];
    const float j00 = fx / t[2];
    const float j02 = -(fx * t[0]) / tz2;
    const float j11 = fy / t[2];
    const float j12 = -(fy * t[1]) / tz2;
    const float *w = u.wsr;
    float T0[3], T1[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        T0[k] = j00 * w[k * 3 + 0] + j02 * w[k * 3 + 2];
        T1[k] = j11 * w[k * 3 + 1] + j12 * w[k * 3 + 2];
    }
    const float V[9] = {c[0], c[1], c[2], c[1], c[3], c[4], c[2], c[4], c[5]};
    float U0[3], U1[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        U0[k] = (T0[0] * V[k * 3 + 0] + T0[1] * V[k * 3 + 1]) + T0[2] * V[k * 3 + 2];
        U1[k] = (T1[0] * V[k * 3 + 0] + T1[1] * V[k * 3 + 1]) + T1[2] * V[k * 3 + 2];
    }
    const float a = (U0[0] * T0[0] + U0[1] * T0[1]) + U0[2] * T0[2];
    const float b = (U0[0] * T1[0] + U0[1] * T1[1]) + U0[2] * T1[2];
    const float cc = (U1[0] * T1[0] + U1[1] * T1[1]) + U1[2] * T1[2];
    const float mid = 0.5f * (a + cc);
    const float h = 0.5f * (a - cc);
    const float radius = len2(h, b);
    const float lmaj = mid + radius;
    const float lmin = mid - radius;
    if (lmin < 0.0f) {
        axes[0] = axes[1] = axes[2] = axes[3] = 0.0f;
        return;
    }
    const float dx = b, dy = lmaj - a;
    float dirx, diry;
    if (dx == 0.0f && dy == 0.0f) {
        dirx = 0.0f;
        diry = 1.0f;
    } else {
        const float l = len2(dx, dy);
        dirx = dx / l;
        diry = dy / l;
    }
    const float majl = minf_wgsl(std_dev * sqrtf(lmaj), 1024.0f);
    const float minl = minf_wgsl(std_dev * sqrtf(lmin), 1024.0f);
    axes[0] = majl * dirx;
    axes[1] = majl * diry;
    axes[2] = minl * diry;
    axes[3] = minl * -dirx;
}

// view_color (utils.wesl:82-135) with the direction of render.wesl:58-73.
template <uint32_t FMT>
__device__ __forceinline__ void view_color(const gs_frame_uniforms &u, const Rec &g,
                                           const float *world, float *rgba) {
    const float vd[3] = {u.cam_pos[0] - world[0], u.cam_pos[1] - world[1], u.cam_pos[2] - world[2]};
    float mvd[3];
    mat3_vec(u.inv_sr, vd, mvd);
    const float l = sqrtf((mvd[0] * mvd[0] + mvd[1] * mvd[1]) + mvd[2] * mvd[2]);
    const float x = -(mvd[0] / l), y = -(mvd[1] / l), z = -(mvd[2] / l);
    const float c1 = 0.4886025f;
    float res[3];
#pragma unroll
    for (int ch = 0; ch < 3; ++ch)
        res[ch] = u.no_sh0 ? 0.5f : (float)((g.color >> (8 * ch)) & 0xFFu) / 255.0f;
    if (u.sh_deg >= 1) {
        float s1[9];
        sh_load<FMT, 0, 9>(g.row, s1);
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) {
            float v = (-s1[0 * 3 + ch]) * y + s1[1 * 3 + ch] * z;
            v = v - s1[2 * 3 + ch] * x;
            res[ch] = res[ch] + c1 * v;
        }
        if (u.sh_deg >= 2) {
            float s2[15];
            sh_load<FMT, 9, 24>(g.row, s2);
            const float xx = x * x, yy = y * y, zz = z * z;
            const float xy = x * y, yz = y * z, xz = x * z;
            const float k0 = 1.0925484f * xy, k1 = -1.0925484f * yz;
            const float k2 = 0.3153916f * ((2.0f * zz - xx) - yy);
            const float k3 = -1.0925484f * xz, k4 = 0.5462742f * (xx - yy);
#pragma unroll
            for (int ch = 0; ch < 3; ++ch) {
                float v = k0 * s2[0 * 3 + ch] + k1 * s2[1 * 3 + ch];
                v = v + k2 * s2[2 * 3 + ch];
                v = v + k3 * s2[3 * 3 + ch];
                v = v + k4 * s2[4 * 3 + ch];
                res[ch] = res[ch] + v;
            }
            if (u.sh_deg >= 3) {
                float s3[21];
                sh_load<FMT, 24, 45>(g.row, s3);
                const float m0 = (-0.5900436f * y) * (3.0f * xx - yy);
                const float m1 = (2.8906114f * xy) * z;
                const float m2 = (-0.4570458f * y) * ((4.0f * zz - xx) - yy);
                const float m3 = (0.3731763f * z) * ((2.0f * zz - 3.0f * xx) - 3.0f * yy);
                const float m4 = (-0.4570458f * x) * ((4.0f * zz - xx) - yy);
                const float m5 = (1.4453057f * z) * (xx - yy);
                const float m6 = (-0.5900436f * x) * (xx - 3.0f * yy);
#pragma unroll
                for (int ch = 0; ch < 3; ++ch) {
                    float v = m0 * s3[0 * 3 + ch] + m1 * s3[1 * 3 + ch];
                    v = v + m2 * s3[2 * 3 + ch];
                    v = v + m3 * s3[3 * 3 + ch];
                    v = v + m4 * s3[4 * 3 + ch];
                    v = v + m5 * s3[5 * 3 + ch];
                    v = v + m6 * s3[6 * 3 + ch];
                    res[ch] = res[ch] + v;
                }
            }
        }
    }
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) rgba[ch] = res[ch] > 0.0f ? res[ch] : 0.0f;
    rgba[3] = (float)((g.color >> 24) & 0xFFu) / 255.0f;
}

// ---- per Gaussian and view -------------------------------------------------------------------
// Projection state of one Gaussian in one view, carried from the cull to the splat record.
struct Proj {
    float nx, ny, world[4], axes[4];
    bool have_axes;
};

// `main` (preprocess.wesl:60-106): NDC cull, then the bound cull along the major axis for
// centres outside the frustum.  Returns visibility; *key = 1 - ndc.z.
__device__ __forceinline__ bool gaussian_visible(const gs_frame_uniforms &u, const Rec &g, Proj &pr, float *key) {
    const float p4[4] = {g.pos[0], g.pos[1], g.pos[2], 1.0f};
    float clip[4];
    mat4_vec(u.model, p4, pr.world);
    mat4_vec(u.pv, pr.world, clip);
    pr.nx = clip[0] / clip[3];
    pr.ny = clip[1] / clip[3];
    const float nz = clip[2] / clip[3];
    pr.have_axes = false;
    bool vis = true;
    if (cull(pr.nx, pr.ny, nz)) {
        cov2d_axes(u, g.cov3d, p4, u.std_dev_scaled, pr.axes);
        pr.have_axes = true;
        const float mx = pr.axes[0] * u.std_dev / u.size[0];
        const float my = pr.axes[1] * u.std_dev / u.size[1];
        const float mlen = len2(mx, my);
        const float nl = len2(pr.nx, pr.ny);
        const float dx = -pr.nx / nl, dy = -pr.ny / nl;
        const float m = minf_wgsl(mlen, nl);
        if (cull(pr.nx + m * dx, pr.ny + m * dy, nz)) vis = false;
    }
    *key = 1.0f - nz;
    return vis;
}

// Per-instance vertex work (render.wesl:75-130): the splat record of a visible Gaussian.
// With `binfo`, also the splat's tiles for a tiles_x x tiles_y grid, as the binning works them out.
template <uint32_t FMT>
__device__ __forceinline__ void write_splat(const gs_frame_uniforms &u, const Rec &g, Proj &pr, gs_splat *out,
                                            uint4 *binfo = nullptr, uint32_t tiles_x = 0, uint32_t tiles_y = 0) {
    float rgba[4];
    view_color<FMT>(u, g, pr.world, rgba);
    const float W = u.viewport[0], H = u.viewport[1];
    const float cx = ((pr.nx + 1.0f) * W) * 0.5f;
    const float cy = ((1.0f - pr.ny) * H) * 0.5f;
    float q0, q1, q2, q3, ex, ey;
    const float std2 = u.std_dev * u.std_dev;
    const float p4[4] = {g.pos[0], g.pos[1], g.pos[2], 1.0f};
    if (u.display_mode == GS_DISPLAY_POINT) {
        float vp[4];
        mat4_vec(u.vm, p4, vp);
        const float l = sqrtf((vp[0] * vp[0] + vp[1] * vp[1]) + vp[2] * vp[2]);
        const float aspect = u.size[1] / u.size[0];
        const float pnd = (0.01f * u.point_size) / l;
        const float hx = (pnd * aspect) * (0.5f * W);
        const float hy = pnd * (0.5f * H);
        q0 = hx;
        q1 = hy;
        q2 = 0.0f;
        q3 = 0.0f;
        if (hx > 0.0f && hy > 0.0f && hx < 1e30f && hy < 1e30f) {
            ex = hx * 1.001f + 0.01f;
            ey = hy * 1.001f + 0.01f;
        } else {
            ex = -1.0f;
            ey = -1.0f;
        }
    } else {
        if (!pr.have_axes) cov2d_axes(u, g.cov3d, p4, u.std_dev_scaled, pr.axes);
        const float *axes = pr.axes;
        const float kx = (0.5f * W) / u.size[0];
        const float ky = (0.5f * H) / u.size[1];
        const float a00 = axes[0] * kx, a01 = axes[2] * kx;
        const float a10 = -axes[1] * ky, a11 = -axes[3] * ky;
        const float det = a00 * a11 - a01 * a10;
        q0 = a11 / det;
        q1 = -a01 / det;
        q2 = -a10 / det;
        q3 = a00 / det;
        const float reach = splat_colour_reach(clamp01(rgba[0]) * 255.0f, clamp01(rgba[1]) * 255.0f,
                                               clamp01(rgba[2]) * 255.0f);
        const float r2 = (u.display_mode == GS_DISPLAY_SPLAT) ? splat_r2_bound(rgba[3], reach, std2) : std2;
        const bool ok = det != 0.0f && isfinite(det) && isfinite(q0) && isfinite(q1) && isfinite(q2) &&
                        isfinite(q3) && r2 >= 0.0f;
        if (ok) {
            ex = sqrtf(r2 * (a00 * a00 + a01 * a01)) * 1.001f + 0.01f;
            ey = sqrtf(r2 * (a10 * a10 + a11 * a11)) * 1.001f + 0.01f;
        } else {
            ex = -1.0f;
            ey = -1.0f;
        }
    }
    const float4 a = make_float4(cx, cy, ex, ey), q = make_float4(q0, q1, q2, q3);
    const float4 c =
        make_float4(clamp01(rgba[0]) * 255.0f, clamp01(rgba[1]) * 255.0f, clamp01(rgba[2]) * 255.0f, rgba[3]);
    float4 *sp = reinterpret_cast<float4 *>(out);
    sp[0] = a;
    sp[1] = q;
    sp[2] = c;
    if (binfo) *binfo = splat_tile_info(a, q, c, tiles_x, tiles_y, u.display_mode, std2);
}

// Selection (preprocess.wesl:68-78): a Gaussian takes part when its bit differs from `invert`.
__device__ __forceinline__ bool gaussian_selected(const uint32_t *selection, uint32_t invert, uint32_t i) {
    if (!selection) return true;
    const bool bit = (selection[i >> 5] >> (i & 31u)) & 1u;
    return (invert != 0u) != bit;
}

// ---- global -> shared staging: 16-byte cp.async chunks, or a bulk copy on an mbarrier -----
__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(bar);
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(bar);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
    const uint32_t b = (uint32_t)__cvta_generic_to_shared(bar);
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(d),
        "l"(src), "r"(bytes), "r"(b)
        : "memory");
}

// Bounded wait for phase `parity` of the barrier; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(bar);
    for (uint32_t i = 0; i < kSpinLimit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Tiles ahead of its own that a CTA asks L2 to fetch: about half a resident wave (152 SMs x 4
// of the 7 CTAs an SM holds), so the CTA that takes that tile later finds its records in L2 and
// DRAM keeps more reads in flight (about 17 MB of FP32 records, an eighth of L2).  Measured at
// 6M: 2, 3 and 4 x 152 tiles ahead equal (0.339 ms, 72 % of HBM, from 0.385 ms without), 8 x
// 152 0.345 ms, 14 x 152 0.483 ms (prefetched records evicted before use).
constexpr uint32_t kPrefetchTiles = 152 * 4;

// Records [first, first + cnt) into shared rows: FP32 records by one bulk copy on the mbarrier
// (phase 0, initialised by the caller before a __syncthreads), half records by 16-byte cp.async
// chunks into padded rows.  Returns with the rows visible to every thread of the CTA.
template <uint32_t FMT>
__device__ __forceinline__ void stage_records(uint4 *s_rec, uint64_t *s_bar, const uint8_t *records, uint32_t first,
                                              uint32_t cnt, uint32_t *status, uint32_t prefetch_n = 0) {
    constexpr uint32_t REC = (FMT == GS_FORMAT_FP32) ? 224u : 128u;
    constexpr uint32_t C16 = REC / 16;
    constexpr uint32_t ROW16 = (FMT == GS_FORMAT_FP32) ? C16 : C16 + 1;
    const uint32_t tid = threadIdx.x;
    if constexpr (FMT == GS_FORMAT_FP32) {
        if (tid == 0) {
            mbar_expect_tx(s_bar, cnt * REC);
            bulk_g2s(s_rec, records + (size_t)first * REC, cnt * REC, s_bar);
            if (prefetch_n > 0) prefetch_l2_bulk(records + (size_t)(first + kPrefetchTiles * kPreThreads) * REC, prefetch_n * REC);
        }
        if (!mbar_wait(s_bar, 0)) atomicOr(status, kStatusTimeout);
    } else {
        if (tid == 0 && prefetch_n > 0)
            prefetch_l2_bulk(records + (size_t)(first + kPrefetchTiles * kPreThreads) * REC, prefetch_n * REC);
        // consecutive threads copy consecutive 16-byte chunks (coalesced); chunk q of the CTA
        // is chunk q % C16 of record q / C16
        const uint4 *src = reinterpret_cast<const uint4 *>(records + (size_t)first * REC);
        const uint32_t chunks = cnt * C16;
#pragma unroll
        for (uint32_t k = 0; k < C16; ++k) {
            const uint32_t q = tid + k * kPreThreads;
            if (q < chunks) {
                const uint32_t r = q / C16;
                cp_async16(&s_rec[r * ROW16 + (q - r * C16)], src + q);
            }
        }
        cp_async_wait_all();
        __syncthreads();
    }
}

template <uint32_t FMT, bool DEV_UNIFORMS>
__global__ void __launch_bounds__(kPreThreads) preprocess_kernel(const __grid_constant__ PreParams P) {
    constexpr uint32_t REC = (FMT == GS_FORMAT_FP32) ? 224u : 128u;
    constexpr uint32_t C16 = REC / 16;  // 16-byte chunks per record
    // FP32 records: one bulk copy of the CTA's records into dense rows (a quarter-warp's 128-bit
    // reads of 224-byte rows meet at most 2 to a bank).  Half records: 16-byte cp.async chunks
    // into rows padded to 144 bytes (dense 128-byte rows would put a quarter-warp on one bank).
    constexpr bool BULK = (FMT == GS_FORMAT_FP32);
    constexpr uint32_t ROW16 = BULK ? C16 : C16 + 1;
    __shared__ __align__(16) uint4 s_rec[kPreThreads * ROW16];
    __shared__ __align__(8) uint64_t s_bar;
    __shared__ uint32_t s_tile, s_epoch, s_base, s_limit, s_stall, s_warp[kPreThreads / 32];
    __shared__ __align__(16) gs_frame_uniforms s_u;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    if constexpr (DEV_UNIFORMS) {
        const uint32_t *src = reinterpret_cast<const uint32_t *>(P.u_dev);
        for (uint32_t i = tid; i < sizeof(gs_frame_uniforms) / 4; i += kPreThreads)
            reinterpret_cast<uint32_t *>(&s_u)[i] = src[i];
    }
    const gs_frame_uniforms &u = DEV_UNIFORMS ? s_u : P.u;

    if (tid == 0) {
        s_epoch = *(volatile uint32_t *)&P.ctrl->epoch;
        s_limit = P.ctrl->spin_limit;
        s_stall = P.ctrl->stall_tile;
        s_tile = blockIdx.x;  // look-back predecessors are lower, earlier-dispatched CTAs
        if (BULK) mbar_init(&s_bar, 1);
    }
    __syncthreads();
    const uint32_t tile = s_tile, epoch = s_epoch;
    const uint32_t first = tile * kPreThreads;
    const uint32_t cnt = min(kPreThreads, P.n - first);
    const uint32_t ahead = tile + kPrefetchTiles;  // records of that tile: [ahead·128, +pcnt)
    const uint32_t pcnt = ahead < P.ntiles ? min(kPreThreads, P.n - ahead * kPreThreads) : 0u;
    stage_records<FMT>(s_rec, &s_bar, P.records, first, cnt, &P.ctrl->status, pcnt);

    const uint32_t i = first + tid;
    bool vis = false;
    float key = 0.0f;
    Proj pr;
    Rec g;
    if (tid < cnt && gaussian_selected(P.selection, P.invert, i)) {
        g = load_rec<FMT>(s_rec + tid * ROW16);
        vis = gaussian_visible(u, g, pr, &key);
    }

    // ---- order-preserving compaction: ballot + block scan; the CTA's count is published now
    // and its global offset is looked up after the vertex work, which hides the wait ----
    const uint32_t bal = __ballot_sync(0xFFFFFFFFu, vis);
    if (lane == 0) s_warp[warp] = __popc(bal);
    __syncthreads();
    if (tid == 0) {
        uint32_t run = 0;
        for (uint32_t w = 0; w < kPreThreads / 32; ++w) {
            const uint32_t c = s_warp[w];
            s_warp[w] = run;
            run += c;
        }
        s_base = run;  // block total until the look-back below
        publish_flag(P.flags + tile, tile, s_stall, pack_flag(epoch, tile == 0 ? kFlagPrefix : kFlagAggregate, run));
    }

    // ---- per-instance vertex work (render.wesl:75-130), written at the Gaussian's index ----
    if (vis && P.splats)
        write_splat<FMT>(u, g, pr, P.splats + i, P.binfo ? P.binfo + i : nullptr, P.tiles_x, P.tiles_y);

    // ---- global offset: warp 0 looks back over the predecessors' published counts ----
    __syncthreads();
    if (warp == 0) {
        const uint32_t total = s_base;
        const uint32_t prefix = tile == 0 ? 0u : look_back_warp(P.flags, tile, epoch, &P.ctrl->status, s_limit);
        if (lane == 0) {
            if (tile > 0) publish_flag(P.flags + tile, tile, s_stall, pack_flag(epoch, kFlagPrefix, prefix + total));
            s_base = prefix;
            if (tile == P.ntiles - 1) {
                // `post` (preprocess.wesl:108-126) and the DrawIndirectArgs instance count.
                const uint32_t v = prefix + total;
                P.ctrl->count = v;
                if (P.indirect) {
                    P.indirect[0] = 6u;
                    P.indirect[1] = v;
                    P.indirect[2] = 0u;
                    P.indirect[3] = 0u;
                }
                if (P.dispatch) {
                    P.dispatch[0] = (v + GS_SORT_BLOCK_KVS - 1) / GS_SORT_BLOCK_KVS;
                    P.dispatch[1] = 1u;
                    P.dispatch[2] = 1u;
                }
            }
        }
    }
    __syncthreads();
    if (tile == P.ntiles - 1) {
        const uint32_t v = min(P.ctrl->count, P.depth_cap);
        const uint32_t padded = min(((v + GS_SORT_BLOCK_KVS - 1) / GS_SORT_BLOCK_KVS) * GS_SORT_BLOCK_KVS, P.depth_cap);
        for (uint32_t k = v + tid; k < padded; k += kPreThreads) P.depths[k] = 2.0f;
    }
    if (vis) {
        // c < n unless a look-back gave up (status already set); never write past the buffers
        const uint32_t c = s_base + s_warp[warp] + __popc(bal & lanemask_lt());
        if (c < P.n) {
            P.indices[c] = i;
            P.depths[c] = key;
        } else {
            atomicOr(&P.ctrl->status, kStatusBounds);
        }
    }
}

// ---- several views of one model in one launch: the records are read once ------------------
// Each CTA stages its 128 records once and runs the per-Gaussian work for every view of the
// launch (each view with its own uniforms, outputs, control block and look-back flags).  Every
// view's tile count is published right after that view's ballot; the look-backs run only after
// all views are done, so predecessors have long published.  Per view the outputs are the ones
// preprocess_kernel writes for that view alone.
template <uint32_t FMT>
__global__ void __launch_bounds__(kPreThreads) preprocess_views_kernel(const __grid_constant__ PreViewsParams P) {
    constexpr uint32_t REC = (FMT == GS_FORMAT_FP32) ? 224u : 128u;
    constexpr uint32_t C16 = REC / 16;
    constexpr uint32_t ROW16 = (FMT == GS_FORMAT_FP32) ? C16 : C16 + 1;
    constexpr uint32_t NW = kPreThreads / 32;
    __shared__ __align__(16) uint4 s_rec[kPreThreads * ROW16];
    __shared__ __align__(8) uint64_t s_bar;
    __shared__ __align__(16) gs_frame_uniforms s_u;
    __shared__ float s_key[kPreMaxViews][kPreThreads];
    __shared__ uint32_t s_bal[kPreMaxViews][NW];
    __shared__ uint32_t s_base[kPreMaxViews];
    __shared__ uint32_t s_epoch[kPreMaxViews];
    __shared__ uint32_t s_tile, s_limit, s_stall;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t nv = P.nviews;
    if (tid == 0) {
        s_tile = blockIdx.x;  // look-back predecessors are lower, earlier-dispatched CTAs
        if (FMT == GS_FORMAT_FP32) mbar_init(&s_bar, 1);
    }
    if (tid < nv) s_epoch[tid] = *(volatile uint32_t *)&P.views[tid].ctrl->epoch;
    if (tid == 0) {
        s_limit = P.group->spin_limit;
        s_stall = P.group->stall_tile;
    }
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t first = tile * kPreThreads;
    const uint32_t cnt = min(kPreThreads, P.n - first);
    stage_records<FMT>(s_rec, &s_bar, P.records, first, cnt, &P.group->status);

    const uint32_t i = first + tid;
    const bool sel = tid < cnt && gaussian_selected(P.selection, P.invert, i);
    Rec g;
    if (sel) g = load_rec<FMT>(s_rec + tid * ROW16);

    for (uint32_t v = 0; v < nv; ++v) {
        const PreView &V = P.views[v];
        for (uint32_t k = tid; k < sizeof(gs_frame_uniforms) / 4; k += kPreThreads)
            reinterpret_cast<uint32_t *>(&s_u)[k] = reinterpret_cast<const uint32_t *>(V.u)[k];
        __syncthreads();
        bool vis = false;
        float key = 0.0f;
        Proj pr;
        if (sel) vis = gaussian_visible(s_u, g, pr, &key);
        const uint32_t bal = __ballot_sync(0xFFFFFFFFu, vis);
        if (lane == 0) s_bal[v][warp] = bal;
        s_key[v][tid] = key;
        if (vis && V.splats) write_splat<FMT>(s_u, g, pr, V.splats + i);
        __syncthreads();  // s_bal[v] complete; s_u free for the next view
        if (tid == 0) {
            uint32_t total = 0;
            for (uint32_t w = 0; w < NW; ++w) total += __popc(s_bal[v][w]);
            s_base[v] = total;  // block total until the look-back
            publish_flag(V.flags + tile, tile, s_stall,
                         pack_flag(s_epoch[v], tile == 0 ? kFlagPrefix : kFlagAggregate, total));
        }
    }
    __syncthreads();

    // ---- global offsets: warp w looks back for views w, w + 4, ... ----
    for (uint32_t v = warp; v < nv; v += NW) {
        const PreView &V = P.views[v];
        const uint32_t total = s_base[v];
        const uint32_t prefix = tile == 0 ? 0u : look_back_warp(V.flags, tile, s_epoch[v], &V.ctrl->status, s_limit);
        if (lane == 0) {
            if (tile > 0) publish_flag(V.flags + tile, tile, s_stall, pack_flag(s_epoch[v], kFlagPrefix, prefix + total));
            s_base[v] = prefix;
            if (tile == P.ntiles - 1) {
                const uint32_t c = prefix + total;
                V.ctrl->count = c;
                if (V.indirect) {
                    V.indirect[0] = 6u;
                    V.indirect[1] = c;
                    V.indirect[2] = 0u;
                    V.indirect[3] = 0u;
                }
                if (V.dispatch) {
                    V.dispatch[0] = (c + GS_SORT_BLOCK_KVS - 1) / GS_SORT_BLOCK_KVS;
                    V.dispatch[1] = 1u;
                    V.dispatch[2] = 1u;
                }
            }
        }
    }
    __syncthreads();
    const uint32_t lt = lanemask_lt();
    for (uint32_t v = 0; v < nv; ++v) {
        const PreView &V = P.views[v];
        if (tile == P.ntiles - 1) {
            const uint32_t c = min(V.ctrl->count, V.depth_cap);
            const uint32_t padded = min(((c + GS_SORT_BLOCK_KVS - 1) / GS_SORT_BLOCK_KVS) * GS_SORT_BLOCK_KVS, V.depth_cap);
            for (uint32_t k = c + tid; k < padded; k += kPreThreads) V.depths[k] = 2.0f;
        }
        const uint32_t bal = s_bal[v][warp];
        if ((bal >> lane) & 1u) {
            uint32_t off = s_base[v];
            for (uint32_t w = 0; w < warp; ++w) off += __popc(s_bal[v][w]);
            const uint32_t c = off + __popc(bal & lt);
            if (c < P.n) {
                V.indices[c] = i;
                V.depths[c] = s_key[v][tid];
            } else {
                atomicOr(&V.ctrl->status, kStatusBounds);
            }
        }
    }
}

// `pre` + `post` for an empty model: zero counts, no padding beyond capacity.
__global__ void preprocess_empty_kernel(uint32_t *indirect, uint32_t *dispatch, Ctrl *ctrl) {
    ctrl->count = 0;
    if (indirect) {
        indirect[0] = 6u;
        indirect[1] = 0u;
        indirect[2] = 0u;
        indirect[3] = 0u;
    }
    if (dispatch) {
        dispatch[0] = 0u;
        dispatch[1] = 1u;
        dispatch[2] = 1u;
    }
}

// A preprocess area holds its control block and look-back flags only, so no stale payload can
// lie where a flag is read: its arena is never cleared (kKeepArena).
__global__ void ctrl_init_views_kernel(const PreView *views, uint32_t nviews, Ctrl *group, WaitCfg cfg) {
    Ctrl *c = blockIdx.x < nviews ? views[blockIdx.x].ctrl : group;
    ctrl_reset(c, 1, c, kKeepArena, cfg);
}

__global__ void preprocess_views_empty_kernel(const PreView *views, uint32_t nviews) {
    for (uint32_t v = threadIdx.x; v < nviews; v += blockDim.x) {
        const PreView &V = views[v];
        V.ctrl->count = 0;
        if (V.indirect) {
            V.indirect[0] = 6u;
            V.indirect[1] = 0u;
            V.indirect[2] = 0u;
            V.indirect[3] = 0u;
        }
        if (V.dispatch) {
            V.dispatch[0] = 0u;
            V.dispatch[1] = 1u;
            V.dispatch[2] = 1u;
        }
    }
}

PreView preprocess_view(const gs_frame_uniforms *u_dev, uint32_t *indirect, uint32_t *dispatch, uint32_t *indices,
                        float *depths, uint32_t depth_cap, gs_splat *splats, void *scratch) {
    PreView V;
    V.u = u_dev;
    V.indirect = indirect;
    V.dispatch = dispatch;
    V.indices = indices;
    V.depths = depths;
    V.depth_cap = depth_cap;
    V.splats = splats;
    V.ctrl = reinterpret_cast<Ctrl *>(scratch);
    V.flags = reinterpret_cast<uint64_t *>((uint8_t *)scratch + align_up(sizeof(Ctrl), 256));
    return V;
}

cudaError_t launch_preprocess_views(const void *records, uint32_t format, uint32_t n, const uint32_t *selection,
                                    int invert, const PreView *views, uint32_t nviews, void *group,
                                    cudaStream_t st) {
    if (nviews == 0) return cudaSuccess;
    if (nviews > kPreMaxViews) return cudaErrorInvalidValue;
    Ctrl *gctrl = reinterpret_cast<Ctrl *>(group);
    ctrl_init_views_kernel<<<nviews + 1, 256, 0, st>>>(views, nviews, gctrl, wait_config());
    count_launches(1);
    if (n == 0) {
        preprocess_views_empty_kernel<<<1, 32, 0, st>>>(views, nviews);
        count_launches(1);
        return cudaGetLastError();
    }
    PreViewsParams P;
    P.records = reinterpret_cast<const uint8_t *>(records);
    P.n = n;
    P.ntiles = (n + kPreThreads - 1) / kPreThreads;
    P.selection = selection;
    P.invert = invert ? 1u : 0u;
    P.views = views;
    P.nviews = nviews;
    P.group = gctrl;
    prof_mark(kProfPreprocess, true, st);
    count_launches(1);
    switch (format) {
        case GS_FORMAT_FP32:
            preprocess_views_kernel<GS_FORMAT_FP32><<<P.ntiles, kPreThreads, 0, st>>>(P);
            break;
        case GS_FORMAT_HALF_SH_FP16:
            preprocess_views_kernel<GS_FORMAT_HALF_SH_FP16><<<P.ntiles, kPreThreads, 0, st>>>(P);
            break;
        default:
            preprocess_views_kernel<GS_FORMAT_HALF_SH_BF16><<<P.ntiles, kPreThreads, 0, st>>>(P);
            break;
    }
    prof_mark(kProfPreprocess, false, st);
    return cudaGetLastError();
}

size_t preprocess_scratch_bytes(uint32_t n) {
    const size_t tiles = (n + kPreThreads - 1) / kPreThreads;
    return align_up(sizeof(Ctrl), 256) + align_up(tiles * sizeof(uint64_t), 256);
}

cudaError_t launch_preprocess(const gs_frame_uniforms &u, const void *records, uint32_t format,
                              uint32_t n, const uint32_t *selection, int invert, uint32_t *indirect,
                              uint32_t *dispatch, uint32_t *indices, float *depths,
                              uint32_t depth_cap, gs_splat *splats, void *scratch, cudaStream_t st,
                              const gs_frame_uniforms *u_dev, uint4 *binfo) {
    Ctrl *ctrl = reinterpret_cast<Ctrl *>(scratch);
    uint64_t *flags = reinterpret_cast<uint64_t *>((uint8_t *)scratch + align_up(sizeof(Ctrl), 256));
    ctrl_init_kernel<<<1, 256, 0, st>>>(ctrl, 1, nullptr, kKeepArena, wait_config());
    count_launches(1);
    if (n == 0) {
        preprocess_empty_kernel<<<1, 1, 0, st>>>(indirect, dispatch, ctrl);
        count_launches(1);
        return cudaGetLastError();
    }
    PreParams P;
    P.u = u;
    P.u_dev = u_dev;
    P.records = reinterpret_cast<const uint8_t *>(records);
    P.n = n;
    P.ntiles = (n + kPreThreads - 1) / kPreThreads;
    P.selection = selection;
    P.invert = invert ? 1u : 0u;
    P.indirect = indirect;
    P.dispatch = dispatch;
    P.indices = indices;
    P.depths = depths;
    P.depth_cap = depth_cap;
    P.splats = splats;
    // the tile records need the viewport on the host (graph-captured uniforms are not read here)
    P.binfo = u_dev ? nullptr : binfo;
    P.tiles_x = ((uint32_t)u.viewport[0] + GS_TILE - 1) / GS_TILE;
    P.tiles_y = ((uint32_t)u.viewport[1] + GS_TILE - 1) / GS_TILE;
    P.ctrl = ctrl;
    P.flags = flags;
    prof_mark(kProfPreprocess, true, st);
    count_launches(1);
    if (u_dev) {
        switch (format) {
            case GS_FORMAT_FP32:
                preprocess_kernel<GS_FORMAT_FP32, true><<<P.ntiles, kPreThreads, 0, st>>>(P);
                break;
            case GS_FORMAT_HALF_SH_FP16:
                preprocess_kernel<GS_FORMAT_HALF_SH_FP16, true><<<P.ntiles, kPreThreads, 0, st>>>(P);
                break;
            default:
                preprocess_kernel<GS_FORMAT_HALF_SH_BF16, true><<<P.ntiles, kPreThreads, 0, st>>>(P);
                break;
        }
    } else {
        switch (format) {
            case GS_FORMAT_FP32:
                preprocess_kernel<GS_FORMAT_FP32, false><<<P.ntiles, kPreThreads, 0, st>>>(P);
                break;
            case GS_FORMAT_HALF_SH_FP16:
                preprocess_kernel<GS_FORMAT_HALF_SH_FP16, false><<<P.ntiles, kPreThreads, 0, st>>>(P);
                break;
            default:
                preprocess_kernel<GS_FORMAT_HALF_SH_BF16, false><<<P.ntiles, kPreThreads, 0, st>>>(P);
                break;
        }
    }
    prof_mark(kProfPreprocess, false, st);
    return cudaGetLastError();
}

}  // namespace gs
