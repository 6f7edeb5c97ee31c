// gs_oracle.cpp — CPU ORACLE (test infrastructure only; never part of the product path).
//
// A plain C++ restatement of the reference's splat render path, used by tests/, the smoke
// check and bench.py's CPU-baseline leg as the checker.  It restates, in one fixed FP32
// evaluation order with no floating-point contraction (build with -ffp-contract=off):
//   * camera matrices          src/camera.rs:70-93 (glam look_to_rh / perspective_rh)
//   * preprocess `main`        src/shader/preprocess.wesl:60-106, `post` :108-126
//   * cull / cov2d / axes / SH src/shader/utils.wesl:18-135, camera.wesl:13-20
//   * per-instance colour      src/shader/render.wesl:58-73
//   * quad + fragment + blend  src/shader/render.wesl:46-56,75-181 with
//                              BlendState::ALPHA_BLENDING onto a cleared Rgba8Unorm target
//                              (src/renderer.rs:162-195, 284-308)
//   * radix sort               std::stable_sort on (u32 key, u32 value): the reference
//                              RadixSorter is a stable LSD sort (src/radix_sorter.rs:73,
//                              src/shader/radix_sort.wgsl:287-529 with subgroup size 1)
//   * multi-model draw order   src/multi_model.rs:491-527
// The un-vendored wgpu-3dgs-core 0.6.0 helpers (model_to_world, model_transform_mat,
// model_scale_rot_mat, model_transform_inv_sr_mat, unpack functions) are restated from their
// documented meaning: model = T·R·S, SR = R·S, inv_SR = (R·S)^-1.
//
// Parity status: the reference (Rust + wgpu) cannot run in this environment, so this oracle
// is pinned to the reference's known-answer tests (tests/e2e/viewer.rs, multi_model.rs,
// tests/buffer/camera.rs) and not to reference outputs; bit layouts of core are unpinned.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "gs_record.h"

namespace {

// ------------------------------------------------------------------------------------------
// Small FP32 linear algebra, column-major (WGSL mat4x4<f32> semantics): m[c*4 + r].
// Sums run left to right; with -ffp-contract=off every * and + rounds on its own.
// ------------------------------------------------------------------------------------------
void mat4_mul(const float *a, const float *b, float *out) {
    float t[16];
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) {
            float s = a[0 * 4 + r] * b[c * 4 + 0];
            s = s + a[1 * 4 + r] * b[c * 4 + 1];
            s = s + a[2 * 4 + r] * b[c * 4 + 2];
            s = s + a[3 * 4 + r] * b[c * 4 + 3];
            t[c * 4 + r] = s;
        }
    std::memcpy(out, t, sizeof(t));
}

void mat4_vec(const float *m, const float *v, float *out) {
    for (int r = 0; r < 4; ++r) {
        float s = m[0 * 4 + r] * v[0];
        s = s + m[1 * 4 + r] * v[1];
        s = s + m[2 * 4 + r] * v[2];
        s = s + m[3 * 4 + r] * v[3];
        out[r] = s;
    }
}

void mat3_mul(const float *a, const float *b, float *out) {
    float t[9];
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) {
            float s = a[0 * 3 + r] * b[c * 3 + 0];
            s = s + a[1 * 3 + r] * b[c * 3 + 1];
            s = s + a[2 * 3 + r] * b[c * 3 + 2];
            t[c * 3 + r] = s;
        }
    std::memcpy(out, t, sizeof(t));
}

void mat3_vec(const float *m, const float *v, float *out) {
    for (int r = 0; r < 3; ++r) {
        float s = m[0 * 3 + r] * v[0];
        s = s + m[1 * 3 + r] * v[1];
        s = s + m[2 * 3 + r] * v[2];
        out[r] = s;
    }
}

// R from a quaternion (x, y, z, w), column-major 3x3.
void quat_to_mat3(const float *q, float *m) {
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

inline float minf_wgsl(float a, float b) { return (b < a) ? b : a; }
inline float clamp01(float v) { return v > 0.0f ? (v < 1.0f ? v : 1.0f) : 0.0f; }
inline float len2(float x, float y) { return std::sqrt(x * x + y * y); }

// utils.wesl:18-20 — true when the point lies outside [-1,1]x[-1,1]x[0,1]; NaN culls.
inline bool cull(float x, float y, float z) {
    return !(x >= -1.0f && y >= -1.0f && z >= 0.0f && x <= 1.0f && y <= 1.0f && z <= 1.0f);
}

// IEEE binary16 / bfloat16 -> float (exact conversions).
float half_to_float(uint16_t h) {
    const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    const uint32_t exp = (h >> 10) & 0x1Fu;
    const uint32_t man = h & 0x3FFu;
    uint32_t bits;
    if (exp == 0) {
        if (man == 0) {
            bits = sign;
        } else {  // subnormal: value = man * 2^-24
            float v = (float)man * 5.9604644775390625e-08f;
            std::memcpy(&bits, &v, 4);
            bits |= sign;
        }
    } else if (exp == 31) {
        bits = sign | 0x7F800000u | (man << 13);
    } else {
        bits = sign | ((exp + 112u) << 23) | (man << 13);
    }
    float f;
    std::memcpy(&f, &bits, 4);
    return f;
}

float bf16_to_float(uint16_t h) {
    uint32_t bits = (uint32_t)h << 16;
    float f;
    std::memcpy(&f, &bits, 4);
    return f;
}

inline uint32_t f2u(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
inline float u2f(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

// Round to nearest even for 0 <= x < 2^22 (as the CUDA kernels do with two adds).
inline float rint_small(float x) {
    const float m = 12582912.0f;  // 1.5 * 2^23; no -ffast-math, so (x + m) - m is kept
    const float t = x + m;
    return t - m;
}

// exp(x) for x in [-10, 0]: Cody–Waite range reduction x = k·ln2 + r with the classic
// two-part ln2 split, then the degree-7 Taylor polynomial of e^r on |r| <= ln2/2 in Horner
// form with fused multiply-adds, scaled by 2^k through the exponent field.  The CUDA
// kernels evaluate the same sequence, so both sides round identically.
float exp_portable(float x) {
    const float log2e = 1.44269504088896341f;
    const float c1 = 0.693359375f;        // ln2 high part (exact in 10 bits)
    const float c2 = -2.12194440e-4f;     // ln2 - c1
    // k = round(x·log2e) as two adds of 1.5·2^23 (round to nearest even).
    const float k = rint_small(x * log2e);
    float r = std::fma(-k, c1, x);
    r = std::fma(-k, c2, r);
    float p = 1.0f / 5040.0f;
    p = std::fma(p, r, 1.0f / 720.0f);
    p = std::fma(p, r, 1.0f / 120.0f);
    p = std::fma(p, r, 1.0f / 24.0f);
    p = std::fma(p, r, 1.0f / 6.0f);
    p = std::fma(p, r, 0.5f);
    p = std::fma(p, r, 1.0f);
    p = std::fma(p, r, 1.0f);
    const int ki = (int)k;
    const float scale = u2f((uint32_t)(ki + 127) << 23);
    return p * scale;
}

// Upper bound on r² beyond which a splat fragment cannot change an 8-bit destination (sizes the
// pixel box of a splat).  A fragment of alpha a moves a channel of destination d in [0, 255] by
// a·(s - d), |s - d| <= reach = max over the channels of max(s, 255 - s); a·reach <= 0.499 keeps
// the rounded result at d.  a = alpha·exp(-r²) <= 0.499/reach whenever r² >= ln(alpha·reach/0.499);
// ln(x) <= ln2·(e + (m - 1) + 0.0861) for x = m·2^e, m in [1, 2).
float colour_reach(float s0, float s1, float s2) {
    const float t0 = s0 > 255.0f - s0 ? s0 : 255.0f - s0;
    const float t1 = s1 > 255.0f - s1 ? s1 : 255.0f - s1;
    const float t2 = s2 > 255.0f - s2 ? s2 : 255.0f - s2;
    const float t01 = t0 > t1 ? t0 : t1;
    return t01 > t2 ? t01 : t2;
}

float splat_r2_bound(float alpha, float reach, float std2) {
    const float x = (alpha * reach) * 2.0041f;
    if (!(x > 0.0f)) return -1.0f;
    const uint32_t bits = f2u(x);
    const float e = (float)((int)((bits >> 23) & 0xFFu) - 127);
    const float mant = u2f((bits & 0x7FFFFFu) | 0x3F800000u);
    float r2 = 0.693147182f * (e + (mant - 1.0f) + 0.0862f) + 0.01f;
    return minf_wgsl(std2, r2);
}

struct Record {
    float pos[3];
    uint32_t color;
    float sh[45];
    float cov3d[6];
};

Record load_record(const void *base, uint32_t format, uint32_t i) {
    Record r;
    if (format == GS_FORMAT_FP32) {
        const gs_gaussian_pod *g = (const gs_gaussian_pod *)base + i;
        std::memcpy(r.pos, g->pos, 12);
        r.color = g->color;
        std::memcpy(r.sh, g->sh, sizeof(r.sh));
        std::memcpy(r.cov3d, g->cov3d, sizeof(r.cov3d));
    } else {
        const gs_gaussian_pod_half *g = (const gs_gaussian_pod_half *)base + i;
        std::memcpy(r.pos, g->pos, 12);
        r.color = g->color;
        for (int k = 0; k < 45; ++k)
            r.sh[k] = (format == GS_FORMAT_HALF_SH_BF16) ? bf16_to_float(g->sh[k])
                                                         : half_to_float(g->sh[k]);
        float q[4], s[3];
        for (int k = 0; k < 4; ++k) q[k] = half_to_float(g->rot[k]);
        for (int k = 0; k < 3; ++k) s[k] = half_to_float(g->scale[k]);
        // Normalise the rotation, then Σ = (R·S)(R·S)ᵀ in FP32.
        float n = std::sqrt(((q[0] * q[0] + q[1] * q[1]) + q[2] * q[2]) + q[3] * q[3]);
        for (int k = 0; k < 4; ++k) q[k] = q[k] / n;
        float R[9];
        quat_to_mat3(q, R);
        float M[9];
        for (int c = 0; c < 3; ++c)
            for (int rr = 0; rr < 3; ++rr) M[c * 3 + rr] = R[c * 3 + rr] * s[c];
        // cov(i, j) = sum_k M(i,k)·M(j,k)
        auto cv = [&](int a, int b) {
            float acc = M[0 * 3 + a] * M[0 * 3 + b];
            acc = acc + M[1 * 3 + a] * M[1 * 3 + b];
            acc = acc + M[2 * 3 + a] * M[2 * 3 + b];
            return acc;
        };
        r.cov3d[0] = cv(0, 0);
        r.cov3d[1] = cv(0, 1);
        r.cov3d[2] = cv(0, 2);
        r.cov3d[3] = cv(1, 1);
        r.cov3d[4] = cv(1, 2);
        r.cov3d[5] = cv(2, 2);
    }
    return r;
}

// utils.wesl:25-48 (cov2d) + 54-79 (cov2d_axes).  Returns (major.xy, minor.xy).
void cov2d_axes(const gs_frame_uniforms &u, const Record &g, const float p4[4], float std_dev,
                float axes[4]) {
    const float *c = g.cov3d;
    float t[4];
    mat4_vec(u.vm, p4, t);
    const float fx = u.focal[0], fy = u.focal[1];
    const float tz2 = t[2] * t[2];
    const float j00 = fx / t[2];
    const float j02 = -(fx * t[0]) / tz2;
    const float j11 = fy / t[2];
    const float j12 = -(fy * t[1]) / tz2;
    const float *w = u.wsr;  // W·SR, column-major
    float T0[3], T1[3];
    for (int k = 0; k < 3; ++k) {
        T0[k] = j00 * w[k * 3 + 0] + j02 * w[k * 3 + 2];
        T1[k] = j11 * w[k * 3 + 1] + j12 * w[k * 3 + 2];
    }
    // V = [c0 c1 c2; c1 c3 c4; c2 c4 c5]; U = T·V (rows), Σ2 = U·Tᵀ.
    const float V[9] = {c[0], c[1], c[2], c[1], c[3], c[4], c[2], c[4], c[5]};
    float U0[3], U1[3];
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
    float dx = b, dy = lmaj - a;
    float dirx, diry;
    if (dx == 0.0f && dy == 0.0f) {
        dirx = 0.0f;
        diry = 1.0f;
    } else {
        const float l = len2(dx, dy);
        dirx = dx / l;
        diry = dy / l;
    }
    const float majl = minf_wgsl(std_dev * std::sqrt(lmaj), 1024.0f);
    const float minl = minf_wgsl(std_dev * std::sqrt(lmin), 1024.0f);
    axes[0] = majl * dirx;
    axes[1] = majl * diry;
    axes[2] = minl * diry;
    axes[3] = minl * -dirx;
}

// utils.wesl:82-135 with the direction of render.wesl:58-73.
void view_color(const gs_frame_uniforms &u, const Record &g, const float world[4], float rgba[4]) {
    const float vd[3] = {u.cam_pos[0] - world[0], u.cam_pos[1] - world[1], u.cam_pos[2] - world[2]};
    float mvd[3];
    mat3_vec(u.inv_sr, vd, mvd);
    const float l = std::sqrt((mvd[0] * mvd[0] + mvd[1] * mvd[1]) + mvd[2] * mvd[2]);
    const float x = -(mvd[0] / l), y = -(mvd[1] / l), z = -(mvd[2] / l);

    const float c1 = 0.4886025f;
    const float c2[5] = {1.0925484f, -1.0925484f, 0.3153916f, -1.0925484f, 0.5462742f};
    const float c3[7] = {-0.5900436f, 2.8906114f, -0.4570458f, 0.3731763f,
                         -0.4570458f, 1.4453057f, -0.5900436f};
    float res[3];
    for (int ch = 0; ch < 3; ++ch)
        res[ch] = u.no_sh0 ? 0.5f : (float)((g.color >> (8 * ch)) & 0xFFu) / 255.0f;
    const float *sh = g.sh;
    if (u.sh_deg >= 1) {
        for (int ch = 0; ch < 3; ++ch) {
            float v = (-sh[0 * 3 + ch]) * y + sh[1 * 3 + ch] * z;
            v = v - sh[2 * 3 + ch] * x;
            res[ch] = res[ch] + c1 * v;
        }
        if (u.sh_deg >= 2) {
            const float xx = x * x, yy = y * y, zz = z * z;
            const float xy = x * y, yz = y * z, xz = x * z;
            const float k0 = c2[0] * xy, k1 = c2[1] * yz;
            const float k2 = c2[2] * ((2.0f * zz - xx) - yy);
            const float k3 = c2[3] * xz, k4 = c2[4] * (xx - yy);
            for (int ch = 0; ch < 3; ++ch) {
                float v = k0 * sh[3 * 3 + ch] + k1 * sh[4 * 3 + ch];
                v = v + k2 * sh[5 * 3 + ch];
                v = v + k3 * sh[6 * 3 + ch];
                v = v + k4 * sh[7 * 3 + ch];
                res[ch] = res[ch] + v;
            }
            if (u.sh_deg >= 3) {
                const float m0 = (c3[0] * y) * (3.0f * xx - yy);
                const float m1 = (c3[1] * xy) * z;
                const float m2 = (c3[2] * y) * ((4.0f * zz - xx) - yy);
                const float m3 = (c3[3] * z) * ((2.0f * zz - 3.0f * xx) - 3.0f * yy);
                const float m4 = (c3[4] * x) * ((4.0f * zz - xx) - yy);
                const float m5 = (c3[5] * z) * (xx - yy);
                const float m6 = (c3[6] * x) * (xx - 3.0f * yy);
                for (int ch = 0; ch < 3; ++ch) {
                    float v = m0 * sh[8 * 3 + ch] + m1 * sh[9 * 3 + ch];
                    v = v + m2 * sh[10 * 3 + ch];
                    v = v + m3 * sh[11 * 3 + ch];
                    v = v + m4 * sh[12 * 3 + ch];
                    v = v + m5 * sh[13 * 3 + ch];
                    v = v + m6 * sh[14 * 3 + ch];
                    res[ch] = res[ch] + v;
                }
            }
        }
    }
    for (int ch = 0; ch < 3; ++ch) rgba[ch] = res[ch] > 0.0f ? res[ch] : 0.0f;  // max(result, 0)
    rgba[3] = (float)((g.color >> 24) & 0xFFu) / 255.0f;
}

struct Pre {
    bool visible;
    float key;
};

// preprocess.wesl:80-105 for one Gaussian; fills `splat` when visible and splat != nullptr.
Pre preprocess_one(const gs_frame_uniforms &u, const Record &g, gs_splat *splat) {
    const float p4[4] = {g.pos[0], g.pos[1], g.pos[2], 1.0f};
    float world[4], clip[4];
    mat4_vec(u.model, p4, world);
    mat4_vec(u.pv, world, clip);
    const float nx = clip[0] / clip[3], ny = clip[1] / clip[3], nz = clip[2] / clip[3];
    float axes[4];
    bool have_axes = false;
    if (cull(nx, ny, nz)) {
        cov2d_axes(u, g, p4, u.std_dev_scaled, axes);
        have_axes = true;
        const float mx = axes[0] * u.std_dev / u.size[0];
        const float my = axes[1] * u.std_dev / u.size[1];
        const float mlen = len2(mx, my);
        const float nl = len2(nx, ny);
        const float dx = -nx / nl, dy = -ny / nl;
        const float m = minf_wgsl(mlen, nl);
        if (cull(nx + m * dx, ny + m * dy, nz)) return {false, 0.0f};
    }
    Pre out{true, 1.0f - nz};
    if (!splat) return out;

    // ---- per-instance vertex work (render.wesl:75-130), once per Gaussian ----
    float rgba[4];
    view_color(u, g, world, rgba);
    const float W = u.viewport[0], H = u.viewport[1];
    splat->cx = ((nx + 1.0f) * W) * 0.5f;
    splat->cy = ((1.0f - ny) * H) * 0.5f;
    splat->s255[0] = clamp01(rgba[0]) * 255.0f;
    splat->s255[1] = clamp01(rgba[1]) * 255.0f;
    splat->s255[2] = clamp01(rgba[2]) * 255.0f;
    splat->alpha = rgba[3];
    const float std2 = u.std_dev * u.std_dev;
    if (u.display_mode == GS_DISPLAY_POINT) {
        // render.wesl:377-389: half side = point_size·s·(aspect, 1)/|view_pos| in NDC.
        float vp[4];
        mat4_vec(u.vm, p4, vp);
        const float l = std::sqrt((vp[0] * vp[0] + vp[1] * vp[1]) + vp[2] * vp[2]);
        const float aspect = u.size[1] / u.size[0];
        const float pnd = (0.01f * u.point_size) / l;
        const float hx = (pnd * aspect) * (0.5f * W);
        const float hy = pnd * (0.5f * H);
        splat->q[0] = hx;
        splat->q[1] = hy;
        splat->q[2] = 0.0f;
        splat->q[3] = 0.0f;
        if (hx > 0.0f && hy > 0.0f && hx < 1e30f && hy < 1e30f) {
            splat->ex = hx * 1.001f + 0.01f;
            splat->ey = hy * 1.001f + 0.01f;
        } else {
            splat->ex = -1.0f;
            splat->ey = -1.0f;
        }
        return out;
    }
    if (!have_axes) cov2d_axes(u, g, p4, u.std_dev_scaled, axes);
    const float kx = (0.5f * W) / u.size[0];
    const float ky = (0.5f * H) / u.size[1];
    const float a00 = axes[0] * kx, a01 = axes[2] * kx;
    const float a10 = -axes[1] * ky, a11 = -axes[3] * ky;
    const float det = a00 * a11 - a01 * a10;
    splat->q[0] = a11 / det;
    splat->q[1] = -a01 / det;
    splat->q[2] = -a10 / det;
    splat->q[3] = a00 / det;
    const float reach = colour_reach(clamp01(rgba[0]) * 255.0f, clamp01(rgba[1]) * 255.0f, clamp01(rgba[2]) * 255.0f);
    const float r2 = (u.display_mode == GS_DISPLAY_SPLAT) ? splat_r2_bound(rgba[3], reach, std2) : std2;
    const bool ok = det != 0.0f && std::isfinite(det) && std::isfinite(splat->q[0]) &&
                    std::isfinite(splat->q[1]) && std::isfinite(splat->q[2]) &&
                    std::isfinite(splat->q[3]) && r2 >= 0.0f;
    if (ok) {
        splat->ex = std::sqrt(r2 * (a00 * a00 + a01 * a01)) * 1.001f + 0.01f;
        splat->ey = std::sqrt(r2 * (a10 * a10 + a11 * a11)) * 1.001f + 0.01f;
    } else {
        splat->ex = -1.0f;
        splat->ey = -1.0f;
    }
    return out;
}

// One fragment of splat `s` at pixel centre offset (dx, dy): returns false when discarded,
// else the fragment alpha.  render.wesl:143-181.
inline bool fragment(const gs_splat &s, uint32_t mode, float std2, float outline2, float dx,
                     float dy, int exp_mode, float *alpha_out) {
    if (mode == GS_DISPLAY_POINT) {
        const float hx = s.q[0], hy = s.q[1];
        if (!(dx >= -hx && dx < hx && dy >= -hy && dy < hy)) return false;
        *alpha_out = 1.0f;
        return true;
    }
    const float qx = std::fma(s.q[0], dx, s.q[1] * dy);
    const float qy = std::fma(s.q[2], dx, s.q[3] * dy);
    const float r2 = std::fma(qx, qx, qy * qy);
    if (!(r2 <= std2)) return false;  // discard (also rejects NaN)
    if (mode == GS_DISPLAY_SPLAT) {
        const float e = exp_mode == 0 ? exp_portable(-r2) : std::exp(-r2);
        *alpha_out = s.alpha * e;
    } else {
        *alpha_out = (r2 > outline2) ? 1.0f : s.alpha;
    }
    return true;
}

// BlendState::ALPHA_BLENDING on an 8-bit target in units of 255:
// rgb' = round(d·(1-α) + s·α), a' = round(a_d·(1-α) + 255·α).
inline void blend(uint8_t *px, const gs_splat &s, float alpha) {
    const float om = 1.0f - alpha;
    for (int ch = 0; ch < 3; ++ch) {
        const float d = (float)px[ch];
        const float x = std::fma(d, om, s.s255[ch] * alpha);
        px[ch] = (uint8_t)rint_small(x);
    }
    const float da = (float)px[3];
    const float xa = std::fma(da, om, 255.0f * alpha);
    px[3] = (uint8_t)rint_small(xa);
}

void raster_brute(const gs_frame_uniforms &u, const gs_splat *splats, const uint32_t *order,
                  uint32_t count, uint8_t *rgba, uint32_t W, uint32_t H, int exp_mode) {
    const float std2 = u.std_dev * u.std_dev;
    const float o = u.std_dev - 0.1f;
    const float outline2 = o * o;
    for (uint32_t k = 0; k < count; ++k) {
        const gs_splat &s = splats[order[k]];
        double ex, ey;
        if (u.display_mode == GS_DISPLAY_POINT) {
            ex = s.q[0];
            ey = s.q[1];
            if (!(ex > 0.0 && ey > 0.0 && ex < 1e30 && ey < 1e30)) continue;
        } else {
            // Quad corners: offset A·(±std, ±std) with A = Q^-1.
            const double q0 = s.q[0], q1 = s.q[1], q2 = s.q[2], q3 = s.q[3];
            const double det = q0 * q3 - q1 * q2;
            if (!(std::isfinite(det) && det != 0.0)) continue;
            const double a00 = q3 / det, a01 = -q1 / det, a10 = -q2 / det, a11 = q0 / det;
            ex = u.std_dev * (std::fabs(a00) + std::fabs(a01));
            ey = u.std_dev * (std::fabs(a10) + std::fabs(a11));
            if (!(std::isfinite(ex) && std::isfinite(ey))) continue;
        }
        const double x0 = std::max(0.0, std::floor(s.cx - ex - 2.0));
        const double x1 = std::min((double)W - 1, std::ceil(s.cx + ex + 2.0));
        const double y0 = std::max(0.0, std::floor(s.cy - ey - 2.0));
        const double y1 = std::min((double)H - 1, std::ceil(s.cy + ey + 2.0));
        if (x0 > x1 || y0 > y1) continue;
        for (uint32_t py = (uint32_t)y0; py <= (uint32_t)y1; ++py)
            for (uint32_t px = (uint32_t)x0; px <= (uint32_t)x1; ++px) {
                const float dx = ((float)px + 0.5f) - s.cx;
                const float dy = ((float)py + 0.5f) - s.cy;
                float a;
                if (!fragment(s, u.display_mode, std2, outline2, dx, dy, exp_mode, &a)) continue;
                blend(rgba + ((size_t)py * W + px) * 4, s, a);
            }
    }
}

// Tile-parallel rasteriser for the CPU baseline: each 16x16 tile keeps the splats whose
// fragment box (ex, ey) touches it, in draw order, and is blended independently.
void raster_tiled(const gs_frame_uniforms &u, const gs_splat *splats, const uint32_t *order,
                  uint32_t count, uint8_t *rgba, uint32_t W, uint32_t H, int exp_mode,
                  int threads) {
    const uint32_t T = GS_TILE;
    const uint32_t tx = (W + T - 1) / T, ty = (H + T - 1) / T;
    const uint32_t ntiles = tx * ty;
    const float std2 = u.std_dev * u.std_dev;
    const float o = u.std_dev - 0.1f;
    const float outline2 = o * o;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
    // Per-thread bins over a contiguous chunk of the draw order keep each tile list ordered
    // once the chunks are concatenated in chunk order.
    int nthreads = 1;
#ifdef _OPENMP
    nthreads = threads > 0 ? threads : omp_get_max_threads();
#endif
    std::vector<std::vector<std::vector<uint32_t>>> bins(nthreads,
                                                         std::vector<std::vector<uint32_t>>(ntiles));
#pragma omp parallel num_threads(nthreads)
    {
        int t = 0;
#ifdef _OPENMP
        t = omp_get_thread_num();
#endif
        const uint64_t lo = (uint64_t)count * t / nthreads, hi = (uint64_t)count * (t + 1) / nthreads;
        for (uint64_t k = lo; k < hi; ++k) {
            const gs_splat &s = splats[order[k]];
            if (!(s.ex >= 0.0f)) continue;
            const float fx0 = std::floor((s.cx - s.ex) / (float)T);
            const float fx1 = std::floor((s.cx + s.ex) / (float)T);
            const float fy0 = std::floor((s.cy - s.ey) / (float)T);
            const float fy1 = std::floor((s.cy + s.ey) / (float)T);
            const int x0 = (int)std::max(0.0f, fx0), x1 = (int)std::min((float)tx - 1, fx1);
            const int y0 = (int)std::max(0.0f, fy0), y1 = (int)std::min((float)ty - 1, fy1);
            for (int yy = y0; yy <= y1; ++yy)
                for (int xx = x0; xx <= x1; ++xx) bins[t][(uint32_t)yy * tx + xx].push_back((uint32_t)k);
        }
    }
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads)
    for (int64_t tile = 0; tile < (int64_t)ntiles; ++tile) {
        const uint32_t bx = (uint32_t)tile % tx, by = (uint32_t)tile / tx;
        for (int t = 0; t < nthreads; ++t)
            for (uint32_t k : bins[t][tile]) {
                const gs_splat &s = splats[order[k]];
                for (uint32_t py = by * T; py < std::min(H, by * T + T); ++py)
                    for (uint32_t px = bx * T; px < std::min(W, bx * T + T); ++px) {
                        const float dx = ((float)px + 0.5f) - s.cx;
                        const float dy = ((float)py + 0.5f) - s.cy;
                        float a;
                        if (!fragment(s, u.display_mode, std2, outline2, dx, dy, exp_mode, &a))
                            continue;
                        blend(rgba + ((size_t)py * W + px) * 4, s, a);
                    }
            }
    }
}

void look_to_rh(const float eye[3], const float dir_in[3], const float up[3], float out[16]) {
    float l = std::sqrt((dir_in[0] * dir_in[0] + dir_in[1] * dir_in[1]) + dir_in[2] * dir_in[2]);
    const float f[3] = {dir_in[0] / l, dir_in[1] / l, dir_in[2] / l};
    float s[3] = {f[1] * up[2] - f[2] * up[1], f[2] * up[0] - f[0] * up[2], f[0] * up[1] - f[1] * up[0]};
    l = std::sqrt((s[0] * s[0] + s[1] * s[1]) + s[2] * s[2]);
    s[0] = s[0] / l;
    s[1] = s[1] / l;
    s[2] = s[2] / l;
    const float uu[3] = {s[1] * f[2] - s[2] * f[1], s[2] * f[0] - s[0] * f[2], s[0] * f[1] - s[1] * f[0]};
    out[0] = s[0]; out[1] = uu[0]; out[2] = -f[0]; out[3] = 0.0f;
    out[4] = s[1]; out[5] = uu[1]; out[6] = -f[1]; out[7] = 0.0f;
    out[8] = s[2]; out[9] = uu[2]; out[10] = -f[2]; out[11] = 0.0f;
    out[12] = -((eye[0] * s[0] + eye[1] * s[1]) + eye[2] * s[2]);
    out[13] = -((eye[0] * uu[0] + eye[1] * uu[1]) + eye[2] * uu[2]);
    out[14] = (eye[0] * f[0] + eye[1] * f[1]) + eye[2] * f[2];
    out[15] = 1.0f;
}

// ------------------------------------------------------------------------------------------
// The reference's vertex stage taken literally (render.wesl:46-56, 75-130), for checking the
// pixel -> quad-offset map that preprocess_one hands the rasterisers: six clip-space vertices
// per instance, proj·(view·(model·pos)) plus the quad corner offsets scaled by w (splat and
// ellipse: along the std-scaled 2D axes; point: the point-size square, aspect H/W, divided by
// |view_pos|); two triangles (vertices 0-2 and 3-5) rasterised at pixel centres under the
// top-left fill rule; quad_offset interpolated at the pixel centre (the six vertices share w,
// so linear interpolation in screen space is the perspective-correct one); frag_main
// (render.wesl:143-181) in FP32; the blend of `blend`.  Screen positions and barycentrics are
// FP64 (hardware snaps to a sub-pixel grid instead), everything the shaders compute is FP32.
// ------------------------------------------------------------------------------------------
struct QuadVert {
    double x, y;  // screen position (pixels, y down)
    float qx, qy; // quad_offset
};

void raster_triangle(QuadVert v0, QuadVert v1, QuadVert v2, uint32_t mode, float std_dev, float alpha_in,
                     const gs_splat &colour, uint8_t *rgba, uint32_t W, uint32_t H) {
    double area = (v1.x - v0.x) * (v2.y - v0.y) - (v1.y - v0.y) * (v2.x - v0.x);
    if (!(std::isfinite(area) && area != 0.0)) return;
    if (area < 0.0) {
        std::swap(v1, v2);
        area = -area;
    }
    const QuadVert v[3] = {v0, v1, v2};
    const double xmin = std::min(v0.x, std::min(v1.x, v2.x)), xmax = std::max(v0.x, std::max(v1.x, v2.x));
    const double ymin = std::min(v0.y, std::min(v1.y, v2.y)), ymax = std::max(v0.y, std::max(v1.y, v2.y));
    const double x0 = std::max(0.0, std::floor(xmin - 1.0)), x1 = std::min((double)W - 1.0, std::ceil(xmax + 1.0));
    const double y0 = std::max(0.0, std::floor(ymin - 1.0)), y1 = std::min((double)H - 1.0, std::ceil(ymax + 1.0));
    if (!(x0 <= x1 && y0 <= y1)) return;
    // With area > 0 in y-down screen space the triangle is clockwise on screen: an edge going
    // up is a left edge, a horizontal edge going right is a top edge.
    bool topleft[3];
    for (int e = 0; e < 3; ++e) {
        const QuadVert &a = v[e], &b = v[(e + 1) % 3];
        topleft[e] = (a.y == b.y && b.x > a.x) || (b.y < a.y);
    }
    const float std2 = std_dev * std_dev;
    const float o = std_dev - 0.1f;
    const float outline2 = o * o;
    for (uint32_t py = (uint32_t)y0; py <= (uint32_t)y1; ++py)
        for (uint32_t px = (uint32_t)x0; px <= (uint32_t)x1; ++px) {
            const double cx = (double)px + 0.5, cy = (double)py + 0.5;
            double w[3];
            bool in = true;
            for (int e = 0; e < 3 && in; ++e) {
                const QuadVert &a = v[e], &b = v[(e + 1) % 3];
                w[e] = (b.x - a.x) * (cy - a.y) - (b.y - a.y) * (cx - a.x);
                in = w[e] > 0.0 || (w[e] == 0.0 && topleft[e]);
            }
            if (!in) continue;
            // edge e lies opposite vertex (e + 2) % 3
            const double l0 = w[1] / area, l1 = w[2] / area, l2 = w[0] / area;
            const float qx = (float)(l0 * v[0].qx + l1 * v[1].qx + l2 * v[2].qx);
            const float qy = (float)(l0 * v[0].qy + l1 * v[1].qy + l2 * v[2].qy);
            float alpha;
            if (mode == GS_DISPLAY_POINT) {
                alpha = 1.0f;
            } else {
                const float r2 = qx * qx + qy * qy;  // dot(in.quad_offset, in.quad_offset)
                if (r2 > std2) continue;             // discard
                if (mode == GS_DISPLAY_SPLAT) {
                    alpha = alpha_in * std::exp(-r2);
                } else {
                    const bool outline = r2 > outline2;
                    alpha = alpha_in + (1.0f - alpha_in) * (outline ? 1.0f : 0.0f);
                }
            }
            blend(rgba + ((size_t)py * W + px) * 4, colour, alpha);
        }
}

// vert_main for the six vertices of one instance, then its two triangles.
void draw_instance(const gs_frame_uniforms &u, const gs_camera_pod &cam, const Record &g, uint8_t *rgba, uint32_t W,
                   uint32_t H) {
    static const float corner[6][2] = {{1.0f, -1.0f}, {-1.0f, -1.0f}, {1.0f, 1.0f},
                                       {-1.0f, 1.0f}, {1.0f, 1.0f}, {-1.0f, -1.0f}};
    const float p4[4] = {g.pos[0], g.pos[1], g.pos[2], 1.0f};
    float world[4], view_pos[4], proj_pos[4];
    mat4_vec(u.model, p4, world);
    mat4_vec(cam.view, world, view_pos);
    mat4_vec(cam.proj, view_pos, proj_pos);
    float rgba_f[4];
    view_color(u, g, world, rgba_f);
    gs_splat colour{};
    colour.s255[0] = clamp01(rgba_f[0]) * 255.0f;  // a Rgba8Unorm attachment clamps the source
    colour.s255[1] = clamp01(rgba_f[1]) * 255.0f;
    colour.s255[2] = clamp01(rgba_f[2]) * 255.0f;
    const float w = proj_pos[3];
    // depth clipping: z / w outside [0, 1] (all vertices share z and w)
    if (!(proj_pos[2] >= 0.0f && proj_pos[2] <= w)) return;
    float clip[6][2], q[6][2];
    if (u.display_mode == GS_DISPLAY_POINT) {
        const float aspect = u.size[1] / u.size[0];  // camera_aspect_ratio = size.y / size.x
        const float len = std::sqrt((view_pos[0] * view_pos[0] + view_pos[1] * view_pos[1]) + view_pos[2] * view_pos[2]);
        for (int k = 0; k < 6; ++k) {
            q[k][0] = (corner[k][0] * 0.01f) * u.point_size;
            q[k][1] = (corner[k][1] * 0.01f) * u.point_size;
            clip[k][0] = proj_pos[0] + ((q[k][0] * w) * aspect) / len;
            clip[k][1] = proj_pos[1] + ((q[k][1] * w) * 1.0f) / len;
        }
    } else {
        float axes[4];
        cov2d_axes(u, g, p4, u.std_dev_scaled, axes);
        if (axes[0] == 0.0f && axes[1] == 0.0f && axes[2] == 0.0f && axes[3] == 0.0f) return;  // clip z = 2
        for (int k = 0; k < 6; ++k) {
            q[k][0] = corner[k][0] * u.std_dev;
            q[k][1] = corner[k][1] * u.std_dev;
            clip[k][0] = (proj_pos[0] + ((q[k][0] * w) * axes[0]) / u.size[0]) + ((q[k][1] * w) * axes[2]) / u.size[0];
            clip[k][1] = (proj_pos[1] + ((q[k][0] * w) * axes[1]) / u.size[1]) + ((q[k][1] * w) * axes[3]) / u.size[1];
        }
    }
    QuadVert vs[6];
    for (int k = 0; k < 6; ++k) {
        const double nx = (double)clip[k][0] / (double)w, ny = (double)clip[k][1] / (double)w;
        vs[k].x = (nx + 1.0) * 0.5 * (double)W;
        vs[k].y = (1.0 - ny) * 0.5 * (double)H;
        vs[k].qx = q[k][0];
        vs[k].qy = q[k][1];
    }
    raster_triangle(vs[0], vs[1], vs[2], u.display_mode, u.std_dev, rgba_f[3], colour, rgba, W, H);
    raster_triangle(vs[3], vs[4], vs[5], u.display_mode, u.std_dev, rgba_f[3], colour, rgba, W, H);
}

}  // namespace

extern "C" {

// CameraPod::new restated (src/buffer/camera.rs:163-172, src/camera.rs:70-93).
void oracle_camera_pod(const gs_camera *cam, uint32_t w, uint32_t h, gs_camera_pod *pod) {
    std::memset(pod, 0, sizeof(*pod));
    const float fwd[3] = {std::cos(cam->pitch) * std::sin(cam->yaw), std::sin(cam->pitch),
                          std::cos(cam->pitch) * std::cos(cam->yaw)};
    const float up[3] = {0.0f, 1.0f, 0.0f};
    look_to_rh(cam->pos, fwd, up, pod->view);
    const float aspect = (float)w / (float)h;
    const float half = 0.5f * cam->vertical_fov;
    const float hh = std::cos(half) / std::sin(half);
    const float ww = hh / aspect;
    const float r = cam->z_far / (cam->z_near - cam->z_far);
    std::memset(pod->proj, 0, sizeof(pod->proj));
    pod->proj[0] = ww;
    pod->proj[5] = hh;
    pod->proj[10] = r;
    pod->proj[11] = -1.0f;
    pod->proj[14] = r * cam->z_near;
    pod->size[0] = (float)w;
    pod->size[1] = (float)h;
}

void oracle_frame_uniforms(const gs_camera_pod *cam, const gs_model_transform_pod *mt,
                           const gs_gaussian_transform_pod *gt, uint32_t vw, uint32_t vh,
                           gs_frame_uniforms *u) {
    std::memset(u, 0, sizeof(*u));
    mat4_mul(cam->proj, cam->view, u->pv);
    float R[9];
    quat_to_mat3(mt->rot, R);
    float SR[9];
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) SR[c * 3 + r] = R[c * 3 + r] * mt->scale[c];
    for (int c = 0; c < 3; ++c) {
        for (int r = 0; r < 3; ++r) u->model[c * 4 + r] = SR[c * 3 + r];
        u->model[c * 4 + 3] = 0.0f;
    }
    u->model[12] = mt->pos[0];
    u->model[13] = mt->pos[1];
    u->model[14] = mt->pos[2];
    u->model[15] = 1.0f;
    mat4_mul(cam->view, u->model, u->vm);
    float Wm[9];
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) Wm[c * 3 + r] = cam->view[c * 4 + r];
    mat3_mul(Wm, SR, u->wsr);
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) u->inv_sr[c * 3 + r] = R[r * 3 + c] / mt->scale[r];
    const float *t = cam->view + 12;
    for (int i = 0; i < 3; ++i)
        u->cam_pos[i] = -((Wm[i * 3 + 0] * t[0] + Wm[i * 3 + 1] * t[1]) + Wm[i * 3 + 2] * t[2]);
    u->size[0] = cam->size[0];
    u->size[1] = cam->size[1];
    u->focal[0] = (cam->proj[0] * cam->size[0]) * 0.5f;
    u->focal[1] = (cam->proj[5] * cam->size[1]) * 0.5f;
    u->viewport[0] = (float)vw;
    u->viewport[1] = (float)vh;
    u->std_dev = gt->max_std_dev;
    u->std_dev_scaled = gt->max_std_dev * gt->size;
    u->point_size = gt->size;
    u->display_mode = gt->display_mode;
    u->sh_deg = gt->sh_deg;
    u->no_sh0 = gt->no_sh0;
}

// Preprocess: visible Gaussians in ascending index order -> indices/depths; returns V.
// `splats` (nullable) is indexed by Gaussian index.  threads > 1 uses OpenMP.
uint32_t oracle_preprocess(const gs_frame_uniforms *u, const void *gaussians, uint32_t format,
                           uint32_t n, const uint32_t *selection, int invert, uint32_t *indices,
                           float *depths, gs_splat *splats, int threads) {
    int nthreads = threads > 0 ? threads : 1;
    std::vector<uint8_t> vis(n);
    std::vector<float> key(n);
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        if (selection) {
            const bool bit = (selection[i / 32] >> (i % 32)) & 1u;
            if ((invert != 0) == bit) {
                vis[i] = 0;
                continue;
            }
        }
        const Record g = load_record(gaussians, format, (uint32_t)i);
        const Pre p = preprocess_one(*u, g, splats ? splats + i : nullptr);
        vis[i] = p.visible;
        key[i] = p.key;
    }
    uint32_t c = 0;
    for (uint32_t i = 0; i < n; ++i)
        if (vis[i]) {
            indices[c] = i;
            depths[c] = key[i];
            ++c;
        }
    return c;
}

void oracle_stable_sort(uint32_t *keys, uint32_t *vals, uint32_t n) {
    std::vector<uint64_t> kv(n);
    for (uint32_t i = 0; i < n; ++i) kv[i] = ((uint64_t)keys[i] << 32) | vals[i];
    std::stable_sort(kv.begin(), kv.end(),
                     [](uint64_t a, uint64_t b) { return (a >> 32) < (b >> 32); });
    for (uint32_t i = 0; i < n; ++i) {
        keys[i] = (uint32_t)(kv[i] >> 32);
        vals[i] = (uint32_t)kv[i];
    }
}

// Parallel stable LSD radix sort (4 x 8 bits) for the CPU baseline.
void oracle_radix_sort(uint32_t *keys, uint32_t *vals, uint32_t n, int threads) {
    int nt = threads > 0 ? threads : 1;
    std::vector<uint32_t> k2(n), v2(n);
    uint32_t *ka = keys, *va = vals, *kb = k2.data(), *vb = v2.data();
    std::vector<uint32_t> hist((size_t)nt * 256);
    for (int pass = 0; pass < 4; ++pass) {
        const int shift = pass * 8;
        std::fill(hist.begin(), hist.end(), 0u);
#pragma omp parallel num_threads(nt)
        {
            int t = 0;
#ifdef _OPENMP
            t = omp_get_thread_num();
#endif
            const uint64_t lo = (uint64_t)n * t / nt, hi = (uint64_t)n * (t + 1) / nt;
            uint32_t *h = &hist[(size_t)t * 256];
            for (uint64_t i = lo; i < hi; ++i) h[(ka[i] >> shift) & 255u]++;
#pragma omp barrier
#pragma omp single
            {
                uint32_t run = 0;
                for (int d = 0; d < 256; ++d)
                    for (int tt = 0; tt < nt; ++tt) {
                        const uint32_t c = hist[(size_t)tt * 256 + d];
                        hist[(size_t)tt * 256 + d] = run;
                        run += c;
                    }
            }
            for (uint64_t i = lo; i < hi; ++i) {
                const uint32_t d = (ka[i] >> shift) & 255u;
                const uint32_t p = h[d]++;
                kb[p] = ka[i];
                vb[p] = va[i];
            }
        }
        std::swap(ka, kb);
        std::swap(va, vb);
    }
    // After 4 passes the data is back in the caller's arrays.
}

void oracle_clear(uint8_t *rgba, uint32_t w, uint32_t h) {
    for (size_t i = 0; i < (size_t)w * h; ++i) {
        rgba[i * 4 + 0] = 0;
        rgba[i * 4 + 1] = 0;
        rgba[i * 4 + 2] = 0;
        rgba[i * 4 + 3] = 255;
    }
}

// Blend `count` splats in `order` onto `rgba` (not cleared here).  exp_mode 0 = the portable
// exp shared with the CUDA bit-exact mode, 1 = libm expf.  threads == 0 runs the literal
// per-instance quad rasteriser; threads >= 1 the tile-parallel one (same result).
void oracle_rasterize(const gs_frame_uniforms *u, const gs_splat *splats, const uint32_t *order,
                      uint32_t count, uint8_t *rgba, uint32_t w, uint32_t h, int exp_mode,
                      int threads) {
    if (threads <= 0)
        raster_brute(*u, splats, order, count, rgba, w, h, exp_mode);
    else
        raster_tiled(*u, splats, order, count, rgba, w, h, exp_mode, threads);
}

float oracle_exp_portable(float x) { return exp_portable(x); }

// The frame through the reference's own vertex stage (draw_instance): the same preprocess,
// stable depth sort and cleared target, then every visible instance's two triangles in draw
// order.  Single-threaded; a parity check of the quad map, sized for small frames.  Returns V.
uint32_t oracle_render_quads(const gs_camera_pod *cam, const gs_frame_uniforms *u, const void *gaussians,
                             uint32_t format, uint32_t n, uint32_t *indices, float *depths, uint8_t *rgba,
                             uint32_t w, uint32_t h, int clear) {
    const uint32_t v = oracle_preprocess(u, gaussians, format, n, nullptr, 0, indices, depths, nullptr, 1);
    oracle_stable_sort((uint32_t *)depths, indices, v);
    if (clear) oracle_clear(rgba, w, h);
    for (uint32_t k = 0; k < v; ++k) draw_instance(*u, *cam, load_record(gaussians, format, indices[k]), rgba, w, h);
    return v;
}

// Full frame: preprocess -> stable sort -> clear -> raster.  Scratch arrays are caller-sized
// (indices/depths: n; splats: n).  Returns V.
uint32_t oracle_render(const gs_frame_uniforms *u, const void *gaussians, uint32_t format,
                       uint32_t n, uint32_t *indices, float *depths, gs_splat *splats,
                       uint8_t *rgba, uint32_t w, uint32_t h, int exp_mode, int threads,
                       int clear) {
    const uint32_t v = oracle_preprocess(u, gaussians, format, n, nullptr, 0, indices, depths,
                                         splats, threads);
    if (threads > 1)
        oracle_radix_sort((uint32_t *)depths, indices, v, threads);
    else
        oracle_stable_sort((uint32_t *)depths, indices, v);
    if (clear) oracle_clear(rgba, w, h);
    oracle_rasterize(u, splats, indices, v, rgba, w, h, exp_mode, threads);
    return v;
}

}  // extern "C"
