// gs_oracle64.cpp — FP64 twin of the CPU oracle (test and measurement infrastructure only).
//
// The same pipeline as gs_oracle.cpp — preprocess (src/shader/preprocess.wesl:60-126,
// utils.wesl:18-135, render.wesl:58-130), stable depth sort, per-fragment back-to-front
// ALPHA_BLENDING with the 8-bit store of a Rgba8Unorm target (render.wesl:143-181,
// renderer.rs:162-195) — evaluated in double precision from the same FP32 pods and records
// (compressed records are decoded exactly).  It is the error reference of the precision tier:
// frames rendered from FP16/BF16 records are compared with it by PSNR.
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

using D = double;

void m4mul(const D *a, const D *b, D *o) {
    D t[16];
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) {
            D s = 0;
            for (int k = 0; k < 4; ++k) s += a[k * 4 + r] * b[c * 4 + k];
            t[c * 4 + r] = s;
        }
    std::memcpy(o, t, sizeof(t));
}

void m4vec(const D *m, const D *v, D *o) {
    for (int r = 0; r < 4; ++r) o[r] = m[r] * v[0] + m[4 + r] * v[1] + m[8 + r] * v[2] + m[12 + r] * v[3];
}

void m3vec(const D *m, const D *v, D *o) {
    for (int r = 0; r < 3; ++r) o[r] = m[r] * v[0] + m[3 + r] * v[1] + m[6 + r] * v[2];
}

void quat3(const D *q, D *m) {
    const D x = q[0], y = q[1], z = q[2], w = q[3];
    m[0] = 1 - 2 * (y * y + z * z);
    m[1] = 2 * (x * y + w * z);
    m[2] = 2 * (x * z - w * y);
    m[3] = 2 * (x * y - w * z);
    m[4] = 1 - 2 * (x * x + z * z);
    m[5] = 2 * (y * z + w * x);
    m[6] = 2 * (x * z + w * y);
    m[7] = 2 * (y * z - w * x);
    m[8] = 1 - 2 * (x * x + y * y);
}

D half_d(uint16_t h) {
    const int s = (h >> 15) & 1, e = (h >> 10) & 31, m = h & 1023;
    D v;
    if (e == 0) v = std::ldexp((D)m, -24);
    else if (e == 31) v = m ? NAN : INFINITY;
    else v = std::ldexp((D)(m | 1024), e - 25);
    return s ? -v : v;
}

D bf16_d(uint16_t h) {
    uint32_t b = (uint32_t)h << 16;
    float f;
    std::memcpy(&f, &b, 4);
    return f;
}

bool cull(D x, D y, D z) { return !(x >= -1 && y >= -1 && z >= 0 && x <= 1 && y <= 1 && z <= 1); }

struct U {
    D pv[16], vm[16], model[16], wsr[9], inv_sr[9], cam[3], size[2], focal[2], vp[2];
    D std, stds, psize;
    uint32_t mode, sh_deg, no_sh0;
};

U make_uniforms(const gs_camera_pod &c, const gs_model_transform_pod &mt, const gs_gaussian_transform_pod &gt,
                uint32_t w, uint32_t h) {
    U u{};
    D view[16], proj[16];
    for (int i = 0; i < 16; ++i) {
        view[i] = c.view[i];
        proj[i] = c.proj[i];
    }
    m4mul(proj, view, u.pv);
    D q[4] = {mt.rot[0], mt.rot[1], mt.rot[2], mt.rot[3]}, R[9], SR[9];
    quat3(q, R);
    for (int cc = 0; cc < 3; ++cc)
        for (int r = 0; r < 3; ++r) SR[cc * 3 + r] = R[cc * 3 + r] * (D)mt.scale[cc];
    std::memset(u.model, 0, sizeof(u.model));
    for (int cc = 0; cc < 3; ++cc)
        for (int r = 0; r < 3; ++r) u.model[cc * 4 + r] = SR[cc * 3 + r];
    u.model[12] = mt.pos[0];
    u.model[13] = mt.pos[1];
    u.model[14] = mt.pos[2];
    u.model[15] = 1;
    m4mul(view, u.model, u.vm);
    D W[9];
    for (int cc = 0; cc < 3; ++cc)
        for (int r = 0; r < 3; ++r) W[cc * 3 + r] = view[cc * 4 + r];
    for (int cc = 0; cc < 3; ++cc)
        for (int r = 0; r < 3; ++r) {
            D s = 0;
            for (int k = 0; k < 3; ++k) s += W[k * 3 + r] * SR[cc * 3 + k];
            u.wsr[cc * 3 + r] = s;
        }
    for (int cc = 0; cc < 3; ++cc)
        for (int r = 0; r < 3; ++r) u.inv_sr[cc * 3 + r] = R[r * 3 + cc] / (D)mt.scale[r];
    for (int i = 0; i < 3; ++i)
        u.cam[i] = -(W[i * 3] * view[12] + W[i * 3 + 1] * view[13] + W[i * 3 + 2] * view[14]);
    u.size[0] = c.size[0];
    u.size[1] = c.size[1];
    u.focal[0] = proj[0] * u.size[0] * 0.5;
    u.focal[1] = proj[5] * u.size[1] * 0.5;
    u.vp[0] = w;
    u.vp[1] = h;
    u.std = gt.max_std_dev;
    u.stds = (D)gt.max_std_dev * (D)gt.size;
    u.psize = gt.size;
    u.mode = gt.display_mode;
    u.sh_deg = gt.sh_deg;
    u.no_sh0 = gt.no_sh0;
    return u;
}

struct Rec {
    D pos[3], sh[45], cov[6];
    uint32_t color;
};

Rec load(const void *base, uint32_t fmt, uint32_t i) {
    Rec r;
    if (fmt == GS_FORMAT_FP32) {
        const gs_gaussian_pod *g = (const gs_gaussian_pod *)base + i;
        for (int k = 0; k < 3; ++k) r.pos[k] = g->pos[k];
        for (int k = 0; k < 45; ++k) r.sh[k] = g->sh[k];
        for (int k = 0; k < 6; ++k) r.cov[k] = g->cov3d[k];
        r.color = g->color;
        return r;
    }
    const gs_gaussian_pod_half *g = (const gs_gaussian_pod_half *)base + i;
    for (int k = 0; k < 3; ++k) r.pos[k] = g->pos[k];
    for (int k = 0; k < 45; ++k) r.sh[k] = fmt == GS_FORMAT_HALF_SH_BF16 ? bf16_d(g->sh[k]) : half_d(g->sh[k]);
    r.color = g->color;
    D q[4], s[3], R[9];
    for (int k = 0; k < 4; ++k) q[k] = half_d(g->rot[k]);
    for (int k = 0; k < 3; ++k) s[k] = half_d(g->scale[k]);
    const D n = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
    for (int k = 0; k < 4; ++k) q[k] /= n;
    quat3(q, R);
    D M[9];
    for (int c = 0; c < 3; ++c)
        for (int rr = 0; rr < 3; ++rr) M[c * 3 + rr] = R[c * 3 + rr] * s[c];
    auto cv = [&](int a, int b) { return M[a] * M[b] + M[3 + a] * M[3 + b] + M[6 + a] * M[6 + b]; };
    r.cov[0] = cv(0, 0);
    r.cov[1] = cv(0, 1);
    r.cov[2] = cv(0, 2);
    r.cov[3] = cv(1, 1);
    r.cov[4] = cv(1, 2);
    r.cov[5] = cv(2, 2);
    return r;
}

void axes_of(const U &u, const Rec &g, const D *p4, D sd, D *ax) {
    D t[4];
    m4vec(u.vm, p4, t);
    const D j00 = u.focal[0] / t[2], j02 = -(u.focal[0] * t[0]) / (t[2] * t[2]);
    const D j11 = u.focal[1] / t[2], j12 = -(u.focal[1] * t[1]) / (t[2] * t[2]);
    D T0[3], T1[3];
    for (int k = 0; k < 3; ++k) {
        T0[k] = j00 * u.wsr[k * 3] + j02 * u.wsr[k * 3 + 2];
        T1[k] = j11 * u.wsr[k * 3 + 1] + j12 * u.wsr[k * 3 + 2];
    }
    const D *c = g.cov;
    const D V[9] = {c[0], c[1], c[2], c[1], c[3], c[4], c[2], c[4], c[5]};
    D U0[3], U1[3];
    for (int k = 0; k < 3; ++k) {
        U0[k] = T0[0] * V[k * 3] + T0[1] * V[k * 3 + 1] + T0[2] * V[k * 3 + 2];
        U1[k] = T1[0] * V[k * 3] + T1[1] * V[k * 3 + 1] + T1[2] * V[k * 3 + 2];
    }
    const D a = U0[0] * T0[0] + U0[1] * T0[1] + U0[2] * T0[2];
    const D b = U0[0] * T1[0] + U0[1] * T1[1] + U0[2] * T1[2];
    const D cc = U1[0] * T1[0] + U1[1] * T1[1] + U1[2] * T1[2];
    const D mid = 0.5 * (a + cc), rad = std::hypot(0.5 * (a - cc), b);
    const D l1 = mid + rad, l2 = mid - rad;
    if (l2 < 0) {
        ax[0] = ax[1] = ax[2] = ax[3] = 0;
        return;
    }
    D dx = b, dy = l1 - a, ux, uy;
    if (dx == 0 && dy == 0) {
        ux = 0;
        uy = 1;
    } else {
        const D l = std::hypot(dx, dy);
        ux = dx / l;
        uy = dy / l;
    }
    const D L1 = std::min(sd * std::sqrt(l1), 1024.0), L2 = std::min(sd * std::sqrt(l2), 1024.0);
    ax[0] = L1 * ux;
    ax[1] = L1 * uy;
    ax[2] = L2 * uy;
    ax[3] = -L2 * ux;
}

void color_of(const U &u, const Rec &g, const D *world, D *rgba) {
    const D vd[3] = {u.cam[0] - world[0], u.cam[1] - world[1], u.cam[2] - world[2]};
    D m[3];
    m3vec(u.inv_sr, vd, m);
    const D l = std::sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
    const D x = -m[0] / l, y = -m[1] / l, z = -m[2] / l;
    const D C1 = 0.4886025, C2[5] = {1.0925484, -1.0925484, 0.3153916, -1.0925484, 0.5462742};
    const D C3[7] = {-0.5900436, 2.8906114, -0.4570458, 0.3731763, -0.4570458, 1.4453057, -0.5900436};
    const D *sh = g.sh;
    for (int ch = 0; ch < 3; ++ch) {
        D r = u.no_sh0 ? 0.5 : (D)((g.color >> (8 * ch)) & 255u) / 255.0;
        if (u.sh_deg >= 1) {
            r += C1 * (-sh[ch] * y + sh[3 + ch] * z - sh[6 + ch] * x);
            if (u.sh_deg >= 2) {
                const D xx = x * x, yy = y * y, zz = z * z, xy = x * y, yz = y * z, xz = x * z;
                r += C2[0] * xy * sh[9 + ch] + C2[1] * yz * sh[12 + ch] + C2[2] * (2 * zz - xx - yy) * sh[15 + ch] +
                     C2[3] * xz * sh[18 + ch] + C2[4] * (xx - yy) * sh[21 + ch];
                if (u.sh_deg >= 3)
                    r += C3[0] * y * (3 * xx - yy) * sh[24 + ch] + C3[1] * xy * z * sh[27 + ch] +
                         C3[2] * y * (4 * zz - xx - yy) * sh[30 + ch] +
                         C3[3] * z * (2 * zz - 3 * xx - 3 * yy) * sh[33 + ch] +
                         C3[4] * x * (4 * zz - xx - yy) * sh[36 + ch] + C3[5] * z * (xx - yy) * sh[39 + ch] +
                         C3[6] * x * (xx - 3 * yy) * sh[42 + ch];
            }
        }
        rgba[ch] = r > 0 ? r : 0;
    }
    rgba[3] = (D)((g.color >> 24) & 255u) / 255.0;
}

struct S64 {
    D cx, cy, ex, ey, q[4], s255[3], alpha;
};

bool pre(const U &u, const Rec &g, S64 *s, D *key) {
    const D p4[4] = {g.pos[0], g.pos[1], g.pos[2], 1};
    D world[4], clip[4];
    m4vec(u.model, p4, world);
    m4vec(u.pv, world, clip);
    const D nx = clip[0] / clip[3], ny = clip[1] / clip[3], nz = clip[2] / clip[3];
    D ax[4];
    bool have = false;
    if (cull(nx, ny, nz)) {
        axes_of(u, g, p4, u.stds, ax);
        have = true;
        const D mx = ax[0] * u.std / u.size[0], my = ax[1] * u.std / u.size[1];
        const D ml = std::hypot(mx, my), nl = std::hypot(nx, ny);
        const D m = std::min(ml, nl);
        if (cull(nx - m * nx / nl, ny - m * ny / nl, nz)) return false;
    }
    *key = 1 - nz;
    D rgba[4];
    color_of(u, g, world, rgba);
    const D W = u.vp[0], H = u.vp[1];
    s->cx = (nx + 1) * W * 0.5;
    s->cy = (1 - ny) * H * 0.5;
    for (int c = 0; c < 3; ++c) s->s255[c] = std::min(std::max(rgba[c], 0.0), 1.0) * 255.0;
    s->alpha = rgba[3];
    const D std2 = u.std * u.std;
    if (u.mode == GS_DISPLAY_POINT) {
        D vp[4];
        m4vec(u.vm, p4, vp);
        const D l = std::sqrt(vp[0] * vp[0] + vp[1] * vp[1] + vp[2] * vp[2]);
        const D pnd = 0.01 * u.psize / l;
        s->q[0] = pnd * (u.size[1] / u.size[0]) * 0.5 * W;
        s->q[1] = pnd * 0.5 * H;
        s->q[2] = s->q[3] = 0;
        s->ex = s->q[0] * 1.001 + 0.01;
        s->ey = s->q[1] * 1.001 + 0.01;
        if (!(s->q[0] > 0 && s->q[1] > 0 && std::isfinite(s->q[0]) && std::isfinite(s->q[1]))) s->ex = -1;
        return true;
    }
    if (!have) axes_of(u, g, p4, u.stds, ax);
    const D kx = 0.5 * W / u.size[0], ky = 0.5 * H / u.size[1];
    const D a00 = ax[0] * kx, a01 = ax[2] * kx, a10 = -ax[1] * ky, a11 = -ax[3] * ky;
    const D det = a00 * a11 - a01 * a10;
    s->q[0] = a11 / det;
    s->q[1] = -a01 / det;
    s->q[2] = -a10 / det;
    s->q[3] = a00 / det;
    D r2 = std2;
    if (u.mode == GS_DISPLAY_SPLAT) r2 = s->alpha > 0 ? std::min(std2, std::log(512.0 * s->alpha) + 0.01) : -1;
    if (det != 0 && std::isfinite(det) && r2 >= 0) {
        s->ex = std::sqrt(r2 * (a00 * a00 + a01 * a01)) * 1.001 + 0.01;
        s->ey = std::sqrt(r2 * (a10 * a10 + a11 * a11)) * 1.001 + 0.01;
    } else {
        s->ex = -1;
    }
    return true;
}

}  // namespace

extern "C" {

// Whole frame in FP64 (clear + preprocess + stable depth sort + tile-parallel blend).
// Returns the number of visible Gaussians.
uint32_t oracle64_render(const gs_camera_pod *cam, const gs_model_transform_pod *mt,
                         const gs_gaussian_transform_pod *gt, const void *records, uint32_t format, uint32_t n,
                         uint8_t *rgba, uint32_t w, uint32_t h, int threads) {
    const U u = make_uniforms(*cam, *mt, *gt, w, h);
    const int nt = threads > 0 ? threads : 1;
    std::vector<S64> spl(n);
    std::vector<D> key(n);
    std::vector<uint8_t> vis(n);
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int64_t i = 0; i < (int64_t)n; ++i) vis[i] = pre(u, load(records, format, (uint32_t)i), &spl[i], &key[i]);
    std::vector<uint32_t> order;
    for (uint32_t i = 0; i < n; ++i)
        if (vis[i]) order.push_back(i);
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return key[a] < key[b]; });
    for (size_t i = 0; i < (size_t)w * h; ++i) {
        rgba[4 * i] = rgba[4 * i + 1] = rgba[4 * i + 2] = 0;
        rgba[4 * i + 3] = 255;
    }
    const uint32_t T = GS_TILE, tx = (w + T - 1) / T, ty = (h + T - 1) / T;
    std::vector<std::vector<uint32_t>> bins((size_t)tx * ty);
    for (uint32_t k = 0; k < order.size(); ++k) {
        const S64 &s = spl[order[k]];
        if (!(s.ex >= 0)) continue;
        const long x0 = std::max(0L, (long)std::floor((s.cx - s.ex) / T)), x1 = std::min((long)tx - 1, (long)std::floor((s.cx + s.ex) / T));
        const long y0 = std::max(0L, (long)std::floor((s.cy - s.ey) / T)), y1 = std::min((long)ty - 1, (long)std::floor((s.cy + s.ey) / T));
        for (long yy = y0; yy <= y1; ++yy)
            for (long xx = x0; xx <= x1; ++xx) bins[(size_t)yy * tx + xx].push_back(order[k]);
    }
    const D std2 = u.std * u.std, o2 = (u.std - 0.1) * (u.std - 0.1);
#pragma omp parallel for schedule(dynamic, 4) num_threads(nt)
    for (int64_t tile = 0; tile < (int64_t)bins.size(); ++tile) {
        const uint32_t bx = (uint32_t)tile % tx, by = (uint32_t)tile / tx;
        for (uint32_t gi : bins[tile]) {
            const S64 &s = spl[gi];
            for (uint32_t py = by * T; py < std::min(h, by * T + T); ++py)
                for (uint32_t px = bx * T; px < std::min(w, bx * T + T); ++px) {
                    const D dx = px + 0.5 - s.cx, dy = py + 0.5 - s.cy;
                    D al;
                    if (u.mode == GS_DISPLAY_POINT) {
                        if (!(dx >= -s.q[0] && dx < s.q[0] && dy >= -s.q[1] && dy < s.q[1])) continue;
                        al = 1;
                    } else {
                        const D qx = s.q[0] * dx + s.q[1] * dy, qy = s.q[2] * dx + s.q[3] * dy, r2 = qx * qx + qy * qy;
                        if (!(r2 <= std2)) continue;
                        al = u.mode == GS_DISPLAY_SPLAT ? s.alpha * std::exp(-r2) : (r2 > o2 ? 1.0 : s.alpha);
                    }
                    uint8_t *p = rgba + ((size_t)py * w + px) * 4;
                    for (int c = 0; c < 3; ++c) p[c] = (uint8_t)std::nearbyint(p[c] * (1 - al) + s.s255[c] * al);
                }
        }
    }
    return (uint32_t)order.size();
}

}  // extern "C"
