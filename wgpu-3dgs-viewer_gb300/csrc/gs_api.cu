// gs_api.cu — the C ABI (include/gs300.h): host-side camera/transform math, stage entry points
// over caller-owned device buffers, and the Viewer / MultiModelViewer facades.
//
// Host FP32 math is compiled with -ffp-contract=off and follows the evaluation order of the
// kernels, so frame uniforms built here are bit-identical to the oracle's.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <thread>
#include <unordered_map>
#include <mutex>
#include <string>
#include <vector>

#include "gs300.h"
#include "gs_internal.h"

using namespace gs;

namespace {

thread_local std::string g_last_error;

gs_status fail(gs_status s, const char *fmt, ...) __attribute__((format(printf, 2, 3)));
gs_status fail(gs_status s, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return s;
}

gs_status cuda_fail(cudaError_t e, const char *what) {
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return fail(GS_ERR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
    }
    return fail(GS_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define GS_CUDA(call)                                      \
    do {                                                   \
        cudaError_t e_ = (call);                           \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

// ---- host FP32 linear algebra (column-major), same order as the kernels ----
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

size_t record_bytes(uint32_t format) {
    return format == GS_FORMAT_FP32 ? sizeof(gs_gaussian_pod) : sizeof(gs_gaussian_pod_half);
}

bool valid_format(uint32_t f) {
    return f == GS_FORMAT_FP32 || f == GS_FORMAT_HALF_SH_FP16 || f == GS_FORMAT_HALF_SH_BF16;
}

gs_status check_gaussian_transform(const gs_gaussian_transform_pod *p) {
    if (!p) return fail(GS_ERR_INVALID_ARG, "gaussian transform pod is NULL");
    if (p->display_mode > GS_DISPLAY_POINT)
        return fail(GS_ERR_INVALID_ARG, "display mode %u is not splat/ellipse/point", p->display_mode);
    if (p->sh_deg > 3) return fail(GS_ERR_INVALID_ARG, "SH degree %u out of range 0..=3", p->sh_deg);
    if (!(p->max_std_dev >= 0.0f && p->max_std_dev <= 3.0f))
        return fail(GS_ERR_INVALID_ARG, "max std dev %g out of range 0..=3", (double)p->max_std_dev);
    return GS_OK;
}

bool aligned(const void *p, size_t a) { return ((uintptr_t)p % a) == 0; }

// Device allocation owned by a facade.
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    ~DevBuf() { release(); }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    cudaError_t ensure(size_t b) {
        if (b <= bytes && ptr) return cudaSuccess;
        release();
        cudaError_t e = cudaMalloc(&ptr, b ? b : 256);
        if (e == cudaSuccess) bytes = b;
        return e;
    }
    // A scratch area: grown when too small, zero-filled only when (re)allocated — a reused area
    // needs no clearing whatever sizes its next calls use (fixed-offset flag arena).
    cudaError_t ensure_zeroed(size_t b) {
        if (b <= bytes && ptr) return cudaSuccess;
        cudaError_t e = ensure(b);
        if (e == cudaSuccess) e = cudaMemset(ptr, 0, bytes);
        return e;
    }
};

gs_status status_from_bits(uint32_t bits, const char *what) {
    if (bits & kStatusTimeout) return fail(GS_ERR_TIMEOUT, "%s: a bounded device wait gave up", what);
    if (bits & kStatusBounds) return fail(GS_ERR_CUDA, "%s: a device index check failed", what);
    if (bits & kStatusCapacity) return fail(GS_ERR_CAPACITY, "%s: tile-pair list exceeded its capacity", what);
    return GS_OK;
}

uint32_t default_pairs(uint32_t n, uint32_t w, uint32_t h) {
    uint64_t p = (uint64_t)n * 8u + (uint64_t)((w + 15) / 16) * ((h + 15) / 16) * 4u + 4096u;
    if (p > 0x7FFFFFFFull) p = 0x7FFFFFFFull;
    return (uint32_t)p;
}

// Per-model device state shared by both facades.
struct Model {
    uint32_t n = 0, format = GS_FORMAT_FP32;
    DevBuf records, control, indices, depths, splats, pre_scratch, sort_scratch, selection;
    DevBuf binfo;  // each visible splat's tiles, written by the preprocess of a one-model view
    int invert = 0;
    bool has_selection = false;
    gs_model_transform_pod model{};
    uint32_t *indirect() { return reinterpret_cast<uint32_t *>(control.ptr); }  // [0..4) args, [4..7) dispatch

    gs_status create(const void *host, uint32_t count, uint32_t fmt) {
        if (count > 0 && !host) return fail(GS_ERR_INVALID_ARG, "records pointer is NULL");
        const gs_status s = alloc(count, fmt);
        if (s != GS_OK) return s;
        if (n) GS_CUDA(cudaMemcpy(records.ptr, host, (size_t)n * record_bytes(fmt), cudaMemcpyHostToDevice));
        return GS_OK;
    }

    // Records converted on the device from the vertex block of a PLY file in host memory.
    gs_status create_from_ply(const void *bytes, size_t len, uint32_t fmt) {
        gs_ply_layout L;
        gs_status s = gs_ply_parse_header(bytes, len, &L);
        if (s != GS_OK) return s;
        const uint64_t block = (uint64_t)L.count * L.stride;
        if (L.data_offset > len || block > len - L.data_offset)
            return fail(GS_ERR_INVALID_ARG, "PLY file holds %zu bytes, its header needs %llu", len,
                        (unsigned long long)(L.data_offset + block));
        s = alloc(L.count, fmt);
        if (s != GS_OK) return s;
        if (!n) return GS_OK;
        DevBuf vertices;
        GS_CUDA(vertices.ensure(block));
        GS_CUDA(cudaMemcpy(vertices.ptr, static_cast<const uint8_t *>(bytes) + L.data_offset, block,
                           cudaMemcpyHostToDevice));
        GS_CUDA(launch_ply_convert(vertices.ptr, L, fmt, records.ptr, nullptr));
        GS_CUDA(cudaStreamSynchronize(nullptr));
        return GS_OK;
    }

    gs_status alloc(uint32_t count, uint32_t fmt) {
        if (!valid_format(fmt)) return fail(GS_ERR_INVALID_ARG, "unknown record format %u", fmt);
        n = count;
        format = fmt;
        model = gs_model_transform_pod{};
        model.rot[3] = 1.0f;
        model.scale[0] = model.scale[1] = model.scale[2] = 1.0f;
        const size_t rb = record_bytes(fmt);
        GS_CUDA(records.ensure((size_t)n * rb));
        GS_CUDA(control.ensure(64));
        GS_CUDA(cudaMemset(control.ptr, 0, 64));
        GS_CUDA(indices.ensure((size_t)n * 4));
        GS_CUDA(depths.ensure((size_t)gs_depth_capacity(n) * 4));
        GS_CUDA(splats.ensure((size_t)n * sizeof(gs_splat)));
        GS_CUDA(pre_scratch.ensure(preprocess_scratch_bytes(n)));
        GS_CUDA(cudaMemset(pre_scratch.ptr, 0, pre_scratch.bytes));
        GS_CUDA(sort_scratch.ensure(sort_scratch_bytes(n, kDepthKeyBits)));
        GS_CUDA(cudaMemset(sort_scratch.ptr, 0, sort_scratch.bytes));
        return GS_OK;
    }

    // Preprocess + depth sort of this model for one frame.  `tiles`: the preprocess also stores
    // each visible splat's tiles for the viewport (binfo), which the binning of a one-model view
    // gathers instead of the whole splat.
    gs_status enqueue(const gs_frame_uniforms &u, cudaStream_t st, bool tiles = false) {
        uint4 *bi = nullptr;
        if (tiles && n) {
            GS_CUDA(binfo.ensure((size_t)n * sizeof(uint4)));
            bi = reinterpret_cast<uint4 *>(binfo.ptr);
        }
        cudaError_t e = launch_preprocess(u, records.ptr, format, n,
                                          has_selection ? (const uint32_t *)selection.ptr : nullptr, invert,
                                          indirect(), indirect() + 4, (uint32_t *)indices.ptr, (float *)depths.ptr,
                                          gs_depth_capacity(n), (gs_splat *)splats.ptr, pre_scratch.ptr, st, nullptr,
                                          bi);
        if (e != cudaSuccess) return cuda_fail(e, "preprocess launch");
        e = launch_sort((uint32_t *)depths.ptr, (uint32_t *)indices.ptr, n, indirect() + 1, kDepthKeyBits,
                        sort_scratch.ptr, st);
        if (e != cudaSuccess) return cuda_fail(e, "sort launch");
        return GS_OK;
    }

    gs_status set_selection(const uint32_t *bits, int inv) {
        if (!bits) {
            has_selection = false;
            return GS_OK;
        }
        const size_t words = ((size_t)n + 31) / 32;
        GS_CUDA(selection.ensure(words * 4 + 4));
        if (words) GS_CUDA(cudaMemcpy(selection.ptr, bits, words * 4, cudaMemcpyHostToDevice));
        has_selection = true;
        invert = inv;
        return GS_OK;
    }

    uint32_t device_status() {
        Ctrl a{}, b{};
        if (pre_scratch.ptr) cudaMemcpy(&a, pre_scratch.ptr, sizeof(Ctrl), cudaMemcpyDeviceToHost);
        if (sort_scratch.ptr) cudaMemcpy(&b, sort_scratch.ptr, sizeof(Ctrl), cudaMemcpyDeviceToHost);
        return a.status | b.status;
    }
};

// Shared render state: camera/Gaussian-transform pods, raster scratch and last-frame args.
struct Frame {
    gs_camera_pod camera{};
    gs_gaussian_transform_pod gt{};
    DevBuf raster_scratch;
    uint32_t max_pairs = 0, scratch_splats = 0, scratch_w = 0, scratch_h = 0;
    uint8_t *last_target = nullptr;
    uint32_t last_w = 0, last_h = 0, last_pitch = 0;
    bool rendered = false;
    int exact_exp = 0;

    Frame() {
        gt.size = 1.0f;
        gt.display_mode = GS_DISPLAY_SPLAT;
        gt.sh_deg = 3;
        gt.no_sh0 = 0;
        gt.max_std_dev = 3.0f;
    }

    // Raster scratch for `splats` splats at w x h.  It only grows: a frame at a smaller size is
    // laid out inside the larger area (its flag arena sits at a fixed offset and is cleared on
    // the device where a layout grows), so changing resolution or models allocates nothing once
    // the largest frame has been seen.
    gs_status ensure_scratch(uint32_t splats, uint32_t w, uint32_t h) {
        const uint32_t want = default_pairs(splats, w, h);
        if (want > max_pairs) max_pairs = want;
        GS_CUDA(raster_scratch.ensure_zeroed(raster_scratch_bytes(splats, w, h, max_pairs)));
        scratch_splats = splats;
        scratch_w = w;
        scratch_h = h;
        return GS_OK;
    }

    gs_status grow_pairs(uint32_t wanted) {
        uint64_t p = (uint64_t)wanted + wanted / 4 + 4096;
        if (p > 0x7FFFFFFFull) p = 0x7FFFFFFFull;
        if (p <= max_pairs) return fail(GS_ERR_CAPACITY, "tile-pair list cannot grow beyond %u", max_pairs);
        max_pairs = (uint32_t)p;
        raster_scratch.release();
        return ensure_scratch(scratch_splats, scratch_w, scratch_h);
    }
};

gs_status check_target(const uint8_t *target, uint32_t w, uint32_t h, uint32_t pitch) {
    if (!target) return fail(GS_ERR_INVALID_ARG, "target is NULL");
    if (w == 0 || h == 0) return fail(GS_ERR_INVALID_ARG, "target size %ux%u is empty", w, h);
    if (pitch < 4u * w || pitch % 4u != 0 || !aligned(target, 4))
        return fail(GS_ERR_INVALID_ARG, "target pitch %u / alignment invalid for width %u", pitch, w);
    return GS_OK;
}

}  // namespace

// ---- stage timers and launch counter ---------------------------------------------------------
namespace gs {
gs_status set_error(gs_status status, const char *message) { return fail(status, "%s", message); }

namespace {
std::atomic<uint64_t> g_launches{0};
std::mutex g_prof_mu;
bool g_prof_on = false;
bool g_prof_count = false;  // splat frames use the counting rasteriser
struct StageEvents {
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pairs;
    size_t used = 0;
    bool open = false;
};
StageEvents g_prof[kProfStages];
}  // namespace

// While a batch graph is being captured on this thread, launches are counted into the graph
// (and charged on every replay) and stage timers are off.
thread_local bool t_capturing = false;
thread_local uint64_t t_captured_launches = 0;

void count_launches(uint32_t n) {
    if (t_capturing) t_captured_launches += n;
    else g_launches.fetch_add(n, std::memory_order_relaxed);
}

bool prof_counting() { return g_prof_on && g_prof_count; }

// Look-back configuration of every launch (spin limit in the low word, stalled tile in the high).
namespace {
std::atomic<uint64_t> g_wait_cfg{((uint64_t)kNoStall << 32) | kSpinLimit};
}  // namespace

WaitCfg wait_config() {
    const uint64_t v = g_wait_cfg.load(std::memory_order_relaxed);
    WaitCfg c;
    c.spin_limit = (uint32_t)v;
    c.stall_tile = (uint32_t)(v >> 32);
    return c;
}

void prof_mark(int stage, bool begin, cudaStream_t st) {
    if (!g_prof_on || t_capturing) return;
    std::lock_guard<std::mutex> g(g_prof_mu);
    StageEvents &e = g_prof[stage];
    if (begin) {
        if (e.used == e.pairs.size()) {
            cudaEvent_t a, b;
            if (cudaEventCreate(&a) != cudaSuccess) return;
            if (cudaEventCreate(&b) != cudaSuccess) return;
            e.pairs.emplace_back(a, b);
        }
        cudaEventRecord(e.pairs[e.used].first, st);
        e.open = true;
    } else if (e.open) {
        cudaEventRecord(e.pairs[e.used].second, st);
        ++e.used;
        e.open = false;
    }
}
}  // namespace gs

// =============================================================================================
extern "C" {

const char *gs_last_error(void) { return g_last_error.c_str(); }
const char *gs_version(void) { return "gs300 0.1.0 sm_103a"; }

uint64_t gs_launch_count(void) { return gs::g_launches.load(); }

gs_status gs_profile_counters(uint64_t out[4]) {
    if (!out) return fail(GS_ERR_INVALID_ARG, "NULL argument");
    GS_CUDA(cudaDeviceSynchronize());
    unsigned long long c[4];
    GS_CUDA(gs::raster_counters(c, false));
    for (int i = 0; i < 4; ++i) out[i] = c[i];
    return GS_OK;
}

gs_status gs_profile_enable(int enable) {
    unsigned long long discard[4];
    GS_CUDA(gs::raster_counters(discard, true));
    std::lock_guard<std::mutex> g(gs::g_prof_mu);
    for (auto &e : gs::g_prof) {
        e.used = 0;
        e.open = false;
    }
    gs::g_prof_on = enable != 0;
    gs::g_prof_count = enable == 2;
    return GS_OK;
}

gs_status gs_profile_read(double *ms, uint32_t *launches) {
    GS_CUDA(cudaDeviceSynchronize());
    std::lock_guard<std::mutex> g(gs::g_prof_mu);
    for (int s = 0; s < gs::kProfStages; ++s) {
        double acc = 0.0;
        for (size_t i = 0; i < gs::g_prof[s].used; ++i) {
            float t = 0.0f;
            GS_CUDA(cudaEventElapsedTime(&t, gs::g_prof[s].pairs[i].first, gs::g_prof[s].pairs[i].second));
            acc += t;
        }
        if (ms) ms[s] = acc;
        if (launches) launches[s] = (uint32_t)gs::g_prof[s].used;
    }
    return GS_OK;
}

gs_status gs_camera_view(const gs_camera *c, float out[16]) {
    if (!c || !out) return fail(GS_ERR_INVALID_ARG, "NULL argument");
    const float f[3] = {std::cos(c->pitch) * std::sin(c->yaw), std::sin(c->pitch), std::cos(c->pitch) * std::cos(c->yaw)};
    // look_to_rh(eye, dir, up = +Y)
    float l = std::sqrt((f[0] * f[0] + f[1] * f[1]) + f[2] * f[2]);
    const float fn[3] = {f[0] / l, f[1] / l, f[2] / l};
    const float up[3] = {0.0f, 1.0f, 0.0f};
    float s[3] = {fn[1] * up[2] - fn[2] * up[1], fn[2] * up[0] - fn[0] * up[2], fn[0] * up[1] - fn[1] * up[0]};
    l = std::sqrt((s[0] * s[0] + s[1] * s[1]) + s[2] * s[2]);
    s[0] = s[0] / l;
    s[1] = s[1] / l;
    s[2] = s[2] / l;
    const float u[3] = {s[1] * fn[2] - s[2] * fn[1], s[2] * fn[0] - s[0] * fn[2], s[0] * fn[1] - s[1] * fn[0]};
    const float *e = c->pos;
    const float m[16] = {s[0], u[0], -fn[0], 0.0f, s[1], u[1], -fn[1], 0.0f, s[2], u[2], -fn[2], 0.0f,
                         -((e[0] * s[0] + e[1] * s[1]) + e[2] * s[2]),
                         -((e[0] * u[0] + e[1] * u[1]) + e[2] * u[2]),
                         (e[0] * fn[0] + e[1] * fn[1]) + e[2] * fn[2], 1.0f};
    std::memcpy(out, m, sizeof(m));
    return GS_OK;
}

gs_status gs_camera_projection(const gs_camera *c, float aspect, float out[16]) {
    if (!c || !out) return fail(GS_ERR_INVALID_ARG, "NULL argument");
    const float half = 0.5f * c->vertical_fov;
    const float h = std::cos(half) / std::sin(half);
    const float w = h / aspect;
    const float r = c->z_far / (c->z_near - c->z_far);
    std::memset(out, 0, 16 * sizeof(float));
    out[0] = w;
    out[5] = h;
    out[10] = r;
    out[11] = -1.0f;
    out[14] = r * c->z_near;
    return GS_OK;
}

gs_status gs_camera_pod_new(const gs_camera *c, uint32_t w, uint32_t h, gs_camera_pod *pod) {
    if (!c || !pod || w == 0 || h == 0) return fail(GS_ERR_INVALID_ARG, "invalid camera pod arguments");
    std::memset(pod, 0, sizeof(*pod));
    gs_camera_view(c, pod->view);
    gs_camera_projection(c, (float)w / (float)h, pod->proj);
    pod->size[0] = (float)w;
    pod->size[1] = (float)h;
    return GS_OK;
}

gs_status gs_gaussian_transform_pod_new(float size, uint32_t mode, uint32_t sh_deg, int no_sh0, float std_dev,
                                        gs_gaussian_transform_pod *out) {
    if (!out) return fail(GS_ERR_INVALID_ARG, "NULL argument");
    gs_gaussian_transform_pod p{};
    p.size = size;
    p.display_mode = mode;
    p.sh_deg = sh_deg;
    p.no_sh0 = no_sh0 ? 1u : 0u;
    p.max_std_dev = std_dev;
    const gs_status s = check_gaussian_transform(&p);
    if (s != GS_OK) return s;
    *out = p;
    return GS_OK;
}

gs_status gs_model_transform_pod_new(const float pos[3], const float rot[4], const float scale[3],
                                     gs_model_transform_pod *out) {
    if (!pos || !rot || !scale || !out) return fail(GS_ERR_INVALID_ARG, "NULL argument");
    gs_model_transform_pod p{};
    std::memcpy(p.pos, pos, 12);
    std::memcpy(p.rot, rot, 16);
    std::memcpy(p.scale, scale, 12);
    *out = p;
    return GS_OK;
}

gs_status gs_gaussian_pack(const gs_gaussian *g, size_t count, gs_gaussian_pod *out) {
    if (count && (!g || !out)) return fail(GS_ERR_INVALID_ARG, "NULL argument");
    for (size_t i = 0; i < count; ++i) {
        gs_gaussian_pod &o = out[i];
        std::memset(&o, 0, sizeof(o));
        std::memcpy(o.pos, g[i].pos, 12);
        o.color = (uint32_t)g[i].color[0] | ((uint32_t)g[i].color[1] << 8) | ((uint32_t)g[i].color[2] << 16) |
                  ((uint32_t)g[i].color[3] << 24);
        std::memcpy(o.sh, g[i].sh, sizeof(o.sh));
        cov3d_from_rot_scale(g[i].rot, g[i].scale, o.cov3d);
    }
    return GS_OK;
}

gs_status gs_frame_uniforms_build(const gs_camera_pod *cam, const gs_model_transform_pod *mt,
                                  const gs_gaussian_transform_pod *gt, uint32_t vw, uint32_t vh,
                                  gs_frame_uniforms *u) {
    if (!cam || !mt || !u) return fail(GS_ERR_INVALID_ARG, "NULL argument");
    const gs_status s = check_gaussian_transform(gt);
    if (s != GS_OK) return s;
    std::memset(u, 0, sizeof(*u));
    mat4_mul(cam->proj, cam->view, u->pv);
    float R[9], SR[9];
    quat_to_mat3(mt->rot, R);
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
    return GS_OK;
}

// ---- stage entry points ----------------------------------------------------------------
uint32_t gs_depth_capacity(uint32_t n) {
    const uint64_t c = ((uint64_t)n + GS_SORT_BLOCK_KVS - 1) / GS_SORT_BLOCK_KVS * GS_SORT_BLOCK_KVS;
    return c > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)c;
}

size_t gs_preprocess_scratch_bytes(uint32_t n) { return preprocess_scratch_bytes(n); }

gs_status gs_preprocess(const gs_frame_uniforms *u, const void *gaussians, uint32_t format, uint32_t n,
                        const uint32_t *selection, int invert, uint32_t *indirect, uint32_t *dispatch,
                        uint32_t *indices, float *depths, uint32_t depth_cap, gs_splat *splats, void *scratch,
                        size_t scratch_bytes, gs_stream stream) {
    if (!u) return fail(GS_ERR_INVALID_ARG, "uniforms are NULL");
    if (!valid_format(format)) return fail(GS_ERR_INVALID_ARG, "unknown record format %u", format);
    if (n && (!gaussians || !indices || !depths)) return fail(GS_ERR_INVALID_ARG, "NULL buffer");
    if (n && !aligned(gaussians, 16)) return fail(GS_ERR_INVALID_ARG, "records must be 16-byte aligned");
    if (splats && !aligned(splats, 16)) return fail(GS_ERR_INVALID_ARG, "splats must be 16-byte aligned");
    if (depth_cap < n) return fail(GS_ERR_INVALID_ARG, "depth capacity %u < n %u", depth_cap, n);
    if (!scratch || scratch_bytes < preprocess_scratch_bytes(n))
        return fail(GS_ERR_INVALID_ARG, "scratch smaller than gs_preprocess_scratch_bytes(n)");
    const cudaError_t e = launch_preprocess(*u, gaussians, format, n, selection, invert, indirect, dispatch,
                                            indices, depths, depth_cap, splats, scratch, (cudaStream_t)stream);
    return e == cudaSuccess ? GS_OK : cuda_fail(e, "gs_preprocess");
}

size_t gs_radix_sort_scratch_bytes(uint32_t max_count) { return sort_scratch_bytes(max_count, 32); }

gs_status gs_radix_sort(uint32_t *keys, uint32_t *values, uint32_t max_count, const uint32_t *count,
                        uint32_t key_bits, void *scratch, size_t scratch_bytes, gs_stream stream) {
    if (key_bits < 1 || key_bits > 32) return fail(GS_ERR_INVALID_ARG, "key_bits %u not in 1..=32", key_bits);
    if (max_count && (!keys || !values)) return fail(GS_ERR_INVALID_ARG, "NULL buffer");
    if (!scratch || scratch_bytes < sort_scratch_bytes(max_count, key_bits))
        return fail(GS_ERR_INVALID_ARG, "scratch smaller than gs_radix_sort_scratch_bytes(max_count)");
    const cudaError_t e = launch_sort(keys, values, max_count, count, key_bits, scratch, (cudaStream_t)stream);
    return e == cudaSuccess ? GS_OK : cuda_fail(e, "gs_radix_sort");
}

size_t gs_rasterize_scratch_bytes(uint32_t max_splats, uint32_t w, uint32_t h, uint32_t max_pairs) {
    return raster_scratch_bytes(max_splats, w, h, max_pairs);
}

gs_status gs_rasterize(const gs_frame_uniforms *u, const gs_splat *splats, const uint32_t *sorted, const uint32_t *count,
                       uint32_t max_splats, uint8_t *target, uint32_t w, uint32_t h, uint32_t pitch, uint32_t max_pairs,
                       void *scratch, size_t scratch_bytes, gs_stream stream) {
    if (!u) return fail(GS_ERR_INVALID_ARG, "uniforms are NULL");
    gs_status s = check_target(target, w, h, pitch);
    if (s != GS_OK) return s;
    if (max_splats && (!splats || !sorted)) return fail(GS_ERR_INVALID_ARG, "NULL buffer");
    if (splats && !aligned(splats, 16)) return fail(GS_ERR_INVALID_ARG, "splats must be 16-byte aligned");
    if (!scratch || scratch_bytes < raster_scratch_bytes(max_splats, w, h, max_pairs))
        return fail(GS_ERR_INVALID_ARG, "scratch smaller than gs_rasterize_scratch_bytes");
    const RasterSegment seg{splats, sorted, count, max_splats};
    const int exact = getenv("GS300_EXACT_EXP") ? 1 : 0;
    const cudaError_t e = launch_raster(&seg, 1, raster_mode(*u), target, w, h, pitch, max_pairs, scratch, exact, (cudaStream_t)stream);
    return e == cudaSuccess ? GS_OK : cuda_fail(e, "gs_rasterize");
}

gs_status gs_debug_set_wait_fault(uint32_t spin_limit, uint32_t stall_tile) {
    if (spin_limit == 0) return fail(GS_ERR_INVALID_ARG, "spin_limit must be >= 1");
    gs::g_wait_cfg.store(((uint64_t)stall_tile << 32) | spin_limit, std::memory_order_relaxed);
    return GS_OK;
}

gs_status gs_scratch_status(const void *scratch, gs_stream stream, uint32_t *pairs) {
    if (!scratch) return fail(GS_ERR_INVALID_ARG, "scratch is NULL");
    GS_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    Ctrl c{};
    GS_CUDA(cudaMemcpy(&c, scratch, sizeof(Ctrl), cudaMemcpyDeviceToHost));
    if (pairs) *pairs = c.total;
    return status_from_bits(c.status, "stage");
}

// ---- Viewer -------------------------------------------------------------------------------
}  // extern "C"

struct gs_viewer {
    Model model;
    Frame frame;
    std::mutex mu;
};

struct gs_target {
    DevBuf buf;
    uint32_t w = 0, h = 0;
};

namespace {

gs_status viewer_render_locked(gs_viewer *v, uint8_t *target, uint32_t w, uint32_t h, uint32_t pitch,
                               cudaStream_t st) {
    gs_status s = check_target(target, w, h, pitch);
    if (s != GS_OK) return s;
    s = v->frame.ensure_scratch(v->model.n, w, h);
    if (s != GS_OK) return s;
    gs_frame_uniforms u;
    s = gs_frame_uniforms_build(&v->frame.camera, &v->model.model, &v->frame.gt, w, h, &u);
    if (s != GS_OK) return s;
    s = v->model.enqueue(u, st, true);
    if (s != GS_OK) return s;
    RasterSegment seg{(const gs_splat *)v->model.splats.ptr, (const uint32_t *)v->model.indices.ptr,
                      v->model.indirect() + 1, v->model.n};
    seg.binfo = reinterpret_cast<const uint4 *>(v->model.binfo.ptr);
    seg.binfo_w = w;
    seg.binfo_h = h;
    const cudaError_t e = launch_raster(&seg, 1, raster_mode(u), target, w, h, pitch, v->frame.max_pairs, v->frame.raster_scratch.ptr,
                                        v->frame.exact_exp, st);
    if (e != cudaSuccess) return cuda_fail(e, "raster launch");
    v->frame.last_target = target;
    v->frame.last_w = w;
    v->frame.last_h = h;
    v->frame.last_pitch = pitch;
    v->frame.rendered = true;
    return GS_OK;
}

}  // namespace

extern "C" {

gs_status gs_viewer_create(const void *host_records, uint32_t count, uint32_t format, gs_viewer **out) {
    if (!out) return fail(GS_ERR_INVALID_ARG, "out is NULL");
    gs_viewer *v = new gs_viewer();
    const gs_status s = v->model.create(host_records, count, format);
    if (s != GS_OK) {
        delete v;
        return s;
    }
    v->frame.exact_exp = getenv("GS300_EXACT_EXP") ? 1 : 0;
    *out = v;
    return GS_OK;
}

gs_status gs_viewer_create_from_ply(const void *ply_bytes, size_t len, uint32_t format, gs_viewer **out) {
    if (!out || !ply_bytes) return fail(GS_ERR_INVALID_ARG, "NULL argument");
    gs_viewer *v = new gs_viewer();
    const gs_status s = v->model.create_from_ply(ply_bytes, len, format);
    if (s != GS_OK) {
        delete v;
        return s;
    }
    v->frame.exact_exp = getenv("GS300_EXACT_EXP") ? 1 : 0;
    *out = v;
    return GS_OK;
}

void gs_viewer_destroy(gs_viewer *v) {
    if (!v) return;
    cudaDeviceSynchronize();
    delete v;
}

uint32_t gs_viewer_len(const gs_viewer *v) { return v ? v->model.n : 0; }

gs_status gs_viewer_update_camera(gs_viewer *v, const gs_camera *c, uint32_t w, uint32_t h) {
    if (!v) return fail(GS_ERR_INVALID_ARG, "viewer is NULL");
    std::lock_guard<std::mutex> g(v->mu);
    return gs_camera_pod_new(c, w, h, &v->frame.camera);
}

gs_status gs_viewer_update_camera_with_pod(gs_viewer *v, const gs_camera_pod *pod) {
    if (!v || !pod) return fail(GS_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> g(v->mu);
    v->frame.camera = *pod;
    return GS_OK;
}

gs_status gs_viewer_update_model_transform(gs_viewer *v, const float pos[3], const float rot[4], const float scale[3]) {
    if (!v) return fail(GS_ERR_INVALID_ARG, "viewer is NULL");
    std::lock_guard<std::mutex> g(v->mu);
    return gs_model_transform_pod_new(pos, rot, scale, &v->model.model);
}

gs_status gs_viewer_update_model_transform_with_pod(gs_viewer *v, const gs_model_transform_pod *pod) {
    if (!v || !pod) return fail(GS_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> g(v->mu);
    v->model.model = *pod;
    return GS_OK;
}

gs_status gs_viewer_update_gaussian_transform(gs_viewer *v, float size, uint32_t mode, uint32_t sh_deg, int no_sh0,
                                              float std_dev) {
    if (!v) return fail(GS_ERR_INVALID_ARG, "viewer is NULL");
    std::lock_guard<std::mutex> g(v->mu);
    return gs_gaussian_transform_pod_new(size, mode, sh_deg, no_sh0, std_dev, &v->frame.gt);
}

gs_status gs_viewer_update_gaussian_transform_with_pod(gs_viewer *v, const gs_gaussian_transform_pod *pod) {
    if (!v) return fail(GS_ERR_INVALID_ARG, "viewer is NULL");
    const gs_status s = check_gaussian_transform(pod);
    if (s != GS_OK) return s;
    std::lock_guard<std::mutex> g(v->mu);
    v->frame.gt = *pod;
    return GS_OK;
}

gs_status gs_viewer_set_selection(gs_viewer *v, const uint32_t *bits, int invert) {
    if (!v) return fail(GS_ERR_INVALID_ARG, "viewer is NULL");
    std::lock_guard<std::mutex> g(v->mu);
    return v->model.set_selection(bits, invert);
}

gs_status gs_viewer_render(gs_viewer *v, uint8_t *target, uint32_t w, uint32_t h, uint32_t pitch, gs_stream stream) {
    if (!v) return fail(GS_ERR_INVALID_ARG, "viewer is NULL");
    std::lock_guard<std::mutex> g(v->mu);
    return viewer_render_locked(v, target, w, h, pitch, (cudaStream_t)stream);
}

gs_status gs_viewer_synchronize(gs_viewer *v, gs_stream stream) {
    if (!v) return fail(GS_ERR_INVALID_ARG, "viewer is NULL");
    std::lock_guard<std::mutex> g(v->mu);
    cudaStream_t st = (cudaStream_t)stream;
    for (int attempt = 0; attempt < 4; ++attempt) {
        GS_CUDA(cudaStreamSynchronize(st));
        if (!v->frame.rendered) return GS_OK;
        Ctrl c{};
        GS_CUDA(cudaMemcpy(&c, v->frame.raster_scratch.ptr, sizeof(Ctrl), cudaMemcpyDeviceToHost));
        const uint32_t bits = c.status | v->model.device_status();
        if (bits & (kStatusTimeout | kStatusBounds)) return status_from_bits(bits, "render");
        if (!(bits & kStatusCapacity)) return GS_OK;
        gs_status s = v->frame.grow_pairs(c.total);
        if (s != GS_OK) return s;
        s = viewer_render_locked(v, v->frame.last_target, v->frame.last_w, v->frame.last_h, v->frame.last_pitch, st);
        if (s != GS_OK) return s;
    }
    return fail(GS_ERR_CAPACITY, "tile-pair list kept overflowing");
}

gs_status gs_viewer_stats(gs_viewer *v, gs_stream stream, uint32_t *visible, uint32_t *pairs) {
    if (!v) return fail(GS_ERR_INVALID_ARG, "viewer is NULL");
    std::lock_guard<std::mutex> g(v->mu);
    GS_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    uint32_t args[4] = {0, 0, 0, 0};
    GS_CUDA(cudaMemcpy(args, v->model.control.ptr, sizeof(args), cudaMemcpyDeviceToHost));
    Ctrl c{};
    if (v->frame.raster_scratch.ptr) GS_CUDA(cudaMemcpy(&c, v->frame.raster_scratch.ptr, sizeof(Ctrl), cudaMemcpyDeviceToHost));
    if (visible) *visible = args[1];
    if (pairs) *pairs = c.total;
    return GS_OK;
}

gs_status gs_viewer_buffers(gs_viewer *v, uint32_t **indices, float **depths, uint32_t **indirect, gs_splat **splats) {
    if (!v) return fail(GS_ERR_INVALID_ARG, "viewer is NULL");
    if (indices) *indices = (uint32_t *)v->model.indices.ptr;
    if (depths) *depths = (float *)v->model.depths.ptr;
    if (indirect) *indirect = v->model.indirect();
    if (splats) *splats = (gs_splat *)v->model.splats.ptr;
    return GS_OK;
}

// ---- targets --------------------------------------------------------------------------------
gs_status gs_target_create(uint32_t w, uint32_t h, gs_target **out) {
    if (!out || w == 0 || h == 0) return fail(GS_ERR_INVALID_ARG, "invalid target arguments");
    gs_target *t = new gs_target();
    const cudaError_t e = t->buf.ensure((size_t)w * h * 4);
    if (e != cudaSuccess) {
        delete t;
        return cuda_fail(e, "target allocation");
    }
    t->w = w;
    t->h = h;
    *out = t;
    return GS_OK;
}

void gs_target_destroy(gs_target *t) {
    if (!t) return;
    cudaDeviceSynchronize();
    delete t;
}

uint8_t *gs_target_data(gs_target *t) { return t ? (uint8_t *)t->buf.ptr : nullptr; }
uint32_t gs_target_pitch(const gs_target *t) { return t ? t->w * 4 : 0; }

gs_status gs_target_download(gs_target *t, uint8_t *host, gs_stream stream) {
    if (!t || !host) return fail(GS_ERR_INVALID_ARG, "NULL argument");
    cudaStream_t st = (cudaStream_t)stream;
    GS_CUDA(cudaMemcpyAsync(host, t->buf.ptr, (size_t)t->w * t->h * 4, cudaMemcpyDeviceToHost, st));
    GS_CUDA(cudaStreamSynchronize(st));
    return GS_OK;
}

gs_status gs_target_download_async(gs_target *t, uint8_t *host, gs_stream stream) {
    if (!t || !host) return fail(GS_ERR_INVALID_ARG, "NULL argument");
    GS_CUDA(cudaMemcpyAsync(host, t->buf.ptr, (size_t)t->w * t->h * 4, cudaMemcpyDeviceToHost,
                            (cudaStream_t)stream));
    return GS_OK;
}

}  // extern "C"

// ---- MultiModelViewer -----------------------------------------------------------------------
struct gs_multi_viewer {
    std::map<std::string, Model *> models;
    Frame frame;
    std::mutex mu;
    std::vector<std::string> last_keys;
    ~gs_multi_viewer() {
        for (auto &kv : models) delete kv.second;
    }
};

namespace {

gs_status multi_render_locked(gs_multi_viewer *v, const std::vector<std::string> &keys, uint8_t *target, uint32_t w,
                              uint32_t h, uint32_t pitch, cudaStream_t st) {
    gs_status s = check_target(target, w, h, pitch);
    if (s != GS_OK) return s;
    std::vector<Model *> ms;
    for (const auto &k : keys) {
        auto it = v->models.find(k);
        if (it == v->models.end()) return fail(GS_ERR_NOT_FOUND, "model '%s' not found", k.c_str());
        ms.push_back(it->second);
    }
    uint64_t total = 0;
    for (Model *m : ms) total += m->n;
    if (total > 0xFFFFFFFFull) return fail(GS_ERR_INVALID_ARG, "too many Gaussians in one render");
    s = v->frame.ensure_scratch((uint32_t)total, w, h);
    if (s != GS_OK) return s;
    std::vector<RasterSegment> segs;
    gs_frame_uniforms u{};
    for (Model *m : ms) {
        s = gs_frame_uniforms_build(&v->frame.camera, &m->model, &v->frame.gt, w, h, &u);
        if (s != GS_OK) return s;
        s = m->enqueue(u, st);
        if (s != GS_OK) return s;
        segs.push_back(RasterSegment{(const gs_splat *)m->splats.ptr, (const uint32_t *)m->indices.ptr, m->indirect() + 1, m->n});
    }
    if (ms.empty()) {
        gs_model_transform_pod identity{};
        identity.rot[3] = 1.0f;
        identity.scale[0] = identity.scale[1] = identity.scale[2] = 1.0f;
        s = gs_frame_uniforms_build(&v->frame.camera, &identity, &v->frame.gt, w, h, &u);
        if (s != GS_OK) return s;
    }
    // Binning and raster read only std dev and display mode (RasterMode), which all models share.
    const cudaError_t e = launch_raster(segs.data(), (uint32_t)segs.size(), raster_mode(u), target, w, h, pitch, v->frame.max_pairs,
                                        v->frame.raster_scratch.ptr, v->frame.exact_exp, st);
    if (e != cudaSuccess) return cuda_fail(e, "raster launch");
    v->last_keys = keys;
    v->frame.last_target = target;
    v->frame.last_w = w;
    v->frame.last_h = h;
    v->frame.last_pitch = pitch;
    v->frame.rendered = true;
    return GS_OK;
}

}  // namespace

extern "C" {

gs_status gs_multi_viewer_create(gs_multi_viewer **out) {
    if (!out) return fail(GS_ERR_INVALID_ARG, "out is NULL");
    gs_multi_viewer *v = new gs_multi_viewer();
    v->frame.exact_exp = getenv("GS300_EXACT_EXP") ? 1 : 0;
    *out = v;
    return GS_OK;
}

void gs_multi_viewer_destroy(gs_multi_viewer *v) {
    if (!v) return;
    cudaDeviceSynchronize();
    delete v;
}

static gs_status multi_insert(gs_multi_viewer *v, const char *key, Model *m) {
    std::lock_guard<std::mutex> g(v->mu);
    auto it = v->models.find(key);
    if (it != v->models.end()) {
        cudaDeviceSynchronize();
        delete it->second;
        it->second = m;
    } else {
        v->models.emplace(key, m);
    }
    return GS_OK;
}

gs_status gs_multi_viewer_insert_model(gs_multi_viewer *v, const char *key, const void *host, uint32_t count,
                                       uint32_t format) {
    if (!v || !key) return fail(GS_ERR_INVALID_ARG, "NULL argument");
    Model *m = new Model();
    const gs_status s = m->create(host, count, format);
    if (s != GS_OK) {
        delete m;
        return s;
    }
    return multi_insert(v, key, m);
}

gs_status gs_multi_viewer_insert_model_from_ply(gs_multi_viewer *v, const char *key, const void *ply_bytes,
                                                size_t len, uint32_t format) {
    if (!v || !key || !ply_bytes) return fail(GS_ERR_INVALID_ARG, "NULL argument");
    Model *m = new Model();
    const gs_status s = m->create_from_ply(ply_bytes, len, format);
    if (s != GS_OK) {
        delete m;
        return s;
    }
    return multi_insert(v, key, m);
}

gs_status gs_multi_viewer_remove_model(gs_multi_viewer *v, const char *key) {
    if (!v || !key) return fail(GS_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> g(v->mu);
    auto it = v->models.find(key);
    if (it == v->models.end()) return fail(GS_ERR_NOT_FOUND, "model '%s' not found", key);
    cudaDeviceSynchronize();
    delete it->second;
    v->models.erase(it);
    return GS_OK;
}

uint32_t gs_multi_viewer_model_count(const gs_multi_viewer *v) { return v ? (uint32_t)v->models.size() : 0; }

gs_status gs_multi_viewer_update_camera(gs_multi_viewer *v, const gs_camera *c, uint32_t w, uint32_t h) {
    if (!v) return fail(GS_ERR_INVALID_ARG, "viewer is NULL");
    std::lock_guard<std::mutex> g(v->mu);
    return gs_camera_pod_new(c, w, h, &v->frame.camera);
}

gs_status gs_multi_viewer_update_camera_with_pod(gs_multi_viewer *v, const gs_camera_pod *pod) {
    if (!v || !pod) return fail(GS_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> g(v->mu);
    v->frame.camera = *pod;
    return GS_OK;
}

gs_status gs_multi_viewer_update_model_transform(gs_multi_viewer *v, const char *key, const float pos[3],
                                                 const float rot[4], const float scale[3]) {
    if (!v || !key) return fail(GS_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> g(v->mu);
    auto it = v->models.find(key);
    if (it == v->models.end()) return fail(GS_ERR_NOT_FOUND, "model '%s' not found", key);
    return gs_model_transform_pod_new(pos, rot, scale, &it->second->model);
}

gs_status gs_multi_viewer_update_model_transform_with_pod(gs_multi_viewer *v, const char *key,
                                                          const gs_model_transform_pod *pod) {
    if (!v || !key || !pod) return fail(GS_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> g(v->mu);
    auto it = v->models.find(key);
    if (it == v->models.end()) return fail(GS_ERR_NOT_FOUND, "model '%s' not found", key);
    it->second->model = *pod;
    return GS_OK;
}

gs_status gs_multi_viewer_update_gaussian_transform(gs_multi_viewer *v, float size, uint32_t mode, uint32_t sh_deg,
                                                    int no_sh0, float std_dev) {
    if (!v) return fail(GS_ERR_INVALID_ARG, "viewer is NULL");
    std::lock_guard<std::mutex> g(v->mu);
    return gs_gaussian_transform_pod_new(size, mode, sh_deg, no_sh0, std_dev, &v->frame.gt);
}

gs_status gs_multi_viewer_update_gaussian_transform_with_pod(gs_multi_viewer *v, const gs_gaussian_transform_pod *pod) {
    if (!v) return fail(GS_ERR_INVALID_ARG, "viewer is NULL");
    const gs_status s = check_gaussian_transform(pod);
    if (s != GS_OK) return s;
    std::lock_guard<std::mutex> g(v->mu);
    v->frame.gt = *pod;
    return GS_OK;
}

gs_status gs_multi_viewer_render(gs_multi_viewer *v, const char *const *keys, uint32_t key_count, uint8_t *target,
                                 uint32_t w, uint32_t h, uint32_t pitch, gs_stream stream) {
    if (!v || (key_count && !keys)) return fail(GS_ERR_INVALID_ARG, "NULL argument");
    std::vector<std::string> ks;
    for (uint32_t i = 0; i < key_count; ++i) {
        if (!keys[i]) return fail(GS_ERR_INVALID_ARG, "key %u is NULL", i);
        ks.emplace_back(keys[i]);
    }
    std::lock_guard<std::mutex> g(v->mu);
    return multi_render_locked(v, ks, target, w, h, pitch, (cudaStream_t)stream);
}

gs_status gs_multi_viewer_synchronize(gs_multi_viewer *v, gs_stream stream) {
    if (!v) return fail(GS_ERR_INVALID_ARG, "viewer is NULL");
    std::lock_guard<std::mutex> g(v->mu);
    cudaStream_t st = (cudaStream_t)stream;
    for (int attempt = 0; attempt < 4; ++attempt) {
        GS_CUDA(cudaStreamSynchronize(st));
        if (!v->frame.rendered) return GS_OK;
        Ctrl c{};
        GS_CUDA(cudaMemcpy(&c, v->frame.raster_scratch.ptr, sizeof(Ctrl), cudaMemcpyDeviceToHost));
        uint32_t bits = c.status;
        for (const auto &k : v->last_keys) {
            auto it = v->models.find(k);
            if (it != v->models.end()) bits |= it->second->device_status();
        }
        if (bits & (kStatusTimeout | kStatusBounds)) return status_from_bits(bits, "render");
        if (!(bits & kStatusCapacity)) return GS_OK;
        gs_status s = v->frame.grow_pairs(c.total);
        if (s != GS_OK) return s;
        s = multi_render_locked(v, v->last_keys, v->frame.last_target, v->frame.last_w, v->frame.last_h,
                                v->frame.last_pitch, st);
        if (s != GS_OK) return s;
    }
    return fail(GS_ERR_CAPACITY, "tile-pair list kept overflowing");
}

}  // extern "C"

namespace {

// ---- Batches: many views (model, camera, target) rendered by one CUDA graph ------------------
struct ViewSlot {
    const Model *model = nullptr;
    uint32_t w = 0, h = 0;
    DevBuf control, indices, depths, splats, pre_scratch, sort_scratch, raster_scratch;
    DevBuf binfo;  // tile records of a view preprocessed alone (serving); grows like the others
    uint32_t max_pairs = 0;

    // Buffers of one view of `m` at w x h; *changed is set when any pointer changed (a captured
    // graph must then be rebuilt).  Buffers only grow: a slot that served a larger scene or
    // resolution keeps its buffers and lays the smaller view out inside them, so a mix of scenes
    // and resolutions stops allocating once each slot has met its largest request.  The tile-pair
    // capacity never shrinks either (it also keeps any growth after an overflow).
    cudaError_t prepare(const Model *m, uint32_t ww, uint32_t hh, bool *changed) {
        const uint32_t n = m->n;
        cudaError_t e = cudaSuccess;
        const void *before[7] = {control.ptr, indices.ptr, depths.ptr, splats.ptr, pre_scratch.ptr, sort_scratch.ptr,
                                 raster_scratch.ptr};
        if ((e = control.ensure_zeroed(64)) != cudaSuccess) return e;
        if ((e = indices.ensure((size_t)n * 4)) != cudaSuccess) return e;
        if ((e = depths.ensure((size_t)gs_depth_capacity(n) * 4)) != cudaSuccess) return e;
        if ((e = splats.ensure((size_t)n * sizeof(gs_splat))) != cudaSuccess) return e;
        if ((e = pre_scratch.ensure_zeroed(preprocess_scratch_bytes(n))) != cudaSuccess) return e;
        if ((e = sort_scratch.ensure_zeroed(sort_scratch_bytes(n, kDepthKeyBits))) != cudaSuccess) return e;
        const uint32_t want = default_pairs(n, ww, hh);
        if (want > max_pairs) max_pairs = want;
        if ((e = raster_scratch.ensure_zeroed(raster_scratch_bytes(n, ww, hh, max_pairs))) != cudaSuccess) return e;
        const void *after[7] = {control.ptr, indices.ptr, depths.ptr, splats.ptr, pre_scratch.ptr, sort_scratch.ptr,
                                raster_scratch.ptr};
        for (int i = 0; i < 7; ++i)
            if (before[i] != after[i]) *changed = true;
        if (model != m || w != ww || h != hh) *changed = true;
        model = m;
        w = ww;
        h = hh;
        return cudaSuccess;
    }
};

}  // namespace

struct gs_batch {
    gs_multi_viewer *mv = nullptr;
    std::vector<std::string> keys;
    std::vector<ViewSlot> slots;
    DevBuf uniforms_dev;
    // Pinned staging of the views' uniforms: a ring of kUniformRing arrays of uniforms_cap, each
    // reused only after the copy that read it (event) has run, so renders issued back to back
    // never upload another render's cameras.
    gs_frame_uniforms *uniforms_host = nullptr;
    uint32_t uniforms_cap = 0, uniforms_ring = 0;
    cudaEvent_t uniforms_copied[4] = {nullptr, nullptr, nullptr, nullptr};
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> events;
    std::vector<cudaEvent_t> chunk_events;  // one per multi-view preprocess launch
    DevBuf views_dev;                       // PreView per view (device), rebuilt with the graph
    DevBuf group_dev;                       // one control block per multi-view launch
    DevBuf jobs_dev, tile_base_dev;         // per view RasterJob and the prefix of tile counts
    DevBuf sort_segs_dev, sort_base_dev;    // per view tile-sort segment and the prefix of its blocks
    uint32_t chunks = 0;
    gs::Tuning tuning = gs::default_tuning();
    cudaStream_t capture = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::string shape;
    uint64_t graph_launches = 0;
    std::vector<gs_batch_view> last;
    std::mutex mu;

    ~gs_batch() {
        if (exec) cudaGraphExecDestroy(exec);
        for (auto s : streams) cudaStreamDestroy(s);
        for (auto e : events) cudaEventDestroy(e);
        for (auto e : chunk_events) cudaEventDestroy(e);
        for (auto e : uniforms_copied)
            if (e) cudaEventDestroy(e);
        if (capture) cudaStreamDestroy(capture);
        if (uniforms_host) cudaFreeHost(uniforms_host);
    }
};

namespace {

constexpr uint32_t kBatchStreams = 16;

gs_status batch_render_locked(gs_batch *b, const gs_batch_view *views, uint32_t n, cudaStream_t st) {
    gs_multi_viewer *mv = b->mv;
    std::lock_guard<std::mutex> g(mv->mu);
    if (n == 0) return GS_OK;
    std::vector<const Model *> ms(n);
    for (uint32_t i = 0; i < n; ++i) {
        if (views[i].model >= b->keys.size()) return fail(GS_ERR_INVALID_ARG, "view %u: model index %u out of range", i, views[i].model);
        auto it = mv->models.find(b->keys[views[i].model]);
        if (it == mv->models.end()) return fail(GS_ERR_NOT_FOUND, "model '%s' not found", b->keys[views[i].model].c_str());
        ms[i] = it->second;
        const gs_status s = check_target(views[i].target, views[i].width, views[i].height, views[i].pitch);
        if (s != GS_OK) return s;
    }
    std::string shape(reinterpret_cast<const char *>(&mv->frame.gt), sizeof(gs_gaussian_transform_pod));
    for (uint32_t i = 0; i < n; ++i) {
        const uintptr_t key[7] = {(uintptr_t)ms[i], ms[i]->n, views[i].width, views[i].height, views[i].pitch,
                                  (uintptr_t)views[i].target, (uintptr_t)ms[i]->has_selection};
        shape.append(reinterpret_cast<const char *>(key), sizeof(key));
    }
    // A new shape rewrites buffers and descriptor arrays that an earlier render of this batch may
    // still be reading on the caller's stream: let the device drain first (shape changes are rare).
    if (shape != b->shape || !b->exec || n > b->uniforms_cap) GS_CUDA(cudaDeviceSynchronize());
    if (n > b->uniforms_cap) {
        if (b->uniforms_host) cudaFreeHost(b->uniforms_host);
        b->uniforms_host = nullptr;
        GS_CUDA(cudaMallocHost(&b->uniforms_host, (size_t)4 * n * sizeof(gs_frame_uniforms)));
        GS_CUDA(b->uniforms_dev.ensure((size_t)n * sizeof(gs_frame_uniforms)));
        b->uniforms_cap = n;
    }
    for (auto &e : b->uniforms_copied)
        if (!e) GS_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    const uint32_t ring = b->uniforms_ring;
    b->uniforms_ring = (ring + 1) % 4;
    GS_CUDA(cudaEventSynchronize(b->uniforms_copied[ring]));  // its previous copy has run
    gs_frame_uniforms *uh = b->uniforms_host + (size_t)ring * b->uniforms_cap;
    if (b->slots.size() < n) b->slots.resize(n);
    bool changed = false;
    for (uint32_t i = 0; i < n; ++i) {
        GS_CUDA(b->slots[i].prepare(ms[i], views[i].width, views[i].height, &changed));
        const gs_status s = gs_frame_uniforms_build(&views[i].camera, &ms[i]->model, &mv->frame.gt, views[i].width,
                                                    views[i].height, &uh[i]);
        if (s != GS_OK) return s;
    }
    if (changed || shape != b->shape || !b->exec) {
        if (b->exec) cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
        if (!b->capture) GS_CUDA(cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking));
        while (b->streams.size() < kBatchStreams) {
            cudaStream_t s;
            GS_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
            b->streams.push_back(s);
        }
        while (b->events.size() < kBatchStreams + 1) {
            cudaEvent_t e;
            GS_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            b->events.push_back(e);
        }
        const uint32_t nstreams = std::min(n, std::min(b->tuning.streams, kBatchStreams));
        const size_t per_launch = std::min(b->tuning.views_per_launch, kPreMaxViews);
        // Views of one model share its record reads: one preprocess launch per chunk of up to
        // `per_launch` views of the same model, in order of first appearance.
        std::vector<std::vector<uint32_t>> chunks;
        {
            std::vector<const Model *> seen;
            std::vector<std::vector<uint32_t>> by_model;
            for (uint32_t i = 0; i < n; ++i) {
                size_t g = 0;
                while (g < seen.size() && seen[g] != ms[i]) ++g;
                if (g == seen.size()) {
                    seen.push_back(ms[i]);
                    by_model.emplace_back();
                }
                by_model[g].push_back(i);
            }
            for (auto &grp : by_model)
                for (size_t k = 0; k < grp.size(); k += per_launch)
                    chunks.emplace_back(grp.begin() + k, grp.begin() + std::min(grp.size(), k + per_launch));
        }
        const gs_frame_uniforms *udev = reinterpret_cast<const gs_frame_uniforms *>(b->uniforms_dev.ptr);
        std::vector<PreView> pv(n);
        std::vector<uint32_t> slot_of(n);  // position of view i in the PreView array
        {
            uint32_t at = 0;
            for (auto &ch : chunks)
                for (uint32_t i : ch) {
                    ViewSlot &v = b->slots[i];
                    uint32_t *ind = reinterpret_cast<uint32_t *>(v.control.ptr);
                    pv[at] = preprocess_view(udev + i, ind, ind + 4, (uint32_t *)v.indices.ptr, (float *)v.depths.ptr,
                                             gs_depth_capacity(ms[i]->n), (gs_splat *)v.splats.ptr, v.pre_scratch.ptr);
                    slot_of[i] = at++;
                }
        }
        GS_CUDA(b->views_dev.ensure((size_t)n * sizeof(PreView)));
        GS_CUDA(cudaMemcpy(b->views_dev.ptr, pv.data(), (size_t)n * sizeof(PreView), cudaMemcpyHostToDevice));
        const size_t gbytes = align_up(sizeof(Ctrl), 256);
        if (b->group_dev.bytes < chunks.size() * gbytes) {
            GS_CUDA(b->group_dev.ensure(chunks.size() * gbytes));
            GS_CUDA(cudaMemset(b->group_dev.ptr, 0, chunks.size() * gbytes));
        }
        while (b->chunk_events.size() < chunks.size()) {
            cudaEvent_t e;
            GS_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            b->chunk_events.push_back(e);
        }
        b->chunks = (uint32_t)chunks.size();
        const PreView *pv_dev = reinterpret_cast<const PreView *>(b->views_dev.ptr);
        // One rasteriser grid over every view's tiles: the views' raster jobs (pointers into
        // their scratch) and the prefix of their tile counts, known before any launch.
        std::vector<RasterJob> jobs(n);
        std::vector<uint32_t> tile_base(n + 1, 0u);
        for (uint32_t i = 0; i < n; ++i) {
            ViewSlot &v = b->slots[i];
            uint32_t *ind = reinterpret_cast<uint32_t *>(v.control.ptr);
            const RasterSegment seg{(const gs_splat *)v.splats.ptr, (const uint32_t *)v.indices.ptr, ind + 1, ms[i]->n};
            jobs[i] = raster_job(&seg, 1, views[i].target, views[i].width, views[i].height, views[i].pitch, v.max_pairs,
                                 v.raster_scratch.ptr);
            tile_base[i + 1] = tile_base[i] + jobs[i].ntiles;
        }
        GS_CUDA(b->jobs_dev.ensure((size_t)n * sizeof(RasterJob)));
        GS_CUDA(cudaMemcpy(b->jobs_dev.ptr, jobs.data(), (size_t)n * sizeof(RasterJob), cudaMemcpyHostToDevice));
        GS_CUDA(b->tile_base_dev.ensure((size_t)(n + 1) * 4));
        GS_CUDA(cudaMemcpy(b->tile_base_dev.ptr, tile_base.data(), (size_t)(n + 1) * 4, cudaMemcpyHostToDevice));
        // With one rasteriser grid, the views' tile sorts run as one segmented sort (one launch per
        // pass over all views' pairs: keys (view, tile) with depth order kept inside each tile)
        // when every target fits two tile-sort passes; else each view sorts its own pairs.
        bool segmented = b->tuning.raster_grid != 0;
        for (uint32_t i = 0; i < n && segmented; ++i) segmented = tile_sort_segmentable(views[i].width, views[i].height);
        std::vector<SortSegment> sort_segs(segmented ? n : 0);
        std::vector<uint32_t> sort_base(n + 1, 0u);
        if (segmented) {
            for (uint32_t i = 0; i < n; ++i) {
                ViewSlot &v = b->slots[i];
                uint32_t *ind = reinterpret_cast<uint32_t *>(v.control.ptr);
                const RasterSegment seg{(const gs_splat *)v.splats.ptr, (const uint32_t *)v.indices.ptr, ind + 1, ms[i]->n};
                sort_segs[i] = tile_sort_segment(&seg, 1, views[i].width, views[i].height, v.max_pairs, v.raster_scratch.ptr);
                sort_base[i + 1] = sort_base[i] + sort_pairs_blocks(v.max_pairs);
            }
            GS_CUDA(b->sort_segs_dev.ensure((size_t)n * sizeof(SortSegment)));
            GS_CUDA(cudaMemcpy(b->sort_segs_dev.ptr, sort_segs.data(), (size_t)n * sizeof(SortSegment),
                               cudaMemcpyHostToDevice));
            GS_CUDA(b->sort_base_dev.ensure((size_t)(n + 1) * 4));
            GS_CUDA(cudaMemcpy(b->sort_base_dev.ptr, sort_base.data(), (size_t)(n + 1) * 4, cudaMemcpyHostToDevice));
        }
        GS_CUDA(cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeThreadLocal));
        t_capturing = true;
        t_captured_launches = 0;
        cudaError_t err = cudaEventRecord(b->events[kBatchStreams], b->capture);
        for (uint32_t s = 0; s < nstreams && err == cudaSuccess; ++s)
            err = cudaStreamWaitEvent(b->streams[s], b->events[kBatchStreams], 0);
        for (size_t c = 0; c < chunks.size() && err == cudaSuccess; ++c) {
            const Model *m = ms[chunks[c][0]];
            cudaStream_t cs = b->streams[c % nstreams];
            err = launch_preprocess_views(m->records.ptr, m->format, m->n,
                                          m->has_selection ? (const uint32_t *)m->selection.ptr : nullptr, m->invert,
                                          pv_dev + slot_of[chunks[c][0]], (uint32_t)chunks[c].size(),
                                          (uint8_t *)b->group_dev.ptr + c * gbytes, cs);
            if (err == cudaSuccess) err = cudaEventRecord(b->chunk_events[c], cs);
            for (uint32_t i : chunks[c]) {
                if (err != cudaSuccess) break;
                ViewSlot &v = b->slots[i];
                cudaStream_t vs = b->streams[i % nstreams];
                uint32_t *ind = reinterpret_cast<uint32_t *>(v.control.ptr);
                if (vs != cs) err = cudaStreamWaitEvent(vs, b->chunk_events[c], 0);
                if (err == cudaSuccess)
                    err = launch_sort((uint32_t *)v.depths.ptr, (uint32_t *)v.indices.ptr, ms[i]->n, ind + 1, kDepthKeyBits,
                                      v.sort_scratch.ptr, vs, kProfDepthSort, &b->tuning);
                if (err == cudaSuccess) {
                    const RasterSegment seg{(const gs_splat *)v.splats.ptr, (const uint32_t *)v.indices.ptr, ind + 1,
                                            ms[i]->n};
                    // The graph is replayed for later cameras: binning and raster take only the
                    // display mode and std dev, which are part of the shape key (frame.gt).
                    if (segmented)
                        err = launch_binning_front(&seg, 1, raster_mode(uh[i]), views[i].width, views[i].height,
                                                   v.max_pairs, v.raster_scratch.ptr, vs);
                    else if (b->tuning.raster_grid)
                        err = launch_binning(&seg, 1, raster_mode(uh[i]), views[i].width, views[i].height, v.max_pairs,
                                             v.raster_scratch.ptr, vs);
                    else
                        err = launch_raster(&seg, 1, raster_mode(uh[i]), views[i].target, views[i].width, views[i].height,
                                            views[i].pitch, v.max_pairs, v.raster_scratch.ptr, mv->frame.exact_exp, vs,
                                            &b->tuning);
                }
            }
        }
        for (uint32_t s = 0; s < nstreams && err == cudaSuccess; ++s) {
            err = cudaEventRecord(b->events[s], b->streams[s]);
            if (err == cudaSuccess) err = cudaStreamWaitEvent(b->capture, b->events[s], 0);
        }
        if (err == cudaSuccess && segmented) {
            err = launch_sort_segments(reinterpret_cast<const SortSegment *>(b->sort_segs_dev.ptr),
                                       reinterpret_cast<const uint32_t *>(b->sort_base_dev.ptr), n, sort_base[n],
                                       b->capture);
            for (uint32_t i = 0; i < n && err == cudaSuccess; ++i) {
                ViewSlot &v = b->slots[i];
                uint32_t *ind = reinterpret_cast<uint32_t *>(v.control.ptr);
                const RasterSegment seg{(const gs_splat *)v.splats.ptr, (const uint32_t *)v.indices.ptr, ind + 1, ms[i]->n};
                err = launch_binning_ranges(&seg, 1, views[i].width, views[i].height, v.max_pairs, v.raster_scratch.ptr,
                                            b->capture);
            }
        }
        if (err == cudaSuccess && b->tuning.raster_grid)
            err = launch_raster_views(reinterpret_cast<const RasterJob *>(b->jobs_dev.ptr),
                                      reinterpret_cast<const uint32_t *>(b->tile_base_dev.ptr), n, tile_base[n],
                                      raster_mode(uh[0]), mv->frame.exact_exp, b->capture, &b->tuning);
        t_capturing = false;
        cudaGraph_t graph = nullptr;
        const cudaError_t end = cudaStreamEndCapture(b->capture, &graph);
        if (err == cudaSuccess) err = end;
        if (err == cudaSuccess) err = cudaGraphInstantiate(&b->exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (err != cudaSuccess) return cuda_fail(err, "batch graph capture");
        b->graph_launches = t_captured_launches;
        b->shape = shape;
    }
    GS_CUDA(cudaMemcpyAsync(b->uniforms_dev.ptr, uh, (size_t)n * sizeof(gs_frame_uniforms), cudaMemcpyHostToDevice,
                            st));
    GS_CUDA(cudaEventRecord(b->uniforms_copied[ring], st));
    GS_CUDA(cudaGraphLaunch(b->exec, st));
    gs::g_launches.fetch_add(b->graph_launches, std::memory_order_relaxed);
    b->last.assign(views, views + n);
    return GS_OK;
}

}  // namespace

extern "C" {

gs_status gs_batch_create(gs_multi_viewer *mv, const char *const *keys, uint32_t key_count, gs_batch **out) {
    if (!mv || !out || (key_count && !keys)) return fail(GS_ERR_INVALID_ARG, "NULL argument");
    gs_batch *b = new gs_batch();
    b->mv = mv;
    for (uint32_t i = 0; i < key_count; ++i) {
        if (!keys[i]) {
            delete b;
            return fail(GS_ERR_INVALID_ARG, "key %u is NULL", i);
        }
        b->keys.emplace_back(keys[i]);
    }
    *out = b;
    return GS_OK;
}

void gs_batch_destroy(gs_batch *b) {
    if (!b) return;
    cudaDeviceSynchronize();
    delete b;
}

gs_status gs_batch_render(gs_batch *b, const gs_batch_view *views, uint32_t view_count, gs_stream stream) {
    if (!b || (view_count && !views)) return fail(GS_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> g(b->mu);
    return batch_render_locked(b, views, view_count, (cudaStream_t)stream);
}

gs_status gs_batch_synchronize(gs_batch *b, gs_stream stream) {
    if (!b) return fail(GS_ERR_INVALID_ARG, "batch is NULL");
    std::lock_guard<std::mutex> g(b->mu);
    cudaStream_t st = (cudaStream_t)stream;
    for (int attempt = 0; attempt < 4; ++attempt) {
        GS_CUDA(cudaStreamSynchronize(st));
        bool regrow = false;
        for (size_t i = 0; i < b->last.size(); ++i) {
            ViewSlot &v = b->slots[i];
            Ctrl c{}, a{}, s{};
            GS_CUDA(cudaMemcpy(&c, v.raster_scratch.ptr, sizeof(Ctrl), cudaMemcpyDeviceToHost));
            GS_CUDA(cudaMemcpy(&a, v.pre_scratch.ptr, sizeof(Ctrl), cudaMemcpyDeviceToHost));
            GS_CUDA(cudaMemcpy(&s, v.sort_scratch.ptr, sizeof(Ctrl), cudaMemcpyDeviceToHost));
            uint32_t bits = c.status | a.status | s.status;
            if (i == 0)
                for (uint32_t k = 0; k < b->chunks; ++k) {
                    Ctrl gc{};
                    GS_CUDA(cudaMemcpy(&gc, (uint8_t *)b->group_dev.ptr + k * align_up(sizeof(Ctrl), 256), sizeof(Ctrl),
                                       cudaMemcpyDeviceToHost));
                    bits |= gc.status;
                }
            if (bits & (kStatusTimeout | kStatusBounds)) return status_from_bits(bits, "batch");
            if (bits & kStatusCapacity) {
                uint64_t p = (uint64_t)c.total + c.total / 4 + 4096;
                v.max_pairs = p > 0x7FFFFFFFull ? 0x7FFFFFFFu : (uint32_t)p;
                v.raster_scratch.release();
                regrow = true;
            }
        }
        if (!regrow) return GS_OK;
        std::vector<gs_batch_view> again = b->last;
        const gs_status s = batch_render_locked(b, again.data(), (uint32_t)again.size(), st);
        if (s != GS_OK) return s;
    }
    return fail(GS_ERR_CAPACITY, "tile-pair list kept overflowing");
}

}  // extern "C"

namespace {

gs_tuning to_public(const gs::Tuning &t) {
    gs_tuning o;
    o.suffix_min = t.suffix_min;
    o.eps = t.eps;
    o.views_per_launch = t.views_per_launch;
    o.streams = t.streams;
    o.sort_match = t.sort_match;
    o.sort_digit_bits = t.sort_digit_bits;
    o.hist_blocks = t.hist_blocks;
    o.raster_grid = t.raster_grid;
    return o;
}

gs_status from_public(const gs_tuning *p, gs::Tuning *t) {
    if (!p) return fail(GS_ERR_INVALID_ARG, "tuning is NULL");
    if (p->suffix_min < 1) return fail(GS_ERR_INVALID_ARG, "suffix_min must be >= 1");
    if (!(p->eps > 0.0f && p->eps <= 0.5f)) return fail(GS_ERR_INVALID_ARG, "eps %g outside (0, 0.5]", (double)p->eps);
    if (p->views_per_launch < 1 || p->views_per_launch > kPreMaxViews)
        return fail(GS_ERR_INVALID_ARG, "views_per_launch %u outside 1..%u", p->views_per_launch, kPreMaxViews);
    if (p->streams < 1 || p->streams > kBatchStreams)
        return fail(GS_ERR_INVALID_ARG, "streams %u outside 1..%u", p->streams, kBatchStreams);
    if (p->sort_match > 1) return fail(GS_ERR_INVALID_ARG, "sort_match must be 0 or 1");
    if (p->sort_digit_bits < 6 || p->sort_digit_bits > 8)
        return fail(GS_ERR_INVALID_ARG, "sort_digit_bits %u outside 6..8", p->sort_digit_bits);
    if (p->hist_blocks > 152 * 8) return fail(GS_ERR_INVALID_ARG, "hist_blocks %u above 1216", p->hist_blocks);
    if (p->raster_grid > 1) return fail(GS_ERR_INVALID_ARG, "raster_grid must be 0 or 1");
    t->suffix_min = p->suffix_min;
    t->eps = p->eps;
    t->views_per_launch = p->views_per_launch;
    t->streams = p->streams;
    t->sort_match = p->sort_match;
    t->sort_digit_bits = p->sort_digit_bits;
    t->hist_blocks = p->hist_blocks;
    t->raster_grid = p->raster_grid;
    return GS_OK;
}

void set_tuning_locked(gs_batch *b, const gs::Tuning &t) {
    b->tuning = t;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;  // the next render captures the graph again
}

}  // namespace

extern "C" {

gs_status gs_tuning_default(gs_tuning *out) {
    if (!out) return fail(GS_ERR_INVALID_ARG, "out is NULL");
    *out = to_public(gs::default_tuning());
    return GS_OK;
}

gs_status gs_batch_set_tuning(gs_batch *b, const gs_tuning *tuning) {
    if (!b) return fail(GS_ERR_INVALID_ARG, "batch is NULL");
    gs::Tuning t;
    const gs_status s = from_public(tuning, &t);
    if (s != GS_OK) return s;
    std::lock_guard<std::mutex> g(b->mu);
    set_tuning_locked(b, t);
    return GS_OK;
}

gs_status gs_batch_get_tuning(gs_batch *b, gs_tuning *out) {
    if (!b || !out) return fail(GS_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> g(b->mu);
    *out = to_public(b->tuning);
    return GS_OK;
}

gs_status gs_batch_autotune(gs_batch *b, const gs_batch_view *views, uint32_t n, uint32_t reps, uint32_t rounds,
                            gs_tuning *out_best, double *out_ms) {
    if (!b || (n && !views)) return fail(GS_ERR_INVALID_ARG, "NULL argument");
    if (n == 0) return fail(GS_ERR_INVALID_ARG, "autotune needs at least one view");
    if (reps == 0) reps = 1;
    if (rounds == 0) rounds = 1;
    std::lock_guard<std::mutex> g(b->mu);
    cudaStream_t st = nullptr;
    GS_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    GS_CUDA(cudaEventCreate(&e0));
    GS_CUDA(cudaEventCreate(&e1));
    // Milliseconds per batch under tuning t (one warm-up render, which also captures the graph
    // and grows any tile-pair list that overflowed, then `reps` timed renders).
    auto measure = [&](const gs::Tuning &t, double *ms) -> gs_status {
        set_tuning_locked(b, t);
        for (int attempt = 0; attempt < 4; ++attempt) {
            gs_status s = batch_render_locked(b, views, n, st);
            if (s != GS_OK) return s;
            GS_CUDA(cudaStreamSynchronize(st));
            bool regrow = false;
            for (uint32_t i = 0; i < n; ++i) {
                Ctrl c{}, a{}, q{};
                GS_CUDA(cudaMemcpy(&c, b->slots[i].raster_scratch.ptr, sizeof(Ctrl), cudaMemcpyDeviceToHost));
                GS_CUDA(cudaMemcpy(&a, b->slots[i].pre_scratch.ptr, sizeof(Ctrl), cudaMemcpyDeviceToHost));
                GS_CUDA(cudaMemcpy(&q, b->slots[i].sort_scratch.ptr, sizeof(Ctrl), cudaMemcpyDeviceToHost));
                const uint32_t bad = (c.status | a.status | q.status) & (kStatusTimeout | kStatusBounds);
                if (bad) return status_from_bits(bad, "autotune");
                if (c.status & kStatusCapacity) {
                    uint64_t p = (uint64_t)c.total + c.total / 4 + 4096;
                    b->slots[i].max_pairs = p > 0x7FFFFFFFull ? 0x7FFFFFFFu : (uint32_t)p;
                    b->slots[i].raster_scratch.release();
                    regrow = true;
                }
            }
            if (!regrow) break;
        }
        GS_CUDA(cudaEventRecord(e0, st));
        for (uint32_t r = 0; r < reps; ++r) {
            const gs_status s = batch_render_locked(b, views, n, st);
            if (s != GS_OK) return s;
        }
        GS_CUDA(cudaEventRecord(e1, st));
        GS_CUDA(cudaEventSynchronize(e1));
        float f = 0.0f;
        GS_CUDA(cudaEventElapsedTime(&f, e0, e1));
        *ms = (double)f / reps;
        return GS_OK;
    };
    gs::Tuning best = b->tuning;
    double best_ms = 0.0;
    gs_status s = measure(best, &best_ms);
    // Candidate values per knob; every combination renders the same frames.
    const uint32_t suffix_c[] = {768, 1024, 1536, 2048};
    const float eps_c[] = {1e-6f, 1e-5f};
    const uint32_t vpl_c[] = {1, 4, 8, 16};
    const uint32_t streams_c[] = {4, 8, 16};
    const uint32_t match_c[] = {0, 1};
    const uint32_t hist_c[] = {0, 304, 608};
    const uint32_t digit_c[] = {6, 7, 8};
    const uint32_t grid_c[] = {0, 1};
    for (uint32_t round = 0; round < rounds && s == GS_OK; ++round) {
        for (int knob = 0; knob < 8 && s == GS_OK; ++knob) {
            const size_t nc = knob == 0   ? 4
                              : knob == 1 ? 2
                              : knob == 2 ? 4
                              : knob == 3 ? 3
                              : knob == 4 ? 2
                              : knob == 5 ? 3
                              : knob == 6 ? 3
                                          : 2;
            for (size_t c = 0; c < nc && s == GS_OK; ++c) {
                gs::Tuning t = best;
                switch (knob) {
                    case 0: t.suffix_min = suffix_c[c]; break;
                    case 1: t.eps = eps_c[c]; break;
                    case 2: t.views_per_launch = vpl_c[c]; break;
                    case 3: t.streams = streams_c[c]; break;
                    case 4: t.sort_match = match_c[c]; break;
                    case 5: t.hist_blocks = hist_c[c]; break;
                    case 6: t.sort_digit_bits = digit_c[c]; break;
                    default: t.raster_grid = grid_c[c]; break;
                }
                if (t.suffix_min == best.suffix_min && t.eps == best.eps && t.views_per_launch == best.views_per_launch &&
                    t.streams == best.streams && t.sort_match == best.sort_match && t.hist_blocks == best.hist_blocks &&
                    t.sort_digit_bits == best.sort_digit_bits &&
                    t.raster_grid == best.raster_grid)
                    continue;
                double ms = 0.0;
                s = measure(t, &ms);
                if (s == GS_OK && ms < best_ms) {
                    best_ms = ms;
                    best = t;
                }
            }
        }
    }
    set_tuning_locked(b, best);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    if (s != GS_OK) return s;
    if (out_best) *out_best = to_public(best);
    if (out_ms) *out_ms = best_ms;
    return GS_OK;
}

}  // extern "C"

// ---- Serving: resident scenes, admission by per-view memory, overlapping requests ------------
namespace {

double now_ms() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Device bytes one request holds while admitted: its key/index/splat buffers, scratch of the
// three stages (tile-pair list at the default capacity) and its render target.
size_t request_bytes(uint32_t n, uint32_t w, uint32_t h) {
    return (size_t)n * (4 + 4 + sizeof(gs_splat)) + preprocess_scratch_bytes(n) + sort_scratch_bytes(n, kDepthKeyBits) +
           raster_scratch_bytes(n, w, h, default_pairs(n, w, h)) + (size_t)w * h * 4;
}

struct ServerReq {
    const Model *model = nullptr;
    gs_camera_pod camera{};
    uint32_t w = 0, h = 0, pitch = 0;
    uint8_t *out = nullptr;
    int out_on_host = 0;
    size_t bytes = 0;
    double t_submit = 0, t_done = 0;
    int state = 0;  // 0 queued, 1 running, 2 done, 3 failed
    int slot = -1;
};

struct ServerSlot {
    ViewSlot view;
    DevBuf target;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    uint64_t req = 0;
    bool busy = false;
    // Dynamic batching: this slot's uniforms on the device; as a group's leader, the group's
    // PreView descriptors and control block, and the pinned staging they are copied from.
    DevBuf u_dev, views_dev, group;
    gs_frame_uniforms *u_host = nullptr;
    PreView *views_host = nullptr;
    cudaEvent_t pre_done = nullptr;
};

}  // namespace

struct gs_server {
    gs_multi_viewer *mv = nullptr;
    size_t budget = 0, reserved = 0;
    uint32_t batch_views = kPreMaxViews;  // requests of one scene sharing a preprocess launch
    double batch_wait_ms = 0.0;           // how long admission may hold for more free slots
    double hold_since = -1.0;             // when the current hold began (-1: not holding)
    std::vector<ServerSlot> slots;
    std::deque<uint64_t> queue;
    std::unordered_map<uint64_t, ServerReq> reqs;
    std::vector<double> lat;
    uint64_t next = 1, completed = 0, failed = 0;
    std::thread worker;
    std::mutex mu;
    std::condition_variable cv, done_cv;
    bool stop = false;
    gs_status error = GS_OK;

    ~gs_server() {
        {
            std::lock_guard<std::mutex> g(mu);
            stop = true;
        }
        cv.notify_all();
        if (worker.joinable()) worker.join();
        for (auto &sl : slots) {
            if (sl.stream) {
                cudaStreamSynchronize(sl.stream);
                cudaStreamDestroy(sl.stream);
            }
            if (sl.done) cudaEventDestroy(sl.done);
            if (sl.pre_done) cudaEventDestroy(sl.pre_done);
            if (sl.u_host) cudaFreeHost(sl.u_host);
            if (sl.views_host) cudaFreeHost(sl.views_host);
        }
    }
};

namespace {

// Buffers, target and uniforms of one admitted request (scheduler thread, server lock held).
gs_status server_prepare(gs_server *sv, ServerReq &r, ServerSlot &sl, uint8_t **target, uint32_t *pitch,
                         gs_frame_uniforms *u) {
    bool changed = false;
    GS_CUDA(sl.view.prepare(r.model, r.w, r.h, &changed));
    *target = r.out;
    *pitch = r.pitch;
    if (r.out_on_host || !r.out) {
        GS_CUDA(sl.target.ensure((size_t)r.w * r.h * 4));
        *target = (uint8_t *)sl.target.ptr;
        *pitch = r.w * 4;
    }
    gs_gaussian_transform_pod gt;
    {
        std::lock_guard<std::mutex> g(sv->mv->mu);
        gt = sv->mv->frame.gt;
    }
    return gs_frame_uniforms_build(&r.camera, &r.model->model, &gt, r.w, r.h, u);
}

// Depth sort, raster, read-back and completion event of a request whose preprocess is enqueued
// (`tiles`: that preprocess also stored the splats' tile records in the slot's binfo).
gs_status server_finish(gs_server *sv, ServerReq &r, ServerSlot &sl, uint8_t *target, uint32_t pitch,
                        const gs_frame_uniforms &u, bool tiles) {
    const Model *m = r.model;
    ViewSlot &v = sl.view;
    uint32_t *ind = reinterpret_cast<uint32_t *>(v.control.ptr);
    cudaError_t e = launch_sort((uint32_t *)v.depths.ptr, (uint32_t *)v.indices.ptr, m->n, ind + 1, kDepthKeyBits,
                                v.sort_scratch.ptr, sl.stream);
    if (e == cudaSuccess) {
        RasterSegment seg{(const gs_splat *)v.splats.ptr, (const uint32_t *)v.indices.ptr, ind + 1, m->n};
        if (tiles) {
            seg.binfo = reinterpret_cast<const uint4 *>(v.binfo.ptr);
            seg.binfo_w = r.w;
            seg.binfo_h = r.h;
        }
        e = launch_raster(&seg, 1, raster_mode(u), target, r.w, r.h, pitch, v.max_pairs, v.raster_scratch.ptr,
                          sv->mv->frame.exact_exp, sl.stream);
    }
    if (e == cudaSuccess && r.out_on_host && r.out)
        e = cudaMemcpyAsync(r.out, target, (size_t)r.w * r.h * 4, cudaMemcpyDeviceToHost, sl.stream);
    if (e == cudaSuccess) e = cudaEventRecord(sl.done, sl.stream);
    if (e != cudaSuccess) return cuda_fail(e, "server launch");
    return GS_OK;
}

// Enqueue one admitted request on its slot's stream (scheduler thread, server lock held).
gs_status server_launch(gs_server *sv, ServerReq &r, ServerSlot &sl) {
    uint8_t *target;
    uint32_t pitch;
    gs_frame_uniforms u;
    gs_status s = server_prepare(sv, r, sl, &target, &pitch, &u);
    if (s != GS_OK) return s;
    const Model *m = r.model;
    ViewSlot &v = sl.view;
    uint32_t *ind = reinterpret_cast<uint32_t *>(v.control.ptr);
    GS_CUDA(v.binfo.ensure((size_t)(m->n ? m->n : 1) * sizeof(uint4)));
    const cudaError_t e = launch_preprocess(u, m->records.ptr, m->format, m->n,
                                            m->has_selection ? (const uint32_t *)m->selection.ptr : nullptr, m->invert,
                                            ind, ind + 4, (uint32_t *)v.indices.ptr, (float *)v.depths.ptr,
                                            gs_depth_capacity(m->n), (gs_splat *)v.splats.ptr, v.pre_scratch.ptr,
                                            sl.stream, nullptr, reinterpret_cast<uint4 *>(v.binfo.ptr));
    if (e != cudaSuccess) return cuda_fail(e, "server launch");
    return server_finish(sv, r, sl, target, pitch, u, true);
}

// Dynamic batching: admitted requests of one scene (group[0] leads) share one preprocess launch
// that reads the scene's records once; each then sorts, rasterises and completes on its own
// slot's stream.  The leader slot's staging stays untouched until the leader completes, which is
// after the shared launch.
gs_status server_launch_group(gs_server *sv, const std::vector<std::pair<ServerReq *, ServerSlot *>> &group) {
    if (group.size() == 1) return server_launch(sv, *group[0].first, *group[0].second);
    ServerSlot &lead = *group[0].second;
    const Model *m = group[0].first->model;
    const size_t nv = group.size();
    if (!lead.views_host) GS_CUDA(cudaMallocHost(&lead.views_host, kPreMaxViews * sizeof(PreView)));
    GS_CUDA(lead.views_dev.ensure(kPreMaxViews * sizeof(PreView)));
    if (!lead.group.ptr) {
        GS_CUDA(lead.group.ensure(align_up(sizeof(Ctrl), 256)));
        GS_CUDA(cudaMemset(lead.group.ptr, 0, align_up(sizeof(Ctrl), 256)));
    }
    if (!lead.pre_done) GS_CUDA(cudaEventCreateWithFlags(&lead.pre_done, cudaEventDisableTiming));
    std::vector<uint8_t *> targets(nv);
    std::vector<uint32_t> pitches(nv);
    std::vector<gs_frame_uniforms> us(nv);
    for (size_t k = 0; k < nv; ++k) {
        ServerReq &r = *group[k].first;
        ServerSlot &sl = *group[k].second;
        gs_status s = server_prepare(sv, r, sl, &targets[k], &pitches[k], &us[k]);
        if (s != GS_OK) return s;
        if (!sl.u_host) GS_CUDA(cudaMallocHost(&sl.u_host, sizeof(gs_frame_uniforms)));
        GS_CUDA(sl.u_dev.ensure(sizeof(gs_frame_uniforms)));
        *sl.u_host = us[k];
        ViewSlot &v = sl.view;
        uint32_t *ind = reinterpret_cast<uint32_t *>(v.control.ptr);
        lead.views_host[k] = preprocess_view((const gs_frame_uniforms *)sl.u_dev.ptr, ind, ind + 4,
                                             (uint32_t *)v.indices.ptr, (float *)v.depths.ptr, gs_depth_capacity(m->n),
                                             (gs_splat *)v.splats.ptr, v.pre_scratch.ptr);
        GS_CUDA(cudaMemcpyAsync(sl.u_dev.ptr, sl.u_host, sizeof(gs_frame_uniforms), cudaMemcpyHostToDevice,
                                lead.stream));
    }
    GS_CUDA(cudaMemcpyAsync(lead.views_dev.ptr, lead.views_host, nv * sizeof(PreView), cudaMemcpyHostToDevice,
                            lead.stream));
    cudaError_t e = launch_preprocess_views(m->records.ptr, m->format, m->n,
                                            m->has_selection ? (const uint32_t *)m->selection.ptr : nullptr, m->invert,
                                            (const PreView *)lead.views_dev.ptr, (uint32_t)nv, lead.group.ptr,
                                            lead.stream);
    if (e == cudaSuccess) e = cudaEventRecord(lead.pre_done, lead.stream);
    if (e != cudaSuccess) return cuda_fail(e, "server group launch");
    for (size_t k = 0; k < nv; ++k) {
        ServerSlot &sl = *group[k].second;
        if (k > 0) GS_CUDA(cudaStreamWaitEvent(sl.stream, lead.pre_done, 0));
        const gs_status s = server_finish(sv, *group[k].first, sl, targets[k], pitches[k], us[k], false);
        if (s != GS_OK) return s;
    }
    return GS_OK;
}

void server_loop(gs_server *sv) {
    std::unique_lock<std::mutex> lk(sv->mu);
    while (!sv->stop) {
        bool busy = false;
        // completions
        for (size_t i = 0; i < sv->slots.size(); ++i) {
            ServerSlot &sl = sv->slots[i];
            if (!sl.busy) continue;
            const cudaError_t q = cudaEventQuery(sl.done);
            if (q == cudaErrorNotReady) {
                busy = true;
                continue;
            }
            ServerReq &r = sv->reqs[sl.req];
            r.t_done = now_ms();
            Ctrl c{};
            uint32_t bits = 0;
            if (q == cudaSuccess && cudaMemcpy(&c, sl.view.raster_scratch.ptr, sizeof(Ctrl), cudaMemcpyDeviceToHost) == cudaSuccess)
                bits = c.status;
            if (q != cudaSuccess || (bits & kStatusTimeout)) {
                r.state = 3;
                ++sv->failed;
            } else if (bits & kStatusCapacity) {
                // grow this slot's tile-pair list and run the request again
                uint64_t p = (uint64_t)c.total + c.total / 4 + 4096;
                sl.view.max_pairs = p > 0x7FFFFFFFull ? 0x7FFFFFFFu : (uint32_t)p;
                sl.view.raster_scratch.release();
                if (server_launch(sv, r, sl) == GS_OK) {
                    busy = true;
                    continue;
                }
                r.state = 3;
                ++sv->failed;
            } else {
                r.state = 2;
                ++sv->completed;
                sv->lat.push_back(r.t_done - r.t_submit);
            }
            sv->reserved -= r.bytes;
            sl.busy = false;
            sv->done_cv.notify_all();
        }
        // admissions, first come first served, while memory and a slot are free; queued requests
        // of the head's scene join its group (dynamic batching, up to batch_views requests)
        while (!sv->queue.empty()) {
            ServerReq &head = sv->reqs[sv->queue.front()];
            if (sv->reserved > 0 && sv->reserved + head.bytes > sv->budget) break;
            std::vector<size_t> free_slots;
            for (size_t i = 0; i < sv->slots.size(); ++i)
                if (!sv->slots[i].busy) free_slots.push_back(i);
            if (free_slots.empty()) break;
            if (sv->batch_wait_ms > 0.0 && free_slots.size() < sv->slots.size()) {
                // batching window: while more of the head's scene's requests are queued than
                // slots are free and busy slots will free up, hold admission for up to
                // batch_wait_ms from when the hold began
                size_t same = 0;
                const size_t scan = std::min(sv->queue.size(), (size_t)64);
                for (size_t q = 0; q < scan; ++q)
                    if (sv->reqs[sv->queue[q]].model == head.model) ++same;
                if (free_slots.size() < std::min<size_t>(same, sv->batch_views)) {
                    const double t = now_ms();
                    if (sv->hold_since < 0.0) sv->hold_since = t;
                    if (t - sv->hold_since < sv->batch_wait_ms) {
                        busy = true;  // poll again soon
                        break;
                    }
                }
            }
            sv->hold_since = -1.0;
            std::vector<std::pair<uint64_t, size_t>> members;  // (request id, slot)
            size_t reserve = 0;
            const size_t scan = std::min(sv->queue.size(), (size_t)64);
            std::vector<size_t> taken;  // queue positions
            for (size_t q = 0; q < scan && members.size() < free_slots.size() && members.size() < sv->batch_views; ++q) {
                const uint64_t id = sv->queue[q];
                ServerReq &r = sv->reqs[id];
                if (q > 0 && r.model != head.model) continue;
                if (q > 0 && sv->reserved + reserve + r.bytes > sv->budget) continue;
                members.emplace_back(id, free_slots[members.size()]);
                taken.push_back(q);
                reserve += r.bytes;
            }
            for (size_t t = taken.size(); t-- > 0;) sv->queue.erase(sv->queue.begin() + (ptrdiff_t)taken[t]);
            std::vector<std::pair<ServerReq *, ServerSlot *>> group;
            for (auto &mb : members) {
                ServerReq &r = sv->reqs[mb.first];
                ServerSlot &sl = sv->slots[mb.second];
                r.slot = (int)mb.second;
                r.state = 1;
                sv->reserved += r.bytes;
                sl.busy = true;
                sl.req = mb.first;
                group.emplace_back(&r, &sl);
            }
            if (server_launch_group(sv, group) != GS_OK) {
                for (auto &g : group) {
                    g.first->state = 3;
                    ++sv->failed;
                    sv->reserved -= g.first->bytes;
                    g.second->busy = false;
                }
                sv->done_cv.notify_all();
            } else {
                busy = true;
            }
        }
        if (busy) {
            lk.unlock();
            std::this_thread::sleep_for(std::chrono::microseconds(20));
            lk.lock();
        } else {
            sv->cv.wait_for(lk, std::chrono::milliseconds(5));
        }
    }
}

}  // namespace

extern "C" {

gs_status gs_server_create(gs_multi_viewer *mv, size_t budget_bytes, uint32_t max_inflight, gs_server **out) {
    if (!mv || !out || max_inflight == 0) return fail(GS_ERR_INVALID_ARG, "invalid server arguments");
    gs_server *sv = new gs_server();
    sv->mv = mv;
    sv->budget = budget_bytes;
    sv->slots.resize(max_inflight);
    for (auto &sl : sv->slots) {
        cudaError_t e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            delete sv;
            return cuda_fail(e, "server streams");
        }
    }
    sv->worker = std::thread(server_loop, sv);
    *out = sv;
    return GS_OK;
}

void gs_server_destroy(gs_server *sv) { delete sv; }

gs_status gs_server_submit(gs_server *sv, const char *key, const gs_camera_pod *camera, uint32_t width, uint32_t height,
                           uint8_t *out, uint32_t out_pitch, int out_on_host, uint64_t *ticket) {
    if (!sv || !key || !camera || !ticket || width == 0 || height == 0) return fail(GS_ERR_INVALID_ARG, "invalid request");
    if (out && !out_on_host && (out_pitch < 4 * width || out_pitch % 4 || !aligned(out, 4)))
        return fail(GS_ERR_INVALID_ARG, "invalid output pitch");
    const Model *m = nullptr;
    {
        std::lock_guard<std::mutex> g(sv->mv->mu);
        auto it = sv->mv->models.find(key);
        if (it == sv->mv->models.end()) return fail(GS_ERR_NOT_FOUND, "model '%s' not found", key);
        m = it->second;
    }
    ServerReq r;
    r.model = m;
    r.camera = *camera;
    r.w = width;
    r.h = height;
    r.out = out;
    r.pitch = out_pitch;
    r.out_on_host = out_on_host;
    r.bytes = request_bytes(m->n, width, height);
    if (r.bytes > sv->budget) return fail(GS_ERR_ADMISSION, "request needs %zu bytes, budget is %zu", r.bytes, sv->budget);
    r.t_submit = now_ms();
    {
        std::lock_guard<std::mutex> g(sv->mu);
        const uint64_t id = sv->next++;
        sv->reqs.emplace(id, r);
        sv->queue.push_back(id);
        *ticket = id;
    }
    sv->cv.notify_all();
    return GS_OK;
}

gs_status gs_server_wait(gs_server *sv, uint64_t ticket, double timeout_s, double *latency_ms) {
    if (!sv) return fail(GS_ERR_INVALID_ARG, "server is NULL");
    std::unique_lock<std::mutex> lk(sv->mu);
    auto it = sv->reqs.find(ticket);
    if (it == sv->reqs.end()) return fail(GS_ERR_NOT_FOUND, "unknown ticket");
    const bool ok = sv->done_cv.wait_for(lk, std::chrono::duration<double>(timeout_s),
                                         [&] { return it->second.state >= 2; });
    if (!ok) return fail(GS_ERR_TIMEOUT, "request still running after %.3f s", timeout_s);
    if (latency_ms) *latency_ms = it->second.t_done - it->second.t_submit;
    const int state = it->second.state;
    sv->reqs.erase(it);
    return state == 2 ? GS_OK : fail(GS_ERR_CUDA, "request failed on the device");
}

gs_status gs_server_stats(gs_server *sv, gs_server_report *out) {
    if (!sv || !out) return fail(GS_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> g(sv->mu);
    out->completed = sv->completed;
    out->failed = sv->failed;
    out->queued = (uint32_t)sv->queue.size();
    uint32_t running = 0;
    for (auto &sl : sv->slots) running += sl.busy ? 1u : 0u;
    out->running = running;
    out->reserved_bytes = sv->reserved;
    std::vector<double> l = sv->lat;
    std::sort(l.begin(), l.end());
    auto pct = [&](double q) { return l.empty() ? 0.0 : l[std::min(l.size() - 1, (size_t)(q * (l.size() - 1) + 0.5))]; };
    out->p50_ms = pct(0.50);
    out->p99_ms = pct(0.99);
    double sum = 0;
    for (double x : l) sum += x;
    out->mean_ms = l.empty() ? 0.0 : sum / l.size();
    out->max_ms = l.empty() ? 0.0 : l.back();
    return GS_OK;
}

gs_status gs_server_reset_stats(gs_server *sv) {
    if (!sv) return fail(GS_ERR_INVALID_ARG, "server is NULL");
    std::lock_guard<std::mutex> g(sv->mu);
    sv->lat.clear();
    sv->completed = 0;
    sv->failed = 0;
    return GS_OK;
}

size_t gs_server_request_bytes(uint32_t n, uint32_t width, uint32_t height) { return request_bytes(n, width, height); }

gs_status gs_server_set_batching(gs_server *sv, uint32_t max_views, double max_wait_ms) {
    if (!sv) return fail(GS_ERR_INVALID_ARG, "server is NULL");
    if (max_views < 1 || max_views > kPreMaxViews)
        return fail(GS_ERR_INVALID_ARG, "max_views %u outside 1..%u", max_views, kPreMaxViews);
    if (!(max_wait_ms >= 0.0 && max_wait_ms <= 1000.0))
        return fail(GS_ERR_INVALID_ARG, "max_wait_ms %g outside 0..1000", max_wait_ms);
    std::lock_guard<std::mutex> g(sv->mu);
    sv->batch_views = max_views;
    sv->batch_wait_ms = max_wait_ms;
    return GS_OK;
}

}  // extern "C"
