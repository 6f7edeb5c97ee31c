// gs_ply.cu — PLY ingest: host scan of the header, device conversion of the vertex block into
// records.
//
// The reference reads scenes with wgpu-3dgs-core's Gaussians::read_from_file(path,
// GaussiansSource::Ply) (examples/simple.rs:157-160) and uploads them with Viewer::new.  Here
// the header (a few hundred bytes of text) is scanned on the host and the vertex block goes to
// the device as it is in the file; one kernel then turns each vertex into a record.
//
// Kernel layout: a CTA owns 128 consecutive vertices.  It copies their bytes (128 × stride)
// into shared memory with coalesced 4-byte loads, so a field at any byte offset is one or two
// shared words joined by a funnel shift (strides need not be multiples of 4).  Each thread
// builds its record in registers and stores it into a dense shared row; one cp.async.bulk
// store then writes the CTA's records (128 × 224 B or 128 × 128 B) to global memory.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_bf16.h>

#include "gs_internal.h"

namespace gs {

constexpr uint32_t kPlyThreads = 128;
constexpr uint32_t kPlyMaxStride = 1024;

// ---- header scan --------------------------------------------------------------------------
namespace {

int ply_type_bytes(const std::string &t) {
    if (t == "char" || t == "uchar" || t == "int8" || t == "uint8") return 1;
    if (t == "short" || t == "ushort" || t == "int16" || t == "uint16") return 2;
    if (t == "int" || t == "uint" || t == "int32" || t == "uint32" || t == "float" || t == "float32") return 4;
    if (t == "double" || t == "float64") return 8;
    return 0;
}

bool is_float32(const std::string &t) { return t == "float" || t == "float32"; }

gs_status ply_fail(const char *fmt, const char *arg = "") {
    char buf[256];
    snprintf(buf, sizeof(buf), fmt, arg);
    return set_error(GS_ERR_INVALID_ARG, buf);
}

std::vector<std::string> split_ws(const std::string &line) {
    std::vector<std::string> out;
    size_t i = 0;
    while (i < line.size()) {
        while (i < line.size() && (line[i] == ' ' || line[i] == '\t' || line[i] == '\r')) ++i;
        size_t j = i;
        while (j < line.size() && !(line[j] == ' ' || line[j] == '\t' || line[j] == '\r')) ++j;
        if (j > i) out.emplace_back(line.substr(i, j - i));
        i = j;
    }
    return out;
}

bool parse_u64(const std::string &s, uint64_t *v) {
    if (s.empty() || s.size() > 19) return false;
    uint64_t x = 0;
    for (char c : s) {
        if (c < '0' || c > '9') return false;
        x = x * 10 + (uint64_t)(c - '0');
    }
    *v = x;
    return true;
}

}  // namespace

// Checks that every field offset the kernel reads lies inside a vertex.
gs_status ply_check_layout(const gs_ply_layout *L) {
    if (!L) return set_error(GS_ERR_INVALID_ARG, "PLY layout is NULL");
    if (L->stride < 4 || L->stride > kPlyMaxStride) return ply_fail("PLY vertex stride out of range 4..1024");
    if (!(L->sh_rest == 0 || L->sh_rest == 3 || L->sh_rest == 8 || L->sh_rest == 15))
        return ply_fail("PLY f_rest coefficients per channel must be 0, 3, 8 or 15");
    auto ok = [&](int32_t off) { return off >= 0 && (uint32_t)off + 4u <= L->stride; };
    for (int k = 0; k < 3; ++k)
        if (!ok(L->pos[k]) || !ok(L->f_dc[k]) || !ok(L->scale[k])) return ply_fail("PLY field offset outside a vertex");
    for (int k = 0; k < 4; ++k)
        if (!ok(L->rot[k])) return ply_fail("PLY field offset outside a vertex");
    if (!ok(L->opacity)) return ply_fail("PLY field offset outside a vertex");
    for (uint32_t k = 0; k < 3 * L->sh_rest; ++k)
        if (!ok(L->f_rest[k])) return ply_fail("PLY field offset outside a vertex");
    return GS_OK;
}

}  // namespace gs

using namespace gs;

extern "C" gs_status gs_ply_parse_header(const void *bytes, size_t len, gs_ply_layout *out) {
    if (!bytes || !out) return set_error(GS_ERR_INVALID_ARG, "NULL argument");
    const char *p = static_cast<const char *>(bytes);
    static const char kEnd[] = "end_header\n";
    const size_t kEndLen = sizeof(kEnd) - 1;
    if (len < 3 || std::memcmp(p, "ply", 3) != 0) return ply_fail("not a PLY file");
    size_t end = std::string::npos;
    for (size_t i = 0; i + kEndLen <= len; ++i) {
        if (p[i] == 'e' && std::memcmp(p + i, kEnd, kEndLen) == 0) {
            end = i;
            break;
        }
    }
    if (end == std::string::npos) return ply_fail("PLY header has no end_header line");
    const std::string head(p, end);

    gs_ply_layout L;
    std::memset(&L, 0, sizeof(L));
    int32_t *req[14] = {&L.pos[0], &L.pos[1], &L.pos[2], &L.f_dc[0], &L.f_dc[1], &L.f_dc[2], &L.opacity,
                        &L.scale[0], &L.scale[1], &L.scale[2], &L.rot[0], &L.rot[1], &L.rot[2], &L.rot[3]};
    static const char *kReq[14] = {"x", "y", "z", "f_dc_0", "f_dc_1", "f_dc_2", "opacity",
                                   "scale_0", "scale_1", "scale_2", "rot_0", "rot_1", "rot_2", "rot_3"};
    for (int k = 0; k < 14; ++k) *req[k] = -1;
    for (int k = 0; k < 45; ++k) L.f_rest[k] = -1;

    struct Element {
        std::string name;
        uint64_t count = 0, stride = 0;
        bool has_list = false;
    };
    std::vector<Element> elems;
    std::string format;
    uint32_t rest_seen = 0;
    size_t pos = 0;
    bool magic = true;
    while (pos < head.size()) {
        size_t nl = head.find('\n', pos);
        if (nl == std::string::npos) nl = head.size();
        const std::vector<std::string> t = split_ws(head.substr(pos, nl - pos));
        pos = nl + 1;
        if (magic) {  // the "ply" line
            magic = false;
            continue;
        }
        if (t.empty() || t[0] == "comment" || t[0] == "obj_info") continue;
        if (t[0] == "format") {
            if (t.size() < 2) return ply_fail("PLY format line is malformed");
            format = t[1];
        } else if (t[0] == "element") {
            Element e;
            if (t.size() < 3 || !parse_u64(t[2], &e.count)) return ply_fail("PLY element line is malformed");
            e.name = t[1];
            if (e.name == "vertex")
                for (const Element &o : elems)
                    if (o.name == "vertex") return ply_fail("PLY has two vertex elements");
            elems.push_back(e);
        } else if (t[0] == "property") {
            if (elems.empty()) return ply_fail("PLY property before any element");
            Element &e = elems.back();
            if (t.size() >= 2 && t[1] == "list") {
                if (e.name == "vertex") return ply_fail("list properties are not supported in the vertex element");
                e.has_list = true;
                continue;
            }
            if (t.size() < 3) return ply_fail("PLY property line is malformed");
            const int b = ply_type_bytes(t[1]);
            if (!b) return ply_fail("unknown PLY property type '%s'", t[1].c_str());
            if (e.name == "vertex") {
                const std::string &name = t[2];
                for (int k = 0; k < 14; ++k) {
                    if (name == kReq[k]) {
                        if (!is_float32(t[1])) return ply_fail("PLY property '%s' must be float", kReq[k]);
                        *req[k] = (int32_t)e.stride;
                    }
                }
                if (name.rfind("f_rest_", 0) == 0) {
                    uint64_t idx = 0;
                    if (!parse_u64(name.substr(7), &idx) || idx >= 45)
                        return ply_fail("PLY property '%s' is beyond SH degree 3", name.c_str());
                    if (!is_float32(t[1])) return ply_fail("PLY property '%s' must be float", name.c_str());
                    L.f_rest[idx] = (int32_t)e.stride;
                    ++rest_seen;
                }
                if (e.stride + (uint64_t)b > kPlyMaxStride) return ply_fail("PLY vertex stride out of range 4..1024");
            }
            e.stride += (uint64_t)b;
        } else {
            return ply_fail("unknown PLY header line '%s'", t[0].c_str());
        }
    }
    if (format != "binary_little_endian") return ply_fail("unsupported PLY format '%s'", format.c_str());
    // the vertex block follows the elements declared before it
    uint64_t before = 0, count = 0, vstride = 0;
    bool seen_vertex = false;
    for (const Element &e : elems) {
        if (e.name == "vertex") {
            seen_vertex = true;
            count = e.count;
            vstride = e.stride;
            break;
        }
        if (e.has_list) return ply_fail("PLY element '%s' before the vertex element has a list property", e.name.c_str());
        before += e.count * e.stride;
    }
    if (!seen_vertex) return ply_fail("PLY has no vertex element");
    if (count > 0xFFFFFFFFull) return ply_fail("PLY vertex count above 2^32 - 1");
    for (int k = 0; k < 14; ++k)
        if (*req[k] < 0) return ply_fail("PLY vertex element lacks property '%s'", kReq[k]);
    if (!(rest_seen == 0 || rest_seen == 9 || rest_seen == 24 || rest_seen == 45))
        return ply_fail("PLY f_rest count must be 0, 9, 24 or 45");
    for (uint32_t k = 0; k < rest_seen; ++k)
        if (L.f_rest[k] < 0) return ply_fail("PLY f_rest properties are not numbered 0..n-1");
    L.data_offset = (uint64_t)end + kEndLen + before;
    L.count = (uint32_t)count;
    L.stride = (uint32_t)vstride;
    L.sh_rest = rest_seen / 3;
    const gs_status s = ply_check_layout(&L);
    if (s != GS_OK) return s;
    *out = L;
    return GS_OK;
}

namespace gs {

struct PlyParams {
    gs_ply_layout L;
    const uint8_t *vertices;
    uint8_t *records;
};

// The float at byte b of the staged words (b need not be a multiple of 4).
__device__ __forceinline__ float staged_f32(const uint32_t *s, uint32_t b) {
    const uint32_t w = b >> 2, sh = (b & 3u) * 8u;
    uint32_t v = s[w];
    if (sh) v = __funnelshift_r(v, s[w + 1], sh);
    return __uint_as_float(v);
}

__device__ __forceinline__ uint32_t f16_bits(float x) { return (uint32_t)__half_as_ushort(__float2half_rn(x)); }
__device__ __forceinline__ uint32_t bf16_bits(float x) {
    return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(x));
}

template <uint32_t FMT>
__global__ void __launch_bounds__(kPlyThreads) ply_convert_kernel(const __grid_constant__ PlyParams P) {
    constexpr uint32_t REC = (FMT == GS_FORMAT_FP32) ? 224u : 128u;
    extern __shared__ __align__(16) uint8_t smem[];
    uint4 *s_out = reinterpret_cast<uint4 *>(smem);                      // kPlyThreads × REC
    uint32_t *s_in = reinterpret_cast<uint32_t *>(smem + kPlyThreads * REC);  // staged vertex words
    const gs_ply_layout &L = P.L;
    const uint32_t tid = threadIdx.x;
    const uint64_t first = (uint64_t)blockIdx.x * kPlyThreads;
    const uint32_t cnt = (uint32_t)min((uint64_t)kPlyThreads, (uint64_t)L.count - first);

    // ---- stage the CTA's vertex bytes [b0, b1) as the words that cover them ----
    const uint64_t total = (uint64_t)L.count * L.stride;
    const uint64_t b0 = first * L.stride, b1 = (first + cnt) * L.stride;
    const uint64_t w0 = b0 >> 2, w1 = (b1 + 3) >> 2;
    const uint32_t nw = (uint32_t)(w1 - w0);
    const uint32_t *v32 = reinterpret_cast<const uint32_t *>(P.vertices);
    const uint64_t whole = total >> 2;  // words lying wholly inside the vertex block
    for (uint32_t k = tid; k < nw; k += kPlyThreads) {
        const uint64_t w = w0 + k;
        uint32_t v;
        if (w < whole) {
            v = __ldcs(v32 + w);
        } else {  // the block's last, partial word: only its bytes below `total`
            v = 0;
            for (uint32_t j = 0; j < 4; ++j)
                if (w * 4 + j < total) v |= (uint32_t)P.vertices[w * 4 + j] << (8 * j);
        }
        s_in[k] = v;
    }
    __syncthreads();

    if (tid < cnt) {
        const uint32_t base = (uint32_t)((first + tid) * L.stride - (w0 << 2));
        auto rd = [&](int32_t off) { return staged_f32(s_in, base + (uint32_t)off); };
        // colour: rgb = 0.5 + SH_C0·f_dc and a = sigmoid(opacity), to 8 bits
        uint32_t color = 0;
#pragma unroll
        for (int c = 0; c < 3; ++c) color |= unorm8_rne(0.5 + kShC0 * (double)rd(L.f_dc[c])) << (8 * c);
        color |= unorm8_rne(1.0 / (1.0 + exp(-(double)rd(L.opacity)))) << 24;
        float scale[3], rot[4];
#pragma unroll
        for (int k = 0; k < 3; ++k) scale[k] = (float)exp((double)rd(L.scale[k]));
        {
            const double q[4] = {rd(L.rot[1]), rd(L.rot[2]), rd(L.rot[3]), rd(L.rot[0])};  // x, y, z, w
            const double nrm = sqrt(((q[0] * q[0] + q[1] * q[1]) + q[2] * q[2]) + q[3] * q[3]);
#pragma unroll
            for (int k = 0; k < 4; ++k) rot[k] = (float)(q[k] / nrm);
        }
        // SH: f_rest is channel-major (K coefficients of R, then G, then B); sh[3k + c]
        const uint32_t K = L.sh_rest;
        auto sh = [&](int k, int c) { return (uint32_t)k < K ? rd(L.f_rest[c * K + k]) : 0.0f; };
        uint4 *row = s_out + tid * (REC / 16);
        if constexpr (FMT == GS_FORMAT_FP32) {
            uint32_t w[56];
            w[0] = __float_as_uint(rd(L.pos[0]));
            w[1] = __float_as_uint(rd(L.pos[1]));
            w[2] = __float_as_uint(rd(L.pos[2]));
            w[3] = color;
#pragma unroll
            for (int k = 0; k < 15; ++k)
#pragma unroll
                for (int c = 0; c < 3; ++c) w[4 + 3 * k + c] = __float_as_uint(sh(k, c));
            float cov[6];
            cov3d_from_rot_scale(rot, scale, cov);
#pragma unroll
            for (int k = 0; k < 6; ++k) w[49 + k] = __float_as_uint(cov[k]);
            w[55] = 0u;
#pragma unroll
            for (int k = 0; k < 14; ++k) row[k] = make_uint4(w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]);
        } else {
            uint32_t h[64];  // the record as 16-bit units
#pragma unroll
            for (int k = 0; k < 64; ++k) h[k] = 0u;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const uint32_t b = __float_as_uint(rd(L.pos[k]));
                h[2 * k] = b & 0xFFFFu;
                h[2 * k + 1] = b >> 16;
            }
            h[6] = color & 0xFFFFu;
            h[7] = color >> 16;
#pragma unroll
            for (int k = 0; k < 4; ++k) h[8 + k] = f16_bits(rot[k]);
#pragma unroll
            for (int k = 0; k < 3; ++k) h[12 + k] = f16_bits(scale[k]);
#pragma unroll
            for (int k = 0; k < 15; ++k)
#pragma unroll
                for (int c = 0; c < 3; ++c)
                    h[15 + 3 * k + c] = (FMT == GS_FORMAT_HALF_SH_FP16) ? f16_bits(sh(k, c)) : bf16_bits(sh(k, c));
#pragma unroll
            for (int k = 0; k < 8; ++k)
                row[k] = make_uint4(h[8 * k] | (h[8 * k + 1] << 16), h[8 * k + 2] | (h[8 * k + 3] << 16),
                                    h[8 * k + 4] | (h[8 * k + 5] << 16), h[8 * k + 6] | (h[8 * k + 7] << 16));
        }
    }

    // ---- one bulk store of the CTA's records (generic-proxy writes made visible to it first) ----
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
        const uint32_t src = (uint32_t)__cvta_generic_to_shared(s_out);
        uint8_t *dst = P.records + first * REC;
        asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(src),
                     "r"(cnt * REC)
                     : "memory");
        asm volatile("cp.async.bulk.commit_group;" ::: "memory");
        asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    }
}

template <uint32_t FMT>
cudaError_t launch_ply_fmt(const PlyParams &P, cudaStream_t st) {
    constexpr uint32_t REC = (FMT == GS_FORMAT_FP32) ? 224u : 128u;
    const size_t smem = kPlyThreads * REC + align_up((size_t)kPlyThreads * P.L.stride + 8, 16);
    cudaError_t e = cudaFuncSetAttribute(ply_convert_kernel<FMT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(kPlyThreads * REC + align_up((size_t)kPlyThreads * kPlyMaxStride + 8, 16)));
    if (e != cudaSuccess) return e;
    const uint32_t grid = (P.L.count + kPlyThreads - 1) / kPlyThreads;
    ply_convert_kernel<FMT><<<grid, kPlyThreads, smem, st>>>(P);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_ply_convert(const void *vertices, const gs_ply_layout &L, uint32_t format, void *records,
                               cudaStream_t st) {
    if (L.count == 0) return cudaSuccess;
    PlyParams P;
    P.L = L;
    P.vertices = static_cast<const uint8_t *>(vertices);
    P.records = static_cast<uint8_t *>(records);
    switch (format) {
        case GS_FORMAT_FP32:
            return launch_ply_fmt<GS_FORMAT_FP32>(P, st);
        case GS_FORMAT_HALF_SH_FP16:
            return launch_ply_fmt<GS_FORMAT_HALF_SH_FP16>(P, st);
        default:
            return launch_ply_fmt<GS_FORMAT_HALF_SH_BF16>(P, st);
    }
}

}  // namespace gs

extern "C" gs_status gs_ply_convert(const void *vertices, const gs_ply_layout *layout, uint32_t format,
                                    void *records, gs_stream stream) {
    const gs_status s = ply_check_layout(layout);
    if (s != GS_OK) return s;
    if (!(format == GS_FORMAT_FP32 || format == GS_FORMAT_HALF_SH_FP16 || format == GS_FORMAT_HALF_SH_BF16))
        return set_error(GS_ERR_INVALID_ARG, "unknown record format");
    if (layout->count == 0) return GS_OK;
    if (!vertices || !records) return set_error(GS_ERR_INVALID_ARG, "NULL argument");
    if ((uintptr_t)vertices % 4 != 0) return set_error(GS_ERR_INVALID_ARG, "vertices must be 4-byte aligned");
    if ((uintptr_t)records % 16 != 0) return set_error(GS_ERR_INVALID_ARG, "records must be 16-byte aligned");
    const cudaError_t e = launch_ply_convert(vertices, *layout, format, records, stream);
    if (e != cudaSuccess) return set_error(GS_ERR_CUDA, cudaGetErrorString(e));
    return GS_OK;
}
