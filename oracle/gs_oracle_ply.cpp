// gs_oracle_ply.cpp — CPU ORACLE for PLY ingest (test infrastructure only; never part of the
// product path).
//
// The reference loads scenes with wgpu-3dgs-core 0.6.0's Gaussians::read_from_file(path,
// GaussiansSource::Ply) (examples/simple.rs:157-160; the crate is un-vendored, Cargo.lock
// 2745-2764), whose input is the standard 3D Gaussian splatting PLY vertex: x, y, z,
// f_dc_0..2, f_rest_0..(3K-1) channel-major, opacity (logit), scale_0..2 (log), rot_0..3
// (w, x, y, z).  This file restates that published convention, one vertex at a time:
//   rgb   = clamp(0.5 + SH_C0 · f_dc, 0, 1), to 8 bits, round half to even
//   alpha = 1 / (1 + e^-opacity), to 8 bits, round half to even
//   scale = e^scale_i;  rot (x, y, z, w) = (rot_1, rot_2, rot_3, rot_0) / |rot|
// in double precision, each rounded once to float, then the record: cov3d = (R·S)(R·S)ᵀ in
// double for the FP32 record; binary16 rotation, scale and SH (bfloat16 SH for the BF16
// record), round to nearest even, for the half records.  The conversion constants are this
// project's (the crate is unpinned); tests pin this restatement to the Python reader
// (gs300/ply.py) and the reference's coverage/model.ply fixture.
#include <cmath>
#include <cstdint>
#include <cstring>

#include "gs_record.h"

namespace {

constexpr double kShC0 = 0.28209479177387814;

float field(const uint8_t *v, int32_t off) {
    float f;
    std::memcpy(&f, v + off, 4);
    return f;
}

uint32_t to_u8(double x) {
    if (!(x > 0.0)) return 0;  // NaN and non-positive values
    if (x > 1.0) x = 1.0;
    return (uint32_t)std::nearbyint(x * 255.0);
}

uint16_t half_bits(float x) {
    const _Float16 h = (_Float16)x;
    uint16_t b;
    std::memcpy(&b, &h, 2);
    return b;
}

uint16_t bf16_bits(float x) {
    uint32_t b;
    std::memcpy(&b, &x, 4);
    if ((b & 0x7FFFFFFFu) > 0x7F800000u) return (uint16_t)((b >> 16) | 0x40u);  // quiet NaN
    return (uint16_t)((b + 0x7FFFu + ((b >> 16) & 1u)) >> 16);
}

void convert_one(const uint8_t *v, const gs_ply_layout &L, uint32_t fmt, uint8_t *rec) {
    float pos[3], sh[45] = {0}, scale[3], rot[4];
    for (int k = 0; k < 3; ++k) pos[k] = field(v, L.pos[k]);
    uint32_t color = 0;
    for (int c = 0; c < 3; ++c) color |= to_u8(0.5 + kShC0 * (double)field(v, L.f_dc[c])) << (8 * c);
    color |= to_u8(1.0 / (1.0 + std::exp(-(double)field(v, L.opacity)))) << 24;
    for (int k = 0; k < 3; ++k) scale[k] = (float)std::exp((double)field(v, L.scale[k]));
    const double q[4] = {field(v, L.rot[1]), field(v, L.rot[2]), field(v, L.rot[3]), field(v, L.rot[0])};
    const double n = std::sqrt(((q[0] * q[0] + q[1] * q[1]) + q[2] * q[2]) + q[3] * q[3]);
    for (int k = 0; k < 4; ++k) rot[k] = (float)(q[k] / n);
    const uint32_t K = L.sh_rest;
    for (uint32_t k = 0; k < K; ++k)
        for (uint32_t c = 0; c < 3; ++c) sh[3 * k + c] = field(v, L.f_rest[c * K + k]);

    if (fmt == GS_FORMAT_FP32) {
        gs_gaussian_pod p;
        std::memset(&p, 0, sizeof(p));
        std::memcpy(p.pos, pos, 12);
        p.color = color;
        std::memcpy(p.sh, sh, sizeof(sh));
        const double x = rot[0], y = rot[1], z = rot[2], w = rot[3];
        const double R[3][3] = {{1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)},
                                {2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)},
                                {2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)}};
        double M[3][3];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) M[r][c] = R[r][c] * (double)scale[c];
        const int A[6] = {0, 0, 0, 1, 1, 2}, B[6] = {0, 1, 2, 1, 2, 2};
        for (int k = 0; k < 6; ++k)
            p.cov3d[k] = (float)((M[A[k]][0] * M[B[k]][0] + M[A[k]][1] * M[B[k]][1]) + M[A[k]][2] * M[B[k]][2]);
        std::memcpy(rec, &p, sizeof(p));
    } else {
        gs_gaussian_pod_half p;
        std::memset(&p, 0, sizeof(p));
        std::memcpy(p.pos, pos, 12);
        p.color = color;
        for (int k = 0; k < 4; ++k) p.rot[k] = half_bits(rot[k]);
        for (int k = 0; k < 3; ++k) p.scale[k] = half_bits(scale[k]);
        for (int k = 0; k < 45; ++k) p.sh[k] = fmt == GS_FORMAT_HALF_SH_FP16 ? half_bits(sh[k]) : bf16_bits(sh[k]);
        std::memcpy(rec, &p, sizeof(p));
    }
}

}  // namespace

extern "C" {

// `vertices` = the file from layout->data_offset on; `out` = layout->count records of `fmt`.
void oracle_ply_convert(const uint8_t *vertices, const gs_ply_layout *layout, uint32_t fmt, void *out) {
    const size_t rb = fmt == GS_FORMAT_FP32 ? sizeof(gs_gaussian_pod) : sizeof(gs_gaussian_pod_half);
    uint8_t *o = static_cast<uint8_t *>(out);
    for (uint32_t i = 0; i < layout->count; ++i)
        convert_one(vertices + (size_t)i * layout->stride, *layout, fmt, o + (size_t)i * rb);
}

}  // extern "C"
