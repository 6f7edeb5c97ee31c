// gs_convert.cuh — record conversions compiled for both the host (gs_gaussian_pack) and the
// device (PLY ingest), so that both produce the same bits.  Every operation is an IEEE double
// or float operation in a fixed order: the library is built with -fmad=false (device) and
// -ffp-contract=off (host), so no multiply-add is contracted on either side.
#pragma once

#include <cmath>
#include <cstdint>

#ifdef __CUDACC__
#define GS_HD __host__ __device__ __forceinline__
#else
#define GS_HD inline
#endif

namespace gs {

// SH band-0 constant of the colour fold rgb = 0.5 + SH_C0 · f_dc.
constexpr double kShC0 = 0.28209479177387814;

// Σ = (R·S)(R·S)ᵀ for a unit quaternion (x, y, z, w) and per-axis scale: (xx, xy, xz, yy, yz,
// zz), accumulated in double and rounded once to float.
GS_HD void cov3d_from_rot_scale(const float rot[4], const float scale[3], float out[6]) {
    const double x = rot[0], y = rot[1], z = rot[2], w = rot[3];
    const double R[3][3] = {{1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)},
                            {2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)},
                            {2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)}};
    double M[3][3];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) M[r][c] = R[r][c] * (double)scale[c];
    const int A[6] = {0, 0, 0, 1, 1, 2}, B[6] = {0, 1, 2, 1, 2, 2};
    for (int k = 0; k < 6; ++k) {
        const int a = A[k], b = B[k];
        out[k] = (float)((M[a][0] * M[b][0] + M[a][1] * M[b][1]) + M[a][2] * M[b][2]);
    }
}

// An 8-bit channel of a value in [0, 1]: clamp, scale by 255, round half to even.  NaN -> 0.
GS_HD uint32_t unorm8_rne(double v) {
    v = v > 0.0 ? (v < 1.0 ? v : 1.0) : 0.0;
    return (uint32_t)rint(v * 255.0);
}

}  // namespace gs
