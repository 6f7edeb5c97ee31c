/*
 * gs_record.h — byte layouts shared by the C ABI (gs300.h), the CUDA kernels and the CPU oracle.
 *
 * The Gaussian record layout of the reference lives in the un-vendored crate
 * wgpu-3dgs-core 0.6.0 (pinned in Cargo.lock); its field list is core::Gaussian
 * {rot, pos, color: U8Vec4, sh: [Vec3; 15], scale} (tests/e2e/viewer.rs:74-80) and the WGSL
 * accessors gaussian_unpack_color / _sh / _cov3d (src/shader/utils.wesl:2-15,95,101-131).
 * The byte layout below is this library's own: FP32 position, the colour as RGBA8 with the
 * DC term folded in (0.5 + SH_C0·dc, src/shader/utils.wesl:94) and opacity in A, 15 RGB SH
 * coefficients of bands 1..3, and the 6 unique entries of the 3D covariance.  It follows
 * WGSL storage-buffer alignment (vec3 aligned to 16 B, struct stride a multiple of 16 B), so
 * a record is 224 B = 14 x 16 B and every record starts on a 16-byte boundary.
 */
#ifndef GS_RECORD_H
#define GS_RECORD_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Display modes (core GaussianDisplayMode; src/shader/render.wesl:377,457-463). */
#define GS_DISPLAY_SPLAT 0u
#define GS_DISPLAY_ELLIPSE 1u
#define GS_DISPLAY_POINT 2u

/* Record formats accepted by gs_preprocess / gs_viewer_create. */
#define GS_FORMAT_FP32 0u         /* gs_gaussian_pod, 224 B */
#define GS_FORMAT_HALF_SH_FP16 1u /* gs_gaussian_pod_half, SH as IEEE binary16 */
#define GS_FORMAT_HALF_SH_BF16 2u /* gs_gaussian_pod_half, SH as bfloat16 */

/* Rasteriser tile edge in pixels. */
#define GS_TILE 16u
/* Keys per radix-sort block (HISTO_BLOCK_KVS = 256 x 15, src/radix_sorter.rs:150-178). */
#define GS_SORT_BLOCK_KVS 3840u

/* core::Gaussian (tests/e2e/viewer.rs:74-80): the CPU-side Gaussian a scene is built from. */
typedef struct gs_gaussian {
    float rot[4];     /* unit quaternion x, y, z, w (glam Quat order) */
    float pos[3];
    uint8_t color[4]; /* RGBA8: rgb = 0.5 + SH_C0·dc, a = opacity */
    float sh[45];     /* 15 x RGB, bands 1..3: sh[3*k + c] */
    float scale[3];
} gs_gaussian;

/* Default device record (DefaultGaussianPod = GaussianPodWithShSingleCov3dSingleConfigs,
 * src/lib.rs:43-44).  224 bytes. */
typedef struct gs_gaussian_pod {
    float pos[3];
    uint32_t color; /* r | g << 8 | b << 16 | a << 24 (WGSL unpack4x8unorm order) */
    float sh[45];   /* 15 x RGB, sh[3*k + c] */
    float cov3d[6]; /* xx, xy, xz, yy, yz, zz of R·S·Sᵀ·Rᵀ */
    uint32_t _pad;
} gs_gaussian_pod;

/* Compressed record (the crate's half-precision GaussianPod variants): FP32 position,
 * FP16 rotation and scale (the covariance is rebuilt in FP32 inside the preprocess
 * kernel), SH as FP16 or BF16 bit patterns.  128 bytes. */
typedef struct gs_gaussian_pod_half {
    float pos[3];
    uint32_t color;
    uint16_t rot[4];   /* binary16 x, y, z, w */
    uint16_t scale[3]; /* binary16 */
    uint16_t sh[45];   /* binary16 or bfloat16 bits, 15 x RGB */
    uint16_t _pad[4];
} gs_gaussian_pod_half;

/* Where the fields of one vertex of a standard 3D Gaussian splatting PLY file lie: binary
 * little-endian vertex element with float properties x, y, z, f_dc_0..2, opacity, scale_0..2,
 * rot_0..3 (w, x, y, z), and optionally f_rest_0..(3K-1) stored channel-major (K = 3, 8 or 15
 * coefficients per channel for SH degree 1, 2, 3).  Other properties are skipped.  Offsets are
 * byte offsets within a vertex.  Written by gs_ply_parse_header. */
typedef struct gs_ply_layout {
    uint64_t data_offset; /* byte offset of the first vertex in the file */
    uint32_t count;       /* vertices */
    uint32_t stride;      /* bytes per vertex */
    uint32_t sh_rest;     /* K: f_rest coefficients per channel (0, 3, 8 or 15) */
    int32_t pos[3];
    int32_t f_dc[3];
    int32_t opacity;
    int32_t scale[3];
    int32_t rot[4];       /* rot_0..rot_3 */
    int32_t f_rest[45];   /* f_rest_0..f_rest_(3K-1); -1 beyond */
} gs_ply_layout;

/* Camera (src/camera.rs:16-29). */
typedef struct gs_camera {
    float pos[3];
    float z_near; /* z.start */
    float z_far;  /* z.end */
    float vertical_fov;
    float pitch;
    float yaw;
} gs_camera;

/* CameraPod (src/buffer/camera.rs:153-161): 144 bytes, column-major matrices. */
typedef struct gs_camera_pod {
    float view[16];
    float proj[16];
    float size[2];
    uint32_t _padding[2];
} gs_camera_pod;

/* ModelTransformPod (wgpu-3dgs-core 0.6.0): translation, rotation quaternion, scale. */
typedef struct gs_model_transform_pod {
    float pos[3];
    float _pad0;
    float rot[4]; /* x, y, z, w */
    float scale[3];
    float _pad1;
} gs_model_transform_pod;

/* GaussianTransformPod (wgpu-3dgs-core 0.6.0; src/lib.rs:236-263): point size multiplier,
 * display mode, SH degree 0..=3, "no SH0" flag, max standard deviation 0..=3. */
typedef struct gs_gaussian_transform_pod {
    float size;
    uint32_t display_mode;
    uint32_t sh_deg;
    uint32_t no_sh0;
    float max_std_dev;
    uint32_t _pad[3];
} gs_gaussian_transform_pod;

/* Screen-space splat written by the preprocess kernel for each visible Gaussian and read by
 * the rasteriser: the per-instance vertex-shader results of src/shader/render.wesl:75-130.
 * 48 bytes.  For a pixel centre at offset d = (px + 0.5 - cx, py + 0.5 - cy) the
 * interpolated quad offset is q = (q[0]*dx + q[1]*dy, q[2]*dx + q[3]*dy).
 * In point mode q[0], q[1] are the exact half sides of the point square.
 * ex < 0 marks a splat that yields no fragments (zero-area quad). */
typedef struct gs_splat {
    float cx, cy;  /* centre in target pixels (y down) */
    float ex, ey;  /* half extents of a pixel box holding every fragment that can change a pixel */
    float q[4];
    float s255[3]; /* colour clamped to [0, 1], times 255 */
    float alpha;   /* colour alpha in [0, 1] */
} gs_splat;

/* Per-frame uniforms derived on the host by gs_frame_uniforms_build. */
typedef struct gs_frame_uniforms {
    float pv[16];     /* proj · view */
    float vm[16];     /* view · model */
    float model[16];  /* model matrix T·R·S */
    float wsr[9];     /* view 3x3 · (R·S), column-major */
    float inv_sr[9];  /* (R·S)^-1, column-major */
    float cam_pos[3]; /* world-space camera position -(Wᵀ·t) */
    float size[2];    /* camera.size */
    float focal[2];   /* (proj[0][0], proj[1][1]) · size · 0.5 */
    float viewport[2];/* target width, height */
    float std_dev;    /* max_std_dev */
    float std_dev_scaled; /* max_std_dev · size (the cov2d_axes argument) */
    float point_size; /* GaussianTransform.size */
    uint32_t display_mode;
    uint32_t sh_deg;
    uint32_t no_sh0;
    uint32_t _pad[2];
} gs_frame_uniforms;

#ifdef __cplusplus
}
#endif

#endif /* GS_RECORD_H */
