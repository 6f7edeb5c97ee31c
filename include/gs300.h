/*
 * gs300.h — C ABI of the GB300-native 3D Gaussian splatting render path.
 *
 * The path is the one behind wgpu-3dgs-viewer's Viewer / Preprocessor / RadixSorter / Renderer
 * (crate wgpu-3dgs-viewer 0.6.1): preprocess (cull, project, SH colour, depth key) -> stable
 * LSD radix sort of the depth keys carrying Gaussian indices -> splat rasterise/blend onto an
 * RGBA8 target cleared to opaque black.  Every entry point is `extern "C"` with plain pointers
 * and sizes; a stream is a `cudaStream_t` passed as `gs_stream` (NULL = legacy default stream).
 *
 * Each declaration cites the reference interface it replaces (file:line inside the crate).
 * Layouts of the records it consumes are in gs_record.h.
 */
#ifndef GS300_H
#define GS300_H

#include <stddef.h>
#include <stdint.h>

#include "gs_record.h"

#ifdef __cplusplus
extern "C" {
#endif

/* A CUDA stream handle (binary-compatible with cudaStream_t / CUstream). */
typedef struct CUstream_st *gs_stream;

/* ------------------------------------------------------------------------------------------ */
/* Status codes.  Replace the Result types of src/error.rs:6-50.                              */
/* ------------------------------------------------------------------------------------------ */
typedef enum gs_status {
    GS_OK = 0,
    GS_ERR_INVALID_ARG = 1,   /* bad pointer/size/enum; GaussianShDegree/GaussianMaxStdDev range */
    GS_ERR_OUT_OF_MEMORY = 2, /* device allocation failed (≙ ModelSizeExceedsDeviceLimit,
                                 src/error.rs:6-33) */
    GS_ERR_NOT_FOUND = 3,     /* ≙ MultiModelViewerAccessError::ModelNotFound (src/error.rs:45-50) */
    GS_ERR_CUDA = 4,          /* a CUDA runtime call failed; see gs_last_error() */
    GS_ERR_TIMEOUT = 5,       /* a bounded device-side wait (decoupled look-back) gave up */
    GS_ERR_CAPACITY = 6,      /* a caller-sized buffer was too small (e.g. tile-pair list) */
    GS_ERR_ADMISSION = 7      /* serving: request does not fit the per-view memory budget */
} gs_status;

/* Message of the last failure on the calling thread ("" if none). */
const char *gs_last_error(void);

/* Library version string, e.g. "gs300 0.1.0 sm_103a". */
const char *gs_version(void);

/* Number of CUDA kernels this library has launched since it was loaded (monotonic). */
uint64_t gs_launch_count(void);

/* Stage timers (no counterpart in the reference, whose timestamp queries are off,
 * src/radix_sorter.rs:504-507).  While enabled, CUDA events are recorded on the launching
 * stream around each stage: GS_PROF_PREPROCESS, _DEPTH_SORT, _BIN, _TILE_SORT, _RANGES,
 * _RASTER.  Enabling (or disabling) clears the accumulated times.  enable: 0 = off, 1 = timers
 * around the kernels every frame runs, 2 = timers, with splat-mode frames rasterised by a
 * counting variant whose work tallies gs_profile_counters returns (its times are the counting
 * kernel's, not the shipped one's). */
#define GS_PROF_STAGES 6
gs_status gs_profile_enable(int enable);
/* Synchronises the device; ms[s] = summed stage time, launches[s] = timed launches. */
gs_status gs_profile_read(double ms[GS_PROF_STAGES], uint32_t launches[GS_PROF_STAGES]);
/* While profiling in mode 2, splat-mode frames use a counting rasteriser; this returns its tallies
 * since gs_profile_enable (synchronises): pixel-splat evaluations, fragment alphas, channel-triple
 * blends, transmittance updates. */
gs_status gs_profile_counters(uint64_t out[4]);

/* ------------------------------------------------------------------------------------------ */
/* Host-side helpers (no device work).                                                         */
/* ------------------------------------------------------------------------------------------ */

/* Camera::view() = Mat4::look_to_rh(pos, forward(yaw, pitch), +Y) (src/camera.rs:70-88),
 * column-major 4x4. */
gs_status gs_camera_view(const gs_camera *camera, float out_view[16]);

/* Camera::projection(aspect) = Mat4::perspective_rh(vertical_fov, aspect, z_near, z_far)
 * (src/camera.rs:90-92), depth range 0..1, column-major 4x4. */
gs_status gs_camera_projection(const gs_camera *camera, float aspect_ratio, float out_proj[16]);

/* CameraPod::new(camera, size) (src/buffer/camera.rs:163-172). */
gs_status gs_camera_pod_new(const gs_camera *camera, uint32_t width, uint32_t height,
                            gs_camera_pod *out_pod);

/* GaussianTransformPod::new(size, display_mode, sh_deg, no_sh0, max_std_dev)
 * (wgpu-3dgs-core 0.6.0; used at src/lib.rs:237-263).  sh_deg must be 0..=3 and
 * max_std_dev 0..=3 (GaussianShDegree::new / GaussianMaxStdDev::new), else GS_ERR_INVALID_ARG. */
gs_status gs_gaussian_transform_pod_new(float size, uint32_t display_mode, uint32_t sh_deg,
                                        int no_sh0, float max_std_dev,
                                        gs_gaussian_transform_pod *out_pod);

/* ModelTransformPod::new(pos, rot, scale) (wgpu-3dgs-core 0.6.0; src/lib.rs:216-234). */
gs_status gs_model_transform_pod_new(const float pos[3], const float rot_xyzw[4],
                                     const float scale[3], gs_model_transform_pod *out_pod);

/* Pack core::Gaussian values (tests/e2e/viewer.rs:74-80) into the default device record
 * (DefaultGaussianPod, src/lib.rs:43-44): cov3d = R·S·Sᵀ·Rᵀ from (rot, scale). */
gs_status gs_gaussian_pack(const gs_gaussian *gaussians, size_t count, gs_gaussian_pod *out_pods);

/* ---- PLY ingest (Gaussians::read_from_file(path, GaussiansSource::Ply), wgpu-3dgs-core 0.6.0,
 * un-vendored; called at examples/simple.rs:157-160 before Viewer::new) ---------------------
 * The file's header is scanned on the host; the vertex block is converted into device records
 * on the GPU.  Conversion: rgb = clamp(0.5 + SH_C0·f_dc, 0, 1) and a = sigmoid(opacity), each
 * rounded to 8 bits (round half to even); scale = exp(scale_i); rotation (x, y, z, w) =
 * (rot_1, rot_2, rot_3, rot_0) normalised; these in double precision and rounded once to
 * float.  SH bands beyond the file's degree are zero.  The FP32 record's cov3d is the one
 * gs_gaussian_pack computes; half records round rotation, scale and SH to binary16 (SH to
 * bfloat16 for GS_FORMAT_HALF_SH_BF16), nearest even. */

/* Scan a PLY header (`len` bytes of the file, at least through "end_header\n") into `out`.
 * GS_ERR_INVALID_ARG for anything but binary_little_endian, a list property in or before the
 * vertex element, a missing or non-float required property, an f_rest count other than
 * 0, 9, 24 or 45, or a vertex stride outside 4..1024 bytes.  Host only. */
gs_status gs_ply_parse_header(const void *bytes, size_t len, gs_ply_layout *out_layout);

/* Convert layout->count vertices at `vertices` (device memory, 4-byte aligned, holding
 * count·stride bytes: the file from data_offset on) into `records` (device memory, 16-byte
 * aligned, count records of `format`), on `stream`.  Asynchronous. */
gs_status gs_ply_convert(const void *vertices, const gs_ply_layout *layout, uint32_t format,
                         void *records, gs_stream stream);

/* Derive the per-frame kernel uniforms (view-projection, model matrices, camera position,
 * decoded GaussianTransform) from the three pods and the viewport size.  The stage entry
 * points below take this struct by pointer (host memory). */
gs_status gs_frame_uniforms_build(const gs_camera_pod *camera,
                                  const gs_model_transform_pod *model_transform,
                                  const gs_gaussian_transform_pod *gaussian_transform,
                                  uint32_t viewport_width, uint32_t viewport_height,
                                  gs_frame_uniforms *out);

/* ------------------------------------------------------------------------------------------ */
/* Stage entry points over caller-owned device buffers (≙ the *_without_bind_group variants   */
/* plus create_bind_group, src/preprocessor.rs:34-68,375-435, src/radix_sorter.rs:19-96,       */
/* src/renderer.rs:20-41,242).  No allocation inside; scratch is caller-provided.             */
/* All pointers are device pointers unless noted.  Work is enqueued on `stream`.              */
/* ------------------------------------------------------------------------------------------ */

/* Capacity of the depth-key buffer for `n` Gaussians: keys_buffer_size(n) in keys
 * (src/radix_sorter.rs:931-934; GaussiansDepthBuffer::new, src/buffer/depth.rs:9-21). */
uint32_t gs_depth_capacity(uint32_t n);

/* Scratch areas of the stage calls must be zero-filled once before their first use.  After
 * that a scratch area can be reused by later calls of the same entry point without clearing,
 * with any sizes (max_count, key_bits, max_splats, width, height, max_pairs) that its byte size
 * covers: its control block and look-back flag arena sit at offsets no size moves, every flag
 * carries the epoch of the call that wrote it, and a call whose flag arena is larger than the
 * previous call's clears the difference on the device before reading any flag.  A scratch area
 * belongs to one entry point (do not pass the same area to two different stage calls), and
 * calls sharing one area must be ordered on the device (one stream, or synchronised). */

/* Bytes of scratch gs_preprocess needs for `n` Gaussians. */
size_t gs_preprocess_scratch_bytes(uint32_t n);

/* Preprocessor::preprocess (src/preprocessor.rs:283-290) = pre + main + post
 * (src/shader/preprocess.wesl:52-126): culls every Gaussian against the frustum (with the
 * major-axis bound test), compacts the visible ones IN ASCENDING GAUSSIAN ORDER into
 * indices[0..V), writes depths[c] = 1 - ndc.z, sets indirect_args = {6, V, 0, 0}
 * (DrawIndirectArgs, src/buffer/indirect_args.rs:15-20), sort_dispatch = {ceil(V/3840), 1, 1}
 * and pads depths[V .. min(ceil(V/3840)*3840, depth_capacity)) with 2.0.
 * When `splats` is non-NULL it also writes, for every visible Gaussian i, the screen-space
 * splat record splats[i] the rasteriser consumes (the per-vertex work of
 * src/shader/render.wesl:75-130 done once per Gaussian).
 * `selection` (nullable) is a bitmask of N bits; with it, Gaussian i is skipped when
 * bit i == invert_selection (src/shader/preprocess.wesl:68-78).
 * `format` is GS_FORMAT_FP32 (gaussians -> gs_gaussian_pod[n]) or GS_FORMAT_HALF_SH_FP16 /
 * GS_FORMAT_HALF_SH_BF16 (gaussians -> gs_gaussian_pod_half[n], the crate's compressed
 * GaussianPod variants); projection, axes and colour are computed in FP32 for all formats. */
gs_status gs_preprocess(const gs_frame_uniforms *uniforms, const void *gaussians, uint32_t format,
                        uint32_t n, const uint32_t *selection, int invert_selection,
                        uint32_t *indirect_args, uint32_t *sort_dispatch, uint32_t *indices,
                        float *depths, uint32_t depth_capacity, gs_splat *splats,
                        void *scratch, size_t scratch_bytes, gs_stream stream);

/* Bytes of scratch gs_radix_sort needs for up to `max_count` pairs. */
size_t gs_radix_sort_scratch_bytes(uint32_t max_count);

/* RadixSorter::sort / GPUSorter::sort_indirect (src/radix_sorter.rs:56-66,658-669,
 * kernels src/shader/radix_sort.wgsl:78-529): stable ascending LSD sort of u32 keys carrying
 * u32 values, 8 bits per pass, in place.  The pair count is read from device memory at
 * `count` (e.g. &indirect_args[1]) when non-NULL, else it is `max_count`.  Sorts bits
 * [0, key_bits) (key_bits 1..32; 32 for depth keys); bits above key_bits are ignored.
 * Bit-exact with a stable sort by (key mod 2^key_bits). */
gs_status gs_radix_sort(uint32_t *keys, uint32_t *values, uint32_t max_count,
                        const uint32_t *count, uint32_t key_bits, void *scratch,
                        size_t scratch_bytes, gs_stream stream);

/* Allocation-free variant of gs_radix_sort (no counterpart in the reference, whose sorter always
 * owns its buffers).  For callers that must not call cudaMalloc: a frame loop that may not
 * allocate or synchronise mid-frame, or a host runtime whose device memory belongs to another
 * allocator and that therefore cannot hand this library a scratch buffer.  Same contract as
 * gs_radix_sort (stable, in place, bits [0, key_bits), device-side `count`), but its scratch is a
 * static device array inside the library: at most 1,048,576 (2^20) pairs per call, and every
 * device that loads the library holds about 18 MB for it until the process exits.  Larger
 * `max_count` returns GS_ERR_INVALID_ARG.  Calls of any size and key width up to that limit may
 * follow one another (the array is zero when the library loads and is then reused like any
 * caller scratch).  The first call on a device looks up the array's device address with that
 * device current (and caches it for the process); make that first call outside any stream
 * capture.  All calls share the one array, so calls whose work overlaps on the GPU (different
 * streams, no ordering between them) race: order them on one stream or synchronise between
 * them. */
gs_status gs_radix_sort_no_alloc(uint32_t *keys, uint32_t *values, uint32_t max_count,
                                 const uint32_t *count, uint32_t key_bits, gs_stream stream);

/* Bytes of scratch gs_rasterize needs for up to `max_splats` visible splats, a
 * width x height target and up to `max_pairs` (tile, splat) pairs. */
size_t gs_rasterize_scratch_bytes(uint32_t max_splats, uint32_t width, uint32_t height,
                                  uint32_t max_pairs);

/* Renderer::render (src/renderer.rs:163-195; src/shader/render.wesl:143-181): clears the
 * RGBA8 target to opaque black and alpha-blends (BlendState::ALPHA_BLENDING) every visible
 * splat in the order of sorted_indices[0..V) (V read from `count`), back to front, one
 * 8-bit re-quantisation per fragment as a Rgba8Unorm attachment does.  `splats` is the
 * array gs_preprocess wrote.  `target` is width x height RGBA8 with row pitch
 * `pitch_bytes`.  Returns GS_ERR_CAPACITY (asynchronously, via gs_status_word) when the
 * tile-pair list exceeds `max_pairs`. */
gs_status gs_rasterize(const gs_frame_uniforms *uniforms, const gs_splat *splats,
                       const uint32_t *sorted_indices, const uint32_t *count, uint32_t max_splats,
                       uint8_t *target, uint32_t width, uint32_t height, uint32_t pitch_bytes,
                       uint32_t max_pairs, void *scratch, size_t scratch_bytes, gs_stream stream);

/* Device status word of a scratch area after a stage ran (synchronises the stream):
 * GS_OK, GS_ERR_TIMEOUT or GS_ERR_CAPACITY.  Also reports the number of tile pairs the
 * last rasterisation produced when `pairs` is non-NULL. */
gs_status gs_scratch_status(const void *scratch, gs_stream stream, uint32_t *pairs);

/* Test hook for the bounded device waits (no counterpart in the reference, whose look-back spin
 * is unbounded, src/shader/radix_sort.wgsl:382-403).  Every look-back of the stage calls and
 * facades enqueued after this call polls a predecessor's flag at most `spin_limit` times before
 * it records GS_ERR_TIMEOUT in its scratch status and carries on (writes whose addresses derive
 * from a look-back stay bounds-checked, so a given-up wait yields a wrong but in-bounds result);
 * with `stall_tile` other than 0xFFFFFFFF, the look-back tile (CTA) of that index publishes
 * nothing, so its successors wait on a flag nothing sets and run out.  gs_debug_set_wait_fault(
 * 4194304, 0xFFFFFFFF) restores the defaults.  spin_limit 0 is GS_ERR_INVALID_ARG. */
gs_status gs_debug_set_wait_fault(uint32_t spin_limit, uint32_t stall_tile);

/* ------------------------------------------------------------------------------------------ */
/* Viewer facade (src/lib.rs:64-275).  Owns device copies of the Gaussians and all buffers.  */
/* ------------------------------------------------------------------------------------------ */
typedef struct gs_viewer gs_viewer;

/* Viewer::new (src/lib.rs:86-197): uploads `count` records (host memory).  `format` is
 * GS_FORMAT_FP32 (gs_gaussian_pod) or GS_FORMAT_HALF_SH_FP16/_BF16 (gs_gaussian_pod_half).
 * With the environment variable GS300_EXACT_EXP=1 set at creation (or at a gs_rasterize
 * call), splat alpha uses a portable exp that the CPU oracle reproduces bit for bit; the
 * default is the SFU exp. */
gs_status gs_viewer_create(const void *host_records, uint32_t count, uint32_t format,
                           gs_viewer **out_viewer);
/* Viewer::new over the Gaussians of a PLY file held in host memory (`len` bytes): header
 * scan, one host-to-device copy of the vertex block, device conversion into `format`
 * records.  GS_ERR_INVALID_ARG if the file is shorter than its header says. */
gs_status gs_viewer_create_from_ply(const void *ply_bytes, size_t len, uint32_t format,
                                    gs_viewer **out_viewer);

void gs_viewer_destroy(gs_viewer *viewer);
uint32_t gs_viewer_len(const gs_viewer *viewer);

/* Viewer::update_camera / update_camera_with_pod (src/lib.rs:201-214). */
gs_status gs_viewer_update_camera(gs_viewer *viewer, const gs_camera *camera, uint32_t width,
                                  uint32_t height);
gs_status gs_viewer_update_camera_with_pod(gs_viewer *viewer, const gs_camera_pod *pod);
/* Viewer::update_model_transform[_with_pod] (src/lib.rs:216-234). */
gs_status gs_viewer_update_model_transform(gs_viewer *viewer, const float pos[3],
                                           const float rot_xyzw[4], const float scale[3]);
gs_status gs_viewer_update_model_transform_with_pod(gs_viewer *viewer,
                                                    const gs_model_transform_pod *pod);
/* Viewer::update_gaussian_transform[_with_pod] (src/lib.rs:236-263). */
gs_status gs_viewer_update_gaussian_transform(gs_viewer *viewer, float size,
                                              uint32_t display_mode, uint32_t sh_deg,
                                              int no_sh0, float max_std_dev);
gs_status gs_viewer_update_gaussian_transform_with_pod(gs_viewer *viewer,
                                                       const gs_gaussian_transform_pod *pod);
/* Optional selection mask (viewer-selection feature, src/lib.rs:134-144): N bits,
 * host memory; NULL clears it. */
gs_status gs_viewer_set_selection(gs_viewer *viewer, const uint32_t *host_bits, int invert);

/* Viewer::render (src/lib.rs:265-275): preprocess -> sort -> render into `target`
 * (device RGBA8, ≙ the TextureView).  Asynchronous on `stream`. */
gs_status gs_viewer_render(gs_viewer *viewer, uint8_t *target, uint32_t width, uint32_t height,
                           uint32_t pitch_bytes, gs_stream stream);
/* Wait for the viewer's last render, check its device status word and, if the tile-pair
 * list overflowed, grow it and render again.  Returns the frame's status. */
gs_status gs_viewer_synchronize(gs_viewer *viewer, gs_stream stream);
/* Counts of the last render (synchronises `stream`): visible splats V (the DrawIndirectArgs
 * instance count, src/buffer/indirect_args.rs:15-20) and (tile, splat) pairs wanted. */
gs_status gs_viewer_stats(gs_viewer *viewer, gs_stream stream, uint32_t *visible, uint32_t *pairs);
/* Stage outputs of the last render (device pointers owned by the viewer): the
 * IndirectIndicesBuffer, GaussiansDepthBuffer, IndirectArgsBuffer and the splat records. */
gs_status gs_viewer_buffers(gs_viewer *viewer, uint32_t **indices, float **depths,
                            uint32_t **indirect_args, gs_splat **splats);

/* ------------------------------------------------------------------------------------------ */
/* Render targets (headless replacement for wgpu::Texture + TextureView, Rgba8Unorm).         */
/* ------------------------------------------------------------------------------------------ */
typedef struct gs_target gs_target;
gs_status gs_target_create(uint32_t width, uint32_t height, gs_target **out_target);
void gs_target_destroy(gs_target *target);
uint8_t *gs_target_data(gs_target *target);
uint32_t gs_target_pitch(const gs_target *target);
/* Copy the target to host memory (width*height*4 bytes, tightly packed) and wait. */
gs_status gs_target_download(gs_target *target, uint8_t *host_rgba, gs_stream stream);
/* The same copy enqueued on `stream` without waiting (the bytes are on the host once the stream
 * reaches it); `host_rgba` should be pinned memory for the copy to overlap other work. */
gs_status gs_target_download_async(gs_target *target, uint8_t *host_rgba, gs_stream stream);

/* ------------------------------------------------------------------------------------------ */
/* MultiModelViewer facade (src/multi_model.rs:289-531).                                      */
/* ------------------------------------------------------------------------------------------ */
typedef struct gs_multi_viewer gs_multi_viewer;

/* MultiModelViewer::new (src/multi_model.rs:307-350). */
gs_status gs_multi_viewer_create(gs_multi_viewer **out_viewer);
void gs_multi_viewer_destroy(gs_multi_viewer *viewer);
/* insert_model (src/multi_model.rs:352-390): a key replaces an existing model of that key. */
gs_status gs_multi_viewer_insert_model(gs_multi_viewer *viewer, const char *key,
                                       const void *host_records, uint32_t count, uint32_t format);
/* insert_model over the Gaussians of a PLY file in host memory (as gs_viewer_create_from_ply). */
gs_status gs_multi_viewer_insert_model_from_ply(gs_multi_viewer *viewer, const char *key,
                                                const void *ply_bytes, size_t len, uint32_t format);
/* remove_model (src/multi_model.rs:392-395): GS_ERR_NOT_FOUND if absent. */
gs_status gs_multi_viewer_remove_model(gs_multi_viewer *viewer, const char *key);
uint32_t gs_multi_viewer_model_count(const gs_multi_viewer *viewer);
gs_status gs_multi_viewer_update_camera(gs_multi_viewer *viewer, const gs_camera *camera,
                                        uint32_t width, uint32_t height);
gs_status gs_multi_viewer_update_camera_with_pod(gs_multi_viewer *viewer,
                                                 const gs_camera_pod *pod);
/* update_model_transform[_with_pod] (src/multi_model.rs:413-443): GS_ERR_NOT_FOUND if absent. */
gs_status gs_multi_viewer_update_model_transform(gs_multi_viewer *viewer, const char *key,
                                                 const float pos[3], const float rot_xyzw[4],
                                                 const float scale[3]);
gs_status gs_multi_viewer_update_model_transform_with_pod(gs_multi_viewer *viewer,
                                                          const char *key,
                                                          const gs_model_transform_pod *pod);
gs_status gs_multi_viewer_update_gaussian_transform(gs_multi_viewer *viewer, float size,
                                                    uint32_t display_mode, uint32_t sh_deg,
                                                    int no_sh0, float max_std_dev);
gs_status gs_multi_viewer_update_gaussian_transform_with_pod(gs_multi_viewer *viewer,
                                                             const gs_gaussian_transform_pod *pod);
/* MultiModelViewer::render (src/multi_model.rs:475-530): every key must exist
 * (GS_ERR_NOT_FOUND otherwise, nothing rendered); each model is preprocessed and sorted on
 * its own, then all are drawn in `keys` order in one pass (model k over models < k). */
gs_status gs_multi_viewer_render(gs_multi_viewer *viewer, const char *const *keys,
                                 uint32_t key_count, uint8_t *target, uint32_t width,
                                 uint32_t height, uint32_t pitch_bytes, gs_stream stream);
gs_status gs_multi_viewer_synchronize(gs_multi_viewer *viewer, gs_stream stream);

/* ------------------------------------------------------------------------------------------ */
/* Batches (no counterpart in the reference): many views, each one model of a MultiModelViewer */
/* seen by its own camera into its own RGBA8 target, rendered by one CUDA graph per batch     */
/* shape.  A shape is the list of (model, target size, target pointer, pitch) plus the        */
/* viewer's GaussianTransform; cameras and model transforms may change between calls (they    */
/* reach the graph through a device uniform buffer).  Views run concurrently on the device.   */
/* ------------------------------------------------------------------------------------------ */
typedef struct gs_batch gs_batch;
typedef struct gs_batch_view {
    uint32_t model; /* index into the keys given to gs_batch_create */
    uint32_t width, height, pitch;
    uint8_t *target;
    gs_camera_pod camera;
} gs_batch_view;
gs_status gs_batch_create(gs_multi_viewer *viewer, const char *const *keys, uint32_t key_count,
                          gs_batch **out_batch);
void gs_batch_destroy(gs_batch *batch);
/* Enqueue all views on `stream` (asynchronous); models missing from the viewer give
 * GS_ERR_NOT_FOUND and nothing is rendered. */
gs_status gs_batch_render(gs_batch *batch, const gs_batch_view *views, uint32_t view_count,
                          gs_stream stream);
/* Wait, check every view's device status, regrow overflowed tile-pair lists and re-render. */
gs_status gs_batch_synchronize(gs_batch *batch, gs_stream stream);

/* Launch choices of a batch that change its speed, never its frames. */
typedef struct gs_tuning {
    uint32_t suffix_min;       /* raster: tile lists at least this long take the exact early-out (>= 1) */
    float eps;                 /* raster: transmittance ending the front-to-back walk, (0, 0.5] */
    uint32_t views_per_launch; /* views of one model sharing a preprocess launch, 1..16 */
    uint32_t streams;          /* streams the captured graph fans out over, 1..16 */
    uint32_t sort_match;       /* depth sort ranking: 1 = match.any, 0 = one ballot per digit bit */
    uint32_t hist_blocks;      /* depth sort key-histogram blocks, 0 (by key count) or 1..1216 */
    uint32_t raster_grid;      /* 0: each view rasterised after its own binning (overlapping other
                                  views' sorting); 1: one rasteriser grid over all views' tiles */
    uint32_t sort_digit_bits;  /* depth sort: widest radix digit of a pass, 6..8 (the key's bits
                                  spread evenly over the passes): narrower digits give longer
                                  runs of equal digits per block at the price of more passes */
} gs_tuning;
/* The library's defaults (GS300_SUFFIX_MIN / GS300_SUFFIX_EPS override the raster knobs,
 * GS300_SORT_DIGIT_BITS the depth sort's digit width, GS300_SORT_MATCH its ranking and
 * GS300_HIST_BLOCKS its key-histogram grid). */
gs_status gs_tuning_default(gs_tuning *out);
/* GS_ERR_INVALID_ARG outside the ranges above.  The next render re-captures the graph. */
gs_status gs_batch_set_tuning(gs_batch *batch, const gs_tuning *tuning);
gs_status gs_batch_get_tuning(gs_batch *batch, gs_tuning *out);
/* Autotuner: renders `views` (into their targets) under candidate tunings, one knob at a time
 * (coordinate descent from the current tuning, `rounds` sweeps), timing `reps` renders of each
 * with CUDA events after one warm-up, and keeps the fastest.  The chosen tuning is set on the
 * batch and returned with its milliseconds per batch.  Synchronous. */
gs_status gs_batch_autotune(gs_batch *batch, const gs_batch_view *views, uint32_t view_count, uint32_t reps,
                            uint32_t rounds, gs_tuning *out_best, double *out_ms);

/* ------------------------------------------------------------------------------------------ */
/* Serving (no counterpart in the reference): scenes stay resident (the models of a           */
/* MultiModelViewer); (scene, camera, resolution) requests are admitted first come first      */
/* served while the device memory their per-view buffers need fits `budget_bytes` and one of  */
/* `max_inflight` slots is free; each admitted request runs on its own stream, so requests     */
/* that arrive while others run overlap with them.  A scheduler thread owns all submission.   */
/* Models must stay in the viewer while requests for them are queued or running.              */
/* ------------------------------------------------------------------------------------------ */
typedef struct gs_server gs_server;
typedef struct gs_server_report {
    uint64_t completed, failed;
    uint32_t queued, running;
    uint64_t reserved_bytes;
    double p50_ms, p99_ms, mean_ms, max_ms; /* submit-to-completion latency */
} gs_server_report;
gs_status gs_server_create(gs_multi_viewer *viewer, size_t budget_bytes, uint32_t max_inflight,
                           gs_server **out_server);
void gs_server_destroy(gs_server *server);
/* Device bytes a request for a scene of `n` Gaussians at width x height holds while admitted. */
size_t gs_server_request_bytes(uint32_t n, uint32_t width, uint32_t height);
/* Queue a request.  `out` (nullable): a device RGBA8 buffer with `out_pitch`, or with
 * out_on_host != 0 a host buffer of width*height*4 bytes filled when the request completes.
 * GS_ERR_ADMISSION if the request alone exceeds the budget. */
gs_status gs_server_submit(gs_server *server, const char *key, const gs_camera_pod *camera,
                           uint32_t width, uint32_t height, uint8_t *out, uint32_t out_pitch,
                           int out_on_host, uint64_t *ticket);
/* Wait for a request (host-side timeout in seconds); reports its latency. */
gs_status gs_server_wait(gs_server *server, uint64_t ticket, double timeout_s, double *latency_ms);
gs_status gs_server_stats(gs_server *server, gs_server_report *out);
gs_status gs_server_reset_stats(gs_server *server);
/* Dynamic batching: up to `max_views` (1..16, default 16) admitted requests of one scene share
 * one preprocess launch that reads the scene's records once; 1 runs every request alone.  With
 * `max_wait_ms` > 0 (0..1000, default 0), while a scene has more requests queued than slots are
 * free, admission holds for up to that long (from when the hold began) for busy slots to free up,
 * so that larger groups form. */
gs_status gs_server_set_batching(gs_server *server, uint32_t max_views, double max_wait_ms);

#ifdef __cplusplus
}
#endif

#endif /* GS300_H */
