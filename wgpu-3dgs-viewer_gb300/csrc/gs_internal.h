// gs_internal.h — declarations shared between the kernel translation units and the C ABI.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "gs_common.cuh"
#include "gs_convert.cuh"
#include "gs300.h"
#include "gs_record.h"

namespace gs {

// Stage timers (CUDA events on the launching stream; recorded only while profiling is on) and
// the count of kernels this library has launched.
enum ProfStage { kProfPreprocess = 0, kProfDepthSort, kProfBin, kProfTileSort, kProfRanges, kProfRaster, kProfStages };
void prof_mark(int stage, bool begin, cudaStream_t st);
// Profiling in counting mode: splat frames run the counting rasteriser instead of the shipped one.
bool prof_counting();
// Work tallies of the counting rasteriser run while profiling: pixel-splat evaluations,
// alphas, channel-triple blends, transmittance updates.
cudaError_t raster_counters(unsigned long long out[4], bool reset);
void count_launches(uint32_t n);

// Records `message` as the calling thread's gs_last_error() and returns `status`.
gs_status set_error(gs_status status, const char *message);

// Resets a control block (see ctrl_reset): owner = the block holding the area's epoch counter
// and arena mark (nullptr: the block itself); arena_words = the flag-arena words of this call
// for the owner's mode-1 reset, kKeepArena when no clearing kernel runs in the call.
__global__ void ctrl_init_kernel(Ctrl *ctrl, int mode, Ctrl *owner, uint32_t arena_words, WaitCfg cfg);

// Look-back configuration every stage launch carries (the poll bound, and the stalled tile of
// the bounded-wait test hook gs_debug_set_wait_fault).
WaitCfg wait_config();

// ---- K1 preprocess (gs_preprocess.cu) ----
size_t preprocess_scratch_bytes(uint32_t n);
cudaError_t launch_preprocess(const gs_frame_uniforms &u, const void *records, uint32_t format,
                              uint32_t n, const uint32_t *selection, int invert, uint32_t *indirect,
                              uint32_t *dispatch, uint32_t *indices, float *depths,
                              uint32_t depth_cap, gs_splat *splats, void *scratch, cudaStream_t st,
                              const gs_frame_uniforms *u_dev = nullptr, uint4 *binfo = nullptr);

// Several views of one model in one launch (records read once).  A view's scratch is the one
// launch_preprocess takes for that model; `group` is a zeroed Ctrl-sized block for the launch.
struct PreView {
    const gs_frame_uniforms *u;  // device
    uint32_t *indirect;
    uint32_t *dispatch;
    uint32_t *indices;
    float *depths;
    uint32_t depth_cap;
    gs_splat *splats;
    Ctrl *ctrl;
    uint64_t *flags;
};
constexpr uint32_t kPreMaxViews = 16;
PreView preprocess_view(const gs_frame_uniforms *u_dev, uint32_t *indirect, uint32_t *dispatch, uint32_t *indices,
                        float *depths, uint32_t depth_cap, gs_splat *splats, void *scratch);
cudaError_t launch_preprocess_views(const void *records, uint32_t format, uint32_t n, const uint32_t *selection,
                                    int invert, const PreView *views_dev, uint32_t nviews, void *group,
                                    cudaStream_t st);

// ---- PLY ingest (gs_ply.cu) ----
gs_status ply_check_layout(const gs_ply_layout *layout);
cudaError_t launch_ply_convert(const void *vertices, const gs_ply_layout &layout, uint32_t format, void *records,
                               cudaStream_t st);

// Launch choices that change speed, never results (gs_tuning in the C ABI).  The defaults are
// the library's; batches can set them or have them picked by gs_batch_autotune.
struct Tuning {
    uint32_t suffix_min = 1024;     // raster: tile lists at least this long take the exact early-out
    float eps = 1e-6f;              // raster: transmittance that ends the front-to-back walk
    uint32_t views_per_launch = 16; // batch: views per shared-read preprocess launch (1..16)
    uint32_t streams = 16;          // batch: streams the captured graph fans out over (1..16)
    uint32_t sort_match = 0;        // depth sort: 1 = match.any ranking, 0 = a ballot per digit bit
    uint32_t sort_digit_bits = 8;   // depth sort: widest digit of a pass (6..8), bits spread evenly
    uint32_t hist_blocks = 0;       // depth sort: key-histogram grid (0 = by key count, <= 1216)
    uint32_t raster_grid = 0;       // batch: 0 = each view rasterised after its own binning,
                                    // 1 = one rasteriser grid over all views after all binning
};
// The defaults, with GS300_SUFFIX_MIN / GS300_SUFFIX_EPS / GS300_HIST_BLOCKS /
// GS300_SORT_DIGIT_BITS overriding them.
Tuning default_tuning();

// ---- K2 onesweep radix sort (gs_sort.cu) ----
// Live bits of a depth key: the key is 1 - ndc.z of a Gaussian whose ndc.z passed the cull test
// (0 <= ndc.z <= 1, src/shader/utils.wesl:18-20), so it lies in [0, 1] and its float bits are at
// most 0x3F800000 < 2^30.  Sorting bits [0, 30) orders every depth key exactly as sorting all 32.
constexpr uint32_t kDepthKeyBits = 30;
// Passes of a sort at most (32-bit keys in 6-bit digits).
constexpr uint32_t kMaxPasses = 6;
size_t sort_scratch_bytes(uint32_t max_count, uint32_t key_bits);
cudaError_t launch_sort(uint32_t *keys, uint32_t *vals, uint32_t max_count, const uint32_t *count,
                        uint32_t key_bits, void *scratch, cudaStream_t st, int prof_stage = kProfDepthSort,
                        const Tuning *tuning = nullptr);

// Digits of the packed-pair sort: the key's bits spread evenly over the fewest passes of at
// most 8 bits (13 bits -> 7 + 6), pass p taking bits [shift[p], shift[p] + bits[p]).
struct PassSplit {
    uint32_t shift[kMaxPasses], bits[kMaxPasses], n;
};
PassSplit even_split(uint32_t key_bits);
// The same spread with digits of at most `max_digit` bits (6..8): fewer digit values per pass
// mean longer runs of equal digits in each block's scatter, at the price of more passes.
PassSplit even_split_max(uint32_t key_bits, uint32_t max_digit);
// Offset of pass p's digit histogram in Ctrl::hist (flat): 256 words a pass for up to 4 passes,
// 1024 / n words a pass beyond (enough for the narrower digits that more passes use).
__host__ __device__ inline uint32_t hist_stride(uint32_t npasses) { return npasses <= 4 ? 256u : 1024u / npasses; }

// Packed (uint2 {key, value}) in-place sort for internal pair lists whose digit histograms
// (split by even_split) the producer accumulated into the control block `ctrl` after
// sort_pairs_begin(): as counts, or (hist_scanned) already as exclusive digit offsets.  Its
// look-back flags (sort_pairs_flag_words of them) lie in the flag arena of the area whose
// control block `owner` is; `alt` holds max_count pairs.
size_t sort_pairs_flag_words(uint32_t max_count, uint32_t key_bits);
cudaError_t sort_pairs_begin(Ctrl *ctrl, Ctrl *owner, cudaStream_t st);
// The split of a tile-pair sort (producers of its digit histograms must use the same one).
PassSplit tile_split(uint32_t key_bits);

// A segmented sort: many independent two-pass tile-pair sorts (one per view of a batch) in one
// launch per pass.  A segment is what launch_sort_pairs would sort for one view.
struct SortSegment {
    uint2 *data, *alt;          // the view's pairs (sorted in place) and its ping-pong buffer
    const uint32_t *count;      // device pair count
    uint32_t max_count;
    uint32_t shift[2], bits[2]; // tile_split of the view's tile-id bits
    uint32_t hist_scanned;      // digit histograms already exclusive offsets
    Ctrl *ctrl;                 // the view's tile-sort control block
    Ctrl *owner;                // the view's raster control block (its status takes the sort's)
    uint64_t *flags[2];         // look-back flags of each pass
};
// CTAs of one segment (blocks of its pairs at capacity).
uint32_t sort_pairs_blocks(uint32_t max_count);
// Both passes over every segment (segs_dev / block_base_dev: device arrays; block_base holds the
// prefix of the segments' block counts, nseg + 1 entries), then the statuses merged.
cudaError_t launch_sort_segments(const SortSegment *segs_dev, const uint32_t *block_base_dev, uint32_t nseg,
                                 uint32_t total_blocks, cudaStream_t st);
cudaError_t launch_sort_pairs(uint2 *data, uint32_t max_count, const uint32_t *count, uint32_t key_bits, Ctrl *ctrl,
                              uint64_t *flags, uint2 *alt, cudaStream_t st, bool hist_scanned);

// ---- K3 binning + K4 raster (gs_raster.cu) ----
// The only frame uniforms binning and rasterisation read: camera, model and SH fields never
// reach them, so a captured graph of these launches stays valid for any camera.
struct RasterMode {
    uint32_t display_mode;
    float std_dev;
};
inline RasterMode raster_mode(const gs_frame_uniforms &u) { return RasterMode{u.display_mode, u.std_dev}; }

struct RasterSegment {
    const gs_splat *splats;       // indexed by Gaussian index
    const uint32_t *sorted_index; // draw order
    const uint32_t *count;        // device: number of entries in sorted_index
    uint32_t max_count;           // capacity of sorted_index
    // Optional: each visible splat's tiles as its preprocess stored them for a binfo_w x
    // binfo_h target (indexed by Gaussian index); used when the binning's target matches.
    const uint4 *binfo = nullptr;
    uint32_t binfo_w = 0, binfo_h = 0;
};
size_t raster_scratch_bytes(uint32_t max_splats, uint32_t width, uint32_t height, uint32_t max_pairs);
// exact_exp: 1 = the portable exp (bit-identical with the CPU oracle), 0 = the SFU exp.
cudaError_t launch_raster(const RasterSegment *segs, uint32_t nseg, const RasterMode &u,
                          uint8_t *target, uint32_t width, uint32_t height, uint32_t pitch,
                          uint32_t max_pairs, void *scratch, int exact_exp, cudaStream_t st,
                          const Tuning *tuning = nullptr);
// Scratch control block of a raster call (status, pair counts).
const Ctrl *raster_ctrl(const void *scratch);

// What the rasteriser needs of one view after binning: its splats, tile-sorted pairs, tile
// ranges, target and status block.  Pure pointer arithmetic on the view's raster scratch, so it
// can be known (and uploaded for a multi-view grid) before any launch.
struct RasterJob {
    const gs_splat *splats;
    const uint2 *pairs;
    const uint2 *ranges;
    const uint32_t *order;  // launch order of the tiles (null: tile = CTA index)
    uint8_t *target;
    uint32_t W, H, pitch, tiles_x, max_splats, ntiles;
    Ctrl *ctrl;
};
RasterJob raster_job(const RasterSegment *segs, uint32_t nseg, uint8_t *target, uint32_t width, uint32_t height,
                     uint32_t pitch, uint32_t max_pairs, void *scratch);
// Binning of one view up to its tile sort (tile rectangles, count scan, pair emission, per-tile
// counts and ranges or the sort's digit histograms).
cudaError_t launch_binning_front(const RasterSegment *segs, uint32_t nseg, const RasterMode &u, uint32_t width,
                                 uint32_t height, uint32_t max_pairs, void *scratch, cudaStream_t st);
// The view's tile sort as a segment of a segmented sort (pointer arithmetic on its scratch), and
// whether its target is small enough for one (two tile-sort passes: at most 65536 tiles).
SortSegment tile_sort_segment(const RasterSegment *segs, uint32_t nseg, uint32_t width, uint32_t height,
                              uint32_t max_pairs, void *scratch);
bool tile_sort_segmentable(uint32_t width, uint32_t height);
// After the view's tile sort: tile ranges from the sorted pairs where the target has more tiles
// than the counting path covers (nothing otherwise).
cudaError_t launch_binning_ranges(const RasterSegment *segs, uint32_t nseg, uint32_t width, uint32_t height,
                                  uint32_t max_pairs, void *scratch, cudaStream_t st);
// Binning, tile sort and tile ranges of one view (everything launch_raster does before the
// rasteriser itself).
cudaError_t launch_binning(const RasterSegment *segs, uint32_t nseg, const RasterMode &u, uint32_t width,
                           uint32_t height, uint32_t max_pairs, void *scratch, cudaStream_t st);
// One rasteriser grid over several binned views (same display mode and std): tile_base holds the
// prefix of the views' tile counts (nviews + 1 entries, device), jobs the views (device).
cudaError_t launch_raster_views(const RasterJob *jobs, const uint32_t *tile_base, uint32_t nviews,
                                uint32_t total_tiles, const RasterMode &u, int exact_exp, cudaStream_t st,
                                const Tuning *tuning = nullptr);

}  // namespace gs
