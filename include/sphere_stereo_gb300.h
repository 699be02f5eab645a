/*
 * sphere_stereo_gb300 -- C ABI of the GB300 (sm_103a) implementation of sphere-sweeping stereo's
 * per-frame path: sphere sweep + matching cost, ISB multiscale cost filter, distance selection,
 * distance post-filter, RGB-D panorama stitcher.
 *
 * Library: libsphere_stereo_gb300.so (built from sphere-stereo_gb300/csrc/*.cu).
 *
 * Conventions
 *   - Every pointer named d_* (or documented as "device") is CUDA device memory of the current
 *     device; other pointers are host memory read during the call only.
 *   - Sizes follow the reference: images are row-major [rows][cols][3]; cost volumes are planar
 *     [candidates][rows][cols] float32 (python/isb_filter.py:69-70) unless a function says
 *     otherwise; resolutions are passed as (cols, rows) pairs where the reference does so.
 *   - `stream` is a cudaStream_t (NULL = legacy default stream).  Every call only enqueues work
 *     on that stream; nothing synchronises the host.
 *   - Every function returns SSG_OK or an error code; ssg_last_error() gives the message of the
 *     calling thread's last failure.  Invalid arguments are rejected before any launch.
 *
 * Each declaration names the reference interface it stands in for (file:line within the
 * reference project, KAIST-VCLAB/sphere-stereo).
 */
#ifndef SPHERE_STEREO_GB300_H
#define SPHERE_STEREO_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define SSG_API __attribute__((visibility("default")))
#else
#define SSG_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

enum {
    SSG_OK = 0,
    SSG_ERR_INVALID_ARGUMENT = 1, /* rejected before launch */
    SSG_ERR_CUDA = 2,             /* a CUDA runtime call or launch failed */
    SSG_ERR_UNSUPPORTED = 3       /* a size beyond a documented compile-time limit */
};

/* Cost storage of the batched path: the level-0 volume is 16-bit, coarser levels float32. */
#define SSG_STORAGE_F16 0     /* IEEE half */
#define SSG_STORAGE_UNORM16 1 /* uint16 q = round(cost * 65535 / 500), costs being in [0, 500] */
#define SSG_STORAGE_F32 2     /* float32 (the coarse levels) */

/* Compile-time limits (also reported by ssg_limits). */
#define SSG_MAX_CAMERAS 16
#define SSG_MAX_CANDIDATES 256
#define SSG_MAX_REFERENCES 16
#define SSG_MAX_LEVELS 24

/* Double-sphere camera in the form the reference's torch code uses it
 * (python/utils.py:57-94 with python/utils.py:40-55): fx, fy, cx, cy are the float32 products
 * `fl * matching_scale` and `principal * matching_scale`; xi and alpha are the calibration's
 * double-precision values (the library rounds derived constants exactly as torch does). */
typedef struct {
    float fx, fy, cx, cy;
    double xi, alpha;
} ssg_camera;

/* Double-sphere intrinsics as the stitcher kernels use them: the `Intrinsics` struct of
 * python/stitcher.cu:31-35, filled by vectorize_calibration (python/stitcher.py:35-46). */
typedef struct {
    float fx, fy, cx, cy, xi, alpha;
} ssg_intrinsics;

/* Launch-shape knobs of the batched kernels (no counterpart in the reference), picked per
 * workload by the Python autotuner (sphere-stereo_gb300/autotune.py).  Process-wide; read when a
 * launch is enqueued, so a captured CUDA graph keeps the values it was captured with. */
#define SSG_TUNE_SWEEP_VARIANT 0      /* sweep block shape: 0 = 256 threads x 4 blocks/SM (64 registers),
                                         1 = 256 x 3 (80 registers), 2 = 128 x 8 (64 registers),
                                         3 = 128 x 7 (72 registers) */
#define SSG_TUNE_HOLE_BLOCKS_PER_SM 1 /* blocks per SM of the hole-filling steps: 2, 4, 8 */
#define SSG_TUNE_MERGE_FRAMES 2       /* frames one thread of the batched merge handles: 2, 4, 8 */
#define SSG_TUNE_UNEVEN_SPAN 3        /* 256-pixel tiles per work item of the uneven sweep: 1, 2, 4 */
#define SSG_TUNE_ISB_UP_BLOCKS 4      /* blocks per SM the chunked ISB upsampling (coarse levels) is
                                         register-bounded for: 2, 3 */
#define SSG_TUNE_ISB_SELECT_BLOCKS 5  /* the same for the last level fused with the selection: 2, 3 */
#define SSG_TUNE_ISB_TILE_TMA 6       /* coarse tiles of the chunked ISB upsampling staged by TMA (1) or by
                                         cp.async (0) */
#define SSG_TUNE_HOLE_PERSISTENT 8    /* hole filling: 1 = the steps after the first in one cooperative
                                         launch, separated by grid-wide barriers; 0 = a launch per
                                         step (default) */
#define SSG_TUNE_SWEEP_TILES 9        /* the batched sweep's blocks: 0 = consecutive pixels of a row;
                                         16 or 32 = tiles that many pixels wide, threads / width rows
                                         high */
#define SSG_TUNE_HOLE_TAIL 10         /* uniform batched hole filling: from this step on, one block per
                                         map runs every remaining step (3, 4, 6 or 8); 0 = a launch per
                                         step to the end */
#define SSG_TUNE_SELECT_WHOLE 11      /* the last ISB level fused with the selection, at most 32
                                         candidates: 1 = every chunk's coarse tile staged at once, no
                                         block barrier between chunks (same bits; default); 0 =
                                         double-buffered chunk tiles */
#define SSG_TUNE_UP_WHOLE 12          /* the same for the chunked coarse upsampling steps (default 0) */
#define SSG_TUNE_ISB_TAIL 13          /* ssg_isb_filter_batch: from the first level of at most this many
                                         pixels (0, 256, 1024 or 4096; 0 = none), the remaining down and
                                         up steps run as one launch, one block per instance (same bits;
                                         default 1024) */
#define SSG_TUNE_POST_TAIL 14         /* the same for the batched single-candidate filter
                                         (ssg_isb_apply_batch with one candidate: the distance
                                         post-filter): 0, 1024, 4096 or 16384 (default 4096) */
#define SSG_TUNE_STAGE_COLUMNS 15     /* image staging (ssg_stage_images, _u8, _resized): 1 = a warp per
                                         strip of texel columns walking down its rows, footprints formed
                                         in registers (default); 0 = blocks of shared-memory texel tiles.
                                         Same bits */
#define SSG_TUNE_TMA_WITHHOLD 7       /* tests of the bounded TMA wait: 1 = the TMA-staged upsampling arms
                                         its tile barriers but issues no copy, so every block's first
                                         wait runs out (after a short limit), it writes nothing and
                                         ssg_take_device_status reports SSG_STATUS_TMA_TIMEOUT; 0 = off */
SSG_API int ssg_tuning_set(int knob, int value);
/* The knob's current value (-1 for an unknown knob). */
SSG_API int ssg_tuning_get(int knob);
/* Writes up to `capacity` allowed values of a knob; returns how many it has (0 if unknown). */
SSG_API int ssg_tuning_choices(int knob, int32_t* values, int capacity);

/* Reads and clears the library's device status words: SSG_STATUS_TMA_TIMEOUT is set when
 * a bounded wait for a TMA tile ran out, SSG_STATUS_BARRIER_TIMEOUT when a grid-wide barrier of the
 * hole filling did.  The block that waited then wrote nothing more (no later
 * chunk, no selection), so the outputs of that launch are incomplete.  The word stays set until
 * this call clears it.  Synchronous. */
#define SSG_STATUS_TMA_TIMEOUT 1u
/* Set when a grid-wide barrier of the cooperative hole filling (SSG_TUNE_HOLE_PERSISTENT) ran
 * out of polls: the launch left its maps partly filled. */
#define SSG_STATUS_BARRIER_TIMEOUT 2u
SSG_API int ssg_take_device_status(uint32_t* status);

/* Message of the calling thread's last failed call ("" if none). */
SSG_API const char* ssg_last_error(void);
/* Library version, major * 10000 + minor * 100 + patch. */
SSG_API int ssg_version(void);
/* Writes {max cameras, max candidates, max references, max levels}. */
SSG_API void ssg_limits(int32_t* out4);

/* ---------------------------------------------------------------------------------------------
 * Guide image
 * ------------------------------------------------------------------------------------------- */

/* rgb2yCbCr followed by the uint8 cast: python/utils.py:144-155 and
 * python/depth_estimation.py:227.  d_rgb: pixels x 3 float32 (channel order as stored);
 * d_guide: pixels x 3 uint8. */
SSG_API int ssg_rgb_to_guide(const float* d_rgb, int64_t pixels, uint8_t* d_guide, void* stream);

/* ---------------------------------------------------------------------------------------------
 * Camera selection and sphere sweep
 * ------------------------------------------------------------------------------------------- */

/* RGBD_Estimator.select_camera for one reference camera: python/depth_estimation.py:83-135.
 * cameras: camera_count entries (host); relative_poses: camera_count x 12 floats (host), rows
 * 0..2 of inverse(camera.rt) @ reference.rt; d_masks: camera_count x rows x cols float32;
 * d_selected: rows x cols int8, -1 where no camera qualifies. */
SSG_API int ssg_select_camera(int cols, int rows, int camera_count, const ssg_camera* cameras, int reference,
                      const float* relative_poses, const float* d_masks, double min_dist, double max_dist,
                      int8_t* d_selected, void* stream);

/* Sphere sweep and per-pixel matching cost for one reference camera:
 * python/depth_estimation.py:141-175 (candidate volume, per-camera transform, projection,
 * bilinear zero-padded grid_sample, L1 over the three channels, clamp at 500).
 * d_images: camera_count device pointers (host array) to rows x cols x 3 float32 images;
 * candidates: candidate_count distances (host), 1 / linspace(1/min_dist, 1/max_dist);
 * d_cost: candidate_count x rows x cols float32. */
SSG_API int ssg_sweep_cost(int cols, int rows, int camera_count, const ssg_camera* cameras, int reference,
                   const float* relative_poses, const float* const* d_images, const int8_t* d_selected,
                   const float* candidates, int candidate_count, float* d_cost, void* stream);

/* ---------------------------------------------------------------------------------------------
 * ISB filter
 * ------------------------------------------------------------------------------------------- */

/* One edge-aware 2x downsampling step: guideDownsample2xKernel, python/isb_filter.cu:44-119
 * (launched by python/isb_filter.py:90-107).  Guides are rows x cols x 3 uint8, costs planar
 * candidate_count x rows x cols float32; var_inv_i = 1 / (2 sigma_i^2). */
SSG_API int ssg_isb_downsample(const uint8_t* d_guide_in, const float* d_cost_in, int rows_in, int cols_in,
                       uint8_t* d_guide_out, float* d_cost_out, int rows_out, int cols_out, int candidate_count,
                       float var_inv_i, void* stream);

/* One edge-aware 2x upsample-and-merge step, fine level updated in place:
 * guideUpsample2xKernel, python/isb_filter.cu:132-329 (python/isb_filter.py:109-134). */
SSG_API int ssg_isb_upsample(const uint8_t* d_guide_in, const float* d_cost_in, int rows_in, int cols_in,
                     uint8_t* d_guide_inout, float* d_cost_inout, int rows_inout, int cols_inout,
                     int candidate_count, float weight_up, float weight_down, float var_inv_i, void* stream);

/* Number of pyramid levels for a cols x rows image: python/isb_filter.py:60. */
SSG_API int ssg_isb_level_count(int cols, int rows);

/* ISB_Filter.apply as one call: python/isb_filter.py:72-136.  d_guides / d_costs: level_count
 * device pointers (host arrays); level 0 is the caller's guide and cost, filtered in place;
 * levels 1.. are scratch of ceil(rows / 2^l) x ceil(cols / 2^l) (python/isb_filter.py:62-70). */
SSG_API int ssg_isb_apply(uint8_t* const* d_guides, float* const* d_costs, int level_count, int rows, int cols,
                  int candidate_count, double sigma_i, double sigma_s, void* stream);

/* Distance selection: python/depth_estimation.py:179-198 (argmin / max over candidates,
 * parabolic sub-candidate step, flat-cost fallback, index -> distance).  d_cost: planar
 * candidate_count x pixels; d_distance: pixels float32; d_index: pixels int32 (may be NULL). */
SSG_API int ssg_select_distance(const float* d_cost, int candidate_count, int64_t pixels, const float* candidates,
                        float* d_distance, int32_t* d_index, void* stream);

/* The last upsampling step of ISB_Filter.apply (level 1 -> level 0) fused with distance
 * selection: python/isb_filter.cu:132-329 followed by python/depth_estimation.py:179-198.
 * Reads the fine cost but never writes it; writes the filtered level-0 guide and the distance. */
SSG_API int ssg_isb_upsample_select(const uint8_t* d_guide_in, const float* d_cost_in, int rows_in, int cols_in,
                            uint8_t* d_guide_inout, const float* d_cost_fine, int rows_fine, int cols_fine,
                            int candidate_count, float weight_up, float weight_down, float var_inv_i,
                            const float* candidates, float* d_distance, int32_t* d_index, void* stream);

/* ---------------------------------------------------------------------------------------------
 * Stitcher
 * ------------------------------------------------------------------------------------------- */

/* createInpaintingWeightsKernel, python/stitcher.cu:212-272.  translation: 3 floats (host),
 * (inverse(rt) @ [viewpoint, 1])[:3] (python/stitcher.py:130); d_table: rows x cols x 2 uint8. */
SSG_API int ssg_inpainting_table(int cols, int rows, const ssg_intrinsics* intrinsics, const float* translation,
                         double min_dist, double max_dist, uint8_t* d_table, void* stream);

/* Box mean over a (2 radius + 1)^2 window of each of `planes` rows x cols float32 planes, with
 * pad_value outside the image: the torch conv2d smoothing of python/stitcher.py:144-148
 * (pad_value 1) and :162-163 (pad_value 0). */
SSG_API int ssg_box_filter(const float* d_in, int planes, int rows, int cols, int radius, float pad_value, float* d_out,
                   void* stream);

/* createBlendingLutKernel, python/stitcher.cu:338-401, for reference_count cameras.
 * intrinsics / rotations (3x3 row-major, inverse of each camera rotation) / translations: host
 * arrays; d_masks: box-filtered masks, reference_count x rows x cols; d_lut:
 * reference_count x pano_rows x pano_cols x 2; d_weights: reference_count x pano_rows x pano_cols. */
SSG_API int ssg_blending_lut(int cols, int rows, int pano_cols, int pano_rows, int reference_count,
                     const ssg_intrinsics* intrinsics, const float* rotations, const float* translations,
                     const float* d_masks, double min_dist, double max_dist, float* d_lut, float* d_weights,
                     void* stream);

/* Blending-weight normalisation over references (python/stitcher.py:164), in place. */
SSG_API int ssg_normalize_weights(float* d_weights, int reference_count, int64_t pixels, void* stream);

/* Distance reprojection to the panorama viewpoint (z-buffer): reprojectDistanceKernel,
 * python/stitcher.cu:181-204, with the fill of python/stitcher.py:184 when fill != 0.
 * Each target pixel receives the minimum distance; targets outside the map are dropped. */
SSG_API int ssg_reproject_distance(const float* d_distance_in, float* d_distance_out, int cols, int rows,
                           const ssg_intrinsics* intrinsics, const float* translation, int fill, void* stream);

/* Hole filling: `iterations` launches of inpaintKernel, python/stitcher.cu:283-323
 * (python/stitcher.py:195-200), each a Jacobi step (every pixel reads the map as it was before
 * the step).  Runs as tiled passes of up to 16 steps each in shared memory, alternating between
 * d_distance and d_scratch (rows x cols float32, caller-owned); the result ends in d_distance.
 * Table entries whose offset field is 3 are ignored (the table kernel never writes one). */
SSG_API int ssg_inpaint(float* d_distance, const uint8_t* d_table, float* d_scratch, int cols, int rows, double max_dist,
                int iterations, void* stream);

/* Hole filling exactly as ssg_inpaint, for callers that cannot allocate device memory (a plugin
 * inside a host application whose memory manager owns the device heap, or a hard real-time loop
 * in which cudaMalloc may synchronise the device): the scratch map lives in a fixed 4 MiB array
 * inside the library, held by every GPU that loads the library until the process exits.  The
 * caller passes only the map and the table.  No counterpart in the reference.
 *   - Maps of up to 1,048,576 pixels (e.g. 1024 x 1024); larger maps return
 *     SSG_ERR_UNSUPPORTED without launching anything.
 *   - The first call on a device looks up the array's device address (cudaGetSymbolAddress)
 *     and enables the kernel's shared memory; make that first call before any stream capture.
 *     The address is kept for the life of the process: do not reset a device (cudaDeviceReset)
 *     after calling this on it, since the reset reloads the library's module and the kept address
 *     would no longer be the array's.
 *   - Every call on a device shares the array: calls that overlap on the GPU (different streams
 *     without ordering) race.  Each pass overwrites the whole scratch map it uses, so nothing a
 *     previous call left there is read.
 *   - No cudaMalloc / cudaFree or allocating library routine is called. */
SSG_API int ssg_inpaint_noalloc(float* d_distance, const uint8_t* d_table, int cols, int rows, double max_dist,
                                int iterations, void* stream);

/* mergeRGBDPanoramaKernel, python/stitcher.cu:423-473.  d_reprojected, d_distances:
 * reference_count x rows x cols; d_images: reference_count x image_rows x image_cols x 3 uint8;
 * outputs pano_rows x pano_cols float32 distance and x 3 uint8 colour. */
SSG_API int ssg_merge_panorama(const float* d_lut, const float* d_weights, const float* d_reprojected,
                       const float* d_distances, const uint8_t* d_images, int image_rows, int image_cols,
                       const float* translations, const ssg_intrinsics* intrinsics, int reference_count, int cols,
                       int rows, int pano_cols, int pano_rows, float* d_distance_panorama, uint8_t* d_rgb_panorama,
                       void* stream);

/* ---------------------------------------------------------------------------------------------
 * Batched path.  A batch holds `frames` frames of one rig; an "instance" is a (frame, reference
 * slot) pair, instance = frame * references + slot.  Buffers of a batch are contiguous arrays of
 * equally sized per-frame / per-instance blocks.  The per-frame steps are those of
 * RGBD_Estimator.estimate_RGBD_panorama (python/depth_estimation.py:205-242); these entry
 * points have no single counterpart in the reference, which processes one frame and one
 * reference camera per call.
 *
 * Cost volumes of the batched path are stored in chunks of 8 candidates, per instance and level
 * [ceil(N / 8)][pixels][8]: the level-0 volume with 16 bits per candidate (SSG_STORAGE_F16 /
 * SSG_STORAGE_UNORM16), the coarser levels as float32; all arithmetic is fp32.  Guides of the
 * batched path are one 32-bit word per pixel, bytes (Y, Cb, Cr, 0) (the reference's 3-byte
 * pixels padded: one load per pixel, the colour distance in one byte-wise absolute-difference
 * sum), rows x cols words per instance and level.
 * ------------------------------------------------------------------------------------------- */

/* Image staging + guides: d_images frames x cameras x rows x cols x 3, float32 (the inputs of
 * estimate_RGBD_panorama, python/depth_estimation.py:205-227) or uint8 (the 8-bit images those
 * inputs are made from, python/utils.py:157-205) -> d_staged: per (frame, camera) a region of
 * 32 x (rows + 2) x (cols + 2) bytes of entries, entry (j, i) holding the bilinear footprint of
 * top-left tap (i - 1, j - 1) -- texels (x0, y0), (x0 + 1, y0), (x0, y0 + 1), (x0 + 1, y0 + 1) --
 * one byte per texel in a 32-bit word per channel, zero outside the image (every entry is
 * written).  Values are staged as 8.8 fixed-point codes round(256 v): float inputs get 32-byte
 * entries (the high-byte words of channels 0, 1, 2, the low-byte word of channel 0, then the
 * low-byte words of channels 1, 2, zero padding); the uint8 variant writes 16-byte entries of
 * high-byte words in the first half of the region.  d_plane_flags frames x cameras int32: the largest
 * class of a plane's values -- 0 integers in [0, 255], 1 values in [0, 65535/256] with fractions
 * (as a linear resize makes them; the sweep then adds the low plane), 2 anything else (the sweep
 * samples that plane from the float images).  d_guides frames x references x rows x cols 32-bit
 * guide words (rgb2yCbCr + uint8 cast of each reference camera, python/utils.py:144-155, from the
 * float values).  Zeroes d_plane_flags first (a 4 x frames x cameras byte memset).  Planes of
 * (rows + 2) x (cols + 2) >= 2^24 entries return SSG_ERR_UNSUPPORTED.  d_staged is 16-byte aligned,
 * 32-byte aligned for float inputs (one 256-bit store per entry); d_guides 4-byte aligned. */
SSG_API int ssg_stage_images(const float* d_images, int frames, int cameras, int cols, int rows,
                             const int* reference_cameras, int references, float* d_staged, uint8_t* d_guides,
                             int32_t* d_plane_flags, void* stream);
SSG_API int ssg_stage_images_u8(const uint8_t* d_images, int frames, int cameras, int cols, int rows,
                                const int* reference_cameras, int references, float* d_staged, uint8_t* d_guides,
                                int32_t* d_plane_flags, void* stream);

/* Resize and staging in one pass, from the decoded 8-bit images (python/utils.py:198-201 resizes
 * each decoded image to the matching resolution before the estimator; python/main.py:73-81):
 * d_images holds frames x cameras images of src_rows x src_cols x 3 bytes, resized to cols x rows
 * with ssg_resize_linear's u8 -> float32 arithmetic and staged as ssg_stage_images stages those
 * float32 images -- the same entries, guides and plane flags bit for bit, without the float32
 * images in memory.  The entries are 32 bytes (sweep with ssg_sweep_cost_batch_entries,
 * entry_bytes 32, d_images NULL: resized 8-bit values never need the float path).  d_staged
 * 32-byte aligned.  SSG_ERR_UNSUPPORTED (resize with ssg_resize_linear and stage the result
 * instead) when d_images is not 4-byte aligned or src_cols x src_rows is not a multiple of 4, and
 * with SSG_TUNE_STAGE_COLUMNS = 0 when a tile's source window exceeds 160 KB of shared memory
 * (reductions beyond about 2.5x). */
SSG_API int ssg_stage_images_resized(const uint8_t* d_images, int src_cols, int src_rows, int frames, int cameras,
                                     int cols, int rows, const int* reference_cameras, int references,
                                     float* d_staged, uint8_t* d_guides, int32_t* d_plane_flags, void* stream);

/* float32 -> uint8 truncation of `count` values in [0, 255] (the float -> uint8 copy of the images
 * to stitch, python/depth_estimation.py:239-240); 16-byte loads and stores where both buffers are
 * 16-byte aligned. */
SSG_API int ssg_convert_u8(const float* d_src, uint8_t* d_dst, int64_t count, void* stream);

/* Sphere sweep + cost for every instance (python/depth_estimation.py:141-175), 16-bit output.
 * relative_poses: references x cameras x 12 floats (host); d_staged / d_plane_flags from
 * ssg_stage_images[_u8]; d_images: the float32 images staged by ssg_stage_images (read for planes
 * of class 2; it also selects the 32-byte entries), NULL after ssg_stage_images_u8; d_selected:
 * references x pixels int8; d_cost: instances x level-0 volume.  d_staged and d_cost are 16-byte
 * aligned, d_staged 32-byte aligned when d_images is given (one 256-bit load per entry). */
SSG_API int ssg_sweep_cost_batch(int cols, int rows, int frames, int camera_count, const ssg_camera* cameras,
                                 int references, const int* reference_cameras, const float* relative_poses,
                                 const float* d_staged, const float* d_images, const int32_t* d_plane_flags,
                                 const int8_t* d_selected, const float* candidates, int candidate_count, int storage,
                                 void* d_cost, void* stream);
/* The same with the entry size given: entry_bytes 16 (ssg_stage_images_u8) or 32
 * (ssg_stage_images, with d_images; ssg_stage_images_resized, d_images NULL).
 * ssg_sweep_cost_batch is this with entry_bytes = d_images ? 32 : 16. */
SSG_API int ssg_sweep_cost_batch_entries(int cols, int rows, int frames, int camera_count,
                                         const ssg_camera* cameras, int references, const int* reference_cameras,
                                         const float* relative_poses, const float* d_staged, int entry_bytes,
                                         const float* d_images, const int32_t* d_plane_flags,
                                         const int8_t* d_selected, const float* candidates, int candidate_count,
                                         int storage, void* d_cost, void* stream);

/* ISB down / up steps (python/isb_filter.cu:44-329) on `instances` contiguous levels.  The
 * downsampling reads a level stored as `storage` and writes float32; the upsampling reads and
 * writes float32 levels (storage must be SSG_STORAGE_F32). */
SSG_API int ssg_isb_downsample_batch(const uint8_t* d_guide_in, const void* d_cost_in, int rows_in, int cols_in,
                                     uint8_t* d_guide_out, void* d_cost_out, int rows_out, int cols_out,
                                     int candidate_count, int instances, int storage, float var_inv_i, void* stream);
SSG_API int ssg_isb_upsample_batch(const uint8_t* d_guide_in, const void* d_cost_in, int rows_in, int cols_in,
                                   uint8_t* d_guide_inout, void* d_cost_inout, int rows_inout, int cols_inout,
                                   int candidate_count, int instances, int storage, float weight_up, float weight_down,
                                   float var_inv_i, void* stream);

/* Last ISB level fused with distance selection (python/isb_filter.cu:132-329 +
 * python/depth_estimation.py:179-198): float32 coarse level, fine (level-0) volume stored as
 * `storage`; d_distance / d_index instances x fine pixels; d_distance_copy (or NULL) receives the
 * same distances (the post-filter's input, which it filters in place). */
/* The cost filter of a batch up to level 1 (python/isb_filter.py:72-134 without the last up
 * step, which ssg_isb_upsample_select_batch fuses with the selection): level 0 (`storage`) down to
 * level level_count - 1, then back up to level 1.  d_guides / d_costs: level_count device pointers
 * to the levels of every instance (the layouts of ssg_isb_downsample_batch; levels from 1 on
 * float32, 32-byte aligned); weight_up / weight_down: host arrays of the up steps' weights, indexed
 * by the fine level.  The small levels run as one fused launch (SSG_TUNE_ISB_TAIL): the same
 * results bit for bit as one ssg_isb_downsample_batch / ssg_isb_upsample_batch call per step. */
SSG_API int ssg_isb_filter_batch(uint8_t* const* d_guides, void* const* d_costs, int level_count, int rows, int cols,
                                 int candidate_count, int instances, int storage, const float* weight_up,
                                 const float* weight_down, float var_inv_i, void* stream);

SSG_API int ssg_isb_upsample_select_batch(const uint8_t* d_guide_in, const void* d_cost_in, int rows_in, int cols_in,
                                          uint8_t* d_guide_inout, const void* d_cost_fine, int rows_fine,
                                          int cols_fine, int candidate_count, int instances, int storage,
                                          float weight_up, float weight_down, float var_inv_i,
                                          const float* candidates, float* d_distance, int32_t* d_index,
                                          float* d_distance_copy, void* stream);

/* Distance selection from a level-0 volume (pyramids of fewer than two levels). */
SSG_API int ssg_select_distance_batch(const void* d_cost, int candidate_count, int64_t pixels, int instances,
                                      int storage, const float* candidates, float* d_distance, int32_t* d_index,
                                      void* stream);

/* ISB_Filter.apply (python/isb_filter.py:72-136) on `instances` contiguous float32 pyramids:
 * level l holds instances x ceil(rows/2^l) x ceil(cols/2^l) 32-bit guide words and instances x
 * (candidate_count x ... ) costs.  flags: 0, or SSG_ISB_SKIP_FINE_GUIDE when the caller wants
 * only the filtered costs (the distance post-filter, python/depth_estimation.py:200-203, keeps
 * the distance and drops the guide): the filtered level-0 guide is then not formed and d_guides[0]
 * keeps its input. */
#define SSG_ISB_SKIP_FINE_GUIDE 1
SSG_API int ssg_isb_apply_batch(uint8_t* const* d_guides, float* const* d_costs, int level_count, int rows, int cols,
                                int candidate_count, int instances, double sigma_i, double sigma_s, int flags,
                                void* stream);

/* Reprojection (python/stitcher.cu:181-204) of `instances` distance maps; instance i uses
 * intrinsics / translation of slot i % references. */
SSG_API int ssg_reproject_distance_batch(const float* d_distance_in, float* d_distance_out, int cols, int rows,
                                         int instances, int references, const ssg_intrinsics* intrinsics,
                                         const float* translations, int fill, void* stream);
/* ssg_reproject_distance_batch with fused multiply-adds and approximate square roots and
 * reciprocal in the projection and the distance (the batched 16-bit path, checked against the
 * fp32 path within tolerances). */
SSG_API int ssg_reproject_distance_batch_approx(const float* d_distance_in, float* d_distance_out, int cols, int rows,
                                                int instances, int references, const ssg_intrinsics* intrinsics,
                                                const float* translations, int fill, void* stream);

/* Inpainting (python/stitcher.cu:283-323) of `instances` maps; d_tables: references x rows x
 * cols x 2 (instance i uses table i % references); d_scratch: instances x rows x cols. */
SSG_API int ssg_inpaint_batch(float* d_distance, const uint8_t* d_tables, float* d_scratch, int cols, int rows,
                              int instances, int references, double max_dist, int iterations, void* stream);

/* Hole filling of `instances` maps with the result of ssg_inpaint_batch (the Jacobi steps of
 * inpaintKernel, python/stitcher.cu:283-323, bit for bit), in place and over lists of holes: a
 * scan stamps every pixel (d_stamps, instances x rows x cols bytes: 0 not a hole, 255 an open
 * hole, s filled at step s); step 1 visits every fillable hole, and step s > 1 only the open holes
 * that read a pixel filled at step s - 1.
 * d_holes: caller-owned int32 scratch of 3 x instances x rows x cols + SSG_HOLE_SCRATCH_HEADER
 * entries (3 rotating counts, the barrier words of the cooperative launch, two lists, a claim word
 * per pixel); instances x rows x cols < 2^31; iterations <= 254.  After a 32-byte memset,
 * launches the scan and step 1, then a kernel per later step, or one cooperative kernel for all of
 * them (SSG_TUNE_HOLE_PERSISTENT = 1, where the device supports cooperative launches). */
#define SSG_HOLE_SCRATCH_HEADER 8
SSG_API int ssg_inpaint_holes_batch(float* d_distance, const uint8_t* d_tables, uint8_t* d_stamps, int32_t* d_holes,
                                    int cols, int rows, int instances, int references, double max_dist,
                                    int iterations, void* stream);

/* Merge (python/stitcher.cu:423-473) of `frames` frames: maps frames x references x rows x
 * cols, images frames x references x image_rows x image_cols x 3, panoramas per frame. */
SSG_API int ssg_merge_panorama_batch(const float* d_lut, const float* d_weights, const float* d_reprojected,
                                     const float* d_distances, const uint8_t* d_images, int image_rows,
                                     int image_cols, const float* translations, const ssg_intrinsics* intrinsics,
                                     int reference_count, int cols, int rows, int pano_cols, int pano_rows, int frames,
                                     float* d_distance_panorama, uint8_t* d_rgb_panorama, void* stream);

/* ssg_merge_panorama_batch with fused multiply-adds and approximate square roots and
 * reciprocals in the same steps (the batched 16-bit path, whose panoramas are checked against the
 * fp32 path within tolerances: PSNR >= 50 dB, inverse-distance MAE <= 1e-4 of the range). */
SSG_API int ssg_merge_panorama_batch_approx(const float* d_lut, const float* d_weights, const float* d_reprojected,
                                            const float* d_distances, const uint8_t* d_images, int image_rows,
                                            int image_cols, const float* translations,
                                            const ssg_intrinsics* intrinsics, int reference_count, int cols, int rows,
                                            int pano_cols, int pano_rows, int frames, float* d_distance_panorama,
                                            uint8_t* d_rgb_panorama, void* stream);

/* The same with the images given as image_count images per frame (image_rows x image_cols x 3
 * bytes each, frames contiguous), reference r stitching image image_slots[r] (host array of
 * reference_count indices): for instance every camera's decoded image of a batch, of which the
 * references' are the images to stitch when the stitch resolution is the decoded one (the
 * reference's input preparation then resizes them to their own size, python/utils.py:198-201).
 * ssg_merge_panorama_batch_approx is this with image_count = reference_count, image_slots = 0, 1,
 * ... */
SSG_API int ssg_merge_panorama_batch_approx_images(const float* d_lut, const float* d_weights,
                                                   const float* d_reprojected, const float* d_distances,
                                                   const uint8_t* d_images, int image_count, const int* image_slots,
                                                   int image_rows, int image_cols, const float* translations,
                                                   const ssg_intrinsics* intrinsics, int reference_count, int cols,
                                                   int rows, int pano_cols, int pano_rows, int frames,
                                                   float* d_distance_panorama, uint8_t* d_rgb_panorama,
                                                   void* stream);

/* ---------------------------------------------------------------------------------------------
 * Differentiable sweep (no counterpart in the reference, whose selection is a hard argmin with
 * a parabolic step, python/depth_estimation.py:179-198).  Forward: the fp32 sweep and ISB filter
 * above, then a soft-argmin inverse distance q = sum_k softmax(-F_k / temperature) / d_k over the
 * filtered costs F, fused with the last filter level.  Backward: the transposes of those linear
 * steps (the filter's weights come from uint8 guides and receive no gradient) and of the sweep.
 * Gradient buffers are float32 planar volumes like the forward's.  Every gradient is
 * bit-reproducible run to run: the filter's transposed steps gather (each output cell sums what
 * it receives in a fixed order), the image gradient is summed in 64-bit fixed point, and the
 * pose gradient by a fixed float64 reduction tree.
 * ------------------------------------------------------------------------------------------- */

/* Last ISB level (level 1 -> 0) fused with the soft-argmin: d_inverse_distance fine pixels. */
SSG_API int ssg_isb_upsample_softargmin(const uint8_t* d_guide_in, const float* d_cost_in, int rows_in, int cols_in,
                                        const uint8_t* d_guide_fine, const float* d_cost_fine, int rows_fine,
                                        int cols_fine, int candidate_count, float weight_up, float weight_down,
                                        float var_inv_i, const float* candidates, float temperature,
                                        float* d_inverse_distance, void* stream);

/* Backward of ssg_isb_upsample_softargmin: writes dL/dF, the gradient with respect to the
 * filtered level-0 costs (candidate planes of the fine level); ssg_isb_upsample_transpose of
 * the same level then splits it into the level-0 cost gradient and the filtered level-1 one. */
SSG_API int ssg_isb_upsample_softargmin_backward(const uint8_t* d_guide_in, const float* d_cost_in, int rows_in,
                                                 int cols_in, const uint8_t* d_guide_fine, const float* d_cost_fine,
                                                 int rows_fine, int cols_fine, int candidate_count, float weight_up,
                                                 float weight_down, float var_inv_i, const float* candidates,
                                                 float temperature, const float* d_grad_inverse_distance,
                                                 float* d_grad_filtered_fine, void* stream);

/* Transpose of one upsampling step (python/isb_filter.cu:132-329): writes the own-pixel part of
 * dL/d(filtered fine level) to d_grad_cost_fine and its coarse-tap part to d_grad_filtered_coarse
 * (every cell of both is written).  d_guide_coarse: filtered coarse guide; d_guide_fine: the fine
 * guide before its own upsampling step. */
SSG_API int ssg_isb_upsample_transpose(const uint8_t* d_guide_coarse, int rows_in, int cols_in,
                                       const uint8_t* d_guide_fine, int rows_fine, int cols_fine,
                                       int candidate_count, float weight_up, float weight_down, float var_inv_i,
                                       const float* d_grad_filtered_fine, float* d_grad_cost_fine,
                                       float* d_grad_filtered_coarse, void* stream);

/* Transpose of one downsampling step (python/isb_filter.cu:44-119): adds the coarse gradient,
 * spread over the 3 x 3 taps, into d_grad_cost_fine (each fine cell gathers its share). */
SSG_API int ssg_isb_downsample_transpose(const uint8_t* d_guide_in, int rows_in, int cols_in, int rows_out,
                                         int cols_out, int candidate_count, float var_inv_i,
                                         const float* d_grad_cost_coarse, float* d_grad_cost_fine, void* stream);

/* Backward of ssg_sweep_cost (python/depth_estimation.py:141-175): adds dL/d(image) into
 * d_grad_images (camera_count device pointers, rows x cols x 3 float32) and the per-camera
 * 6-DoF gradient into d_grad_pose (camera_count x 6 float64: rotation, then translation, of a
 * right perturbation T <- T [Exp(omega), v] evaluated at zero).  The image gradient of the call
 * is summed in 64-bit fixed point: multiples of 2^-e, with 2^e the largest power of two for which
 * 2 x pixels x candidates x max |d_grad_cost| x 2^e stays below 2^62 (a contribution is rounded by
 * at most 2^-(e+1)); a non-finite d_grad_cost makes it NaN.  d_scratch: 256-byte aligned,
 * ssg_sweep_backward_scratch_bytes(cols, rows, camera_count) bytes, not shared by calls in
 * flight at once. */
SSG_API size_t ssg_sweep_backward_scratch_bytes(int cols, int rows, int camera_count);
SSG_API int ssg_sweep_cost_backward(int cols, int rows, int camera_count, const ssg_camera* cameras, int reference,
                                    const float* relative_poses, const float* const* d_images,
                                    float* const* d_grad_images, const int8_t* d_selected, const float* candidates,
                                    int candidate_count, const float* d_grad_cost, double* d_grad_pose,
                                    void* d_scratch, void* stream);

/* ---------------------------------------------------------------------------------------------
 * Uneven batches (no counterpart in the reference, which estimates one rig's frame per call of
 * estimate_RGBD_panorama, python/depth_estimation.py:205-242): many RGB-D panorama jobs of
 * different rigs, matching resolutions and candidate counts in one fixed sequence of launches --
 * one persistent sweep launch over every instance (a work queue of 256-pixel tiles, largest
 * instances first), one launch per cost-filter step, one fused selection, one launch per
 * post-filter step, then fill, reprojection, hole filling and merge over every job.  The 16-bit
 * path's arithmetic (ssg_sweep_cost_batch, ssg_isb_*_batch, ssg_merge_panorama_batch_approx).
 * ------------------------------------------------------------------------------------------- */

/* One instance: one reference camera of one rig, with its own buffers (device pointers, the
 * layouts of the batched functions above for one instance). */
typedef struct {
    int cols, rows;               /* matching resolution; at least 2 filter levels */
    int camera_count;             /* cameras of the rig */
    int reference_camera;         /* the reference camera, in [0, camera_count) */
    int candidate_count;
    const ssg_camera* cameras;    /* host, camera_count */
    const float* relative_poses;  /* host, camera_count x 12: rows 0..2 of inverse(camera.rt) @ reference.rt */
    const float* candidates;      /* host, candidate_count distances */
    double sigma_i, sigma_s;      /* cost filter; the distance post-filter uses half of each */
    const float* d_staged;        /* the rig frame's planes from ssg_stage_images (2 x camera_count planes) */
    const float* d_images;        /* the frame's float32 images staged (or NULL for 8-bit inputs) */
    const int32_t* d_plane_flags; /* the frame's camera_count plane flags from ssg_stage_images */
    const int8_t* d_selected;     /* rows x cols selected cameras */
    uint8_t* const* d_guides;     /* host array of level_count pointers: the guide pyramid (level 0 staged) */
    void* const* d_costs;         /* host array: level 0 16-bit chunked (written by the sweep), others float32 */
    uint8_t* const* d_df_guides;  /* host array of level_count pointers: post-filter guides (level 0 may be
                                     d_guides[0], which the 16-bit selection leaves unchanged) */
    float* const* d_df_costs;     /* host array of level_count - 1 pointers: post-filter levels 1.. */
    float* d_distance_raw;        /* rows x cols: the selection's distance */
    float* d_distance;            /* rows x cols: the filtered distance */
    int32_t* d_index;             /* rows x cols selected candidate index, or NULL */
} ssg_uneven_instance;

/* One job: the stitch of one rig's instances (python/stitcher.py:166-220). */
typedef struct {
    int cols, rows, references, pano_cols, pano_rows, image_cols, image_rows;
    const ssg_intrinsics* intrinsics; /* host, references */
    const float* translations;        /* host, references x 3 */
    const float* d_distance;          /* references x rows x cols: the instances' d_distance maps, contiguous */
    const uint8_t* d_tables;          /* references x rows x cols x 2 inpainting tables */
    const float* d_lut;               /* references x pano_rows x pano_cols x 2 */
    const float* d_weights;           /* references x pano_rows x pano_cols */
    const uint8_t* d_images;          /* references x image_rows x image_cols x 3 */
    float* d_pano_distance;           /* pano_rows x pano_cols */
    uint8_t* d_rgb;                   /* pano_rows x pano_cols x 3 */
} ssg_uneven_job;

typedef struct ssg_uneven_batch ssg_uneven_batch;

/* Validates the instances and jobs and lays out their descriptors; gives the sizes of the device
 * plan and scratch the caller allocates (256-byte aligned).  storage: SSG_STORAGE_F16 or
 * SSG_STORAGE_UNORM16.  The host arrays are read during the call only. */
SSG_API int ssg_uneven_create(const ssg_uneven_instance* instances, int instance_count, const ssg_uneven_job* jobs,
                              int job_count, int storage, double max_dist, int inpainting_iterations,
                              size_t* plan_bytes, size_t* scratch_bytes, ssg_uneven_batch** batch);
/* Writes the descriptors into d_plan (synchronising `stream`: call it at set-up, outside a
 * capture) and binds d_scratch (the sweep's work counter, the reprojected maps, hole lists). */
SSG_API int ssg_uneven_upload(ssg_uneven_batch* batch, void* d_plan, void* d_scratch, void* stream);
/* Enqueues the batch's launches on `stream` (capturable in a CUDA graph). */
SSG_API int ssg_uneven_run(const ssg_uneven_batch* batch, void* stream);
/* Kernels one ssg_uneven_run launches. */
SSG_API int ssg_uneven_launches(const ssg_uneven_batch* batch);
SSG_API void ssg_uneven_destroy(ssg_uneven_batch* batch);

/* ---------------------------------------------------------------------------------------------
 * Input preparation: the resize of decoded images to the matching and stitching resolutions
 * (python/utils.py:198-201), on the device.
 * ------------------------------------------------------------------------------------------- */
#define SSG_PIXEL_U8 0
#define SSG_PIXEL_F32 1

/* Linear resize of `images` images (contiguous) of src_cols x src_rows x channels (1..4,
 * interleaved) to dst_cols x dst_rows: the interpolation the reference's
 * cv2.resize(image, size, cv2.INTER_AREA) call performs (its third positional argument is `dst`,
 * so the default INTER_LINEAR applies), restated from OpenCV's published algorithm: pixel-centre
 * mapping, edge clamping, separately rounded float products and sums; an exact 2x reduction is a
 * 2x2 average.  Types: uint8 -> float32 (the reference converts decoded images to float32 and
 * resizes those), float32 -> float32, and uint8 -> uint8 with 11-bit fixed-point weights (its
 * ground-truth resize, utils.py:221-222).  One launch. */
SSG_API int ssg_resize_linear(const void* d_src, int src_type, int src_cols, int src_rows, int channels, void* d_dst,
                              int dst_type, int dst_cols, int dst_rows, int images, void* stream);

/* ---------------------------------------------------------------------------------------------
 * Evaluation against ground truth (python/utils.py:206-250, evaluate_rgbd_panorama): the
 * reference computes these per frame on the host with scikit-image and numpy; here a batch of
 * frames is reduced on the device.
 * ------------------------------------------------------------------------------------------- */
#define SSG_EVAL_MAX_THRESHOLDS 16
#define SSG_EVAL_FIXED_METRICS 4 /* psnr, ssim, mae, rmse */

/* Bytes of the scratch ssg_eval_panoramas needs (8-byte aligned); 0 for invalid arguments. */
SSG_API size_t ssg_eval_scratch_bytes(int frames, int threshold_count);
/* Metrics of `frames` RGB-D panoramas of cols x rows (contiguous per frame) against their ground
 * truth: d_rgb / d_gt_rgb uint8 [rows][cols][3], d_inv_distance / d_gt_inv_distance float32
 * [rows][cols] (inverse distances, python/main.py:114).  d_metrics (float64, device) receives per
 * frame psnr, ssim, mae, rmse, then threshold_count bad-pixel ratios in percent (thresholds: host
 * array), with the definitions of peak_signal_noise_ratio(gt, est), structural_similarity(gt, est,
 * multichannel=True) on x / 255 float32 images and the reference's numpy expressions
 * (utils.py:230-244).  Panoramas must be at least 7 x 7 (the SSIM window).  Deterministic: fixed
 * reduction order.  Three launches. */
SSG_API int ssg_eval_panoramas(int cols, int rows, int frames, const uint8_t* d_rgb, const uint8_t* d_gt_rgb,
                               const float* d_inv_distance, const float* d_gt_inv_distance, const float* thresholds,
                               int threshold_count, void* d_scratch, double* d_metrics, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SPHERE_STEREO_GB300_H */
