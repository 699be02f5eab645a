// Uneven batches: per-instance descriptors in device memory, read by the descriptor-driven
// kernels of ssg_sweep_batch.cu, ssg_isb.cu and ssg_stitch.cu and launched by ssg_uneven.cu.
// An instance is one reference camera of one rig at its own resolution and candidate count; a job
// is one rig's RGB-D panorama (its instances plus the stitch).
#pragma once

#include "ssg_cells.cuh"
#include "ssg_isb_common.cuh"

namespace ssg {

constexpr int kSweepTile = kBatchBlock;  // reference pixels per work item of the persistent sweep

// One instance of the persistent sweep.  Instances are ordered by decreasing work
// (pixels x chunks) and tile_begin is the prefix of their tile counts, so the work queue hands
// out the expensive tiles first.
struct SweepInst {
    int cols, rows, cameras, ncand;
    int chunks, ref_camera, tile_begin, tiles;
    int storage, pad0, pad1, pad2;
    const uint4* staged;     // camera 0's plane of footprints of the instance's frame
    const float* floats;     // camera 0's float image of the frame (planes with flags set), or NULL
    const int* plane_flags;  // per camera of the frame: 1 where the plane is sampled from `floats`
    const int8_t* selected;  // rows x cols
    void* cost;              // chunks x rows x cols x 8, 16-bit
    TorchCam ref_cam;
    FastCam cam[SSG_MAX_CAMERAS];
    float pose[SSG_MAX_CAMERAS][12];
    alignas(8) float cand[SSG_MAX_CANDIDATES];  // padded to whole chunks with the last candidate
};

// One instance's share of one filter launch (a down step, an up step, or the selecting step)
struct LevelDesc {
    LevelGeom g;
    int chunks, ncand;
    float weight_up, weight_down, var_inv_i;
    int pad;
    const uint8_t* guide_in;
    const void* cost_in;
    uint8_t* guide_out;  // down: the coarse guide; up: the fine guide (read, and written if not the select)
    void* cost_out;      // down: coarse costs; up: fine costs (in place; read only by the select)
    SelectOut so;        // the selecting step
    const float* lut;    // the range-weight table of var_inv_i (range_table()), or nullptr
};

// Stitch of one job (python/stitcher.py:166-220): `references` maps of cols x rows, contiguous
struct StitchJob {
    int cols, rows, references, pano_cols, pano_rows, image_cols, image_rows;
    int map_begin;        // flat index of the job's first map pixel in the concatenated maps
    float ratio_x, ratio_y;
    int word_rows;  // `images` starts and ends on 4-byte boundaries: texel pairs read as words
    int pad1;
    const float* distance;      // references x rows x cols, filtered distance maps
    float* reprojected;         // references x rows x cols, in the concatenated maps
    const uint8_t* tables;      // references x rows x cols x 2 inpainting tables
    const float2* lut;          // references x pano_rows x pano_cols
    const float* weights;       // references x pano_rows x pano_cols
    const uint8_t* images;      // references x image_rows x image_cols x 3
    float* pano_distance;       // pano_rows x pano_cols
    uint8_t* rgb;               // pano_rows x pano_cols x 3
    Intr k[SSG_MAX_REFERENCES];
    float t[SSG_MAX_REFERENCES][3];
};

// ISB constants of a pyramid (python/isb_filter.py:87-88, :110-112)
struct Levels {
    float var_inv_i;
    float weight_up[SSG_MAX_LEVELS], weight_down[SSG_MAX_LEVELS];
};
Levels isb_constants(int level_count, double sigma_i, double sigma_s);
int level_rows(int rows, int s);  // ceil(rows / 2^s)
SelectOut select_constants(const float* candidates, int ncand, float* distance, int32_t* index);

// launchers (descriptor arrays in device memory)
int launch_sweep_uneven(const SweepInst* d_insts, int instances, int total_tiles, int storage, int* d_counter,
                        cudaStream_t st);
int launch_down_uneven(const LevelDesc* d_descs, int count, int max_rows_out, int max_cols_out, int width,
                       int storage_in, cudaStream_t st);
// guide = false: the single-candidate step does not form the filtered fine guide
int launch_up_uneven(const LevelDesc* d_descs, int count, int max_rows_in, int max_cols_in, int width,
                     int storage_fine, bool select, bool guide, cudaStream_t st);
// fill + reprojection + hole filling + merge of every job: maps concatenated job by job
// (total_map_pixels), d_stamps one byte per map pixel, d_holes 3 x total_map_pixels + 4 int32
int launch_stitch_uneven(const StitchJob* d_jobs, int jobs, float* d_maps, int64_t total_map_pixels,
                         int max_map_pixels, int max_pano_pixels, int max_references, double max_dist,
                         int iterations, uint8_t* d_stamps, int32_t* d_holes, cudaStream_t st);

}  // namespace ssg
