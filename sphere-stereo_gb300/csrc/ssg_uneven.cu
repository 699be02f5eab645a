// Uneven batches: many RGB-D panorama jobs of different rigs, matching resolutions and candidate
// counts in one sequence of launches (no counterpart in the reference, which runs one rig's frame
// per call of estimate_RGBD_panorama, python/depth_estimation.py:205-242).
//
//   sweep + cost           one persistent launch: a work queue of 256-pixel tiles over every
//                          instance, largest instances first
//   cost filter            one launch per pyramid step over the instances that have the step
//   selection              one launch (the last up step, fused), writing the raw and the
//                          post-filter's level-0 distance
//   distance post-filter   one launch per step (single candidate, sigma / 2)
//   stitch                 fill, reprojection, hole lists and merge over every job's maps
//
// ssg_uneven_create validates the specs and lays out the descriptors on the host;
// ssg_uneven_upload writes them into caller-owned device memory; ssg_uneven_run enqueues the
// launches (no allocation, no host synchronisation: the sequence can be captured in a CUDA graph).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "ssg_uneven.cuh"

namespace ssg {

namespace {

struct Step {
    size_t offset;  // byte offset of the step's LevelDesc array in the plan
    int count, rows, cols, width, storage;
    bool down, select;
    bool guide;  // an upsampling step forms the filtered fine guide
};

constexpr size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

}  // namespace

}  // namespace ssg

struct ssg_uneven_batch {
    std::vector<ssg::SweepInst> sweep;
    std::vector<ssg::LevelDesc> levels;  // every step's descriptors, back to back
    std::vector<ssg::Step> steps;
    std::vector<ssg::StitchJob> jobs;
    size_t sweep_offset = 0, levels_offset = 0, jobs_offset = 0, plan_bytes = 0;
    size_t maps_offset = 0, stamps_offset = 0, holes_offset = 0, scratch_bytes = 0;
    int total_tiles = 0, storage = SSG_STORAGE_F16, iterations = 0, max_references = 1;
    int max_map_pixels = 0, max_pano_pixels = 0;
    int64_t total_map_pixels = 0;
    double max_dist = 0;
    unsigned char* d_plan = nullptr;
    unsigned char* d_scratch = nullptr;
};

using namespace ssg;

static int check_instance(const ssg_uneven_instance& in, int i)
{
    SSG_REQUIRE(in.cols > 0 && in.rows > 0 && (int64_t)(in.cols + 2) * (in.rows + 2) < ((int64_t)1 << 31),
                "instance %d: invalid resolution", i);
    SSG_REQUIRE(in.camera_count >= 1 && in.camera_count <= SSG_MAX_CAMERAS, "instance %d: camera_count out of range",
                i);
    SSG_REQUIRE(in.reference_camera >= 0 && in.reference_camera < in.camera_count,
                "instance %d: reference camera out of range", i);
    SSG_REQUIRE(in.candidate_count >= 1 && in.candidate_count <= SSG_MAX_CANDIDATES,
                "instance %d: candidate_count out of range", i);
    SSG_REQUIRE(in.cameras && in.relative_poses && in.candidates, "instance %d: null host array", i);
    SSG_REQUIRE(in.sigma_i > 0 && in.sigma_s > 0, "instance %d: sigmas must be positive", i);
    SSG_REQUIRE(in.d_staged && in.d_plane_flags && in.d_selected && in.d_guides && in.d_costs && in.d_df_guides &&
                    in.d_df_costs && in.d_distance_raw && in.d_distance,
                "instance %d: null device pointer", i);
    SSG_REQUIRE(((uintptr_t)in.d_staged & 15) == 0, "instance %d: staged planes must be 16-byte aligned", i);
    SSG_REQUIRE(!in.d_images || ((uintptr_t)in.d_staged & 31) == 0,
                "instance %d: the staged planes of float images (32-byte entries) must be 32-byte aligned", i);
    const int L = ssg_isb_level_count(in.cols, in.rows);
    SSG_REQUIRE(L >= 2 && L <= SSG_MAX_LEVELS, "instance %d: a %dx%d image has %d filter levels (2 or more needed)",
                i, in.cols, in.rows, L);
    for (int l = 0; l < L; ++l) {
        SSG_REQUIRE(in.d_guides[l] && in.d_costs[l] && in.d_df_guides[l], "instance %d: level %d is NULL", i, l);
        // whole cells: 16 bytes of the 16-bit level 0, 32 bytes (one 256-bit access) of float32 levels
        const uintptr_t mask = l == 0 ? 15 : 31;
        SSG_REQUIRE(((uintptr_t)in.d_costs[l] & mask) == 0, "instance %d: cost level %d must be %d-byte aligned", i, l,
                    (int)mask + 1);
    }
    for (int l = 1; l < L; ++l) SSG_REQUIRE(in.d_df_costs[l - 1], "instance %d: post-filter level %d is NULL", i, l);
    for (int c = 0; c < in.camera_count; ++c) {
        const ssg_camera& k = in.cameras[c];
        SSG_REQUIRE(std::isfinite(k.xi) && std::isfinite(k.alpha) && k.alpha > 0.0 && k.alpha <= 1.0,
                    "instance %d camera %d: xi must be finite and alpha in (0, 1]", i, c);
    }
    return SSG_OK;
}

static int check_job(const ssg_uneven_job& j, int i)
{
    SSG_REQUIRE(j.cols > 1 && j.rows > 1 && j.pano_cols > 0 && j.pano_rows > 0 && j.image_cols > 1 && j.image_rows > 1,
                "job %d: invalid sizes", i);
    SSG_REQUIRE(j.references >= 1 && j.references <= SSG_MAX_REFERENCES, "job %d: references out of range", i);
    SSG_REQUIRE(j.intrinsics && j.translations && j.d_distance && j.d_tables && j.d_lut && j.d_weights &&
                    j.d_images && j.d_pano_distance && j.d_rgb,
                "job %d: null pointer", i);
    for (int r = 0; r < j.references; ++r) {
        const ssg_intrinsics& k = j.intrinsics[r];
        SSG_REQUIRE(std::isfinite(k.xi) && std::isfinite(k.alpha) && k.alpha > 0.0f && k.alpha <= 1.0f &&
                        k.fx != 0.0f && k.fy != 0.0f,
                    "job %d intrinsics %d: invalid", i, r);
    }
    return SSG_OK;
}

extern "C" int ssg_uneven_create(const ssg_uneven_instance* instances, int instance_count,
                                 const ssg_uneven_job* jobs, int job_count, int storage, double max_dist,
                                 int inpainting_iterations, size_t* plan_bytes, size_t* scratch_bytes,
                                 ssg_uneven_batch** out)
{
    SSG_REQUIRE(out && plan_bytes && scratch_bytes, "null output pointer");
    *out = nullptr;
    SSG_REQUIRE(instances && instance_count >= 1 && instance_count <= 65535, "instance_count out of range");
    SSG_REQUIRE(job_count >= 0 && job_count <= 65535 && (job_count == 0 || jobs), "job_count out of range");
    SSG_REQUIRE(storage == SSG_STORAGE_F16 || storage == SSG_STORAGE_UNORM16, "storage must be 16-bit");
    SSG_REQUIRE(inpainting_iterations >= 0 && inpainting_iterations <= 254, "inpainting_iterations out of range");
    for (int i = 0; i < instance_count; ++i)
        if (int e = check_instance(instances[i], i)) return e;
    for (int j = 0; j < job_count; ++j)
        if (int e = check_job(jobs[j], j)) return e;

    ssg_uneven_batch* b = new ssg_uneven_batch();
    b->storage = storage;
    b->iterations = inpainting_iterations;
    b->max_dist = max_dist;

    // --- sweep: instances by decreasing work, tiles prefixed in that order
    std::vector<int> order(instance_count);
    for (int i = 0; i < instance_count; ++i) order[i] = i;
    auto work = [&](int i) {
        const ssg_uneven_instance& in = instances[i];
        return (int64_t)in.cols * in.rows * ((in.candidate_count + 7) / 8);
    };
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return work(a) > work(c); });
    int64_t tiles = 0;
    for (int i : order) {
        const ssg_uneven_instance& in = instances[i];
        SweepInst s{};
        s.cols = in.cols;
        s.rows = in.rows;
        s.cameras = in.camera_count;
        s.ncand = in.candidate_count;
        s.chunks = (in.candidate_count + 7) / 8;
        s.ref_camera = in.reference_camera;
        s.tiles = (int)(((int64_t)in.cols * in.rows + kSweepTile - 1) / kSweepTile);
        s.tile_begin = (int)tiles;
        tiles += s.tiles;
        s.storage = storage;
        s.staged = reinterpret_cast<const uint4*>(in.d_staged);
        s.floats = in.d_images;
        s.plane_flags = in.d_plane_flags;
        s.selected = in.d_selected;
        s.cost = in.d_costs[0];
        s.ref_cam = make_torch_cam(in.cameras[in.reference_camera]);
        for (int c = 0; c < in.camera_count; ++c) {
            const ssg_camera& k = in.cameras[c];
            s.cam[c] = FastCam{k.fx, k.fy, k.cx, k.cy, (float)k.xi, (float)k.alpha, (float)(1.0 - k.alpha)};
            std::memcpy(s.pose[c], in.relative_poses + 12 * c, sizeof(float) * 12);
        }
        for (int k = 0; k < 8 * s.chunks; ++k)
            s.cand[k] = in.candidates[k < in.candidate_count ? k : in.candidate_count - 1];
        b->sweep.push_back(s);
    }
    if (tiles >= ((int64_t)1 << 31)) {
        delete b;
        return fail(SSG_ERR_UNSUPPORTED, "uneven batch of %lld sweep tiles is too large", (long long)tiles);
    }
    b->total_tiles = (int)tiles;

    // --- filter steps
    std::vector<int> L(instance_count);
    int max_levels = 0;
    for (int i = 0; i < instance_count; ++i) {
        L[i] = ssg_isb_level_count(instances[i].cols, instances[i].rows);
        max_levels = std::max(max_levels, L[i]);
    }
    auto geom = [&](int i, int fine, int coarse, bool down) {
        const ssg_uneven_instance& in = instances[i];
        const int rf = level_rows(in.rows, fine), cf = level_rows(in.cols, fine);
        const int rc = level_rows(in.rows, coarse), cc = level_rows(in.cols, coarse);
        return down ? LevelGeom{rf, cf, rc, cc} : LevelGeom{rc, cc, rf, cf};
    };
    auto add_step = [&](bool down, bool select, int width, int st, const std::vector<LevelDesc>& descs,
                        bool guide = true) {
        if (descs.empty()) return;
        Step step{};
        step.guide = guide;
        step.offset = b->levels.size();  // index for now, bytes after layout
        step.count = (int)descs.size();
        step.down = down;
        step.select = select;
        step.width = width;
        step.storage = st;
        for (const LevelDesc& d : descs) {
            step.rows = std::max(step.rows, down ? d.g.rows_out : d.g.rows_in);
            step.cols = std::max(step.cols, down ? d.g.cols_out : d.g.cols_in);
        }
        b->levels.insert(b->levels.end(), descs.begin(), descs.end());
        b->steps.push_back(step);
    };
    // cost filter (python/isb_filter.py:72-136): downsampling, then upsampling to level 1
    for (int s = 1; s < max_levels; ++s) {
        std::vector<LevelDesc> descs;
        for (int i = 0; i < instance_count; ++i) {
            if (L[i] <= s) continue;
            const ssg_uneven_instance& in = instances[i];
            LevelDesc d{};
            d.g = geom(i, s - 1, s, true);
            d.chunks = (in.candidate_count + 7) / 8;
            d.ncand = in.candidate_count;
            d.var_inv_i = isb_constants(L[i], in.sigma_i, in.sigma_s).var_inv_i;
            d.guide_in = in.d_guides[s - 1];
            d.cost_in = in.d_costs[s - 1];
            d.guide_out = in.d_guides[s];
            d.cost_out = in.d_costs[s];
            descs.push_back(d);
        }
        add_step(true, false, 8, s == 1 ? storage : SSG_STORAGE_F32, descs);
    }
    for (int s = max_levels - 2; s >= 1; --s) {
        std::vector<LevelDesc> descs;
        for (int i = 0; i < instance_count; ++i) {
            if (s > L[i] - 2) continue;
            const ssg_uneven_instance& in = instances[i];
            const Levels c = isb_constants(L[i], in.sigma_i, in.sigma_s);
            LevelDesc d{};
            d.g = geom(i, s, s + 1, false);
            d.chunks = (in.candidate_count + 7) / 8;
            d.ncand = d.chunks * 8;
            d.var_inv_i = c.var_inv_i;
            d.weight_up = c.weight_up[s];
            d.weight_down = c.weight_down[s];
            d.guide_in = in.d_guides[s + 1];
            d.cost_in = in.d_costs[s + 1];
            d.guide_out = in.d_guides[s];
            d.cost_out = in.d_costs[s];
            descs.push_back(d);
        }
        add_step(false, false, 8, SSG_STORAGE_F32, descs);
    }
    // the last up step fused with the selection (python/depth_estimation.py:179-198); it also writes
    // the distance the post-filter starts from
    {
        std::vector<LevelDesc> descs;
        for (int i = 0; i < instance_count; ++i) {
            const ssg_uneven_instance& in = instances[i];
            const Levels c = isb_constants(L[i], in.sigma_i, in.sigma_s);
            LevelDesc d{};
            d.g = geom(i, 0, 1, false);
            d.chunks = (in.candidate_count + 7) / 8;
            d.ncand = in.candidate_count;
            d.var_inv_i = c.var_inv_i;
            d.weight_up = c.weight_up[0];
            d.weight_down = c.weight_down[0];
            d.guide_in = in.d_guides[1];
            d.cost_in = in.d_costs[1];
            d.guide_out = in.d_guides[0];
            d.cost_out = in.d_costs[0];
            d.so = select_constants(in.candidates, in.candidate_count, in.d_distance_raw, in.d_index);
            d.so.distance2 = in.d_distance;
            descs.push_back(d);
        }
        add_step(false, true, 8, storage, descs);
    }
    // distance post-filter (python/depth_estimation.py:200-203): one candidate, sigma / 2
    for (int s = 1; s < max_levels; ++s) {
        std::vector<LevelDesc> descs;
        for (int i = 0; i < instance_count; ++i) {
            if (L[i] <= s) continue;
            const ssg_uneven_instance& in = instances[i];
            LevelDesc d{};
            d.g = geom(i, s - 1, s, true);
            d.chunks = 1;
            d.ncand = 1;
            d.var_inv_i = isb_constants(L[i], in.sigma_i / 2, in.sigma_s / 2).var_inv_i;
            d.guide_in = in.d_df_guides[s - 1];
            d.cost_in = s == 1 ? in.d_distance : in.d_df_costs[s - 2];
            d.guide_out = in.d_df_guides[s];
            d.cost_out = in.d_df_costs[s - 1];
            descs.push_back(d);
        }
        add_step(true, false, 1, SSG_STORAGE_F32, descs);
    }
    for (int s = max_levels - 2; s >= 0; --s) {
        std::vector<LevelDesc> descs;
        for (int i = 0; i < instance_count; ++i) {
            if (s > L[i] - 2) continue;
            const ssg_uneven_instance& in = instances[i];
            const Levels c = isb_constants(L[i], in.sigma_i / 2, in.sigma_s / 2);
            LevelDesc d{};
            d.g = geom(i, s, s + 1, false);
            d.chunks = 1;
            d.ncand = 1;
            d.var_inv_i = c.var_inv_i;
            d.weight_up = c.weight_up[s];
            d.weight_down = c.weight_down[s];
            d.guide_in = in.d_df_guides[s + 1];
            d.cost_in = in.d_df_costs[s];
            d.guide_out = in.d_df_guides[s];
            d.cost_out = s == 0 ? static_cast<void*>(in.d_distance) : static_cast<void*>(in.d_df_costs[s - 1]);
            descs.push_back(d);
        }
        // the estimator keeps the post-filtered distance only: no filtered level-0 guide
        add_step(false, false, 1, SSG_STORAGE_F32, descs, s > 0);
    }

    // --- stitch jobs: maps concatenated job by job
    int64_t maps = 0;
    for (int j = 0; j < job_count; ++j) {
        const ssg_uneven_job& in = jobs[j];
        StitchJob s{};
        s.cols = in.cols;
        s.rows = in.rows;
        s.references = in.references;
        s.pano_cols = in.pano_cols;
        s.pano_rows = in.pano_rows;
        s.image_cols = in.image_cols;
        s.image_rows = in.image_rows;
        s.map_begin = (int)maps;
        s.ratio_x = (float)in.image_cols / (float)in.cols;
        s.ratio_y = (float)in.image_rows / (float)in.rows;
        s.distance = in.d_distance;
        s.tables = in.d_tables;
        s.lut = reinterpret_cast<const float2*>(in.d_lut);
        s.weights = in.d_weights;
        s.images = in.d_images;
        s.word_rows = ((uintptr_t)in.d_images & 3) == 0 &&
                      (((int64_t)in.references * in.image_rows * in.image_cols * 3) & 3) == 0;
        s.pano_distance = in.d_pano_distance;
        s.rgb = in.d_rgb;
        for (int r = 0; r < in.references; ++r) {
            s.k[r] = to_intr(in.intrinsics[r]);
            std::memcpy(s.t[r], in.translations + 3 * r, sizeof(float) * 3);
        }
        const int64_t P = (int64_t)in.cols * in.rows;
        maps += P * in.references;
        b->max_references = std::max(b->max_references, in.references);
        b->max_map_pixels = (int)std::max<int64_t>(b->max_map_pixels, P);
        b->max_pano_pixels = (int)std::max<int64_t>(b->max_pano_pixels, (int64_t)in.pano_cols * in.pano_rows);
        b->jobs.push_back(s);
    }
    if (maps >= ((int64_t)1 << 31)) {
        delete b;
        return fail(SSG_ERR_UNSUPPORTED, "uneven batch of %lld map pixels is too large", (long long)maps);
    }
    b->total_map_pixels = maps;

    // --- layouts
    size_t off = 0;
    b->sweep_offset = off;
    off = align_up(off + sizeof(SweepInst) * b->sweep.size(), 256);
    b->levels_offset = off;
    for (Step& st : b->steps) st.offset = off + st.offset * sizeof(LevelDesc);
    off = align_up(off + sizeof(LevelDesc) * b->levels.size(), 256);
    b->jobs_offset = off;
    off = align_up(off + sizeof(StitchJob) * b->jobs.size(), 256);
    b->plan_bytes = off;
    size_t so = 256;  // the sweep's work counter
    b->maps_offset = so;
    so = align_up(so + sizeof(float) * (size_t)maps, 256);
    b->stamps_offset = so;
    so = align_up(so + (size_t)maps, 256);
    b->holes_offset = so;
    so = align_up(so + sizeof(int32_t) * (3 * (size_t)maps + SSG_HOLE_SCRATCH_HEADER), 256);
    b->scratch_bytes = so;
    *plan_bytes = b->plan_bytes;
    *scratch_bytes = b->scratch_bytes;
    *out = b;
    return SSG_OK;
}

extern "C" int ssg_uneven_upload(ssg_uneven_batch* b, void* d_plan, void* d_scratch, void* stream)
{
    SSG_REQUIRE(b && d_plan && d_scratch, "null pointer");
    SSG_REQUIRE(((uintptr_t)d_plan & 255) == 0 && ((uintptr_t)d_scratch & 255) == 0,
                "plan and scratch must be 256-byte aligned");
    unsigned char* scratch = static_cast<unsigned char*>(d_scratch);
    for (StitchJob& j : b->jobs) j.reprojected = reinterpret_cast<float*>(scratch + b->maps_offset) + j.map_begin;
    cudaStream_t st = as_stream(stream);
    for (LevelDesc& d : b->levels) d.lut = range_table(d.var_inv_i, st);  // nullptr: evaluated per block
    std::vector<unsigned char> host(b->plan_bytes, 0);
    std::memcpy(host.data() + b->sweep_offset, b->sweep.data(), sizeof(SweepInst) * b->sweep.size());
    std::memcpy(host.data() + b->levels_offset, b->levels.data(), sizeof(LevelDesc) * b->levels.size());
    if (!b->jobs.empty())
        std::memcpy(host.data() + b->jobs_offset, b->jobs.data(), sizeof(StitchJob) * b->jobs.size());
    cudaError_t e = cudaMemcpyAsync(d_plan, host.data(), host.size(), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return fail(SSG_ERR_CUDA, "cudaMemcpyAsync(plan): %s", cudaGetErrorString(e));
    // the host buffer is released below: wait for the copy (set-up, outside any capture)
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(SSG_ERR_CUDA, "cudaStreamSynchronize: %s", cudaGetErrorString(e));
    b->d_plan = static_cast<unsigned char*>(d_plan);
    b->d_scratch = scratch;
    return SSG_OK;
}

extern "C" int ssg_uneven_run(const ssg_uneven_batch* b, void* stream)
{
    SSG_REQUIRE(b && b->d_plan && b->d_scratch, "the batch has not been uploaded");
    cudaStream_t st = as_stream(stream);
    const SweepInst* insts = reinterpret_cast<const SweepInst*>(b->d_plan + b->sweep_offset);
    if (int e = launch_sweep_uneven(insts, (int)b->sweep.size(), b->total_tiles, b->storage,
                                    reinterpret_cast<int*>(b->d_scratch), st))
        return e;
    for (const Step& s : b->steps) {
        const LevelDesc* d = reinterpret_cast<const LevelDesc*>(b->d_plan + s.offset);
        const int e = s.down ? launch_down_uneven(d, s.count, s.rows, s.cols, s.width, s.storage, st)
                             : launch_up_uneven(d, s.count, s.rows, s.cols, s.width, s.storage, s.select, s.guide, st);
        if (e) return e;
    }
    if (b->jobs.empty()) return SSG_OK;
    return launch_stitch_uneven(reinterpret_cast<const StitchJob*>(b->d_plan + b->jobs_offset), (int)b->jobs.size(),
                                reinterpret_cast<float*>(b->d_scratch + b->maps_offset), b->total_map_pixels,
                                b->max_map_pixels, b->max_pano_pixels, b->max_references, b->max_dist, b->iterations,
                                b->d_scratch + b->stamps_offset,
                                reinterpret_cast<int32_t*>(b->d_scratch + b->holes_offset), st);
}

extern "C" int ssg_uneven_launches(const ssg_uneven_batch* b)
{
    if (!b) return 0;
    const int stitch = b->jobs.empty() ? 0 : 3 + (b->iterations > 0 ? 1 + b->iterations : 0);
    return 1 + (int)b->steps.size() + stitch;
}

extern "C" void ssg_uneven_destroy(ssg_uneven_batch* b) { delete b; }
