// ISB multiscale edge-aware cost filter (python/isb_filter.cu, python/isb_filter.py) and the
// distance selection of python/depth_estimation.py:179-198, for one cost volume in the reference's
// planar layout [candidates][rows][cols] and for batches of volumes in the chunked layout of
// ssg_cells.cuh.
//
// Both layouts run the same kernels, templated on the cell width W (1 = planar, 8 = chunked):
//   - downsampling: one thread per coarse pixel; its 3x3 range weights are computed once from the
//     uint8 guides and shared by all candidates;
//   - upsampling: one thread per fine pixel, with the coarse neighbourhood of a block staged in
//     shared memory per chunk of candidates;
//   - the last upsampling step can be fused with the selection, so that the filtered level-0
//     volume is never written.
// Guides, range weights and cost sums use the reference's arithmetic in its order
// (ssg_isb_common.cuh), so both layouts give the same bits; the batched path differs from the
// reference only by the 16-bit rounding of its level-0 volume.
#include <cmath>

#include "ssg_cells.cuh"
#include "ssg_isb_common.cuh"

namespace ssg {

// ---------------------------------------------------------------------------------------------
// ISB filter on the chunked layout. Guides and range weights come from the same device functions
// as the fp32 path (ssg_isb_common.cuh), so the guide pyramid is bit-identical to it: the uint8
// truncation of the filtered guide turns a one-ulp change of a weight into a step of one grey
// level on a sizeable share of coarse pixels, which then moves the argmin. The costs are summed
// in the fp32 path's order as well; the level-0 rounding is the only difference.
// ---------------------------------------------------------------------------------------------
struct LevelGeom {
    int rows_in, cols_in, rows_out, cols_out;
};

// Downsampling, one thread per coarse pixel; level 0 (any storage) or a float32 level in,
// float32 out.
template <int W, typename Tin>
__global__ void __launch_bounds__(kBatchBlock) isb_down_kernel(const uint8_t* __restrict__ guide_in,
                                                                   const Tin* __restrict__ cost_in,
                                                                   uint8_t* __restrict__ guide_out,
                                                                   float* __restrict__ cost_out, LevelGeom g,
                                                                   int chunks, float var_inv_i)
{
    const int64_t pin = (int64_t)g.rows_in * g.cols_in, pout = (int64_t)g.rows_out * g.cols_out;
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= pout) return;
    const int inst = blockIdx.y;
    guide_in += (int64_t)inst * pin * 3;
    guide_out += (int64_t)inst * pout * 3;
    cost_in += (int64_t)inst * chunks * pin * W;
    cost_out += (int64_t)inst * chunks * pout * W;
    DownTapsT<int> t;
    down_weights(guide_in, g.rows_in, g.cols_in, (int)(o % g.cols_out), (int)(o / g.cols_out), var_inv_i,
                 guide_out + 3 * o, t);
    for (int c = 0; c < chunks; ++c) {
        const Tin* src = cost_in + (int64_t)c * pin * W;
        float acc[W];
        CellIO<W, Tin>::load(src + (int64_t)t.centre * W, acc);
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            float v[W];
            CellIO<W, Tin>::load(src + (int64_t)t.idx[i] * W, v);
#pragma unroll
            for (int j = 0; j < W; ++j) acc[j] = fadd(acc[j], fmul(v[j], t.w[i]));
        }
#pragma unroll
        for (int j = 0; j < W; ++j) acc[j] = fdiv(acc[j], t.wsum);
        CellIO<W, float>::store(cost_out + ((int64_t)c * pout + o) * W, acc);
    }
}

// ---------------------------------------------------------------------------------------------
// Upsampling, one thread per fine pixel.  A block covers kUpTileX coarse pixels of one coarse
// row: warp w takes fine pixel F = w % 4 (UpTaps<F>) of coarse pixels 32 * (w / 4) + lane, so
// that all lanes of a warp follow one tap list.  The coarse costs of the block's 3 x (kUpTileX + 2)
// neighbourhood (edge-clamped, as the taps are) are staged per chunk in shared memory with
// cp.async, double-buffered: each coarse cell is read from memory once per block instead of
// once per tap, and the next chunk streams in while this one is filtered.
// ---------------------------------------------------------------------------------------------
constexpr int kUpTileX = kBatchBlock / 4;
constexpr int kUpTileCols = kUpTileX + 2;

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem));
}
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_one() { asm volatile("cp.async.wait_group 1;\n" ::); }

// Tile of one chunk: [part][row 0..2][col 0..kUpTileCols-1] with parts of 4 floats (W = 8: two
// parts, float4 elements) or one part of single floats (W = 1).
template <int W>
struct UpTile {
    static constexpr int parts = W == 8 ? 2 : 1;
    static constexpr int elem = W == 8 ? 4 : 1;
    static constexpr int floats = parts * 3 * kUpTileCols * elem;
};

template <int W>
__device__ __forceinline__ void load_tile_async(float* __restrict__ buf, const float* __restrict__ chunk,
                                                int rows_in, int cols_in, int x0, int y)
{
    constexpr int cells = 3 * kUpTileCols;
    for (int e = threadIdx.x; e < UpTile<W>::parts * cells; e += blockDim.x) {
        const int part = e / cells, rc = e % cells;
        const int row = rc / kUpTileCols, col = rc % kUpTileCols;
        const int gx = min(max(x0 - 1 + col, 0), cols_in - 1), gy = min(max(y - 1 + row, 0), rows_in - 1);
        const float* src = chunk + ((int64_t)gy * cols_in + gx) * W + part * 4;
        if constexpr (W == 8)
            cp_async16(buf + e * 4, src);
        else
            cp_async4(buf + e, src);
    }
}

// coarse tap (row a, col b) of local coarse column lx, all W candidates
template <int W>
__device__ __forceinline__ void tile_tap(const float* __restrict__ buf, int a, int b, int lx, float v[W])
{
    const int cell = a * kUpTileCols + lx + b;
    if constexpr (W == 8) {
        const float4 lo = reinterpret_cast<const float4*>(buf)[cell];
        const float4 hi = reinterpret_cast<const float4*>(buf)[3 * kUpTileCols + cell];
        v[0] = lo.x; v[1] = lo.y; v[2] = lo.z; v[3] = lo.w;
        v[4] = hi.x; v[5] = hi.y; v[6] = hi.z; v[7] = hi.w;
    } else {
        v[0] = buf[cell];
    }
}

// filtered costs of fine pixel F (the arithmetic and order of up_costs)
template <int F, int W>
__device__ __forceinline__ void tile_filter(const float* __restrict__ buf, int lx, const float (&w)[9], float inv,
                                            float weight_up, float acc[W])
{
#pragma unroll
    for (int j = 0; j < W; ++j) acc[j] = fmul(weight_up, acc[j]);
#pragma unroll
    for (int i = 0; i < UpTaps<F>::n; ++i) {
        const int t = UpTaps<F>::tap(i);
        float v[W];
        tile_tap<W>(buf, t / 3, t % 3, lx, v);
#pragma unroll
        for (int j = 0; j < W; ++j) acc[j] = fadd(acc[j], fmul(w[i], v[j]));
    }
#pragma unroll
    for (int j = 0; j < W; ++j) acc[j] = fmul(acc[j], inv);
}

template <int F>
__device__ __forceinline__ float fine_weights_padded(const float (&gd)[9][3], const float up[3], float weight_up,
                                                     float weight_down, float var_inv_i, float (&w)[9], float g[3])
{
    float wf[UpTaps<F>::n];
    const float inv = fine_weights<F>(gd, up, weight_up, weight_down, var_inv_i, wf, g);
#pragma unroll
    for (int i = 0; i < 9; ++i) w[i] = i < UpTaps<F>::n ? wf[i < UpTaps<F>::n ? i : 0] : 0.0f;  // (no dead-branch index past n)
    return inv;
}

struct SelectOut {
    float d0, dl, q;
    float* distance;
    int32_t* index;
    bool write_guide;  // the selecting step also writes the filtered level-0 guide
};

// kSelect = false: coarse float32 -> fine float32 in place (and the fine guide);
// kSelect = true: the last step, fine level-0 costs of type Tf in, the selection out.
template <int W, typename Tf, bool kSelect>
__global__ void __launch_bounds__(kBatchBlock) isb_up_kernel(const uint8_t* __restrict__ guide_in,
                                                                 const float* __restrict__ cost_in,
                                                                 uint8_t* __restrict__ guide_io,
                                                                 Tf* __restrict__ cost_fine, LevelGeom g, int chunks,
                                                                 int ncand, float weight_up, float weight_down,
                                                                 float var_inv_i, SelectOut so)
{
    __shared__ __align__(16) float tile[2][UpTile<W>::floats];
    const int64_t pin = (int64_t)g.rows_in * g.cols_in, pio = (int64_t)g.rows_out * g.cols_out;
    const int inst = blockIdx.z, y = blockIdx.y, x0 = blockIdx.x * kUpTileX;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int F = warp & 3;
    const int lx = (warp >> 2) * 32 + lane, x = x0 + lx;
    guide_in += (int64_t)inst * pin * 3;
    guide_io += (int64_t)inst * pio * 3;
    cost_in += (int64_t)inst * chunks * pin * W;
    cost_fine += (int64_t)inst * chunks * pio * W;
    const int fx = 2 * x + (F >= 2 ? 1 : 0), fy = 2 * y + (F & 1);
    // a fine pixel outside the level is the clamped duplicate of another one and is skipped
    const bool active = x < g.cols_in && fx < g.cols_out && fy < g.rows_out;
    const int fi = fy * g.cols_out + fx;
    float w[9], inv = 0.0f;
    if (active) {
        int ci[9];
        float gd[9][3], up[3], gsum[3];
        coarse_neighbourhood(guide_in, g.rows_in, g.cols_in, x, y, ci, gd);
        load_guide(guide_io, fi, up);
        switch (F) {
            case 0: inv = fine_weights_padded<0>(gd, up, weight_up, weight_down, var_inv_i, w, gsum); break;
            case 1: inv = fine_weights_padded<1>(gd, up, weight_up, weight_down, var_inv_i, w, gsum); break;
            case 2: inv = fine_weights_padded<2>(gd, up, weight_up, weight_down, var_inv_i, w, gsum); break;
            default: inv = fine_weights_padded<3>(gd, up, weight_up, weight_down, var_inv_i, w, gsum); break;
        }
        if (!kSelect || so.write_guide)
#pragma unroll
            for (int ch = 0; ch < 3; ++ch) guide_io[3 * fi + ch] = (uint8_t)__float2uint_rz(fmul(gsum[ch], inv));
    }
    Selector s;
    load_tile_async<W>(tile[0], cost_in, g.rows_in, g.cols_in, x0, y);
    cp_async_commit();
    for (int c = 0; c < chunks; ++c) {
        if (c + 1 < chunks)
            load_tile_async<W>(tile[(c + 1) & 1], cost_in + (int64_t)(c + 1) * pin * W, g.rows_in, g.cols_in, x0, y);
        cp_async_commit();
        cp_async_wait_one();  // this chunk's tile has landed
        __syncthreads();
        if (active) {
            Tf* fc = cost_fine + ((int64_t)c * pio + fi) * W;
            const float* buf = tile[c & 1];
            float acc[W];
            CellIO<W, Tf>::load(fc, acc);
            switch (F) {
                case 0: tile_filter<0, W>(buf, lx, w, inv, weight_up, acc); break;
                case 1: tile_filter<1, W>(buf, lx, w, inv, weight_up, acc); break;
                case 2: tile_filter<2, W>(buf, lx, w, inv, weight_up, acc); break;
                default: tile_filter<3, W>(buf, lx, w, inv, weight_up, acc); break;
            }
            if constexpr (kSelect) {
#pragma unroll
                for (int j = 0; j < W; ++j)
                    if (c * W + j < ncand) s.push(c * W + j, acc[j]);
            } else {
                CellIO<W, float>::store(reinterpret_cast<float*>(fc), acc);
            }
        }
        __syncthreads();  // the tile is refilled two chunks on
    }
    if constexpr (kSelect) {
        if (active) {
            so.distance[(int64_t)inst * pio + fi] = select_from(s, ncand, so.d0, so.dl, so.q);
            if (so.index) so.index[(int64_t)inst * pio + fi] = s.idx;
        }
    }
}

// Selection from an unfiltered level-0 volume (pyramids of fewer than two levels, or the
// reference's own select_distance on a filtered planar volume)
template <int W, typename T>
__global__ void __launch_bounds__(kBatchBlock) select_kernel(const T* __restrict__ cost, int64_t P, int chunks,
                                                            int ncand, float d0, float dl, float q,
                                                            float* __restrict__ distance,
                                                            int32_t* __restrict__ index)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    const int inst = blockIdx.y;
    cost += (int64_t)inst * chunks * P * W;
    Selector s;
    for (int c = 0; c < chunks; ++c) {
        float v[W];
        CellIO<W, T>::load(cost + ((int64_t)c * P + i) * W, v);
#pragma unroll
        for (int j = 0; j < W; ++j)
            if (c * W + j < ncand) s.push(c * W + j, v[j]);
    }
    distance[(int64_t)inst * P + i] = select_from(s, ncand, d0, dl, q);
    if (index) index[(int64_t)inst * P + i] = s.idx;
}

static int chunks_of(int n) { return (n + 7) / 8; }

// blocks of kUpTileX coarse pixels of one coarse row, per instance
static dim3 up_grid(int cols_in, int rows_in, int instances)
{
    return dim3((unsigned)((cols_in + kUpTileX - 1) / kUpTileX), (unsigned)rows_in, (unsigned)instances);
}

static int level_rows(int rows, int s) { return (int)std::ceil(rows / std::pow(2.0, s)); }

struct Levels {
    float var_inv_i;
    float weight_up[SSG_MAX_LEVELS], weight_down[SSG_MAX_LEVELS];
};

// python/isb_filter.py:87-88, :110-112 in double, rounded to float32 as cupy.float32 does
static Levels isb_constants(int level_count, double sigma_i, double sigma_s)
{
    Levels l{};
    const double vs = 1 / (2 * sigma_s * sigma_s), vi = 1 / (2 * sigma_i * sigma_i);
    l.var_inv_i = (float)vi;
    for (int s = 0; s + 1 < level_count; ++s) {
        const double dist = std::pow(2.0, s) - 0.5;
        const double wd = std::exp(-(dist * dist) * vs);
        l.weight_down[s] = (float)wd;
        l.weight_up[s] = (float)(1 - wd);
    }
    return l;
}

// (candidates[0] / candidates[-1] - 1) in float32, depth_estimation.py:195-196
static SelectOut select_constants(const float* candidates, int ncand, float* distance, int32_t* index,
                                  bool write_guide)
{
    const float d0 = candidates[0], dl = candidates[ncand - 1];
    return SelectOut{d0, dl, d0 / dl - 1.0f, distance, index, write_guide};
}

static int check_levels(int rows_in, int cols_in, int rows_out, int cols_out)
{
    SSG_REQUIRE(rows_in > 0 && cols_in > 0 && rows_out > 0 && cols_out > 0, "sizes must be positive");
    SSG_REQUIRE((int64_t)rows_in * cols_in < ((int64_t)1 << 31) && rows_in <= 65535 && rows_out <= 65535,
                "a level of %dx%d pixels is too large", rows_in, cols_in);
    SSG_REQUIRE(2 * (rows_out - 1) < rows_in && 2 * (cols_out - 1) < cols_in && (rows_in + 1) / 2 <= rows_out &&
                    (cols_in + 1) / 2 <= cols_out,
                "level %dx%d is not the 2x downsampling of %dx%d", rows_out, cols_out, rows_in, cols_in);
    return SSG_OK;
}

// --- launches shared by both layouts ---------------------------------------------------------
template <int W, typename Tin>
static int launch_down(const uint8_t* gi, const Tin* ci, int ri, int cl_i, uint8_t* go, float* co, int ro, int cl_o,
                       int chunks, int instances, float var_inv_i, cudaStream_t st)
{
    const LevelGeom g{ri, cl_i, ro, cl_o};
    const dim3 grid(grid_1d((int64_t)ro * cl_o, kBatchBlock), instances);
    isb_down_kernel<W, Tin><<<grid, kBatchBlock, 0, st>>>(gi, ci, go, co, g, chunks, var_inv_i);
    return launch_status("isb_down_kernel");
}

template <int W, typename Tf, bool kSelect>
static int launch_up(const uint8_t* gi, const float* ci, int rc, int cc, uint8_t* gio, Tf* cf, int rf, int cf_cols,
                     int chunks, int ncand, int instances, float wu, float wd, float var_inv_i, const SelectOut& so,
                     cudaStream_t st)
{
    const LevelGeom g{rc, cc, rf, cf_cols};
    isb_up_kernel<W, Tf, kSelect><<<up_grid(cc, rc, instances), kBatchBlock, 0, st>>>(gi, ci, gio, cf, g, chunks,
                                                                                      ncand, wu, wd, var_inv_i, so);
    return launch_status(kSelect ? "isb_up_kernel<select>" : "isb_up_kernel");
}

// the whole filter on planar levels (W = 1, chunks = candidates): python/isb_filter.py:72-136
static int apply_planar(uint8_t* const* d_guides, float* const* d_costs, int level_count, int rows, int cols,
                        int candidate_count, int instances, double sigma_i, double sigma_s, cudaStream_t st)
{
    const Levels c = isb_constants(level_count, sigma_i, sigma_s);
    for (int s = 1; s < level_count; ++s) {
        const int ri = level_rows(rows, s - 1), ci = level_rows(cols, s - 1), ro = level_rows(rows, s),
                  co = level_rows(cols, s);
        if (int e = check_levels(ri, ci, ro, co)) return e;
        if (int e = launch_down<1, float>(d_guides[s - 1], d_costs[s - 1], ri, ci, d_guides[s], d_costs[s], ro, co,
                                          candidate_count, instances, c.var_inv_i, st))
            return e;
    }
    for (int s = level_count - 2; s >= 0; --s) {
        const int rc = level_rows(rows, s + 1), cc = level_rows(cols, s + 1), rf = level_rows(rows, s),
                  cf = level_rows(cols, s);
        if (int e = launch_up<1, float, false>(d_guides[s + 1], d_costs[s + 1], rc, cc, d_guides[s], d_costs[s], rf, cf,
                                               candidate_count, candidate_count, instances, c.weight_up[s],
                                               c.weight_down[s], c.var_inv_i, SelectOut{}, st))
            return e;
    }
    return SSG_OK;
}

static int check_apply_args(uint8_t* const* d_guides, float* const* d_costs, int level_count, int rows, int cols,
                            int candidate_count, double sigma_i, double sigma_s)
{
    SSG_REQUIRE(d_guides && d_costs, "null level arrays");
    const int expected = cols > 0 && rows > 0 ? (int)(std::fmin(std::log2((double)cols), std::log2((double)rows)) - 1) : 0;
    SSG_REQUIRE(level_count == expected, "level_count %d differs from the pyramid of a %dx%d image (%d)", level_count,
                cols, rows, expected);
    SSG_REQUIRE(level_count <= SSG_MAX_LEVELS, "too many levels");
    SSG_REQUIRE(candidate_count >= 1 && candidate_count <= 65535, "candidate_count out of range");
    SSG_REQUIRE(sigma_i > 0 && sigma_s > 0, "sigmas must be positive");
    for (int s = 0; s < level_count; ++s) SSG_REQUIRE(d_guides[s] && d_costs[s], "level %d is NULL", s);
    return SSG_OK;
}

}  // namespace ssg

using namespace ssg;

// ---------------------------------------------------------------------------------------------
// One planar volume, the reference's layout (python/isb_filter.py, depth_estimation.py:179-198)
// ---------------------------------------------------------------------------------------------
extern "C" int ssg_isb_level_count(int cols, int rows)
{
    if (cols <= 0 || rows <= 0) return 0;
    return (int)(std::fmin(std::log2((double)cols), std::log2((double)rows)) - 1);
}

extern "C" int ssg_isb_downsample(const uint8_t* d_guide_in, const float* d_cost_in, int rows_in, int cols_in,
                                  uint8_t* d_guide_out, float* d_cost_out, int rows_out, int cols_out,
                                  int candidate_count, float var_inv_i, void* stream)
{
    SSG_REQUIRE(d_guide_in && d_cost_in && d_guide_out && d_cost_out, "null device pointer");
    if (int e = check_levels(rows_in, cols_in, rows_out, cols_out)) return e;
    SSG_REQUIRE(candidate_count >= 1, "candidate_count must be positive");
    return launch_down<1, float>(d_guide_in, d_cost_in, rows_in, cols_in, d_guide_out, d_cost_out, rows_out, cols_out,
                                 candidate_count, 1, var_inv_i, as_stream(stream));
}

extern "C" int ssg_isb_upsample(const uint8_t* d_guide_in, const float* d_cost_in, int rows_in, int cols_in,
                                uint8_t* d_guide_inout, float* d_cost_inout, int rows_inout, int cols_inout,
                                int candidate_count, float weight_up, float weight_down, float var_inv_i,
                                void* stream)
{
    SSG_REQUIRE(d_guide_in && d_cost_in && d_guide_inout && d_cost_inout, "null device pointer");
    if (int e = check_levels(rows_inout, cols_inout, rows_in, cols_in)) return e;
    SSG_REQUIRE(candidate_count >= 1, "candidate_count must be positive");
    return launch_up<1, float, false>(d_guide_in, d_cost_in, rows_in, cols_in, d_guide_inout, d_cost_inout,
                                      rows_inout, cols_inout, candidate_count, candidate_count, 1, weight_up,
                                      weight_down, var_inv_i, SelectOut{}, as_stream(stream));
}

extern "C" int ssg_isb_apply(uint8_t* const* d_guides, float* const* d_costs, int level_count, int rows, int cols,
                             int candidate_count, double sigma_i, double sigma_s, void* stream)
{
    if (int e = check_apply_args(d_guides, d_costs, level_count, rows, cols, candidate_count, sigma_i, sigma_s))
        return e;
    return apply_planar(d_guides, d_costs, level_count, rows, cols, candidate_count, 1, sigma_i, sigma_s,
                        as_stream(stream));
}

extern "C" int ssg_isb_apply_batch(uint8_t* const* d_guides, float* const* d_costs, int level_count, int rows,
                                   int cols, int candidate_count, int instances, double sigma_i, double sigma_s,
                                   void* stream)
{
    if (int e = check_apply_args(d_guides, d_costs, level_count, rows, cols, candidate_count, sigma_i, sigma_s))
        return e;
    SSG_REQUIRE(instances >= 1 && instances <= 65535, "instances out of range");
    return apply_planar(d_guides, d_costs, level_count, rows, cols, candidate_count, instances, sigma_i, sigma_s,
                        as_stream(stream));
}

extern "C" int ssg_select_distance(const float* d_cost, int candidate_count, int64_t pixels, const float* candidates,
                                   float* d_distance, int32_t* d_index, void* stream)
{
    SSG_REQUIRE(d_cost && d_distance && candidates, "null pointer");
    SSG_REQUIRE(candidate_count >= 1, "candidate_count must be positive");
    SSG_REQUIRE(pixels >= 0, "negative pixel count");
    if (pixels == 0) return SSG_OK;
    const SelectOut so = select_constants(candidates, candidate_count, d_distance, d_index, false);
    select_kernel<1, float><<<dim3(grid_1d(pixels, kBatchBlock), 1), kBatchBlock, 0, as_stream(stream)>>>(
        d_cost, pixels, candidate_count, candidate_count, so.d0, so.dl, so.q, d_distance, d_index);
    return launch_status("select_kernel");
}

extern "C" int ssg_isb_upsample_select(const uint8_t* d_guide_in, const float* d_cost_in, int rows_in, int cols_in,
                                       uint8_t* d_guide_inout, const float* d_cost_fine, int rows_fine, int cols_fine,
                                       int candidate_count, float weight_up, float weight_down, float var_inv_i,
                                       const float* candidates, float* d_distance, int32_t* d_index, void* stream)
{
    SSG_REQUIRE(d_guide_in && d_cost_in && d_guide_inout && d_cost_fine && d_distance && candidates,
                "null pointer");
    if (int e = check_levels(rows_fine, cols_fine, rows_in, cols_in)) return e;
    SSG_REQUIRE(candidate_count >= 1, "candidate_count must be positive");
    const SelectOut so = select_constants(candidates, candidate_count, d_distance, d_index, true);
    return launch_up<1, float, true>(d_guide_in, d_cost_in, rows_in, cols_in, d_guide_inout,
                                     const_cast<float*>(d_cost_fine), rows_fine, cols_fine, candidate_count,
                                     candidate_count, 1, weight_up, weight_down, var_inv_i, so, as_stream(stream));
}

// ---------------------------------------------------------------------------------------------
// Batches of chunked volumes (the batched path)
// ---------------------------------------------------------------------------------------------
extern "C" int ssg_isb_downsample_batch(const uint8_t* d_guide_in, const void* d_cost_in, int rows_in, int cols_in,
                                        uint8_t* d_guide_out, void* d_cost_out, int rows_out, int cols_out,
                                        int candidate_count, int instances, int storage, float var_inv_i,
                                        void* stream)
{
    SSG_REQUIRE(d_guide_in && d_cost_in && d_guide_out && d_cost_out, "null pointer");
    if (int e = check_levels(rows_in, cols_in, rows_out, cols_out)) return e;
    SSG_REQUIRE(storage == SSG_STORAGE_F16 || storage == SSG_STORAGE_UNORM16 || storage == SSG_STORAGE_F32,
                "unknown input storage %d", storage);
    SSG_REQUIRE(candidate_count >= 1 && candidate_count <= SSG_MAX_CANDIDATES, "candidate_count out of range");
    SSG_REQUIRE(instances >= 1 && instances <= 65535, "instances out of range");
    const int chunks = chunks_of(candidate_count);
    float* out = static_cast<float*>(d_cost_out);
    cudaStream_t st = as_stream(stream);
    if (storage == SSG_STORAGE_F16)
        return launch_down<8, __half>(d_guide_in, static_cast<const __half*>(d_cost_in), rows_in, cols_in, d_guide_out,
                                      out, rows_out, cols_out, chunks, instances, var_inv_i, st);
    if (storage == SSG_STORAGE_UNORM16)
        return launch_down<8, uint16_t>(d_guide_in, static_cast<const uint16_t*>(d_cost_in), rows_in, cols_in,
                                        d_guide_out, out, rows_out, cols_out, chunks, instances, var_inv_i, st);
    return launch_down<8, float>(d_guide_in, static_cast<const float*>(d_cost_in), rows_in, cols_in, d_guide_out, out,
                                 rows_out, cols_out, chunks, instances, var_inv_i, st);
}

extern "C" int ssg_isb_upsample_batch(const uint8_t* d_guide_in, const void* d_cost_in, int rows_in, int cols_in,
                                      uint8_t* d_guide_inout, void* d_cost_inout, int rows_inout, int cols_inout,
                                      int candidate_count, int instances, int storage, float weight_up,
                                      float weight_down, float var_inv_i, void* stream)
{
    SSG_REQUIRE(d_guide_in && d_cost_in && d_guide_inout && d_cost_inout, "null pointer");
    if (int e = check_levels(rows_inout, cols_inout, rows_in, cols_in)) return e;
    SSG_REQUIRE(storage == SSG_STORAGE_F32, "coarse levels are float32 (storage must be SSG_STORAGE_F32)");
    SSG_REQUIRE(candidate_count >= 1 && candidate_count <= SSG_MAX_CANDIDATES, "candidate_count out of range");
    SSG_REQUIRE(instances >= 1 && instances <= 65535, "instances out of range");
    const int chunks = chunks_of(candidate_count);
    return launch_up<8, float, false>(d_guide_in, static_cast<const float*>(d_cost_in), rows_in, cols_in,
                                      d_guide_inout, static_cast<float*>(d_cost_inout), rows_inout, cols_inout, chunks,
                                      chunks * 8, instances, weight_up, weight_down, var_inv_i, SelectOut{},
                                      as_stream(stream));
}

extern "C" int ssg_isb_upsample_select_batch(const uint8_t* d_guide_in, const void* d_cost_in, int rows_in,
                                             int cols_in, uint8_t* d_guide_inout, const void* d_cost_fine,
                                             int rows_fine, int cols_fine, int candidate_count, int instances,
                                             int storage, float weight_up, float weight_down, float var_inv_i,
                                             const float* candidates, float* d_distance, int32_t* d_index,
                                             void* stream)
{
    SSG_REQUIRE(d_guide_in && d_cost_in && d_guide_inout && d_cost_fine && d_distance && candidates, "null pointer");
    if (int e = check_levels(rows_fine, cols_fine, rows_in, cols_in)) return e;
    SSG_REQUIRE(storage == SSG_STORAGE_F16 || storage == SSG_STORAGE_UNORM16 || storage == SSG_STORAGE_F32,
                "unknown fine-level storage %d", storage);
    SSG_REQUIRE(candidate_count >= 1 && candidate_count <= SSG_MAX_CANDIDATES, "candidate_count out of range");
    SSG_REQUIRE(instances >= 1 && instances <= 65535, "instances out of range");
    const int chunks = chunks_of(candidate_count);
    // the level-0 guide is not needed after the selection and is left as it was
    const SelectOut so = select_constants(candidates, candidate_count, d_distance, d_index, false);
    const float* coarse = static_cast<const float*>(d_cost_in);
    void* fine = const_cast<void*>(d_cost_fine);  // read only in the selecting variant
    cudaStream_t st = as_stream(stream);
    if (storage == SSG_STORAGE_F16)
        return launch_up<8, __half, true>(d_guide_in, coarse, rows_in, cols_in, d_guide_inout,
                                          static_cast<__half*>(fine), rows_fine, cols_fine, chunks, candidate_count,
                                          instances, weight_up, weight_down, var_inv_i, so, st);
    if (storage == SSG_STORAGE_UNORM16)
        return launch_up<8, uint16_t, true>(d_guide_in, coarse, rows_in, cols_in, d_guide_inout,
                                            static_cast<uint16_t*>(fine), rows_fine, cols_fine, chunks,
                                            candidate_count, instances, weight_up, weight_down, var_inv_i, so, st);
    return launch_up<8, float, true>(d_guide_in, coarse, rows_in, cols_in, d_guide_inout, static_cast<float*>(fine),
                                     rows_fine, cols_fine, chunks, candidate_count, instances, weight_up, weight_down,
                                     var_inv_i, so, st);
}

extern "C" int ssg_select_distance_batch(const void* d_cost, int candidate_count, int64_t pixels, int instances,
                                         int storage, const float* candidates, float* d_distance, int32_t* d_index,
                                         void* stream)
{
    SSG_REQUIRE(d_cost && d_distance && candidates, "null pointer");
    SSG_REQUIRE(pixels > 0 && instances >= 1 && instances <= 65535, "invalid sizes");
    SSG_REQUIRE(candidate_count >= 1 && candidate_count <= SSG_MAX_CANDIDATES, "candidate_count out of range");
    SSG_REQUIRE(storage == SSG_STORAGE_F16 || storage == SSG_STORAGE_UNORM16 || storage == SSG_STORAGE_F32,
                "unknown storage %d", storage);
    const SelectOut so = select_constants(candidates, candidate_count, d_distance, d_index, false);
    const dim3 grid(grid_1d(pixels, kBatchBlock), instances);
    const int chunks = chunks_of(candidate_count);
    cudaStream_t st = as_stream(stream);
    if (storage == SSG_STORAGE_F16)
        select_kernel<8, __half><<<grid, kBatchBlock, 0, st>>>(static_cast<const __half*>(d_cost), pixels, chunks,
                                                               candidate_count, so.d0, so.dl, so.q, d_distance, d_index);
    else if (storage == SSG_STORAGE_UNORM16)
        select_kernel<8, uint16_t><<<grid, kBatchBlock, 0, st>>>(static_cast<const uint16_t*>(d_cost), pixels, chunks,
                                                                 candidate_count, so.d0, so.dl, so.q, d_distance,
                                                                 d_index);
    else
        select_kernel<8, float><<<grid, kBatchBlock, 0, st>>>(static_cast<const float*>(d_cost), pixels, chunks,
                                                              candidate_count, so.d0, so.dl, so.q, d_distance, d_index);
    return launch_status("select_kernel");
}
