// ISB multiscale edge-aware cost filter (python/isb_filter.cu, python/isb_filter.py) and the
// distance selection of python/depth_estimation.py:179-198, fp32 planar cost volumes
// [candidates][rows][cols] as the reference's API has them.
//
// One thread per coarse pixel, as in the reference: the range weights of its 3x3 neighbourhood
// are computed once from the uint8 guides and shared by all candidates.  Consecutive threads
// touch consecutive pixels of each candidate plane, so loads and stores coalesce.  Arithmetic
// is the reference's, in its order, with the exponential of ssg_common.cuh.
#include <cmath>

#include "ssg_common.cuh"

namespace ssg {

constexpr int kIsbBlock = 256;
constexpr float kIsbEps = 0.01f;  // isb_filter.cu:32

__device__ __forceinline__ float range_weight(float d, float var_inv_i)
{
    // __expf(-diff * diff * varInvI) + EPS  (isb_filter.cu:87, :229)
    return fadd(cw_expf(fmul(fmul(-d, d), var_inv_i)), kIsbEps);
}

__device__ __forceinline__ float abs_sum(const float a[3], const float b[3])
{
    return fadd(fadd(fabsf(fsub(a[0], b[0])), fabsf(fsub(a[1], b[1]))), fabsf(fsub(a[2], b[2])));
}

__device__ __forceinline__ void load_guide(const uint8_t* __restrict__ g, int64_t idx, float out[3])
{
    out[0] = (float)g[3 * idx];
    out[1] = (float)g[3 * idx + 1];
    out[2] = (float)g[3 * idx + 2];
}

// guideDownsample2xKernel, isb_filter.cu:44-119
__global__ void __launch_bounds__(kIsbBlock) isb_down_kernel(const uint8_t* __restrict__ guide_in,
                                                             const float* __restrict__ cost_in, int rows_in,
                                                             int cols_in, uint8_t* __restrict__ guide_out,
                                                             float* __restrict__ cost_out, int rows_out,
                                                             int cols_out, int ncand, float var_inv_i)
{
    const int64_t pout = (int64_t)rows_out * cols_out, pin = (int64_t)rows_in * cols_in;
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= pout) return;
    // blockIdx.y: instance of a batch of equally sized, contiguous levels
    guide_in += (int64_t)blockIdx.y * pin * 3;
    guide_out += (int64_t)blockIdx.y * pout * 3;
    cost_in += (int64_t)blockIdx.y * ncand * pin;
    cost_out += (int64_t)blockIdx.y * ncand * pout;
    const int x = (int)(o % cols_out), y = (int)(o / cols_out);
    const int x2 = 2 * x, y2 = 2 * y;
    const int px = min(x2 + 1, cols_in - 1), py = min(y2 + 1, rows_in - 1);
    const int mx = max(x2 - 1, 0), my = max(y2 - 1, 0);
    const int64_t idx[8] = {(int64_t)my * cols_in + mx, (int64_t)y2 * cols_in + mx, (int64_t)py * cols_in + mx,
                            (int64_t)py * cols_in + x2, (int64_t)py * cols_in + px, (int64_t)y2 * cols_in + px,
                            (int64_t)my * cols_in + px, (int64_t)my * cols_in + x2};
    const int64_t ic = (int64_t)y2 * cols_in + x2;
    float cur[3];
    load_guide(guide_in, ic, cur);
    float w[8] = {0.25f, 0.5f, 0.25f, 0.5f, 0.25f, 0.5f, 0.25f, 0.5f};
    float wsum = 1.0f, g[3] = {cur[0], cur[1], cur[2]};
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        float nb[3];
        load_guide(guide_in, idx[i], nb);
        w[i] = fmul(w[i], range_weight(abs_sum(cur, nb), var_inv_i));
        wsum = fadd(wsum, w[i]);
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) g[ch] = fadd(g[ch], fmul(nb[ch], w[i]));
    }
    const float den = fdiv(1.0f, wsum);
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) guide_out[3 * o + ch] = (uint8_t)__float2uint_rz(fmul(g[ch], den));
    for (int z = 0; z < ncand; ++z) {
        const float* c = cost_in + (int64_t)z * pin;
        float s = __ldg(c + ic);
#pragma unroll
        for (int i = 0; i < 8; ++i) s = fadd(s, fmul(__ldg(c + idx[i]), w[i]));
        cost_out[(int64_t)z * pout + o] = fdiv(s, wsum);
    }
}

// Weights of the four fine pixels of one coarse pixel (isb_filter.cu:142-267): taps index the
// 3x3 coarse neighbourhood [row][col] flattened as 3 * row + col.
struct UpWeights {
    float w1[9], w2[6], w3[6], w4[4];
    float inv[4];
    int64_t cidx[9];
    int64_t fidx[4];
    bool set[4];
};

// Tap lists of the fine pixels below, right and below-right (isb_filter.cu:185-208), as indices
// into the flattened 3x3 neighbourhood; written out so that every index is a compile-time
// constant and the neighbourhood stays in registers.
#define SSG_TAPS2(a) {a[4], a[7], a[3], a[6], a[5], a[8]}  // (1,1),(2,1),(1,0),(2,0),(1,2),(2,2)
#define SSG_TAPS3(a) {a[4], a[5], a[1], a[2], a[7], a[8]}  // (1,1),(1,2),(0,1),(0,2),(2,1),(2,2)
#define SSG_TAPS4(a) {a[4], a[5], a[7], a[8]}              // (1,1),(1,2),(2,1),(2,2)

__device__ __forceinline__ void up_weights(const uint8_t* __restrict__ guide_in, int rows_in, int cols_in,
                                           uint8_t* __restrict__ guide_io, int rows_io, int cols_io, int x, int y,
                                           float weight_up, float weight_down, float var_inv_i, UpWeights& u)
{
    const int mdx = max(x - 1, 0), mdy = max(y - 1, 0);
    const int pdx = min(x + 1, cols_in - 1), pdy = min(y + 1, rows_in - 1);
    const int x2 = 2 * x, y2 = 2 * y;
    const int pux = min(x2 + 1, cols_io - 1), puy = min(y2 + 1, rows_io - 1);
    const int rr[3] = {mdy, y, pdy}, cc[3] = {mdx, x, pdx};
    float gd[9][3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            u.cidx[3 * a + b] = (int64_t)rr[a] * cols_in + cc[b];
            load_guide(guide_in, u.cidx[3 * a + b], gd[3 * a + b]);
        }
    u.fidx[0] = (int64_t)y2 * cols_io + x2;
    u.fidx[1] = (int64_t)puy * cols_io + x2;
    u.fidx[2] = (int64_t)y2 * cols_io + pux;
    u.fidx[3] = (int64_t)puy * cols_io + pux;
    u.set[0] = true;
    u.set[1] = y2 != puy;
    u.set[2] = x2 != pux;
    u.set[3] = u.set[1] && u.set[2];
    float up[4][3];
#pragma unroll
    for (int f = 0; f < 4; ++f) load_guide(guide_io, u.fidx[f], up[f]);
    const float b1[9] = {1, 1, 1, 1, 8, 1, 1, 1, 1};
    const float b23[6] = {8, 8, 1, 1, 1, 1};
    float g[4][3], ws[4];
#pragma unroll
    for (int f = 0; f < 4; ++f) {
        ws[f] = weight_up;
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) g[f][ch] = fmul(weight_up, up[f][ch]);
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const float* nb = gd[i];
        u.w1[i] = fmul(b1[i], fmul(weight_down, range_weight(abs_sum(nb, up[0]), var_inv_i)));
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) g[0][ch] = fadd(g[0][ch], fmul(nb[ch], u.w1[i]));
        ws[0] = fadd(ws[0], u.w1[i]);
    }
    const float* g2[6] = SSG_TAPS2(gd);
    const float* g3[6] = SSG_TAPS3(gd);
    const float* g4[4] = SSG_TAPS4(gd);
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        const float* nb2 = g2[i];
        u.w2[i] = fmul(b23[i], fmul(weight_down, range_weight(abs_sum(nb2, up[1]), var_inv_i)));
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) g[1][ch] = fadd(g[1][ch], fmul(nb2[ch], u.w2[i]));
        ws[1] = fadd(ws[1], u.w2[i]);
        const float* nb3 = g3[i];
        u.w3[i] = fmul(b23[i], fmul(weight_down, range_weight(abs_sum(nb3, up[2]), var_inv_i)));
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) g[2][ch] = fadd(g[2][ch], fmul(nb3[ch], u.w3[i]));
        ws[2] = fadd(ws[2], u.w3[i]);
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float* nb = g4[i];
        u.w4[i] = fmul(weight_down, range_weight(abs_sum(nb, up[3]), var_inv_i));
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) g[3][ch] = fadd(g[3][ch], fmul(nb[ch], u.w4[i]));
        ws[3] = fadd(ws[3], u.w4[i]);
    }
#pragma unroll
    for (int f = 0; f < 4; ++f) {
        u.inv[f] = fdiv(1.0f, ws[f]);
        if (u.set[f])
#pragma unroll
            for (int ch = 0; ch < 3; ++ch)
                guide_io[3 * u.fidx[f] + ch] = (uint8_t)__float2uint_rz(fmul(g[f][ch], u.inv[f]));
    }
}

// Filtered fine costs of one candidate plane (isb_filter.cu:270-327)
__device__ __forceinline__ void up_costs(const UpWeights& u, const float* __restrict__ c,
                                         const float* __restrict__ fine, float weight_up, float out[4])
{
    float cd[9];
#pragma unroll
    for (int t = 0; t < 9; ++t) cd[t] = __ldg(c + u.cidx[t]);
    float s = fmul(weight_up, fine[u.fidx[0]]);
#pragma unroll
    for (int i = 0; i < 9; ++i) s = fadd(s, fmul(u.w1[i], cd[i]));
    out[0] = fmul(s, u.inv[0]);
    const float c2[6] = SSG_TAPS2(cd);
    const float c3[6] = SSG_TAPS3(cd);
    const float c4[4] = SSG_TAPS4(cd);
    if (u.set[1]) {
        s = fmul(weight_up, fine[u.fidx[1]]);
#pragma unroll
        for (int i = 0; i < 6; ++i) s = fadd(s, fmul(u.w2[i], c2[i]));
        out[1] = fmul(s, u.inv[1]);
    }
    if (u.set[2]) {
        s = fmul(weight_up, fine[u.fidx[2]]);
#pragma unroll
        for (int i = 0; i < 6; ++i) s = fadd(s, fmul(u.w3[i], c3[i]));
        out[2] = fmul(s, u.inv[2]);
    }
    if (u.set[3]) {
        s = fmul(weight_up, fine[u.fidx[3]]);
#pragma unroll
        for (int i = 0; i < 4; ++i) s = fadd(s, fmul(u.w4[i], c4[i]));
        out[3] = fmul(s, u.inv[3]);
    }
}

// guideUpsample2xKernel, isb_filter.cu:132-329
__global__ void __launch_bounds__(kIsbBlock) isb_up_kernel(const uint8_t* __restrict__ guide_in,
                                                           const float* __restrict__ cost_in, int rows_in,
                                                           int cols_in, uint8_t* __restrict__ guide_io,
                                                           float* __restrict__ cost_io, int rows_io, int cols_io,
                                                           int ncand, float weight_up, float weight_down,
                                                           float var_inv_i)
{
    const int64_t pin = (int64_t)rows_in * cols_in, pio = (int64_t)rows_io * cols_io;
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= pin) return;
    guide_in += (int64_t)blockIdx.y * pin * 3;
    guide_io += (int64_t)blockIdx.y * pio * 3;
    cost_in += (int64_t)blockIdx.y * ncand * pin;
    cost_io += (int64_t)blockIdx.y * ncand * pio;
    UpWeights u;
    up_weights(guide_in, rows_in, cols_in, guide_io, rows_io, cols_io, (int)(o % cols_in), (int)(o / cols_in),
               weight_up, weight_down, var_inv_i, u);
    for (int z = 0; z < ncand; ++z) {
        float* fine = cost_io + (int64_t)z * pio;
        float out[4];
        up_costs(u, cost_in + (int64_t)z * pin, fine, weight_up, out);
#pragma unroll
        for (int f = 0; f < 4; ++f)
            if (u.set[f]) fine[u.fidx[f]] = out[f];
    }
}

// Running argmin / max with the neighbours of the argmin (depth_estimation.py:180-187):
// the first minimum wins ties, as torch.min(dim) does.
struct Selector {
    float m, M, L, R, prev;
    int idx;
    bool need_right;
    __device__ __forceinline__ void push(int z, float c)
    {
        if (z == 0) {
            m = M = L = prev = c;
            idx = 0;
            need_right = true;
            return;
        }
        if (need_right) {
            R = c;
            need_right = false;
        }
        if (c < m) {
            m = c;
            idx = z;
            L = prev;
            need_right = true;
        }
        if (c > M) M = c;
        prev = c;
    }
};

// depth_estimation.py:188-198
__device__ __forceinline__ float select_from(Selector s, int ncand, float d0, float dl, float q)
{
    if (s.need_right) s.R = s.m;  // argmin at the last candidate: clamp(idx + 1) = idx
    float var = fdiv(fmul(0.5f, fsub(s.L, s.R)), fadd(fsub(fadd(s.L, s.R), fmul(2.0f, s.m)), 1e-8f));
    var = var < -0.5f ? -0.5f : (var > 0.5f ? 0.5f : var);
    if (s.idx == ncand - 1 || s.idx == 0) var = 0.0f;
    float sel = fadd((float)s.idx, var);
    if (s.M == s.m) sel = (float)(ncand - 1);
    float d = fdiv(d0, fadd(fdiv(fmul(q, sel), (float)(ncand - 1)), 1.0f));
    if (fabsf(fsub(s.M, s.m)) < 1e-8f) d = dl;
    return d;
}

__global__ void __launch_bounds__(kIsbBlock) select_distance_kernel(const float* __restrict__ cost, int ncand,
                                                                    int64_t P, float d0, float dl, float q,
                                                                    float* __restrict__ distance,
                                                                    int32_t* __restrict__ index)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    Selector s;
    for (int z = 0; z < ncand; ++z) s.push(z, __ldg(cost + (int64_t)z * P + i));
    distance[i] = select_from(s, ncand, d0, dl, q);
    if (index) index[i] = s.idx;
}

// Last upsampling step fused with the selection: the level-0 filtered costs stay in registers
__global__ void __launch_bounds__(kIsbBlock) isb_up_select_kernel(
    const uint8_t* __restrict__ guide_in, const float* __restrict__ cost_in, int rows_in, int cols_in,
    uint8_t* __restrict__ guide_io, const float* __restrict__ cost_fine, int rows_io, int cols_io, int ncand,
    float weight_up, float weight_down, float var_inv_i, float d0, float dl, float q, float* __restrict__ distance,
    int32_t* __restrict__ index)
{
    const int64_t pin = (int64_t)rows_in * cols_in, pio = (int64_t)rows_io * cols_io;
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= pin) return;
    UpWeights u;
    up_weights(guide_in, rows_in, cols_in, guide_io, rows_io, cols_io, (int)(o % cols_in), (int)(o / cols_in),
               weight_up, weight_down, var_inv_i, u);
    Selector s[4];
    for (int z = 0; z < ncand; ++z) {
        float out[4];
        up_costs(u, cost_in + (int64_t)z * pin, cost_fine + (int64_t)z * pio, weight_up, out);
#pragma unroll
        for (int f = 0; f < 4; ++f)
            if (u.set[f]) s[f].push(z, out[f]);
    }
#pragma unroll
    for (int f = 0; f < 4; ++f)
        if (u.set[f]) {
            distance[u.fidx[f]] = select_from(s[f], ncand, d0, dl, q);
            if (index) index[u.fidx[f]] = s[f].idx;
        }
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

static void candidate_constants(const float* candidates, int ncand, float& d0, float& dl, float& q)
{
    d0 = candidates[0];
    dl = candidates[ncand - 1];
    q = d0 / dl - 1.0f;  // (candidates[0] / candidates[-1] - 1), float32
}

}  // namespace ssg

using namespace ssg;

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
    SSG_REQUIRE(rows_in > 0 && cols_in > 0 && rows_out > 0 && cols_out > 0, "sizes must be positive");
    SSG_REQUIRE(2 * (rows_out - 1) < rows_in && 2 * (cols_out - 1) < cols_in,
                "output %dx%d is not a 2x downsampling of %dx%d", rows_out, cols_out, rows_in, cols_in);
    SSG_REQUIRE(candidate_count >= 1, "candidate_count must be positive");
    const int64_t pout = (int64_t)rows_out * cols_out;
    isb_down_kernel<<<grid_1d(pout, kIsbBlock), kIsbBlock, 0, as_stream(stream)>>>(
        d_guide_in, d_cost_in, rows_in, cols_in, d_guide_out, d_cost_out, rows_out, cols_out, candidate_count,
        var_inv_i);
    return launch_status("isb_down_kernel");
}

extern "C" int ssg_isb_upsample(const uint8_t* d_guide_in, const float* d_cost_in, int rows_in, int cols_in,
                                uint8_t* d_guide_inout, float* d_cost_inout, int rows_inout, int cols_inout,
                                int candidate_count, float weight_up, float weight_down, float var_inv_i,
                                void* stream)
{
    SSG_REQUIRE(d_guide_in && d_cost_in && d_guide_inout && d_cost_inout, "null device pointer");
    SSG_REQUIRE(rows_in > 0 && cols_in > 0 && rows_inout > 0 && cols_inout > 0, "sizes must be positive");
    SSG_REQUIRE(2 * (rows_in - 1) < rows_inout && 2 * (cols_in - 1) < cols_inout,
                "coarse %dx%d is not the 2x downsampling of %dx%d", rows_in, cols_in, rows_inout, cols_inout);
    SSG_REQUIRE((rows_inout + 1) / 2 <= rows_in && (cols_inout + 1) / 2 <= cols_in,
                "coarse %dx%d does not cover fine %dx%d", rows_in, cols_in, rows_inout, cols_inout);
    SSG_REQUIRE(candidate_count >= 1, "candidate_count must be positive");
    const int64_t pin = (int64_t)rows_in * cols_in;
    isb_up_kernel<<<grid_1d(pin, kIsbBlock), kIsbBlock, 0, as_stream(stream)>>>(
        d_guide_in, d_cost_in, rows_in, cols_in, d_guide_inout, d_cost_inout, rows_inout, cols_inout, candidate_count,
        weight_up, weight_down, var_inv_i);
    return launch_status("isb_up_kernel");
}

extern "C" int ssg_isb_apply(uint8_t* const* d_guides, float* const* d_costs, int level_count, int rows, int cols,
                             int candidate_count, double sigma_i, double sigma_s, void* stream)
{
    SSG_REQUIRE(d_guides && d_costs, "null level arrays");
    SSG_REQUIRE(level_count == ssg_isb_level_count(cols, rows),
                "level_count %d differs from the pyramid of a %dx%d image (%d)", level_count, cols, rows,
                ssg_isb_level_count(cols, rows));
    SSG_REQUIRE(level_count <= SSG_MAX_LEVELS, "too many levels");
    SSG_REQUIRE(sigma_i > 0 && sigma_s > 0, "sigmas must be positive");
    for (int s = 0; s < level_count; ++s) SSG_REQUIRE(d_guides[s] && d_costs[s], "level %d is NULL", s);
    const Levels c = isb_constants(level_count, sigma_i, sigma_s);
    for (int s = 1; s < level_count; ++s) {
        int e = ssg_isb_downsample(d_guides[s - 1], d_costs[s - 1], level_rows(rows, s - 1), level_rows(cols, s - 1),
                                   d_guides[s], d_costs[s], level_rows(rows, s), level_rows(cols, s), candidate_count,
                                   c.var_inv_i, stream);
        if (e) return e;
    }
    for (int s = level_count - 2; s >= 0; --s) {
        int e = ssg_isb_upsample(d_guides[s + 1], d_costs[s + 1], level_rows(rows, s + 1), level_rows(cols, s + 1),
                                 d_guides[s], d_costs[s], level_rows(rows, s), level_rows(cols, s), candidate_count,
                                 c.weight_up[s], c.weight_down[s], c.var_inv_i, stream);
        if (e) return e;
    }
    return SSG_OK;
}

extern "C" int ssg_isb_apply_batch(uint8_t* const* d_guides, float* const* d_costs, int level_count, int rows,
                                   int cols, int candidate_count, int instances, double sigma_i, double sigma_s,
                                   void* stream)
{
    SSG_REQUIRE(d_guides && d_costs, "null level arrays");
    SSG_REQUIRE(level_count == ssg_isb_level_count(cols, rows),
                "level_count %d differs from the pyramid of a %dx%d image (%d)", level_count, cols, rows,
                ssg_isb_level_count(cols, rows));
    SSG_REQUIRE(level_count <= SSG_MAX_LEVELS, "too many levels");
    SSG_REQUIRE(instances >= 1 && instances <= 65535, "instances out of range");
    SSG_REQUIRE(candidate_count >= 1, "candidate_count must be positive");
    SSG_REQUIRE(sigma_i > 0 && sigma_s > 0, "sigmas must be positive");
    for (int s = 0; s < level_count; ++s) SSG_REQUIRE(d_guides[s] && d_costs[s], "level %d is NULL", s);
    const Levels c = isb_constants(level_count, sigma_i, sigma_s);
    cudaStream_t st = as_stream(stream);
    for (int s = 1; s < level_count; ++s) {
        const int ri = level_rows(rows, s - 1), ci = level_rows(cols, s - 1), ro = level_rows(rows, s),
                  co = level_rows(cols, s);
        dim3 grid(grid_1d((int64_t)ro * co, kIsbBlock), instances);
        isb_down_kernel<<<grid, kIsbBlock, 0, st>>>(d_guides[s - 1], d_costs[s - 1], ri, ci, d_guides[s], d_costs[s], ro,
                                                    co, candidate_count, c.var_inv_i);
        if (int e = launch_status("isb_down_kernel")) return e;
    }
    for (int s = level_count - 2; s >= 0; --s) {
        const int rc = level_rows(rows, s + 1), cc = level_rows(cols, s + 1), rf = level_rows(rows, s),
                  cf = level_rows(cols, s);
        dim3 grid(grid_1d((int64_t)rc * cc, kIsbBlock), instances);
        isb_up_kernel<<<grid, kIsbBlock, 0, st>>>(d_guides[s + 1], d_costs[s + 1], rc, cc, d_guides[s], d_costs[s], rf,
                                                  cf, candidate_count, c.weight_up[s], c.weight_down[s], c.var_inv_i);
        if (int e = launch_status("isb_up_kernel")) return e;
    }
    return SSG_OK;
}

extern "C" int ssg_select_distance(const float* d_cost, int candidate_count, int64_t pixels, const float* candidates,
                                   float* d_distance, int32_t* d_index, void* stream)
{
    SSG_REQUIRE(d_cost && d_distance && candidates, "null pointer");
    SSG_REQUIRE(candidate_count >= 1, "candidate_count must be positive");
    SSG_REQUIRE(pixels >= 0, "negative pixel count");
    if (pixels == 0) return SSG_OK;
    float d0, dl, q;
    candidate_constants(candidates, candidate_count, d0, dl, q);
    select_distance_kernel<<<grid_1d(pixels, kIsbBlock), kIsbBlock, 0, as_stream(stream)>>>(
        d_cost, candidate_count, pixels, d0, dl, q, d_distance, d_index);
    return launch_status("select_distance_kernel");
}

extern "C" int ssg_isb_upsample_select(const uint8_t* d_guide_in, const float* d_cost_in, int rows_in, int cols_in,
                                       uint8_t* d_guide_inout, const float* d_cost_fine, int rows_fine, int cols_fine,
                                       int candidate_count, float weight_up, float weight_down, float var_inv_i,
                                       const float* candidates, float* d_distance, int32_t* d_index, void* stream)
{
    SSG_REQUIRE(d_guide_in && d_cost_in && d_guide_inout && d_cost_fine && d_distance && candidates,
                "null pointer");
    SSG_REQUIRE(rows_in > 0 && cols_in > 0 && rows_fine > 0 && cols_fine > 0, "sizes must be positive");
    SSG_REQUIRE(2 * (rows_in - 1) < rows_fine && 2 * (cols_in - 1) < cols_fine &&
                    (rows_fine + 1) / 2 <= rows_in && (cols_fine + 1) / 2 <= cols_in,
                "coarse %dx%d does not match fine %dx%d", rows_in, cols_in, rows_fine, cols_fine);
    SSG_REQUIRE(candidate_count >= 1, "candidate_count must be positive");
    float d0, dl, q;
    candidate_constants(candidates, candidate_count, d0, dl, q);
    const int64_t pin = (int64_t)rows_in * cols_in;
    isb_up_select_kernel<<<grid_1d(pin, kIsbBlock), kIsbBlock, 0, as_stream(stream)>>>(
        d_guide_in, d_cost_in, rows_in, cols_in, d_guide_inout, d_cost_fine, rows_fine, cols_fine, candidate_count,
        weight_up, weight_down, var_inv_i, d0, dl, q, d_distance, d_index);
    return launch_status("isb_up_select_kernel");
}
