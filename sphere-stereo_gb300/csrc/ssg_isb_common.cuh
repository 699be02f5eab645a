// ISB filter device functions shared by the forward kernels (ssg_isb.cu) and the transposed
// operators of the backward pass (ssg_backward.cu): range weights of python/isb_filter.cu, in
// the reference's arithmetic and order.
#pragma once

#include "ssg_common.cuh"

namespace ssg {

constexpr float kIsbEps = 0.01f;  // isb_filter.cu:32

// Sizes of a level pair (down: in = fine, out = coarse; up: in = coarse, out = fine)
struct LevelGeom {
    int rows_in, cols_in, rows_out, cols_out;
};

// Outputs of the selecting step (depth_estimation.py:179-198): d0, dl the first and last
// candidates, q = d0 / dl - 1
struct SelectOut {
    float d0, dl, q;
    float* distance;
    int32_t* index;
    float* distance2;  // optional second copy of the distance
};

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

__device__ __forceinline__ void load_guide(const uint8_t* __restrict__ g, int64_t idx, int out[3])
{
    out[0] = g[3 * idx];
    out[1] = g[3 * idx + 1];
    out[2] = g[3 * idx + 2];
}

// Guides are 8-bit, so the colour distance of two guide pixels, |a0 - b0| + |a1 - b1| + |a2 - b2|,
// is an integer in [0, 765]: the reference computes it in float32 exactly, and a range weight is
// a function of that integer alone.  The forward kernels therefore read range weights from a
// shared-memory table of all 766 values, filled per block with range_weight, which gives the
// same bits as evaluating the exponential per tap.
constexpr int kRangeLutSize = 766;
constexpr int kRangeLutStride = 768;  // a table padded to whole 16-byte words

__device__ __forceinline__ int colour_distance(const int a[3], const int b[3])
{
    return abs(a[0] - b[0]) + abs(a[1] - b[1]) + abs(a[2] - b[2]);
}

// Guide layouts.  G3: [rows][cols][3] bytes, the reference's (isb_filter.py:64).  G4: one 32-bit
// word per pixel, bytes (Y, Cb, Cr, 0): one load per pixel, and the colour distance of two pixels
// is one sum of absolute byte differences (__vsadu4), equal to G3's since the fourth bytes are 0.
struct G3 {
    struct Pix {
        int c[3];
    };
    static constexpr int bytes = 3;
    __device__ static __forceinline__ Pix load(const uint8_t* __restrict__ g, int64_t idx)
    {
        Pix p;
        load_guide(g, idx, p.c);
        return p;
    }
    __device__ static __forceinline__ int dist(const Pix& a, const Pix& b) { return colour_distance(a.c, b.c); }
    __device__ static __forceinline__ int ch(const Pix& p, int k) { return p.c[k]; }
    __device__ static __forceinline__ void store(uint8_t* __restrict__ g, int64_t idx, const uint32_t v[3])
    {
#pragma unroll
        for (int k = 0; k < 3; ++k) g[3 * idx + k] = (uint8_t)v[k];
    }
};

struct G4 {
    using Pix = uint32_t;
    static constexpr int bytes = 4;
    __device__ static __forceinline__ Pix load(const uint8_t* __restrict__ g, int64_t idx)
    {
        return reinterpret_cast<const uint32_t*>(g)[idx];
    }
    __device__ static __forceinline__ int dist(Pix a, Pix b) { return (int)__vsadu4(a, b); }
    __device__ static __forceinline__ int ch(Pix p, int k) { return (int)((p >> (8 * k)) & 255u); }
    __device__ static __forceinline__ void store(uint8_t* __restrict__ g, int64_t idx, const uint32_t v[3])
    {
        reinterpret_cast<uint32_t*>(g)[idx] = v[0] | (v[1] << 8) | (v[2] << 16);
    }
};

// G4 read through L2 (ld.global.cg): for kernels that read guides written earlier in the same
// launch, where the read-only path is not coherent
struct G4C : G4 {
    __device__ static __forceinline__ Pix load(const uint8_t* g, int64_t idx)
    {
        return __ldcg(reinterpret_cast<const uint32_t*>(g) + idx);
    }
};

struct ExpRange {  // evaluates the weight of a colour distance
    float var_inv_i;
    __device__ __forceinline__ float operator()(int d) const { return range_weight((float)d, var_inv_i); }
};

struct LutRange {  // reads it from the block's table
    const float* lut;
    __device__ __forceinline__ float operator()(int d) const { return lut[d]; }
};

// fills the table of a block (the caller synchronises the block before reading it)
__device__ __forceinline__ void fill_range_lut(float* lut, float var_inv_i)
{
    for (int d = threadIdx.x; d < kRangeLutSize; d += blockDim.x) lut[d] = range_weight((float)d, var_inv_i);
}

// the block's table (16-byte aligned, kRangeLutStride floats): copied from the precomputed table
// `table` (range_table()) when there is one, else evaluated; the caller synchronises the block
__device__ __forceinline__ void load_range_lut(float* lut, const float* __restrict__ table, float var_inv_i)
{
    if (table) {
        for (int q = threadIdx.x; q < kRangeLutStride / 4; q += blockDim.x)
            reinterpret_cast<float4*>(lut)[q] = __ldg(reinterpret_cast<const float4*>(table) + q);
    } else {
        fill_range_lut(lut, var_inv_i);
    }
}

// The range-weight table of var_inv_i in device memory (filled once per device and value, on
// `stream`, which is synchronised then), or nullptr when it cannot be had now (the stream is
// being captured, or all slots are taken): kernels then evaluate the table per block.
const float* range_table(float var_inv_i, cudaStream_t stream);

// Guide weights of one coarse pixel of guideDownsample2xKernel (isb_filter.cu:44-119): the
// centre tap (weight 1) and its 8 neighbours in the reference's order, edge-clamped. Writes the
// coarse guide (uint8 truncation, isb_filter.cu:93).
template <typename I>
struct DownTapsT {
    I centre;
    I idx[8];
    float w[8];
    float wsum;
};
using DownTaps = DownTapsT<int64_t>;

// guide_out points at the layout's array; the coarse pixel's index is o
template <typename I, typename RW, typename GL = G3>
__device__ __forceinline__ void down_weights(const uint8_t* __restrict__ guide_in, int rows_in, int cols_in, int x,
                                             int y, const RW& range, uint8_t* __restrict__ guide_out, int64_t o,
                                             DownTapsT<I>& t)
{
    const int x2 = 2 * x, y2 = 2 * y;
    const int px = min(x2 + 1, cols_in - 1), py = min(y2 + 1, rows_in - 1);
    const int mx = max(x2 - 1, 0), my = max(y2 - 1, 0);
    const int rows8[8] = {my, y2, py, py, py, y2, my, my};
    const int cols8[8] = {mx, mx, mx, x2, px, px, px, x2};
    t.centre = (I)y2 * cols_in + x2;
    const typename GL::Pix cur = GL::load(guide_in, t.centre);
    const float base[8] = {0.25f, 0.5f, 0.25f, 0.5f, 0.25f, 0.5f, 0.25f, 0.5f};
    float wsum = 1.0f, g[3] = {(float)GL::ch(cur, 0), (float)GL::ch(cur, 1), (float)GL::ch(cur, 2)};
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        t.idx[i] = (I)rows8[i] * cols_in + cols8[i];
        const typename GL::Pix nb = GL::load(guide_in, t.idx[i]);
        t.w[i] = fmul(base[i], range(GL::dist(cur, nb)));
        wsum = fadd(wsum, t.w[i]);
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) g[ch] = fadd(g[ch], fmul((float)GL::ch(nb, ch), t.w[i]));
    }
    t.wsum = wsum;
    const float den = fdiv(1.0f, wsum);
    uint32_t v[3];
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) v[ch] = __float2uint_rz(fmul(g[ch], den));
    GL::store(guide_out, o, v);
}

// The four fine pixels of a coarse pixel (x, y) of guideUpsample2xKernel (isb_filter.cu:142-267):
// F = 0 (2x, 2y), 1 (2x, 2y + 1), 2 (2x + 1, 2y), 3 (2x + 1, 2y + 1). Each reads a fixed list of
// the coarse 3x3 neighbourhood (taps indexed 3 * row + col, isb_filter.cu:185-208), with a base
// weight of 8 on its nearest taps (none for F = 3).
template <int F>
struct UpTaps;
template <>
struct UpTaps<0> {
    static constexpr int n = 9;
    static constexpr bool weighted = true;
    __device__ static constexpr int tap(int i) { return i; }
    __device__ static constexpr float base(int i) { return i == 4 ? 8.0f : 1.0f; }
};
template <>
struct UpTaps<1> {  // (1,1),(2,1),(1,0),(2,0),(1,2),(2,2)
    static constexpr int n = 6;
    static constexpr bool weighted = true;
    __device__ static constexpr int tap(int i) { return i == 0 ? 4 : i == 1 ? 7 : i == 2 ? 3 : i == 3 ? 6 : i == 4 ? 5 : 8; }
    __device__ static constexpr float base(int i) { return i < 2 ? 8.0f : 1.0f; }
};
template <>
struct UpTaps<2> {  // (1,1),(1,2),(0,1),(0,2),(2,1),(2,2)
    static constexpr int n = 6;
    static constexpr bool weighted = true;
    __device__ static constexpr int tap(int i) { return i == 0 ? 4 : i == 1 ? 5 : i == 2 ? 1 : i == 3 ? 2 : i == 4 ? 7 : 8; }
    __device__ static constexpr float base(int i) { return i < 2 ? 8.0f : 1.0f; }
};
template <>
struct UpTaps<3> {  // (1,1),(1,2),(2,1),(2,2)
    static constexpr int n = 4;
    static constexpr bool weighted = false;
    __device__ static constexpr int tap(int i) { return i == 0 ? 4 : i == 1 ? 5 : i == 2 ? 7 : 8; }
    __device__ static constexpr float base(int) { return 1.0f; }
};

// Range weights of fine pixel F from the coarse guides `gd` and its own guide `up`; returns
// 1 / (sum of weights) and the weighted guide sum `g` (isb_filter.cu:142-267).
template <int F, typename RW, typename GL = G3>
__device__ __forceinline__ float fine_weights(const typename GL::Pix (&gd)[9], const typename GL::Pix& up,
                                              float weight_up, float weight_down, const RW& range,
                                              float (&w)[UpTaps<F>::n], float g[3])
{
    float ws = weight_up;
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) g[ch] = fmul(weight_up, (float)GL::ch(up, ch));
#pragma unroll
    for (int i = 0; i < UpTaps<F>::n; ++i) {
        const typename GL::Pix& nb = gd[UpTaps<F>::tap(i)];
        const float rw = fmul(weight_down, range(GL::dist(nb, up)));
        w[i] = UpTaps<F>::weighted ? fmul(UpTaps<F>::base(i), rw) : rw;
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) g[ch] = fadd(g[ch], fmul((float)GL::ch(nb, ch), w[i]));
        ws = fadd(ws, w[i]);
    }
    return fdiv(1.0f, ws);
}

// Coarse 3x3 neighbourhood of (x, y), edge-clamped: flat indices and guides
template <typename I, typename GL = G3>
__device__ __forceinline__ void coarse_neighbourhood(const uint8_t* __restrict__ guide_in, int rows_in, int cols_in,
                                                     int x, int y, I (&cidx)[9], typename GL::Pix (&gd)[9])
{
    const int rr[3] = {max(y - 1, 0), y, min(y + 1, rows_in - 1)};
    const int cc[3] = {max(x - 1, 0), x, min(x + 1, cols_in - 1)};
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            cidx[3 * a + b] = (I)rr[a] * cols_in + cc[b];
            gd[3 * a + b] = GL::load(guide_in, cidx[3 * a + b]);
        }
}

// Weights of the four fine pixels of one coarse pixel: taps index the 3x3 coarse neighbourhood
// [row][col] flattened as 3 * row + col.
struct UpWeights {
    float w1[9], w2[6], w3[6], w4[4];
    float inv[4];
    int64_t cidx[9];
    int64_t fidx[4];
    bool set[4];
};

// Tap lists of the fine pixels below, right and below-right (UpTaps<1..3>) as macros over an
// array, so that every index is a compile-time constant and the values stay in registers.
#define SSG_TAPS2(a) {a[4], a[7], a[3], a[6], a[5], a[8]}
#define SSG_TAPS3(a) {a[4], a[5], a[1], a[2], a[7], a[8]}
#define SSG_TAPS4(a) {a[4], a[5], a[7], a[8]}

__device__ __forceinline__ void up_weights(const uint8_t* __restrict__ guide_in, int rows_in, int cols_in,
                                           uint8_t* __restrict__ guide_io, int rows_io, int cols_io, int x, int y,
                                           float weight_up, float weight_down, float var_inv_i, bool write_guide,
                                           UpWeights& u)
{
    G3::Pix gd[9];
    coarse_neighbourhood<int64_t, G3>(guide_in, rows_in, cols_in, x, y, u.cidx, gd);
    const int x2 = 2 * x, y2 = 2 * y;
    const int pux = min(x2 + 1, cols_io - 1), puy = min(y2 + 1, rows_io - 1);
    u.fidx[0] = (int64_t)y2 * cols_io + x2;
    u.fidx[1] = (int64_t)puy * cols_io + x2;
    u.fidx[2] = (int64_t)y2 * cols_io + pux;
    u.fidx[3] = (int64_t)puy * cols_io + pux;
    u.set[0] = true;
    u.set[1] = y2 != puy;
    u.set[2] = x2 != pux;
    u.set[3] = u.set[1] && u.set[2];
    G3::Pix up[4];
#pragma unroll
    for (int f = 0; f < 4; ++f) up[f] = G3::load(guide_io, u.fidx[f]);
    float g[4][3];
    const ExpRange range{var_inv_i};
    u.inv[0] = fine_weights<0, ExpRange, G3>(gd, up[0], weight_up, weight_down, range, u.w1, g[0]);
    u.inv[1] = fine_weights<1, ExpRange, G3>(gd, up[1], weight_up, weight_down, range, u.w2, g[1]);
    u.inv[2] = fine_weights<2, ExpRange, G3>(gd, up[2], weight_up, weight_down, range, u.w3, g[2]);
    u.inv[3] = fine_weights<3, ExpRange, G3>(gd, up[3], weight_up, weight_down, range, u.w4, g[3]);
    if (write_guide)
#pragma unroll
        for (int f = 0; f < 4; ++f)
            if (u.set[f])
#pragma unroll
                for (int ch = 0; ch < 3; ++ch)
                    guide_io[3 * u.fidx[f] + ch] = (uint8_t)__float2uint_rz(fmul(g[f][ch], u.inv[f]));
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

// Running argmin / max with the neighbours of the argmin (depth_estimation.py:180-187):
// the first minimum wins ties, as torch.min(dim) does.  Candidates are pushed in order
// z = 0, 1, ...; L is the value before the argmin (read only when the argmin is not the first
// candidate), R the value after it (read only when it is not the last).  Branch-free: every
// push is a handful of compares and selects.  Costs are finite (the sweep clamps them).
struct Selector {
    float m = __builtin_huge_valf(), M = -__builtin_huge_valf(), L = 0.0f, R = 0.0f, prev = 0.0f;
    int idx = 0;
    bool need_right = false;
    // the first strict minimum and the maximum as the reference's min / max take them; fminf and
    // fmaxf give the same values (a NaN cost leaves both unchanged, as the comparisons do)
    __device__ __forceinline__ void push(int z, float c)
    {
        R = need_right ? c : R;
        const bool lt = c < m;
        m = fminf(c, m);
        idx = lt ? z : idx;
        L = lt ? prev : L;
        need_right = lt;
        M = fmaxf(c, M);
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

}  // namespace ssg
