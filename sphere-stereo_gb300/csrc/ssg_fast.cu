// Batched path with 16-bit cost storage and fp32 arithmetic.
//
// A batch is `instances` independent (frame, reference camera) pairs of one rig; every kernel
// takes the whole batch in one launch (blockIdx.y = instance), so the small pyramid levels are
// not launch-latency bound and a whole batch is a few dozen launches.
//
// Cost volume layout, per instance and level: [chunks][pixels][8] of a 16-bit type, candidate
// k = 8 * chunk + j.  One thread per (coarse) pixel loops over chunks: every load and store is a
// 16-byte vector, consecutive threads touch consecutive 16-byte cells (coalesced), the range
// weights of a pixel are computed once for all candidates, and the last ISB level streams the
// candidates in order through the same running argmin as the fp32 path, without writing the
// level-0 volume back.
//
// Storage: the level-0 volume (the sweep's output, the largest buffer) is 16-bit, __half (fp16)
// or unorm16 (uint16 q = round(c * 65535 / 500); costs are clamped to [0, 500] by the sweep);
// the coarser levels are float32.  Quantising the coarse levels moves the argmin: they are
// averages whose differences between candidates are small next to their magnitude, and the
// coarse scales carry much of the final weight.  Measured on the reference's golden frames:
// 16-bit coarse levels keep 73-99 % of the reference's candidate indices, float32 coarse
// levels 99.99-100 %.  Arithmetic is fp32 with fused multiply-adds and fast transcendentals;
// the fp32 path (ssg_sweep.cu, ssg_isb.cu) is the one that reproduces the reference bit for bit.
#include <cmath>

#include "ssg_common.cuh"

namespace ssg {

constexpr int kFastBlock = 256;
constexpr float kUnormScale = 65535.0f / 500.0f;
constexpr float kUnormInv = 500.0f / 65535.0f;

__device__ __forceinline__ float sqrt_approx(float x)
{
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float rcp_approx(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// 8 costs <-> one 16-byte cell
template <typename T>
struct Cell;

template <>
struct Cell<__half> {
    __device__ static __forceinline__ void unpack(uint4 v, float c[8])
    {
        const __half2* h = reinterpret_cast<const __half2*>(&v);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const float2 f = __half22float2(h[i]);
            c[2 * i] = f.x;
            c[2 * i + 1] = f.y;
        }
    }
    __device__ static __forceinline__ uint4 pack(const float c[8])
    {
        uint4 v;
        __half2* h = reinterpret_cast<__half2*>(&v);
#pragma unroll
        for (int i = 0; i < 4; ++i) h[i] = __floats2half2_rn(c[2 * i], c[2 * i + 1]);
        return v;
    }
};

template <>
struct Cell<uint16_t> {
    __device__ static __forceinline__ void unpack(uint4 v, float c[8])
    {
        const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            c[2 * i] = (float)(w[i] & 0xFFFFu) * kUnormInv;
            c[2 * i + 1] = (float)(w[i] >> 16) * kUnormInv;
        }
    }
    __device__ static __forceinline__ uint32_t q(float c)
    {
        return (uint32_t)__float2uint_rn(fminf(fmaxf(c, 0.0f), 500.0f) * kUnormScale);
    }
    __device__ static __forceinline__ uint4 pack(const float c[8])
    {
        return make_uint4(q(c[0]) | (q(c[1]) << 16), q(c[2]) | (q(c[3]) << 16), q(c[4]) | (q(c[5]) << 16),
                          q(c[6]) | (q(c[7]) << 16));
    }
};

template <>
struct Cell<float> {};

__device__ __forceinline__ uint4 ldg16(const void* p) { return __ldg(reinterpret_cast<const uint4*>(p)); }

// 8 consecutive candidates of one cell, any storage type
template <typename T>
__device__ __forceinline__ void load8(const T* __restrict__ p, float v[8])
{
    Cell<T>::unpack(ldg16(p), v);
}
template <>
__device__ __forceinline__ void load8<float>(const float* __restrict__ p, float v[8])
{
    const float4 a = __ldg(reinterpret_cast<const float4*>(p)), b = __ldg(reinterpret_cast<const float4*>(p) + 1);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}
template <typename T>
__device__ __forceinline__ void store8(T* p, const float v[8])
{
    reinterpret_cast<uint4*>(p)[0] = Cell<T>::pack(v);
}
template <>
__device__ __forceinline__ void store8<float>(float* p, const float v[8])
{
    reinterpret_cast<float4*>(p)[0] = make_float4(v[0], v[1], v[2], v[3]);
    reinterpret_cast<float4*>(p)[1] = make_float4(v[4], v[5], v[6], v[7]);
}

// ---------------------------------------------------------------------------------------------
// Image staging: HWC float32 -> RGBx float4 (16-byte texels for the sweep's bilinear taps), with
// the guide of every reference camera (rgb2yCbCr + uint8 cast) written in the same pass.
// ---------------------------------------------------------------------------------------------
struct StageParams {
    int cameras, references;
    int64_t pixels;
    int ref_slot[SSG_MAX_CAMERAS];  // reference slot of each camera, -1 if not a reference
};

__global__ void __launch_bounds__(kFastBlock) stage_images_kernel(const __grid_constant__ StageParams p,
                                                                  const float* __restrict__ images,
                                                                  float4* __restrict__ staged,
                                                                  uint8_t* __restrict__ guides)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.pixels) return;
    const int inst = blockIdx.y;  // frame * cameras + camera
    const int frame = inst / p.cameras, cam = inst % p.cameras;
    const float* src = images + ((int64_t)inst * p.pixels + i) * 3;
    const float c0 = src[0], c1 = src[1], c2 = src[2];
    staged[(int64_t)inst * p.pixels + i] = make_float4(c0, c1, c2, 0.0f);
    const int slot = p.ref_slot[cam];
    if (slot >= 0) {
        float y = fadd(fadd(fadd(fmul(c0, 0.1826f), 16.0f), fmul(c1, 0.6142f)), fmul(c2, 0.062f));
        float cb = fadd(fsub(fsub(128.0f, fmul(c0, 0.1006f)), fmul(c1, 0.3386f)), fmul(c2, 0.4392f));
        float cr = fsub(fsub(fadd(fmul(c0, 0.4392f), 128.0f), fmul(c1, 0.3989f)), fmul(c2, 0.0403f));
        uint8_t* g = guides + (((int64_t)frame * p.references + slot) * p.pixels + i) * 3;
        g[0] = (uint8_t)__float2uint_rz(fminf(fmaxf(y, 16.0f), 235.0f));
        g[1] = (uint8_t)__float2uint_rz(fminf(fmaxf(cb, 16.0f), 240.0f));
        g[2] = (uint8_t)__float2uint_rz(fminf(fmaxf(cr, 16.0f), 240.0f));
    }
}

// ---------------------------------------------------------------------------------------------
// Sweep + cost, batched, 16-bit output
// ---------------------------------------------------------------------------------------------
struct FastCam {
    float fx, fy, cx, cy, xi, alpha, one_minus_alpha;
};

struct FastSweepParams {
    int cols, rows, cameras, references, ncand, chunks;
    TorchCam ref_cam[SSG_MAX_REFERENCES];
    int ref_index[SSG_MAX_REFERENCES];
    FastCam cam[SSG_MAX_CAMERAS];
    float pose[SSG_MAX_REFERENCES][SSG_MAX_CAMERAS][12];  // reference -> camera, rows 0..2
    float cand[SSG_MAX_CANDIDATES];
};

__device__ __forceinline__ void fast_project(float x, float y, float z, const FastCam& k, float& u, float& v)
{
    const float rxy = fmaf(y, y, x * x);
    const float d1 = sqrt_approx(fmaf(z, z, rxy));
    const float c = fmaf(k.xi, d1, z);
    const float d2 = sqrt_approx(fmaf(c, c, rxy));
    const float inv = rcp_approx(fmaf(k.alpha, d2, k.one_minus_alpha * c));
    u = fmaf(k.fx * x, inv, k.cx);
    v = fmaf(k.fy * y, inv, k.cy);
}

// bilinear, zero padding, corner order nw, ne, sw, se (torch grid_sample)
__device__ __forceinline__ void fast_sample(const float4* __restrict__ img, int cols, int rows, float ix, float iy,
                                            float& s0, float& s1, float& s2)
{
    const float x0 = floorf(ix), y0 = floorf(iy);
    const float fx = ix - x0, fy = iy - y0;
    const float gx = 1.0f - fx, gy = 1.0f - fy;
    const int xi = (int)x0, yi = (int)y0;
    const bool in_x0 = x0 >= 0.0f && x0 < (float)cols, in_x1 = x0 >= -1.0f && x0 < (float)(cols - 1);
    const bool in_y0 = y0 >= 0.0f && y0 < (float)rows, in_y1 = y0 >= -1.0f && y0 < (float)(rows - 1);
    s0 = s1 = s2 = 0.0f;
    const int64_t row0 = (int64_t)yi * cols, row1 = row0 + cols;
    if (in_y0) {
        if (in_x0) {
            const float4 t = __ldg(img + row0 + xi);
            const float w = gx * gy;
            s0 = t.x * w; s1 = t.y * w; s2 = t.z * w;
        }
        if (in_x1) {
            const float4 t = __ldg(img + row0 + xi + 1);
            const float w = fx * gy;
            s0 = fmaf(t.x, w, s0); s1 = fmaf(t.y, w, s1); s2 = fmaf(t.z, w, s2);
        }
    }
    if (in_y1) {
        if (in_x0) {
            const float4 t = __ldg(img + row1 + xi);
            const float w = gx * fy;
            s0 = fmaf(t.x, w, s0); s1 = fmaf(t.y, w, s1); s2 = fmaf(t.z, w, s2);
        }
        if (in_x1) {
            const float4 t = __ldg(img + row1 + xi + 1);
            const float w = fx * fy;
            s0 = fmaf(t.x, w, s0); s1 = fmaf(t.y, w, s1); s2 = fmaf(t.z, w, s2);
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(kFastBlock) sweep_fast_kernel(const __grid_constant__ FastSweepParams p,
                                                                const float4* __restrict__ staged,
                                                                const int8_t* __restrict__ selected,
                                                                T* __restrict__ cost)
{
    const int64_t P = (int64_t)p.cols * p.rows;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    const int inst = blockIdx.y;  // frame * references + slot
    const int frame = inst / p.references, slot = inst % p.references;
    const float4* frame_img = staged + (int64_t)frame * p.cameras * P;
    const float4 rp = __ldg(frame_img + (int64_t)p.ref_index[slot] * P + i);
    T* out = cost + (int64_t)inst * p.chunks * P * 8;
    const int sel = selected[(int64_t)slot * P + i];
    if (sel < 0 || sel >= p.cameras) {
        float c = fabsf(rp.x) + fabsf(rp.y) + fabsf(rp.z);
        c = fminf(c, 500.0f);
        float cc[8] = {c, c, c, c, c, c, c, c};
        const uint4 v = Cell<T>::pack(cc);
        for (int ch = 0; ch < p.chunks; ++ch) reinterpret_cast<uint4*>(out + ((int64_t)ch * P + i) * 8)[0] = v;
        return;
    }
    float pu[3];
    unproject_torch((float)(i % p.cols), (float)(i / p.cols), p.ref_cam[slot], pu);
    const float* m = p.pose[slot][sel];
    // p_cam = R (d u) + t = d (R u) + t
    const float ax = fmaf(m[2], pu[2], fmaf(m[1], pu[1], m[0] * pu[0]));
    const float ay = fmaf(m[6], pu[2], fmaf(m[5], pu[1], m[4] * pu[0]));
    const float az = fmaf(m[10], pu[2], fmaf(m[9], pu[1], m[8] * pu[0]));
    const float tx = m[3], ty = m[7], tz = m[11];
    const FastCam k = p.cam[sel];
    const float4* img = frame_img + (int64_t)sel * P;
    for (int ch = 0; ch < p.chunks; ++ch) {
        float cc[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int kk = ch * 8 + j;
            const float d = p.cand[kk < p.ncand ? kk : p.ncand - 1];
            float u, v, s0, s1, s2;
            fast_project(fmaf(d, ax, tx), fmaf(d, ay, ty), fmaf(d, az, tz), k, u, v);
            fast_sample(img, p.cols, p.rows, u, v, s0, s1, s2);
            cc[j] = fminf(fabsf(s0 - rp.x) + fabsf(s1 - rp.y) + fabsf(s2 - rp.z), 500.0f);
        }
        reinterpret_cast<uint4*>(out + ((int64_t)ch * P + i) * 8)[0] = Cell<T>::pack(cc);
    }
}

// ---------------------------------------------------------------------------------------------
// ISB filter on the chunked 16-bit layout
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ float fast_range_weight(float d, float var_inv_i)
{
    return __expf(-d * d * var_inv_i) + 0.01f;
}

__device__ __forceinline__ float abs_sum3(const float a[3], const float b[3])
{
    return fabsf(a[0] - b[0]) + fabsf(a[1] - b[1]) + fabsf(a[2] - b[2]);
}

__device__ __forceinline__ void guide3(const uint8_t* __restrict__ g, int64_t idx, float out[3])
{
    out[0] = (float)g[3 * idx];
    out[1] = (float)g[3 * idx + 1];
    out[2] = (float)g[3 * idx + 2];
}

struct LevelGeom {
    int rows_in, cols_in, rows_out, cols_out;
};

template <typename Tin, typename Tout>
__global__ void __launch_bounds__(kFastBlock) isb_down_fast_kernel(const uint8_t* __restrict__ guide_in,
                                                                   const Tin* __restrict__ cost_in,
                                                                   uint8_t* __restrict__ guide_out,
                                                                   Tout* __restrict__ cost_out, LevelGeom g, int chunks,
                                                                   float var_inv_i)
{
    const int64_t pin = (int64_t)g.rows_in * g.cols_in, pout = (int64_t)g.rows_out * g.cols_out;
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= pout) return;
    const int inst = blockIdx.y;
    guide_in += (int64_t)inst * pin * 3;
    guide_out += (int64_t)inst * pout * 3;
    cost_in += (int64_t)inst * chunks * pin * 8;
    cost_out += (int64_t)inst * chunks * pout * 8;
    const int x = (int)(o % g.cols_out), y = (int)(o / g.cols_out);
    const int x2 = 2 * x, y2 = 2 * y;
    const int px = min(x2 + 1, g.cols_in - 1), py = min(y2 + 1, g.rows_in - 1);
    const int mx = max(x2 - 1, 0), my = max(y2 - 1, 0);
    const int64_t idx[9] = {(int64_t)y2 * g.cols_in + x2, (int64_t)my * g.cols_in + mx, (int64_t)y2 * g.cols_in + mx,
                            (int64_t)py * g.cols_in + mx, (int64_t)py * g.cols_in + x2, (int64_t)py * g.cols_in + px,
                            (int64_t)y2 * g.cols_in + px, (int64_t)my * g.cols_in + px, (int64_t)my * g.cols_in + x2};
    float cur[3];
    guide3(guide_in, idx[0], cur);
    const float base[8] = {0.25f, 0.5f, 0.25f, 0.5f, 0.25f, 0.5f, 0.25f, 0.5f};
    float w[9];
    w[0] = 1.0f;
    float wsum = 1.0f, gs[3] = {cur[0], cur[1], cur[2]};
#pragma unroll
    for (int t = 1; t < 9; ++t) {
        float nb[3];
        guide3(guide_in, idx[t], nb);
        w[t] = base[t - 1] * fast_range_weight(abs_sum3(cur, nb), var_inv_i);
        wsum += w[t];
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) gs[ch] = fmaf(nb[ch], w[t], gs[ch]);
    }
    const float inv = 1.0f / wsum;
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) guide_out[3 * o + ch] = (uint8_t)__float2uint_rz(gs[ch] * inv);
#pragma unroll
    for (int t = 0; t < 9; ++t) w[t] *= inv;
    for (int c = 0; c < chunks; ++c) {
        const Tin* src = cost_in + (int64_t)c * pin * 8;
        float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
        for (int t = 0; t < 9; ++t) {
            float v[8];
            load8<Tin>(src + idx[t] * 8, v);
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[j] = fmaf(v[j], w[t], acc[j]);
        }
        store8<Tout>(cost_out + ((int64_t)c * pout + o) * 8, acc);
    }
}

// Weights of the four fine pixels of a coarse pixel (isb_filter.cu:142-267), normalised: the
// fine pixel's own weight `up` and the coarse taps' weights, each divided by its sum.
struct FastUp {
    float w1[9], w2[6], w3[6], w4[4], up[4];
    int64_t cidx[9], fidx[4];
    bool set[4];
};

#define SSG_T2(a) {a[4], a[7], a[3], a[6], a[5], a[8]}
#define SSG_T3(a) {a[4], a[5], a[1], a[2], a[7], a[8]}
#define SSG_T4(a) {a[4], a[5], a[7], a[8]}

__device__ __forceinline__ void fast_up_weights(const uint8_t* __restrict__ gin, const LevelGeom& g,
                                                uint8_t* __restrict__ gio, int x, int y, float weight_up,
                                                float weight_down, float var_inv_i, bool write_guide, FastUp& u)
{
    const int mdx = max(x - 1, 0), mdy = max(y - 1, 0);
    const int pdx = min(x + 1, g.cols_in - 1), pdy = min(y + 1, g.rows_in - 1);
    const int x2 = 2 * x, y2 = 2 * y;
    const int pux = min(x2 + 1, g.cols_out - 1), puy = min(y2 + 1, g.rows_out - 1);
    const int rr[3] = {mdy, y, pdy}, cc[3] = {mdx, x, pdx};
    float gd[9][3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            u.cidx[3 * a + b] = (int64_t)rr[a] * g.cols_in + cc[b];
            guide3(gin, u.cidx[3 * a + b], gd[3 * a + b]);
        }
    u.fidx[0] = (int64_t)y2 * g.cols_out + x2;
    u.fidx[1] = (int64_t)puy * g.cols_out + x2;
    u.fidx[2] = (int64_t)y2 * g.cols_out + pux;
    u.fidx[3] = (int64_t)puy * g.cols_out + pux;
    u.set[0] = true;
    u.set[1] = y2 != puy;
    u.set[2] = x2 != pux;
    u.set[3] = u.set[1] && u.set[2];
    float up[4][3];
#pragma unroll
    for (int f = 0; f < 4; ++f) guide3(gio, u.fidx[f], up[f]);
    const float b1[9] = {1, 1, 1, 1, 8, 1, 1, 1, 1};
    const float b23[6] = {8, 8, 1, 1, 1, 1};
    const float* g2[6] = SSG_T2(gd);
    const float* g3[6] = SSG_T3(gd);
    const float* g4[4] = SSG_T4(gd);
    float gs[4][3], ws[4];
#pragma unroll
    for (int f = 0; f < 4; ++f) {
        ws[f] = weight_up;
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) gs[f][ch] = weight_up * up[f][ch];
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        u.w1[i] = b1[i] * weight_down * fast_range_weight(abs_sum3(gd[i], up[0]), var_inv_i);
        ws[0] += u.w1[i];
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) gs[0][ch] = fmaf(gd[i][ch], u.w1[i], gs[0][ch]);
    }
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        u.w2[i] = b23[i] * weight_down * fast_range_weight(abs_sum3(g2[i], up[1]), var_inv_i);
        ws[1] += u.w2[i];
        u.w3[i] = b23[i] * weight_down * fast_range_weight(abs_sum3(g3[i], up[2]), var_inv_i);
        ws[2] += u.w3[i];
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) {
            gs[1][ch] = fmaf(g2[i][ch], u.w2[i], gs[1][ch]);
            gs[2][ch] = fmaf(g3[i][ch], u.w3[i], gs[2][ch]);
        }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        u.w4[i] = weight_down * fast_range_weight(abs_sum3(g4[i], up[3]), var_inv_i);
        ws[3] += u.w4[i];
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) gs[3][ch] = fmaf(g4[i][ch], u.w4[i], gs[3][ch]);
    }
    float inv[4];
#pragma unroll
    for (int f = 0; f < 4; ++f) {
        inv[f] = 1.0f / ws[f];
        u.up[f] = weight_up * inv[f];
        if (write_guide && u.set[f])
#pragma unroll
            for (int ch = 0; ch < 3; ++ch) gio[3 * u.fidx[f] + ch] = (uint8_t)__float2uint_rz(gs[f][ch] * inv[f]);
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) u.w1[i] *= inv[0];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        u.w2[i] *= inv[1];
        u.w3[i] *= inv[2];
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) u.w4[i] *= inv[3];
}

// 8 candidates of the four fine pixels from 9 coarse cells and the fine cells
template <typename Tc, typename Tf>
__device__ __forceinline__ void fast_up_chunk(const FastUp& u, const Tc* __restrict__ coarse,
                                              const Tf* __restrict__ fine, float out[4][8])
{
    float cd[9][8];
#pragma unroll
    for (int t = 0; t < 9; ++t) load8<Tc>(coarse + u.cidx[t] * 8, cd[t]);
    const float* c2[6] = SSG_T2(cd);
    const float* c3[6] = SSG_T3(cd);
    const float* c4[4] = SSG_T4(cd);
#pragma unroll
    for (int f = 0; f < 4; ++f) {
        float fv[8];
        load8<Tf>(fine + u.fidx[f] * 8, fv);
#pragma unroll
        for (int j = 0; j < 8; ++j) out[f][j] = u.up[f] * fv[j];
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
#pragma unroll
        for (int i = 0; i < 9; ++i) out[0][j] = fmaf(u.w1[i], cd[i][j], out[0][j]);
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            out[1][j] = fmaf(u.w2[i], c2[i][j], out[1][j]);
            out[2][j] = fmaf(u.w3[i], c3[i][j], out[2][j]);
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) out[3][j] = fmaf(u.w4[i], c4[i][j], out[3][j]);
    }
}

__global__ void __launch_bounds__(kFastBlock) isb_up_fast_kernel(const uint8_t* __restrict__ guide_in,
                                                                 const float* __restrict__ cost_in,
                                                                 uint8_t* __restrict__ guide_io,
                                                                 float* __restrict__ cost_io, LevelGeom g, int chunks,
                                                                 float weight_up, float weight_down, float var_inv_i)
{
    const int64_t pin = (int64_t)g.rows_in * g.cols_in, pio = (int64_t)g.rows_out * g.cols_out;
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= pin) return;
    const int inst = blockIdx.y;
    guide_in += (int64_t)inst * pin * 3;
    guide_io += (int64_t)inst * pio * 3;
    cost_in += (int64_t)inst * chunks * pin * 8;
    cost_io += (int64_t)inst * chunks * pio * 8;
    FastUp u;
    fast_up_weights(guide_in, g, guide_io, (int)(o % g.cols_in), (int)(o / g.cols_in), weight_up, weight_down,
                    var_inv_i, true, u);
    for (int c = 0; c < chunks; ++c) {
        float out[4][8];
        float* fine = cost_io + (int64_t)c * pio * 8;
        fast_up_chunk<float, float>(u, cost_in + (int64_t)c * pin * 8, fine, out);
#pragma unroll
        for (int f = 0; f < 4; ++f)
            if (u.set[f]) store8<float>(fine + u.fidx[f] * 8, out[f]);
    }
}

// Running argmin / max with the argmin's neighbours (python/depth_estimation.py:180-187)
struct FastSelector {
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
        M = fmaxf(M, c);
        prev = c;
    }
    // python/depth_estimation.py:188-198
    __device__ __forceinline__ float distance(int ncand, float d0, float dl, float q) const
    {
        const float r = need_right ? m : R;
        float var = 0.5f * (L - r) / ((L + r) - 2.0f * m + 1e-8f);
        var = fminf(fmaxf(var, -0.5f), 0.5f);
        if (idx == ncand - 1 || idx == 0) var = 0.0f;
        float sel = (float)idx + var;
        if (M == m) sel = (float)(ncand - 1);
        float d = d0 / (q * sel / (float)(ncand - 1) + 1.0f);
        if (fabsf(M - m) < 1e-8f) d = dl;
        return d;
    }
};

template <typename T>
__global__ void __launch_bounds__(kFastBlock) isb_up_select_fast_kernel(
    const uint8_t* __restrict__ guide_in, const float* __restrict__ cost_in, uint8_t* __restrict__ guide_io,
    const T* __restrict__ cost_fine, LevelGeom g, int chunks, int ncand, float weight_up, float weight_down,
    float var_inv_i, float d0, float dl, float q, float* __restrict__ distance, int32_t* __restrict__ index)
{
    const int64_t pin = (int64_t)g.rows_in * g.cols_in, pio = (int64_t)g.rows_out * g.cols_out;
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= pin) return;
    const int inst = blockIdx.y;
    guide_in += (int64_t)inst * pin * 3;
    guide_io += (int64_t)inst * pio * 3;
    cost_in += (int64_t)inst * chunks * pin * 8;
    cost_fine += (int64_t)inst * chunks * pio * 8;
    distance += (int64_t)inst * pio;
    if (index) index += (int64_t)inst * pio;
    FastUp u;
    fast_up_weights(guide_in, g, guide_io, (int)(o % g.cols_in), (int)(o / g.cols_in), weight_up, weight_down,
                    var_inv_i, false, u);
    FastSelector s[4];
    for (int c = 0; c < chunks; ++c) {
        float out[4][8];
        fast_up_chunk<float, T>(u, cost_in + (int64_t)c * pin * 8, cost_fine + (int64_t)c * pio * 8, out);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int k = c * 8 + j;
            if (k < ncand) {
#pragma unroll
                for (int f = 0; f < 4; ++f) s[f].push(k, out[f][j]);
            }
        }
    }
#pragma unroll
    for (int f = 0; f < 4; ++f)
        if (u.set[f]) {
            distance[u.fidx[f]] = s[f].distance(ncand, d0, dl, q);
            if (index) index[u.fidx[f]] = s[f].idx;
        }
}

// Plain selection from a level-0 volume (pyramids of fewer than two levels)
template <typename T>
__global__ void __launch_bounds__(kFastBlock) select_fast_kernel(const T* __restrict__ cost, int64_t P, int chunks,
                                                                 int ncand, float d0, float dl, float q,
                                                                 float* __restrict__ distance,
                                                                 int32_t* __restrict__ index)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    const int inst = blockIdx.y;
    cost += (int64_t)inst * chunks * P * 8;
    FastSelector s;
    for (int c = 0; c < chunks; ++c) {
        float v[8];
        load8<T>(cost + ((int64_t)c * P + i) * 8, v);
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (c * 8 + j < ncand) s.push(c * 8 + j, v[j]);
    }
    distance[(int64_t)inst * P + i] = s.distance(ncand, d0, dl, q);
    if (index) index[(int64_t)inst * P + i] = s.idx;
}

static int check_storage(int storage)
{
    SSG_REQUIRE(storage == SSG_STORAGE_F16 || storage == SSG_STORAGE_UNORM16, "unknown cost storage %d", storage);
    return SSG_OK;
}

static int chunks_of(int n) { return (n + 7) / 8; }

}  // namespace ssg

using namespace ssg;

extern "C" int ssg_stage_images(const float* d_images, int frames, int cameras, int64_t pixels,
                                const int* reference_cameras, int references, float* d_staged, uint8_t* d_guides,
                                void* stream)
{
    SSG_REQUIRE(d_images && d_staged && d_guides && reference_cameras, "null pointer");
    SSG_REQUIRE(frames >= 1 && frames <= 65535 / SSG_MAX_CAMERAS, "frames %d outside [1, %d]", frames,
                65535 / SSG_MAX_CAMERAS);
    SSG_REQUIRE(cameras >= 1 && cameras <= SSG_MAX_CAMERAS && references >= 1 && references <= SSG_MAX_REFERENCES,
                "camera or reference count out of range");
    SSG_REQUIRE(pixels > 0, "pixels must be positive");
    SSG_REQUIRE(((uintptr_t)d_staged & 15) == 0, "staged images must be 16-byte aligned");
    StageParams p{};
    p.cameras = cameras;
    p.references = references;
    p.pixels = pixels;
    for (int c = 0; c < SSG_MAX_CAMERAS; ++c) p.ref_slot[c] = -1;
    for (int r = 0; r < references; ++r) {
        SSG_REQUIRE(reference_cameras[r] >= 0 && reference_cameras[r] < cameras, "reference camera out of range");
        p.ref_slot[reference_cameras[r]] = r;
    }
    dim3 grid(grid_1d(pixels, kFastBlock), frames * cameras);
    stage_images_kernel<<<grid, kFastBlock, 0, as_stream(stream)>>>(p, d_images, reinterpret_cast<float4*>(d_staged),
                                                                    d_guides);
    return launch_status("stage_images_kernel");
}

extern "C" int ssg_sweep_cost_batch(int cols, int rows, int frames, int camera_count, const ssg_camera* cameras,
                                    int references, const int* reference_cameras, const float* relative_poses,
                                    const float* d_staged, const int8_t* d_selected, const float* candidates,
                                    int candidate_count, int storage, void* d_cost, void* stream)
{
    SSG_REQUIRE(cols > 0 && rows > 0, "resolution must be positive");
    SSG_REQUIRE(cameras && reference_cameras && relative_poses && d_staged && d_selected && candidates && d_cost,
                "null pointer");
    SSG_REQUIRE(camera_count >= 1 && camera_count <= SSG_MAX_CAMERAS, "camera_count out of range");
    SSG_REQUIRE(references >= 1 && references <= SSG_MAX_REFERENCES, "references out of range");
    SSG_REQUIRE(frames >= 1 && frames * references <= 65535, "frames out of range");
    SSG_REQUIRE(candidate_count >= 1 && candidate_count <= SSG_MAX_CANDIDATES, "candidate_count %d outside [1, %d]",
                candidate_count, SSG_MAX_CANDIDATES);
    SSG_REQUIRE(((uintptr_t)d_staged & 15) == 0 && ((uintptr_t)d_cost & 15) == 0, "buffers must be 16-byte aligned");
    if (int e = check_storage(storage)) return e;
    FastSweepParams p{};
    p.cols = cols;
    p.rows = rows;
    p.cameras = camera_count;
    p.references = references;
    p.ncand = candidate_count;
    p.chunks = chunks_of(candidate_count);
    for (int c = 0; c < camera_count; ++c) {
        const ssg_camera& k = cameras[c];
        SSG_REQUIRE(std::isfinite(k.xi) && std::isfinite(k.alpha) && k.alpha > 0.0 && k.alpha <= 1.0,
                    "camera %d: xi must be finite and alpha in (0, 1]", c);
        p.cam[c] = FastCam{k.fx, k.fy, k.cx, k.cy, (float)k.xi, (float)k.alpha, (float)(1.0 - k.alpha)};
    }
    for (int r = 0; r < references; ++r) {
        const int rc = reference_cameras[r];
        SSG_REQUIRE(rc >= 0 && rc < camera_count, "reference camera out of range");
        p.ref_index[r] = rc;
        p.ref_cam[r] = make_torch_cam(cameras[rc]);
        for (int c = 0; c < camera_count; ++c)
            for (int j = 0; j < 12; ++j) p.pose[r][c][j] = relative_poses[((int64_t)r * camera_count + c) * 12 + j];
    }
    for (int k = 0; k < candidate_count; ++k) p.cand[k] = candidates[k];
    const int64_t P = (int64_t)cols * rows;
    dim3 grid(grid_1d(P, kFastBlock), frames * references);
    const float4* staged = reinterpret_cast<const float4*>(d_staged);
    if (storage == SSG_STORAGE_F16)
        sweep_fast_kernel<__half><<<grid, kFastBlock, 0, as_stream(stream)>>>(p, staged, d_selected,
                                                                              static_cast<__half*>(d_cost));
    else
        sweep_fast_kernel<uint16_t><<<grid, kFastBlock, 0, as_stream(stream)>>>(p, staged, d_selected,
                                                                                static_cast<uint16_t*>(d_cost));
    return launch_status("sweep_fast_kernel");
}

static int check_levels(int rows_in, int cols_in, int rows_out, int cols_out)
{
    SSG_REQUIRE(rows_in > 0 && cols_in > 0 && rows_out > 0 && cols_out > 0, "sizes must be positive");
    SSG_REQUIRE(2 * (rows_out - 1) < rows_in && 2 * (cols_out - 1) < cols_in && (rows_in + 1) / 2 <= rows_out &&
                    (cols_in + 1) / 2 <= cols_out,
                "level %dx%d is not the 2x downsampling of %dx%d", rows_out, cols_out, rows_in, cols_in);
    return SSG_OK;
}

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
    const LevelGeom g{rows_in, cols_in, rows_out, cols_out};
    dim3 grid(grid_1d((int64_t)rows_out * cols_out, kFastBlock), instances);
    const int chunks = chunks_of(candidate_count);
    float* out = static_cast<float*>(d_cost_out);
    cudaStream_t st = as_stream(stream);
    if (storage == SSG_STORAGE_F16)
        isb_down_fast_kernel<__half, float><<<grid, kFastBlock, 0, st>>>(
            d_guide_in, static_cast<const __half*>(d_cost_in), d_guide_out, out, g, chunks, var_inv_i);
    else if (storage == SSG_STORAGE_UNORM16)
        isb_down_fast_kernel<uint16_t, float><<<grid, kFastBlock, 0, st>>>(
            d_guide_in, static_cast<const uint16_t*>(d_cost_in), d_guide_out, out, g, chunks, var_inv_i);
    else
        isb_down_fast_kernel<float, float><<<grid, kFastBlock, 0, st>>>(
            d_guide_in, static_cast<const float*>(d_cost_in), d_guide_out, out, g, chunks, var_inv_i);
    return launch_status("isb_down_fast_kernel");
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
    const LevelGeom g{rows_in, cols_in, rows_inout, cols_inout};
    dim3 grid(grid_1d((int64_t)rows_in * cols_in, kFastBlock), instances);
    isb_up_fast_kernel<<<grid, kFastBlock, 0, as_stream(stream)>>>(
        d_guide_in, static_cast<const float*>(d_cost_in), d_guide_inout, static_cast<float*>(d_cost_inout), g,
        chunks_of(candidate_count), weight_up, weight_down, var_inv_i);
    return launch_status("isb_up_fast_kernel");
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
    const LevelGeom g{rows_in, cols_in, rows_fine, cols_fine};
    dim3 grid(grid_1d((int64_t)rows_in * cols_in, kFastBlock), instances);
    const int chunks = chunks_of(candidate_count);
    const float d0 = candidates[0], dl = candidates[candidate_count - 1], q = d0 / dl - 1.0f;
    const float* coarse = static_cast<const float*>(d_cost_in);
    cudaStream_t st = as_stream(stream);
    if (storage == SSG_STORAGE_F16)
        isb_up_select_fast_kernel<__half><<<grid, kFastBlock, 0, st>>>(
            d_guide_in, coarse, d_guide_inout, static_cast<const __half*>(d_cost_fine), g, chunks, candidate_count,
            weight_up, weight_down, var_inv_i, d0, dl, q, d_distance, d_index);
    else if (storage == SSG_STORAGE_UNORM16)
        isb_up_select_fast_kernel<uint16_t><<<grid, kFastBlock, 0, st>>>(
            d_guide_in, coarse, d_guide_inout, static_cast<const uint16_t*>(d_cost_fine), g, chunks, candidate_count,
            weight_up, weight_down, var_inv_i, d0, dl, q, d_distance, d_index);
    else
        isb_up_select_fast_kernel<float><<<grid, kFastBlock, 0, st>>>(
            d_guide_in, coarse, d_guide_inout, static_cast<const float*>(d_cost_fine), g, chunks, candidate_count,
            weight_up, weight_down, var_inv_i, d0, dl, q, d_distance, d_index);
    return launch_status("isb_up_select_fast_kernel");
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
    const float d0 = candidates[0], dl = candidates[candidate_count - 1], q = d0 / dl - 1.0f;
    dim3 grid(grid_1d(pixels, kFastBlock), instances);
    const int chunks = chunks_of(candidate_count);
    if (storage == SSG_STORAGE_F16)
        select_fast_kernel<__half><<<grid, kFastBlock, 0, as_stream(stream)>>>(
            static_cast<const __half*>(d_cost), pixels, chunks, candidate_count, d0, dl, q, d_distance, d_index);
    else if (storage == SSG_STORAGE_UNORM16)
        select_fast_kernel<uint16_t><<<grid, kFastBlock, 0, as_stream(stream)>>>(
            static_cast<const uint16_t*>(d_cost), pixels, chunks, candidate_count, d0, dl, q, d_distance, d_index);
    else
        select_fast_kernel<float><<<grid, kFastBlock, 0, as_stream(stream)>>>(
            static_cast<const float*>(d_cost), pixels, chunks, candidate_count, d0, dl, q, d_distance, d_index);
    return launch_status("select_fast_kernel");
}
