// Differentiable sweep: soft-argmin inverse distance and its backward pass.
//
// Forward (no counterpart in the reference, whose selection is a hard argmin + parabola,
// python/depth_estimation.py:179-198): the fp32 sweep and ISB filter of ssg_sweep.cu /
// ssg_isb.cu, then per pixel q = sum_k softmax(-F_k / tau) / d_k over the filtered costs F,
// fused with the last filter level.
//
// Backward, with the cost volume recomputed instead of stored, and every sum formed in an order
// that does not depend on thread timing (the gradients are bit-reproducible run to run):
//   * seed: the last level recomputes F and runs an online softmax over the candidates (two
//     passes); dL/dF is written per fine pixel;
//   * the ISB filter is linear in the cost for a fixed guide (its weights come from uint8 guides
//     and get no gradient), so each up step and each down step is run transposed, from level 0's
//     dL/dF up to the coarsest level and back down to level 0.  Each transposed step is a
//     gather: every output cell recomputes the weights with which the forward step read it and
//     sums its contributions in a fixed order, so that no two threads write one cell;
//   * the sweep's backward recomputes every sample, maps dL/dcost through the clamp, the L1 and
//     the bilinear sample to the images and through the double-sphere projection to the 6-DoF
//     pose deltas of the source and reference cameras.  A source texel receives contributions
//     from any sample that lands on it, so the image gradient is accumulated in 64-bit fixed
//     point (multiples of 2^-e, e from the largest |dL/dcost| and the number of samples):
//     integer sums do not depend on the order of the atomic adds.  The pose gradient is reduced
//     per block by a fixed warp-shuffle tree in float64, and the block sums are added in block
//     order.
// Pose deltas are right perturbations, T_c <- T_c exp(delta_c), delta = (omega, v): the
// relative pose reference -> camera becomes exp(-delta_c) rel exp(delta_ref).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "ssg_isb_common.cuh"

namespace ssg {

constexpr int kBwdBlock = 256;

struct SoftParams {
    int ncand;
    float tau;
    float inv_cand[SSG_MAX_CANDIDATES];  // 1 / d_k
};

// q = sum_k w_k / d_k with w = softmax(-F / tau), by an online softmax
struct OnlineSoftmax {
    float m, s, t;
    __device__ __forceinline__ void init() { m = -INFINITY, s = 0.0f, t = 0.0f; }
    __device__ __forceinline__ void push(float x, float invd)
    {
        if (x > m) {
            const float r = expf(m - x);
            s *= r;
            t *= r;
            m = x;
        }
        const float e = expf(x - m);
        s += e;
        t = fmaf(e, invd, t);
    }
};

// Filtered level-0 costs of the four fine pixels for candidate z (the arithmetic of up_costs)
__device__ __forceinline__ void fine_costs(const UpWeights& u, const float* __restrict__ coarse,
                                           const float* __restrict__ fine, float weight_up, float out[4])
{
    out[0] = out[1] = out[2] = out[3] = 0.0f;
    up_costs(u, coarse, fine, weight_up, out);
}

__global__ void __launch_bounds__(kBwdBlock) isb_up_softargmin_kernel(
    const uint8_t* __restrict__ guide_in, const float* __restrict__ cost_in, int rows_in, int cols_in,
    const uint8_t* __restrict__ guide_fine, const float* __restrict__ cost_fine, int rows_io, int cols_io,
    float weight_up, float weight_down, float var_inv_i, const __grid_constant__ SoftParams sp,
    float* __restrict__ q)
{
    const int64_t pin = (int64_t)rows_in * cols_in, pio = (int64_t)rows_io * cols_io;
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= pin) return;
    UpWeights u;
    up_weights(guide_in, rows_in, cols_in, const_cast<uint8_t*>(guide_fine), rows_io, cols_io, (int)(o % cols_in),
               (int)(o / cols_in), weight_up, weight_down, var_inv_i, false, u);
    OnlineSoftmax sm[4];
#pragma unroll
    for (int f = 0; f < 4; ++f) sm[f].init();
    const float inv_tau = 1.0f / sp.tau;
    for (int z = 0; z < sp.ncand; ++z) {
        float c[4];
        fine_costs(u, cost_in + (int64_t)z * pin, cost_fine + (int64_t)z * pio, weight_up, c);
#pragma unroll
        for (int f = 0; f < 4; ++f)
            if (u.set[f]) sm[f].push(-c[f] * inv_tau, sp.inv_cand[z]);
    }
#pragma unroll
    for (int f = 0; f < 4; ++f)
        if (u.set[f]) q[u.fidx[f]] = sm[f].t / sm[f].s;
}

// dL/dF of the soft-argmin for every fine pixel and candidate, written to grad_F (candidate
// planes of the fine level); ssg_isb_upsample_transpose then takes it through the last level.
__global__ void __launch_bounds__(kBwdBlock) isb_up_softargmin_backward_kernel(
    const uint8_t* __restrict__ guide_in, const float* __restrict__ cost_in, int rows_in, int cols_in,
    const uint8_t* __restrict__ guide_fine, const float* __restrict__ cost_fine, int rows_io, int cols_io,
    float weight_up, float weight_down, float var_inv_i, const __grid_constant__ SoftParams sp,
    const float* __restrict__ grad_q, float* __restrict__ grad_F)
{
    const int64_t pin = (int64_t)rows_in * cols_in, pio = (int64_t)rows_io * cols_io;
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= pin) return;
    UpWeights u;
    up_weights(guide_in, rows_in, cols_in, const_cast<uint8_t*>(guide_fine), rows_io, cols_io, (int)(o % cols_in),
               (int)(o / cols_in), weight_up, weight_down, var_inv_i, false, u);
    const float inv_tau = 1.0f / sp.tau;
    OnlineSoftmax sm[4];
#pragma unroll
    for (int f = 0; f < 4; ++f) sm[f].init();
    for (int z = 0; z < sp.ncand; ++z) {
        float c[4];
        fine_costs(u, cost_in + (int64_t)z * pin, cost_fine + (int64_t)z * pio, weight_up, c);
#pragma unroll
        for (int f = 0; f < 4; ++f)
            if (u.set[f]) sm[f].push(-c[f] * inv_tau, sp.inv_cand[z]);
    }
    float qv[4], gq[4];
#pragma unroll
    for (int f = 0; f < 4; ++f) {
        qv[f] = u.set[f] ? sm[f].t / sm[f].s : 0.0f;
        gq[f] = u.set[f] ? grad_q[u.fidx[f]] : 0.0f;
    }
    for (int z = 0; z < sp.ncand; ++z) {
        float c[4];
        fine_costs(u, cost_in + (int64_t)z * pin, cost_fine + (int64_t)z * pio, weight_up, c);
#pragma unroll
        for (int f = 0; f < 4; ++f) {
            if (!u.set[f]) continue;
            const float w = expf(-c[f] * inv_tau - sm[f].m) / sm[f].s;
            grad_F[(int64_t)z * pio + u.fidx[f]] = gq[f] * (-inv_tau) * w * (sp.inv_cand[z] - qv[f]);
        }
    }
}

// Transpose of one up step s (fine level s, coarse level s + 1):
//   f_s = a * c_s + B f_{s+1}   =>   g_c_s = a * g_f_s ,  g_f_{s+1} = B^T g_f_s
// One thread per coarse cell (X, Y): the own-pixel part of the four fine pixels of (X, Y) is
// written, and g_f_{s+1}(X, Y) gathers the fine gradients of every fine pixel that read the cell
// in the forward step -- the fine pixels of the coarse 3 x 3 neighbourhood whose edge-clamped tap
// lists hold (X, Y), with the weights the forward step gave those taps.  Contributions are summed
// in a fixed order (neighbour, then fine pixel).
__device__ __forceinline__ void add_tap_weights(const UpWeights& u, int64_t me, float (&k)[4])
{
    const int64_t c2[6] = SSG_TAPS2(u.cidx);
    const int64_t c3[6] = SSG_TAPS3(u.cidx);
    const int64_t c4[4] = SSG_TAPS4(u.cidx);
    k[0] = k[1] = k[2] = k[3] = 0.0f;
#pragma unroll
    for (int i = 0; i < 9; ++i)
        if (u.cidx[i] == me) k[0] += u.w1[i] * u.inv[0];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        if (c2[i] == me) k[1] += u.w2[i] * u.inv[1];
        if (c3[i] == me) k[2] += u.w3[i] * u.inv[2];
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
        if (c4[i] == me) k[3] += u.w4[i] * u.inv[3];
#pragma unroll
    for (int f = 0; f < 4; ++f)
        if (!u.set[f]) k[f] = 0.0f;
}

__global__ void __launch_bounds__(kBwdBlock) isb_up_transpose_kernel(
    const uint8_t* __restrict__ guide_coarse, int rows_in, int cols_in, const uint8_t* __restrict__ guide_fine,
    int rows_io, int cols_io, int ncand, float weight_up, float weight_down, float var_inv_i,
    const float* __restrict__ grad_f_fine, float* __restrict__ grad_c_fine, float* __restrict__ grad_f_coarse)
{
    const int64_t pin = (int64_t)rows_in * cols_in, pio = (int64_t)rows_io * cols_io;
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= pin) return;
    const int X = (int)(o % cols_in), Y = (int)(o / cols_in);
    // per neighbour n = 3 (dy + 1) + (dx + 1): the fine index of its pixel F = 0 (the others
    // are + cols_io, + 1, + cols_io + 1 when set) and the weights k[n][F] with which they read (X, Y)
    int base[9];
    float k[9][4];
    float own[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int n = 0; n < 9; ++n) {
        const int x = X + n % 3 - 1, y = Y + n / 3 - 1;
        base[n] = 0;
#pragma unroll
        for (int f = 0; f < 4; ++f) k[n][f] = 0.0f;
        if (x < 0 || y < 0 || x >= cols_in || y >= rows_in) continue;
        UpWeights u;
        up_weights(guide_coarse, rows_in, cols_in, const_cast<uint8_t*>(guide_fine), rows_io, cols_io, x, y,
                   weight_up, weight_down, var_inv_i, false, u);
        add_tap_weights(u, o, k[n]);
        base[n] = (int)u.fidx[0];
        if (n == 4)
#pragma unroll
            for (int f = 0; f < 4; ++f) own[f] = u.set[f] ? weight_up * u.inv[f] : 0.0f;
    }
    const int x2 = 2 * X, y2 = 2 * Y;
    const bool set1 = y2 + 1 < rows_io, set2 = x2 + 1 < cols_io;
    const int64_t fo[4] = {(int64_t)y2 * cols_io + x2, (int64_t)(y2 + 1) * cols_io + x2, (int64_t)y2 * cols_io + x2 + 1,
                           (int64_t)(y2 + 1) * cols_io + x2 + 1};
    const bool fset[4] = {true, set1, set2, set1 && set2};
    for (int z = 0; z < ncand; ++z) {
        const float* gf = grad_f_fine + (int64_t)z * pio;
        float acc = 0.0f;
#pragma unroll
        for (int n = 0; n < 9; ++n) {
            const float* g = gf + base[n];
            if (k[n][0] != 0.0f) acc += k[n][0] * g[0];
            if (k[n][1] != 0.0f) acc += k[n][1] * g[cols_io];
            if (k[n][2] != 0.0f) acc += k[n][2] * g[1];
            if (k[n][3] != 0.0f) acc += k[n][3] * g[cols_io + 1];
        }
        grad_f_coarse[(int64_t)z * pin + o] = acc;
        float* gc = grad_c_fine + (int64_t)z * pio;
#pragma unroll
        for (int f = 0; f < 4; ++f)
            if (fset[f]) gc[fo[f]] = own[f] * gf[fo[f]];
    }
}

// Transpose of one down step s (fine level s - 1, coarse level s):
//   c_s[o] = sum_t w_t c_{s-1}[idx_t] / wsum   =>   g_c_{s-1}[i] += sum_{o, t: idx_t(o) = i} w_t / wsum * g_c_s[o]
// One thread per fine cell i = (X, Y): the coarse pixels whose edge-clamped 3 x 3 taps can hold
// it are those with |X - 2 x| <= 1 and |Y - 2 y| <= 1 (at most four); their normalised weights
// are recomputed as the forward step forms them, and the cell adds their gradients in a fixed
// order to what it holds (the up transpose's own-pixel part).
__device__ __forceinline__ void down_taps(int x, int y, int rows_in, int cols_in, int64_t (&idx)[9])
{
    const int x2 = 2 * x, y2 = 2 * y;
    const int px = min(x2 + 1, cols_in - 1), py = min(y2 + 1, rows_in - 1);
    const int mx = max(x2 - 1, 0), my = max(y2 - 1, 0);
    idx[0] = (int64_t)y2 * cols_in + x2;
    idx[1] = (int64_t)my * cols_in + mx;
    idx[2] = (int64_t)y2 * cols_in + mx;
    idx[3] = (int64_t)py * cols_in + mx;
    idx[4] = (int64_t)py * cols_in + x2;
    idx[5] = (int64_t)py * cols_in + px;
    idx[6] = (int64_t)y2 * cols_in + px;
    idx[7] = (int64_t)my * cols_in + px;
    idx[8] = (int64_t)my * cols_in + x2;
}

// normalised weights of the 3 x 3 taps of coarse pixel (x, y) (isb_filter.cu:44-119)
__device__ __forceinline__ void down_weights(const uint8_t* __restrict__ guide_in, const int64_t (&idx)[9],
                                             float var_inv_i, float (&w)[9])
{
    float cur[3];
    load_guide(guide_in, idx[0], cur);
    const float base[8] = {0.25f, 0.5f, 0.25f, 0.5f, 0.25f, 0.5f, 0.25f, 0.5f};
    w[0] = 1.0f;
    float wsum = 1.0f;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        float nb[3];
        load_guide(guide_in, idx[i + 1], nb);
        w[i + 1] = fmul(base[i], range_weight(abs_sum(cur, nb), var_inv_i));
        wsum = fadd(wsum, w[i + 1]);
    }
#pragma unroll
    for (int t = 0; t < 9; ++t) w[t] = w[t] / wsum;
}

__global__ void __launch_bounds__(kBwdBlock) isb_down_transpose_kernel(const uint8_t* __restrict__ guide_in,
                                                                       int rows_in, int cols_in, int rows_out,
                                                                       int cols_out, int ncand, float var_inv_i,
                                                                       const float* __restrict__ grad_c_coarse,
                                                                       float* __restrict__ grad_c_fine)
{
    const int64_t pout = (int64_t)rows_out * cols_out, pin = (int64_t)rows_in * cols_in;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= pin) return;
    const int X = (int)(i % cols_in), Y = (int)(i / cols_in);
    int64_t co[4];
    float k[4];
#pragma unroll
    for (int n = 0; n < 4; ++n) {
        // odd X: x in {(X - 1) / 2, (X + 1) / 2}; even X: x = X / 2 only (n & 1 = 1 is skipped)
        const int x = (X >> 1) + (n & 1), y = (Y >> 1) + (n >> 1);
        co[n] = 0;
        k[n] = 0.0f;
        const bool none = ((n & 1) && !(X & 1)) || ((n >> 1) && !(Y & 1));
        if (none || x >= cols_out || y >= rows_out) continue;
        int64_t idx[9];
        down_taps(x, y, rows_in, cols_in, idx);
        float w[9];
        down_weights(guide_in, idx, var_inv_i, w);
        float kk = 0.0f;
#pragma unroll
        for (int t = 0; t < 9; ++t)
            if (idx[t] == i) kk += w[t];
        co[n] = (int64_t)y * cols_out + x;
        k[n] = kk;
    }
    for (int z = 0; z < ncand; ++z) {
        const float* gc = grad_c_coarse + (int64_t)z * pout;
        float acc = 0.0f;
#pragma unroll
        for (int n = 0; n < 4; ++n)
            if (k[n] != 0.0f) acc += k[n] * gc[co[n]];
        grad_c_fine[(int64_t)z * pin + i] += acc;
    }
}

// --------------------------------------------------------------------------------------------
// Sweep backward
// --------------------------------------------------------------------------------------------
struct SweepBwdParams {
    int cols, rows, ncam, ncand, reference;
    float colsf, rowsf, inv_cols, inv_rows;
    int cols_pow2, rows_pow2;
    TorchCam ref;
    TorchCam cams[SSG_MAX_CAMERAS];
    float rt[SSG_MAX_CAMERAS][12];
    const float* images[SSG_MAX_CAMERAS];
    float cand[SSG_MAX_CANDIDATES];
};

__device__ __forceinline__ float sample_coord(float uv, float size, float inv_size, bool pow2)
{
    const float t = fadd(uv, 0.5f);
    const float qq = pow2 ? fmul(t, inv_size) : fdiv(t, size);
    const float g = fsub(fmul(qq, 2.0f), 1.0f);
    return fmul(fsub(fmul(fadd(g, 1.0f), size), 1.0f), 0.5f);
}

// d(uv)/d(point) of the double-sphere projection (python/utils.py:75-94), rows u and v
__device__ __forceinline__ void project_jacobian(const float p[3], const TorchCam& k, float ju[3], float jv[3])
{
    const float x = p[0], y = p[1], z = p[2];
    const float d1 = sqrtf(x * x + y * y + z * z);
    const float c = k.xi * d1 + z;
    const float d2 = sqrtf(x * x + y * y + c * c);
    const float nrm = k.alpha * d2 + k.one_minus_alpha * c;
    const float dc[3] = {k.xi * x / d1, k.xi * y / d1, k.xi * z / d1 + 1.0f};
    float dn[3];
    dn[0] = k.alpha * (x + c * dc[0]) / d2 + k.one_minus_alpha * dc[0];
    dn[1] = k.alpha * (y + c * dc[1]) / d2 + k.one_minus_alpha * dc[1];
    dn[2] = k.alpha * (c * dc[2]) / d2 + k.one_minus_alpha * dc[2];
    const float in = 1.0f / nrm, in2 = in * in;
    ju[0] = k.fx * (in - x * dn[0] * in2);
    ju[1] = k.fx * (-x * dn[1] * in2);
    ju[2] = k.fx * (-x * dn[2] * in2);
    jv[0] = k.fy * (-y * dn[0] * in2);
    jv[1] = k.fy * (in - y * dn[1] * in2);
    jv[2] = k.fy * (-y * dn[2] * in2);
}

// The image gradient's fixed-point scale: 2^e with e = 62 - ceil(log2 count) - ceil(log2 m), m the
// largest |dL/dcost| (its float bits) and count a bound on the contributions one texel can receive
// (each at most m x the candidates in magnitude): no sum leaves the int64 range, and a
// contribution is rounded by at most m 2^-(63 - log2 count).  0 when m is 0, inf or NaN.
__device__ __forceinline__ float fixed_scale(uint32_t absmax_bits, double count)
{
    const float m = __uint_as_float(absmax_bits);
    if (!(m > 0.0f) || !(m <= 3.0e38f)) return 0.0f;
    int em, ec;
    frexpf(m, &em);     // m < 2^em
    frexp(count, &ec);  // count < 2^ec
    const int e = max(-120, min(62 - ec - em, 120));
    return ldexpf(1.0f, e);
}

__device__ __forceinline__ void fixed_add(long long* acc, float x, float scale)
{
    const long long q = __float2ll_rn(x * scale);
    if (q) atomicAdd(reinterpret_cast<unsigned long long*>(acc), (unsigned long long)q);
}

// largest |x| over n values, as float bits (monotonic for non-negative floats; NaN above inf)
__global__ void __launch_bounds__(kBwdBlock) absmax_kernel(const float* __restrict__ x, int64_t n,
                                                           uint32_t* __restrict__ out)
{
    uint32_t m = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        m = max(m, __float_as_uint(x[i]) & 0x7FFFFFFFu);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) m = max(m, __shfl_down_sync(0xFFFFFFFFu, m, off));
    if ((threadIdx.x & 31) == 0 && m) atomicMax(out, m);
}

__global__ void __launch_bounds__(kBwdBlock) sweep_backward_kernel(const __grid_constant__ SweepBwdParams p,
                                                                   const int8_t* __restrict__ selected,
                                                                   const float* __restrict__ grad_cost,
                                                                   const uint32_t* __restrict__ absmax,
                                                                   long long* __restrict__ image_acc,
                                                                   double* __restrict__ pose_partial)
{
    const int64_t P = (int64_t)p.cols * p.rows;
    const float scale = fixed_scale(*absmax, 2.0 * (double)P * p.ncand);
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int sel = i < P ? selected[i] : -1;
    const bool active = i < P && sel >= 0 && sel < p.ncam;
    float gsrc[6] = {0, 0, 0, 0, 0, 0}, gref6[6] = {0, 0, 0, 0, 0, 0};
    if (active) {
        float pu[3];
        unproject_torch((float)(i % p.cols), (float)(i / p.cols), p.ref, pu);
        const float* refimg = p.images[p.reference] + 3 * i;
        const float r[3] = {refimg[0], refimg[1], refimg[2]};
        const TorchCam cam = p.cams[sel];
        float rt[12];
#pragma unroll
        for (int j = 0; j < 12; ++j) rt[j] = p.rt[sel][j];
        const float* img = p.images[sel];
        long long* gimg = image_acc + (int64_t)sel * P * 3;
        float gref[3] = {0.0f, 0.0f, 0.0f};
        for (int k = 0; k < p.ncand; ++k) {
            const float g = grad_cost[(int64_t)k * P + i];
            if (g == 0.0f) continue;
            const float d = p.cand[k];
            const float pv[3] = {fmul(d, pu[0]), fmul(d, pu[1]), fmul(d, pu[2])};
            float q[3], uv[2];
            transform_torch(rt, pv, q);
            project_torch(q, cam, uv);
            const float ix = sample_coord(uv[0], p.colsf, p.inv_cols, p.cols_pow2);
            const float iy = sample_coord(uv[1], p.rowsf, p.inv_rows, p.rows_pow2);
            const float x0 = floorf(ix), y0 = floorf(iy), x1 = x0 + 1.0f, y1 = y0 + 1.0f;
            const float xs[4] = {x0, x1, x0, x1}, ys[4] = {y0, y0, y1, y1};
            const float w[4] = {(x1 - ix) * (y1 - iy), (ix - x0) * (y1 - iy), (x1 - ix) * (iy - y0),
                                (ix - x0) * (iy - y0)};
            // d w / d ix and d w / d iy
            const float wx[4] = {-(y1 - iy), (y1 - iy), -(iy - y0), (iy - y0)};
            const float wy[4] = {-(x1 - ix), -(ix - x0), (x1 - ix), (ix - x0)};
            float tv[4][3], sx[3] = {0, 0, 0}, sy[3] = {0, 0, 0};
            bool in[4];
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                in[t] = xs[t] >= 0.0f && xs[t] < p.colsf && ys[t] >= 0.0f && ys[t] < p.rowsf;
                tv[t][0] = tv[t][1] = tv[t][2] = 0.0f;  // zero padding
                if (in[t]) {
                    const float* v = img + 3 * ((int64_t)(int)ys[t] * p.cols + (int)xs[t]);
#pragma unroll
                    for (int ch = 0; ch < 3; ++ch) tv[t][ch] = v[ch];
                }
#pragma unroll
                for (int ch = 0; ch < 3; ++ch) {
                    sx[ch] += tv[t][ch] * wx[t];
                    sy[ch] += tv[t][ch] * wy[t];
                }
            }
            // the sample as two horizontal interpolations and a vertical one (the value of the four
            // weighted taps): four equal taps give exactly their value, so a sample in a flat
            // region equal to the reference texel has a residual of exactly 0 and the L1 kink's
            // zero subgradient, as in the float64 reference
            const float fx = ix - x0, fy = iy - y0;
            float res[3];
#pragma unroll
            for (int ch = 0; ch < 3; ++ch) {
                const float top = tv[0][ch] + fx * (tv[1][ch] - tv[0][ch]);
                const float bot = tv[2][ch] + fx * (tv[3][ch] - tv[2][ch]);
                res[ch] = top + fy * (bot - top) - r[ch];
            }
            const float cost = fabsf(res[0]) + fabsf(res[1]) + fabsf(res[2]);
            if (cost > 500.0f) continue;  // clamp(max=500) passes no gradient above the bound
            float gs[3];
#pragma unroll
            for (int ch = 0; ch < 3; ++ch) {
                const float sg = res[ch] > 0.0f ? 1.0f : (res[ch] < 0.0f ? -1.0f : 0.0f);
                gs[ch] = g * sg;
                gref[ch] -= gs[ch];
            }
#pragma unroll
            for (int t = 0; t < 4; ++t)
                if (in[t]) {
                    long long* gv = gimg + 3 * ((int64_t)(int)ys[t] * p.cols + (int)xs[t]);
#pragma unroll
                    for (int ch = 0; ch < 3; ++ch) fixed_add(gv + ch, gs[ch] * w[t], scale);
                }
            // d ix / d u = d iy / d v = 1 (the normalisation round trip is the identity)
            const float gu = gs[0] * sx[0] + gs[1] * sx[1] + gs[2] * sx[2];
            const float gv = gs[0] * sy[0] + gs[1] * sy[1] + gs[2] * sy[2];
            float ju[3], jv[3];
            project_jacobian(q, cam, ju, jv);
            const float gp[3] = {gu * ju[0] + gv * jv[0], gu * ju[1] + gv * jv[1], gu * ju[2] + gv * jv[2]};
            // source camera: p' = exp(-delta) p  ->  dL/domega = g x p, dL/dv = -g
            gsrc[0] += gp[1] * q[2] - gp[2] * q[1];
            gsrc[1] += gp[2] * q[0] - gp[0] * q[2];
            gsrc[2] += gp[0] * q[1] - gp[1] * q[0];
            gsrc[3] -= gp[0];
            gsrc[4] -= gp[1];
            gsrc[5] -= gp[2];
            // reference camera: p' = R (exp(delta) p_ref) + t  ->  with h = R^T g:
            // dL/domega = p_ref x h, dL/dv = h
            const float h[3] = {rt[0] * gp[0] + rt[4] * gp[1] + rt[8] * gp[2],
                                rt[1] * gp[0] + rt[5] * gp[1] + rt[9] * gp[2],
                                rt[2] * gp[0] + rt[6] * gp[1] + rt[10] * gp[2]};
            gref6[0] += pv[1] * h[2] - pv[2] * h[1];
            gref6[1] += pv[2] * h[0] - pv[0] * h[2];
            gref6[2] += pv[0] * h[1] - pv[1] * h[0];
            gref6[3] += h[0];
            gref6[4] += h[1];
            gref6[5] += h[2];
        }
        long long* gr = image_acc + ((int64_t)p.reference * P + i) * 3;
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) fixed_add(gr + ch, gref[ch], scale);
    }
    // the pose gradient of the block, per camera: a pixel's candidates were summed in float32;
    // pixels are summed in float64 by a fixed shuffle tree per warp and the warps in order
    __shared__ double warp_sum[kBwdBlock / 32][6];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int c = 0; c < p.ncam; ++c) {
        double v[6];
#pragma unroll
        for (int j = 0; j < 6; ++j) {
            v[j] = 0.0;
            if (active && sel == c) v[j] += (double)gsrc[j];
            if (active && c == p.reference) v[j] += (double)gref6[j];
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1)
#pragma unroll
            for (int j = 0; j < 6; ++j) v[j] += __shfl_down_sync(0xFFFFFFFFu, v[j], off);
        if (lane == 0)
#pragma unroll
            for (int j = 0; j < 6; ++j) warp_sum[warp][j] = v[j];
        __syncthreads();
        if (threadIdx.x < 6) {
            double t = 0.0;
            for (int w = 0; w < kBwdBlock / 32; ++w) t += warp_sum[w][threadIdx.x];
            pose_partial[((int64_t)blockIdx.x * p.ncam + c) * 6 + threadIdx.x] = t;
        }
        __syncthreads();
    }
}

// grad_images[c] += image_acc[c] * 2^-e, every camera (NaN where the incoming gradient was not finite)
struct GradImages {
    float* ptr[SSG_MAX_CAMERAS];
};

__global__ void __launch_bounds__(kBwdBlock) image_grad_convert_kernel(const long long* __restrict__ image_acc,
                                                                       int64_t per_camera, int cameras,
                                                                       const uint32_t* __restrict__ absmax,
                                                                       double count, GradImages out)
{
    const float scale = fixed_scale(*absmax, count);
    const bool finite = __uint_as_float(*absmax) <= 3.0e38f;
    const float inv = scale > 0.0f ? 1.0f / scale : 0.0f;  // a power of two: exact
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < per_camera * cameras;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(k / per_camera);
        const int64_t e = k - (int64_t)c * per_camera;
        const long long q = image_acc[k];
        if (!finite) out.ptr[c][e] = __int_as_float(0x7FFFFFFF);
        else if (q) out.ptr[c][e] += __ll2float_rn(q) * inv;
    }
}

// grad_pose[c][j] += the block sums in block order
__global__ void pose_grad_sum_kernel(const double* __restrict__ pose_partial, int blocks, int cameras,
                                     double* __restrict__ grad_pose)
{
    const int k = threadIdx.x;
    if (k >= cameras * 6) return;
    double t = 0.0;
    for (int b = 0; b < blocks; ++b) t += pose_partial[(int64_t)b * cameras * 6 + k];
    grad_pose[k] += t;
}

static SoftParams soft_params(const float* candidates, int ncand, float tau)
{
    SoftParams sp{};
    sp.ncand = ncand;
    sp.tau = tau;
    for (int k = 0; k < ncand; ++k) sp.inv_cand[k] = 1.0f / candidates[k];
    return sp;
}

}  // namespace ssg

using namespace ssg;

static int check_up_sizes(int rows_in, int cols_in, int rows_io, int cols_io)
{
    SSG_REQUIRE(rows_in > 0 && cols_in > 0 && rows_io > 0 && cols_io > 0, "sizes must be positive");
    SSG_REQUIRE(2 * (rows_in - 1) < rows_io && 2 * (cols_in - 1) < cols_io && (rows_io + 1) / 2 <= rows_in &&
                    (cols_io + 1) / 2 <= cols_in,
                "coarse %dx%d does not match fine %dx%d", rows_in, cols_in, rows_io, cols_io);
    return SSG_OK;
}

extern "C" int ssg_isb_upsample_softargmin(const uint8_t* d_guide_in, const float* d_cost_in, int rows_in, int cols_in,
                                           const uint8_t* d_guide_fine, const float* d_cost_fine, int rows_fine,
                                           int cols_fine, int candidate_count, float weight_up, float weight_down,
                                           float var_inv_i, const float* candidates, float temperature,
                                           float* d_inverse_distance, void* stream)
{
    SSG_REQUIRE(d_guide_in && d_cost_in && d_guide_fine && d_cost_fine && candidates && d_inverse_distance,
                "null pointer");
    if (int e = check_up_sizes(rows_in, cols_in, rows_fine, cols_fine)) return e;
    SSG_REQUIRE(candidate_count >= 1 && candidate_count <= SSG_MAX_CANDIDATES, "candidate_count out of range");
    SSG_REQUIRE(temperature > 0.0f, "temperature must be positive");
    const SoftParams sp = soft_params(candidates, candidate_count, temperature);
    isb_up_softargmin_kernel<<<grid_1d((int64_t)rows_in * cols_in, kBwdBlock), kBwdBlock, 0, as_stream(stream)>>>(
        d_guide_in, d_cost_in, rows_in, cols_in, d_guide_fine, d_cost_fine, rows_fine, cols_fine, weight_up,
        weight_down, var_inv_i, sp, d_inverse_distance);
    return launch_status("isb_up_softargmin_kernel");
}

extern "C" int ssg_isb_upsample_softargmin_backward(const uint8_t* d_guide_in, const float* d_cost_in, int rows_in,
                                                    int cols_in, const uint8_t* d_guide_fine, const float* d_cost_fine,
                                                    int rows_fine, int cols_fine, int candidate_count,
                                                    float weight_up, float weight_down, float var_inv_i,
                                                    const float* candidates, float temperature,
                                                    const float* d_grad_inverse_distance, float* d_grad_filtered_fine,
                                                    void* stream)
{
    SSG_REQUIRE(d_guide_in && d_cost_in && d_guide_fine && d_cost_fine && candidates && d_grad_inverse_distance &&
                    d_grad_filtered_fine,
                "null pointer");
    if (int e = check_up_sizes(rows_in, cols_in, rows_fine, cols_fine)) return e;
    SSG_REQUIRE(candidate_count >= 1 && candidate_count <= SSG_MAX_CANDIDATES, "candidate_count out of range");
    SSG_REQUIRE(temperature > 0.0f, "temperature must be positive");
    const SoftParams sp = soft_params(candidates, candidate_count, temperature);
    isb_up_softargmin_backward_kernel<<<grid_1d((int64_t)rows_in * cols_in, kBwdBlock), kBwdBlock, 0,
                                        as_stream(stream)>>>(d_guide_in, d_cost_in, rows_in, cols_in, d_guide_fine,
                                                             d_cost_fine, rows_fine, cols_fine, weight_up, weight_down,
                                                             var_inv_i, sp, d_grad_inverse_distance,
                                                             d_grad_filtered_fine);
    return launch_status("isb_up_softargmin_backward_kernel");
}

extern "C" int ssg_isb_upsample_transpose(const uint8_t* d_guide_coarse, int rows_in, int cols_in,
                                          const uint8_t* d_guide_fine, int rows_fine, int cols_fine,
                                          int candidate_count, float weight_up, float weight_down, float var_inv_i,
                                          const float* d_grad_filtered_fine, float* d_grad_cost_fine,
                                          float* d_grad_filtered_coarse, void* stream)
{
    SSG_REQUIRE(d_guide_coarse && d_guide_fine && d_grad_filtered_fine && d_grad_cost_fine && d_grad_filtered_coarse,
                "null pointer");
    if (int e = check_up_sizes(rows_in, cols_in, rows_fine, cols_fine)) return e;
    SSG_REQUIRE(candidate_count >= 1, "candidate_count must be positive");
    isb_up_transpose_kernel<<<grid_1d((int64_t)rows_in * cols_in, kBwdBlock), kBwdBlock, 0, as_stream(stream)>>>(
        d_guide_coarse, rows_in, cols_in, d_guide_fine, rows_fine, cols_fine, candidate_count, weight_up, weight_down,
        var_inv_i, d_grad_filtered_fine, d_grad_cost_fine, d_grad_filtered_coarse);
    return launch_status("isb_up_transpose_kernel");
}

extern "C" int ssg_isb_downsample_transpose(const uint8_t* d_guide_in, int rows_in, int cols_in, int rows_out,
                                            int cols_out, int candidate_count, float var_inv_i,
                                            const float* d_grad_cost_coarse, float* d_grad_cost_fine, void* stream)
{
    SSG_REQUIRE(d_guide_in && d_grad_cost_coarse && d_grad_cost_fine, "null pointer");
    if (int e = check_up_sizes(rows_out, cols_out, rows_in, cols_in)) return e;
    SSG_REQUIRE(candidate_count >= 1, "candidate_count must be positive");
    isb_down_transpose_kernel<<<grid_1d((int64_t)rows_in * cols_in, kBwdBlock), kBwdBlock, 0, as_stream(stream)>>>(
        d_guide_in, rows_in, cols_in, rows_out, cols_out, candidate_count, var_inv_i, d_grad_cost_coarse,
        d_grad_cost_fine);
    return launch_status("isb_down_transpose_kernel");
}

// scratch of ssg_sweep_cost_backward: the largest |dL/dcost| (256 bytes), the fixed-point image
// sums (camera_count x pixels x 3 int64) and the block sums of the pose gradient
static int64_t sweep_backward_blocks(int cols, int rows) { return grid_1d((int64_t)cols * rows, kBwdBlock); }

extern "C" size_t ssg_sweep_backward_scratch_bytes(int cols, int rows, int camera_count)
{
    if (cols <= 0 || rows <= 0 || camera_count < 1 || camera_count > SSG_MAX_CAMERAS) return 0;
    const int64_t P = (int64_t)cols * rows;
    return (size_t)(256 + (int64_t)camera_count * P * 3 * 8 +
                    sweep_backward_blocks(cols, rows) * camera_count * 6 * 8);
}

extern "C" int ssg_sweep_cost_backward(int cols, int rows, int camera_count, const ssg_camera* cameras, int reference,
                                       const float* relative_poses, const float* const* d_images,
                                       float* const* d_grad_images, const int8_t* d_selected,
                                       const float* candidates, int candidate_count, const float* d_grad_cost,
                                       double* d_grad_pose, void* d_scratch, void* stream)
{
    SSG_REQUIRE(cols > 0 && rows > 0, "resolution must be positive");
    SSG_REQUIRE(cameras && relative_poses && d_images && d_grad_images && d_selected && candidates && d_grad_cost &&
                    d_grad_pose && d_scratch,
                "null pointer");
    SSG_REQUIRE(((uintptr_t)d_scratch & 255) == 0, "d_scratch must be 256-byte aligned");
    SSG_REQUIRE(camera_count >= 1 && camera_count <= SSG_MAX_CAMERAS, "camera_count out of range");
    SSG_REQUIRE(reference >= 0 && reference < camera_count, "reference out of range");
    SSG_REQUIRE(candidate_count >= 1 && candidate_count <= SSG_MAX_CANDIDATES, "candidate_count out of range");
    SweepBwdParams p{};
    p.cols = cols;
    p.rows = rows;
    p.ncam = camera_count;
    p.ncand = candidate_count;
    p.reference = reference;
    p.colsf = (float)cols;
    p.rowsf = (float)rows;
    p.cols_pow2 = (cols & (cols - 1)) == 0;
    p.rows_pow2 = (rows & (rows - 1)) == 0;
    p.inv_cols = 1.0f / (float)cols;
    p.inv_rows = 1.0f / (float)rows;
    p.ref = make_torch_cam(cameras[reference]);
    GradImages out{};
    for (int c = 0; c < camera_count; ++c) {
        SSG_REQUIRE(d_images[c] && d_grad_images[c], "image %d or its gradient is NULL", c);
        p.cams[c] = make_torch_cam(cameras[c]);
        p.images[c] = d_images[c];
        out.ptr[c] = d_grad_images[c];
        std::memcpy(p.rt[c], relative_poses + 12 * c, sizeof(float) * 12);
    }
    for (int k = 0; k < candidate_count; ++k) p.cand[k] = candidates[k];
    const int64_t P = (int64_t)cols * rows;
    const int64_t blocks = sweep_backward_blocks(cols, rows);
    uint8_t* scratch = static_cast<uint8_t*>(d_scratch);
    uint32_t* absmax = reinterpret_cast<uint32_t*>(scratch);
    long long* image_acc = reinterpret_cast<long long*>(scratch + 256);
    double* pose_partial = reinterpret_cast<double*>(scratch + 256 + (int64_t)camera_count * P * 3 * 8);
    cudaStream_t st = as_stream(stream);
    const cudaError_t e = cudaMemsetAsync(scratch, 0, 256 + (size_t)camera_count * P * 3 * 8, st);
    if (e != cudaSuccess) return fail(SSG_ERR_CUDA, "cudaMemsetAsync: %s", cudaGetErrorString(e));
    const int64_t volume = P * candidate_count;
    absmax_kernel<<<(unsigned)std::min<int64_t>(grid_1d(volume, kBwdBlock), 4096), kBwdBlock, 0, st>>>(d_grad_cost,
                                                                                                       volume, absmax);
    sweep_backward_kernel<<<(unsigned)blocks, kBwdBlock, 0, st>>>(p, d_selected, d_grad_cost, absmax, image_acc,
                                                                  pose_partial);
    const double count = 2.0 * (double)P * candidate_count;  // the sweep kernel's bound
    image_grad_convert_kernel<<<(unsigned)std::min<int64_t>(grid_1d(P * 3 * camera_count, kBwdBlock), 8192),
                                kBwdBlock, 0, st>>>(image_acc, P * 3, camera_count, absmax, count, out);
    pose_grad_sum_kernel<<<1, 32 * ((camera_count * 6 + 31) / 32), 0, st>>>(pose_partial, (int)blocks, camera_count,
                                                                             d_grad_pose);
    return launch_status("sweep_backward_kernel");
}
