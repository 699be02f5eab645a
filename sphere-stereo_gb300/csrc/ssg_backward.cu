// Differentiable sweep: soft-argmin inverse distance and its backward pass.
//
// Forward (no counterpart in the reference, whose selection is a hard argmin + parabola,
// python/depth_estimation.py:179-198): the fp32 sweep and ISB filter of ssg_sweep.cu /
// ssg_isb.cu, then per pixel q = sum_k softmax(-F_k / tau) / d_k over the filtered costs F,
// fused with the last filter level.
//
// Backward, with the cost volume recomputed instead of stored:
//   * seed: the last level recomputes F, runs an online softmax over the candidates (two passes)
//     and writes dL/dF mapped through the level's linear operator: its own-pixel part to the
//     level-0 cost gradient, its coarse-tap part to the level-1 gradient (atomic adds);
//   * the ISB filter is linear in the cost for a fixed guide (its weights come from uint8 guides
//     and get no gradient), so each up step and each down step is run transposed, from the
//     coarsest level back to level 0;
//   * the sweep's backward recomputes every sample, maps dL/dcost through the clamp, the L1 and
//     the bilinear sample to the images (atomic scatter into the source image, direct sum into
//     the reference image) and through the double-sphere projection to the 6-DoF pose deltas of
//     the source and reference cameras, reduced per block and added in float64.
// Pose deltas are right perturbations, T_c <- T_c exp(delta_c), delta = (omega, v): the
// relative pose reference -> camera becomes exp(-delta_c) rel exp(delta_ref).
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

// dL/dF of the soft-argmin, pushed through the last level: level-0 part (own pixel) written,
// level-1 part (coarse taps) added atomically.
__global__ void __launch_bounds__(kBwdBlock) isb_up_softargmin_backward_kernel(
    const uint8_t* __restrict__ guide_in, const float* __restrict__ cost_in, int rows_in, int cols_in,
    const uint8_t* __restrict__ guide_fine, const float* __restrict__ cost_fine, int rows_io, int cols_io,
    float weight_up, float weight_down, float var_inv_i, const __grid_constant__ SoftParams sp,
    const float* __restrict__ grad_q, float* __restrict__ grad_c0, float* __restrict__ grad_f1)
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
    float qv[4], gq[4], own[4];
#pragma unroll
    for (int f = 0; f < 4; ++f) {
        qv[f] = u.set[f] ? sm[f].t / sm[f].s : 0.0f;
        gq[f] = u.set[f] ? grad_q[u.fidx[f]] : 0.0f;
        own[f] = weight_up * u.inv[f];  // d F / d (level-0 cost) of the own pixel
    }
    // normalised coarse-tap weights of each fine pixel
    float w1[9], w2[6], w3[6], w4[4];
#pragma unroll
    for (int i = 0; i < 9; ++i) w1[i] = u.w1[i] * u.inv[0];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        w2[i] = u.w2[i] * u.inv[1];
        w3[i] = u.w3[i] * u.inv[2];
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) w4[i] = u.w4[i] * u.inv[3];
    const int64_t c2[6] = SSG_TAPS2(u.cidx);
    const int64_t c3[6] = SSG_TAPS3(u.cidx);
    const int64_t c4[4] = SSG_TAPS4(u.cidx);
    for (int z = 0; z < sp.ncand; ++z) {
        float c[4];
        fine_costs(u, cost_in + (int64_t)z * pin, cost_fine + (int64_t)z * pio, weight_up, c);
        float gF[4];
#pragma unroll
        for (int f = 0; f < 4; ++f) {
            if (!u.set[f]) {
                gF[f] = 0.0f;
                continue;
            }
            const float w = expf(-c[f] * inv_tau - sm[f].m) / sm[f].s;
            gF[f] = gq[f] * (-inv_tau) * w * (sp.inv_cand[z] - qv[f]);
            grad_c0[(int64_t)z * pio + u.fidx[f]] = own[f] * gF[f];
        }
        float* g1 = grad_f1 + (int64_t)z * pin;
#pragma unroll
        for (int i = 0; i < 9; ++i) atomicAdd(g1 + u.cidx[i], w1[i] * gF[0]);
        if (u.set[1])
#pragma unroll
            for (int i = 0; i < 6; ++i) atomicAdd(g1 + c2[i], w2[i] * gF[1]);
        if (u.set[2])
#pragma unroll
            for (int i = 0; i < 6; ++i) atomicAdd(g1 + c3[i], w3[i] * gF[2]);
        if (u.set[3])
#pragma unroll
            for (int i = 0; i < 4; ++i) atomicAdd(g1 + c4[i], w4[i] * gF[3]);
    }
}

// Transpose of one up step s (fine level s, coarse level s + 1):
//   f_s = a * c_s + B f_{s+1}   =>   g_c_s += a * g_f_s ,  g_f_{s+1} += B^T g_f_s
__global__ void __launch_bounds__(kBwdBlock) isb_up_transpose_kernel(
    const uint8_t* __restrict__ guide_coarse, int rows_in, int cols_in, const uint8_t* __restrict__ guide_fine,
    int rows_io, int cols_io, int ncand, float weight_up, float weight_down, float var_inv_i,
    const float* __restrict__ grad_f_fine, float* __restrict__ grad_c_fine, float* __restrict__ grad_f_coarse)
{
    const int64_t pin = (int64_t)rows_in * cols_in, pio = (int64_t)rows_io * cols_io;
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= pin) return;
    UpWeights u;
    up_weights(guide_coarse, rows_in, cols_in, const_cast<uint8_t*>(guide_fine), rows_io, cols_io, (int)(o % cols_in),
               (int)(o / cols_in), weight_up, weight_down, var_inv_i, false, u);
    float own[4], w1[9], w2[6], w3[6], w4[4];
#pragma unroll
    for (int f = 0; f < 4; ++f) own[f] = weight_up * u.inv[f];
#pragma unroll
    for (int i = 0; i < 9; ++i) w1[i] = u.w1[i] * u.inv[0];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        w2[i] = u.w2[i] * u.inv[1];
        w3[i] = u.w3[i] * u.inv[2];
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) w4[i] = u.w4[i] * u.inv[3];
    const int64_t c2[6] = SSG_TAPS2(u.cidx);
    const int64_t c3[6] = SSG_TAPS3(u.cidx);
    const int64_t c4[4] = SSG_TAPS4(u.cidx);
    for (int z = 0; z < ncand; ++z) {
        const float* gf = grad_f_fine + (int64_t)z * pio;
        float* gc = grad_c_fine + (int64_t)z * pio;
        float* g1 = grad_f_coarse + (int64_t)z * pin;
        float g[4];
#pragma unroll
        for (int f = 0; f < 4; ++f) {
            g[f] = u.set[f] ? gf[u.fidx[f]] : 0.0f;
            if (u.set[f]) gc[u.fidx[f]] += own[f] * g[f];
        }
#pragma unroll
        for (int i = 0; i < 9; ++i) atomicAdd(g1 + u.cidx[i], w1[i] * g[0]);
        if (u.set[1])
#pragma unroll
            for (int i = 0; i < 6; ++i) atomicAdd(g1 + c2[i], w2[i] * g[1]);
        if (u.set[2])
#pragma unroll
            for (int i = 0; i < 6; ++i) atomicAdd(g1 + c3[i], w3[i] * g[2]);
        if (u.set[3])
#pragma unroll
            for (int i = 0; i < 4; ++i) atomicAdd(g1 + c4[i], w4[i] * g[3]);
    }
}

// Transpose of one down step s (fine level s - 1, coarse level s):
//   c_s[o] = sum_t w_t c_{s-1}[idx_t] / wsum   =>   g_c_{s-1}[idx_t] += w_t / wsum * g_c_s[o]
__global__ void __launch_bounds__(kBwdBlock) isb_down_transpose_kernel(const uint8_t* __restrict__ guide_in,
                                                                       int rows_in, int cols_in, int rows_out,
                                                                       int cols_out, int ncand, float var_inv_i,
                                                                       const float* __restrict__ grad_c_coarse,
                                                                       float* __restrict__ grad_c_fine)
{
    const int64_t pout = (int64_t)rows_out * cols_out, pin = (int64_t)rows_in * cols_in;
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= pout) return;
    const int x = (int)(o % cols_out), y = (int)(o / cols_out);
    const int x2 = 2 * x, y2 = 2 * y;
    const int px = min(x2 + 1, cols_in - 1), py = min(y2 + 1, rows_in - 1);
    const int mx = max(x2 - 1, 0), my = max(y2 - 1, 0);
    const int64_t idx[9] = {(int64_t)y2 * cols_in + x2,  (int64_t)my * cols_in + mx, (int64_t)y2 * cols_in + mx,
                            (int64_t)py * cols_in + mx,  (int64_t)py * cols_in + x2, (int64_t)py * cols_in + px,
                            (int64_t)y2 * cols_in + px,  (int64_t)my * cols_in + px, (int64_t)my * cols_in + x2};
    float cur[3];
    load_guide(guide_in, idx[0], cur);
    const float base[8] = {0.25f, 0.5f, 0.25f, 0.5f, 0.25f, 0.5f, 0.25f, 0.5f};
    float w[9];
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
    (void)pin;
    for (int z = 0; z < ncand; ++z) {
        const float g = grad_c_coarse[(int64_t)z * pout + o];
        if (g == 0.0f) continue;
        float* gf = grad_c_fine + (int64_t)z * pin;
#pragma unroll
        for (int t = 0; t < 9; ++t) atomicAdd(gf + idx[t], w[t] * g);
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
    float* grad_images[SSG_MAX_CAMERAS];
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

__global__ void __launch_bounds__(kBwdBlock) sweep_backward_kernel(const __grid_constant__ SweepBwdParams p,
                                                                   const int8_t* __restrict__ selected,
                                                                   const float* __restrict__ grad_cost,
                                                                   double* __restrict__ grad_pose)
{
    // the extrinsic-gradient reduction in float64: a pixel's candidates are summed in float32,
    // pixels and blocks in float64
    __shared__ double pose_acc[SSG_MAX_CAMERAS][6];
    for (int j = threadIdx.x; j < SSG_MAX_CAMERAS * 6; j += blockDim.x) (&pose_acc[0][0])[j] = 0.0;
    __syncthreads();
    const int64_t P = (int64_t)p.cols * p.rows;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int sel = i < P ? selected[i] : -1;
    if (i < P && sel >= 0 && sel < p.ncam) {
        float pu[3];
        unproject_torch((float)(i % p.cols), (float)(i / p.cols), p.ref, pu);
        const float* refimg = p.images[p.reference] + 3 * i;
        const float r[3] = {refimg[0], refimg[1], refimg[2]};
        const TorchCam cam = p.cams[sel];
        float rt[12];
#pragma unroll
        for (int j = 0; j < 12; ++j) rt[j] = p.rt[sel][j];
        const float* img = p.images[sel];
        float* gimg = p.grad_images[sel];
        float gref[3] = {0.0f, 0.0f, 0.0f};
        float gsrc[6] = {0, 0, 0, 0, 0, 0}, gref6[6] = {0, 0, 0, 0, 0, 0};
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
                    float* gv = gimg + 3 * ((int64_t)(int)ys[t] * p.cols + (int)xs[t]);
#pragma unroll
                    for (int ch = 0; ch < 3; ++ch) atomicAdd(gv + ch, gs[ch] * w[t]);
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
        float* gr = p.grad_images[p.reference] + 3 * i;
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) atomicAdd(gr + ch, gref[ch]);
#pragma unroll
        for (int j = 0; j < 6; ++j) {
            atomicAdd(&pose_acc[sel][j], (double)gsrc[j]);
            atomicAdd(&pose_acc[p.reference][j], (double)gref6[j]);
        }
    }
    __syncthreads();
    for (int j = threadIdx.x; j < p.ncam * 6; j += blockDim.x) {
        const double v = (&pose_acc[0][0])[j];
        if (v != 0.0) atomicAdd(grad_pose + j, v);
    }
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
                                                    const float* d_grad_inverse_distance, float* d_grad_cost_fine,
                                                    float* d_grad_filtered_coarse, void* stream)
{
    SSG_REQUIRE(d_guide_in && d_cost_in && d_guide_fine && d_cost_fine && candidates && d_grad_inverse_distance &&
                    d_grad_cost_fine && d_grad_filtered_coarse,
                "null pointer");
    if (int e = check_up_sizes(rows_in, cols_in, rows_fine, cols_fine)) return e;
    SSG_REQUIRE(candidate_count >= 1 && candidate_count <= SSG_MAX_CANDIDATES, "candidate_count out of range");
    SSG_REQUIRE(temperature > 0.0f, "temperature must be positive");
    const SoftParams sp = soft_params(candidates, candidate_count, temperature);
    isb_up_softargmin_backward_kernel<<<grid_1d((int64_t)rows_in * cols_in, kBwdBlock), kBwdBlock, 0,
                                        as_stream(stream)>>>(d_guide_in, d_cost_in, rows_in, cols_in, d_guide_fine,
                                                             d_cost_fine, rows_fine, cols_fine, weight_up, weight_down,
                                                             var_inv_i, sp, d_grad_inverse_distance, d_grad_cost_fine,
                                                             d_grad_filtered_coarse);
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
    isb_down_transpose_kernel<<<grid_1d((int64_t)rows_out * cols_out, kBwdBlock), kBwdBlock, 0, as_stream(stream)>>>(
        d_guide_in, rows_in, cols_in, rows_out, cols_out, candidate_count, var_inv_i, d_grad_cost_coarse,
        d_grad_cost_fine);
    return launch_status("isb_down_transpose_kernel");
}

extern "C" int ssg_sweep_cost_backward(int cols, int rows, int camera_count, const ssg_camera* cameras, int reference,
                                       const float* relative_poses, const float* const* d_images,
                                       float* const* d_grad_images, const int8_t* d_selected,
                                       const float* candidates, int candidate_count, const float* d_grad_cost,
                                       double* d_grad_pose, void* stream)
{
    SSG_REQUIRE(cols > 0 && rows > 0, "resolution must be positive");
    SSG_REQUIRE(cameras && relative_poses && d_images && d_grad_images && d_selected && candidates && d_grad_cost &&
                    d_grad_pose,
                "null pointer");
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
    for (int c = 0; c < camera_count; ++c) {
        SSG_REQUIRE(d_images[c] && d_grad_images[c], "image %d or its gradient is NULL", c);
        p.cams[c] = make_torch_cam(cameras[c]);
        p.images[c] = d_images[c];
        p.grad_images[c] = d_grad_images[c];
        std::memcpy(p.rt[c], relative_poses + 12 * c, sizeof(float) * 12);
    }
    for (int k = 0; k < candidate_count; ++k) p.cand[k] = candidates[k];
    const int64_t P = (int64_t)cols * rows;
    sweep_backward_kernel<<<grid_1d(P, kBwdBlock), kBwdBlock, 0, as_stream(stream)>>>(p, d_selected, d_grad_cost,
                                                                                      d_grad_pose);
    return launch_status("sweep_backward_kernel");
}
