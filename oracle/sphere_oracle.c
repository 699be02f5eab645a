/*
 * TEST INFRASTRUCTURE -- the CPU oracle.  Only tests/, the smoke check and the CPU-baseline leg
 * of the benchmark load this code, as the checker; the product library never links it.
 *
 * A plain-C restatement of the reference's per-frame path (sphere sweep + matching cost,
 * ISB filter, distance selection, distance post-filter, stitcher).  Every function cites the
 * reference lines it restates.  Built twice:
 *   REAL=float  -> libsphere_oracle_f32.so: the reference's own arithmetic, operation by
 *                  operation (float32, same evaluation order; fused multiply-adds exactly where
 *                  the reference's torch CPU kernels use them: the 3-component norm and the 4x4
 *                  point transform; see oracle/sphere_oracle.py).  Pinned against the reference
 *                  itself run on this host (tests/golden/).
 *   REAL=double -> libsphere_oracle_f64.so: the same algorithm in float64, for the error
 *                  statements of the fp16/fp32 device paths.
 * Compiled with -ffp-contract=off so that no multiply-add is fused behind the code's back.
 *
 * Races of the reference GPU code get one fixed, documented schedule:
 *   - the distance z-buffer (python/stitcher.cu:181-204) keeps the minimum distance per target
 *     pixel, and drops targets outside the map (the reference writes out of bounds there);
 *   - inpainting (python/stitcher.cu:283-323) is a Jacobi step per launch: every pixel reads the
 *     map as it was before the launch.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef REAL
#define REAL float
#endif

#define IS_F32 (sizeof(REAL) == sizeof(float))
static inline REAL r_sqrt(REAL x) { return IS_F32 ? (REAL)sqrtf((float)x) : (REAL)sqrt((double)x); }
/* Exponential used where the reference calls __expf / expf.  Mode 0 (default): libm, the
 * function the reference's kernels get when compiled for the host; mode 1: the Cody-Waite
 * exponential of the CUDA library (sphere-stereo_gb300/csrc/ssg_common.cuh), restated below
 * operation by operation, so that the oracle and the device agree bit for bit.  Float builds
 * only; the double build always uses libm's exp. */
static int g_exp_mode = 0;
void sso_set_exp_mode(int mode) { g_exp_mode = mode; }

static float scale_by_pow2(float p, int n)
{
    union { int32_t i; float f; } s, a, b;
    if (n > 127) return p * 1.7014118e38f * 2.0f;
    if (n >= -125) { s.i = (n + 127) << 23; return p * s.f; }
    if (n < -152) return 0.0f;
    a.i = (n + 100 + 127) << 23;
    b.i = (-100 + 127) << 23;
    return (p * a.f) * b.f;
}

float sso_cw_expf(float x)
{
    if (!(x == x)) return x;
    if (x > 88.8f) return INFINITY;
    if (x < -104.0f) return 0.0f;
    const float n = rintf(x * 1.44269504088896341f);
    float r = fmaf(n, -0.693145751953125f, x);
    r = fmaf(n, -1.42860682030941723e-06f, r);
    float p = 1.98412698e-04f;
    p = fmaf(p, r, 1.38888889e-03f);
    p = fmaf(p, r, 8.33333333e-03f);
    p = fmaf(p, r, 4.16666667e-02f);
    p = fmaf(p, r, 1.66666667e-01f);
    p = fmaf(p, r, 0.5f);
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    return scale_by_pow2(p, (int)n);
}

static inline REAL r_exp(REAL x)
{
    if (!IS_F32) return (REAL)exp((double)x);
    return g_exp_mode ? (REAL)sso_cw_expf((float)x) : (REAL)expf((float)x);
}
static inline REAL r_sin(REAL x) { return IS_F32 ? (REAL)sinf((float)x) : (REAL)sin((double)x); }
static inline REAL r_cos(REAL x) { return IS_F32 ? (REAL)cosf((float)x) : (REAL)cos((double)x); }
static inline REAL r_fma(REAL a, REAL b, REAL c)
{
    return IS_F32 ? (REAL)fmaf((float)a, (float)b, (float)c) : (REAL)fma((double)a, (double)b, (double)c);
}
static inline REAL r_hypot(REAL a, REAL b) { return IS_F32 ? (REAL)hypotf((float)a, (float)b) : (REAL)hypot(a, b); }
/* norm3df of the CUDA kernels: the correctly rounded Euclidean norm */
static inline REAL r_norm3(REAL a, REAL b, REAL c)
{
    double n = sqrt((double)a * a + (double)b * b + (double)c * c);
    return (REAL)n;
}
static inline REAL r_fmin(REAL a, REAL b) { return IS_F32 ? (REAL)fminf((float)a, (float)b) : (REAL)fmin(a, b); }
static inline REAL r_fmax(REAL a, REAL b) { return IS_F32 ? (REAL)fmaxf((float)a, (float)b) : (REAL)fmax(a, b); }
static inline REAL r_abs(REAL a) { return a < 0 ? -a : a; }

/* __float2int_rn / __float2int_rd: to nearest even / down, NaN -> 0, saturating */
static inline int sat_int(double v)
{
    if (v != v) return 0;
    if (v >= 2147483647.0) return INT32_MAX;
    if (v <= -2147483648.0) return INT32_MIN;
    return (int)v;
}
static inline int rn_int(REAL x) { return sat_int(nearbyint((double)x)); }
static inline int rd_int(REAL x) { return sat_int(floor((double)x)); }

/* ---------------------------------------------------------------------------------------------
 * Camera model, torch form (python/utils.py:57-94).  cam = {fx*s, fy*s, cx*s, cy*s, xi, alpha}:
 * the first four are the float32 products `fl * matching_scale`, `principal * matching_scale`;
 * xi, alpha are the calibration's Python floats, rounded where torch rounds them (a Python
 * scalar meets a float32 tensor).
 * ------------------------------------------------------------------------------------------- */
typedef struct {
    REAL fx, fy, cx, cy;
    REAL xi, alpha, alpha2, k1, one_minus_xi2, one_minus_alpha, minus_w2;
} torch_cam;

static torch_cam make_torch_cam(const double* c)
{
    torch_cam k;
    double xi = c[4], al = c[5];
    k.fx = (REAL)c[0]; k.fy = (REAL)c[1]; k.cx = (REAL)c[2]; k.cy = (REAL)c[3];
    k.xi = (REAL)xi; k.alpha = (REAL)al;
    k.alpha2 = (REAL)(al * al);                 /* calib.alpha**2          utils.py:65 */
    k.k1 = (REAL)(2 * al - 1);                  /* (2 * calib.alpha - 1)   utils.py:66,72 */
    k.one_minus_xi2 = (REAL)(1 - xi * xi);      /* (1 - calib.xi**2)       utils.py:69 */
    k.one_minus_alpha = (REAL)(1 - al);         /* (1 - calib.alpha)       utils.py:84 */
    double w1 = al > 0.5 ? (1 - al) / al : al / (1 - al);          /* utils.py:86-89 */
    double w2 = (w1 + xi) / sqrt(2 * w1 * xi + xi * xi + 1);       /* utils.py:90 */
    k.minus_w2 = (REAL)(-w2);
    return k;
}

/* utils.py:57-73 */
static int unproject_torch(REAL u, REAL v, const torch_cam* k, REAL p[3])
{
    REAL mx = (u - k->cx) / k->fx;
    REAL my = (v - k->cy) / k->fy;
    REAL r2 = mx * mx + my * my;
    REAL disc = 1 - k->k1 * r2;
    REAL mz = (1 - k->alpha2 * r2) / (k->alpha * r_sqrt(disc > 0 ? disc : 0) + 1 - k->alpha);
    REAL mz2 = mz * mz;
    REAL s = (mz * k->xi + r_sqrt(mz2 + k->one_minus_xi2 * r2)) / (mz2 + r2);
    p[0] = s * mx;
    p[1] = s * my;
    p[2] = s * mz - k->xi;
    return disc >= 0;
}

/* torch.norm(., dim=-1) of a 3-vector on the reference's CPU kernels: fma(z, z, fma(y, y, x*x)) */
static inline REAL norm3_torch(REAL x, REAL y, REAL z) { return r_sqrt(r_fma(z, z, r_fma(y, y, x * x))); }

/* utils.py:75-94 */
static int project_torch(const REAL p[3], const torch_cam* k, REAL uv[2])
{
    REAL d1 = norm3_torch(p[0], p[1], p[2]);
    REAL c = k->xi * d1 + p[2];
    REAL d2 = norm3_torch(p[0], p[1], c);
    REAL nrm = k->alpha * d2 + k->one_minus_alpha * c;
    uv[0] = (k->fx * p[0]) / nrm + k->cx;
    uv[1] = (k->fy * p[1]) / nrm + k->cy;
    return p[2] > k->minus_w2 * d1;
}

/* [p, 1] @ rt.T on the reference's CPU matmul: fma chain over x, y, z, then + t.
 * rt = 12 floats, rows 0..2 of torch.matmul(torch.inverse(cam.rt), ref.rt). */
static inline void transform_torch(const float* rt, const REAL p[3], REAL q[3])
{
    for (int i = 0; i < 3; ++i) {
        REAL acc = p[0] * (REAL)rt[4 * i + 0];
        acc = r_fma(p[1], (REAL)rt[4 * i + 1], acc);
        acc = r_fma(p[2], (REAL)rt[4 * i + 2], acc);
        q[i] = acc + (REAL)rt[4 * i + 3];
    }
}

/* utils.py:144-155 then .type(torch.uint8) (depth_estimation.py:227).  rgb: n x 3 channels as
 * stored (the reference's images come from cv2, i.e. BGR order; coefficients apply to the stored
 * channel order). */
void sso_rgb2ycbcr(const REAL* rgb, long n, uint8_t* guide)
{
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i) {
        REAL c0 = rgb[3 * i], c1 = rgb[3 * i + 1], c2 = rgb[3 * i + 2];
        REAL y = 16 + (REAL)0.1826f * c0 + (REAL)0.6142f * c1 + (REAL)0.062f * c2;
        REAL cb = 128 - (REAL)0.1006f * c0 - (REAL)0.3386f * c1 + (REAL)0.4392f * c2;
        REAL cr = 128 + (REAL)0.4392f * c0 - (REAL)0.3989f * c1 - (REAL)0.0403f * c2;
        if (!IS_F32) {
            y = 16 + 0.1826 * c0 + 0.6142 * c1 + 0.062 * c2;
            cb = 128 - 0.1006 * c0 - 0.3386 * c1 + 0.4392 * c2;
            cr = 128 + 0.4392 * c0 - 0.3989 * c1 - 0.0403 * c2;
        }
        y = y < 16 ? 16 : (y > 235 ? 235 : y);
        cb = cb < 16 ? 16 : (cb > 240 ? 240 : cb);
        cr = cr < 16 ? 16 : (cr > 240 ? 240 : cr);
        guide[3 * i] = (uint8_t)y;
        guide[3 * i + 1] = (uint8_t)cb;
        guide[3 * i + 2] = (uint8_t)cr;
    }
}

/* unproject of every pixel of a W x H grid (python/utils.py:57-73 on the meshgrid of
 * depth_estimation.py:141-143); rays: H*W*3, valid: H*W */
void sso_unproject_grid(int W, int H, const double* cam, REAL* rays, uint8_t* valid)
{
    torch_cam k = make_torch_cam(cam);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)W * H; ++i) {
        REAL p[3];
        int v = unproject_torch((REAL)(i % W), (REAL)(i / W), &k, p);
        rays[3 * i] = p[0]; rays[3 * i + 1] = p[1]; rays[3 * i + 2] = p[2];
        valid[i] = (uint8_t)v;
    }
}

/* grid_sample, 4-D input [1,1,H,W], bilinear, zero padding, align_corners=False, at pixel uv
 * after the reference's normalisation ((uv + 0.5) / [W, H]) * 2 - 1 (depth_estimation.py:117-123) */
static REAL sample_mask(const REAL* mask, int W, int H, REAL u, REAL v)
{
    REAL gx = ((u + (REAL)0.5) / (REAL)W) * 2 - 1;
    REAL gy = ((v + (REAL)0.5) / (REAL)H) * 2 - 1;
    REAL ix = ((gx + 1) * (REAL)W - 1) / 2;
    REAL iy = ((gy + 1) * (REAL)H - 1) / 2;
    REAL x0 = floor(ix), y0 = floor(iy), x1 = x0 + 1, y1 = y0 + 1;
    REAL nw = (x1 - ix) * (y1 - iy), ne = (ix - x0) * (y1 - iy);
    REAL sw = (x1 - ix) * (iy - y0), se = (ix - x0) * (iy - y0);
    REAL xs[4] = {x0, x1, x0, x1}, ys[4] = {y0, y0, y1, y1}, ws[4] = {nw, ne, sw, se};
    REAL out = 0;
    for (int t = 0; t < 4; ++t) {
        if (xs[t] >= 0 && xs[t] < W && ys[t] >= 0 && ys[t] < H)
            out = out + mask[(long)ys[t] * W + (long)xs[t]] * ws[t];
    }
    return out;
}

/* RGBD_Estimator.select_camera for one reference (depth_estimation.py:83-135).
 * cams: C x 6 (see torch_cam); rts: C x 12; masks: C x H x W; selected: H x W (-1 = none). */
void sso_select_camera(int W, int H, int C, const double* cams, int ref, const float* rts, const REAL* masks,
                       double min_dist, double max_dist, int8_t* selected)
{
    torch_cam kr = make_torch_cam(cams + 6 * ref);
    const REAL dmin = (REAL)min_dist, dmax = (REAL)max_dist;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)W * H; ++i) {
        REAL pu[3];
        int ref_valid = unproject_torch((REAL)(i % W), (REAL)(i / W), &kr, pu);
        REAL max_disp = 1;
        int sel = -1;
        for (int c = 0; c < C; ++c) {
            torch_cam kc = make_torch_cam(cams + 6 * c);
            REAL pn[3] = {pu[0] * dmin, pu[1] * dmin, pu[2] * dmin};
            REAL pf[3] = {pu[0] * dmax, pu[1] * dmax, pu[2] * dmax};
            REAL qn[3], qf[3];
            transform_torch(rts + 12 * c, pn, qn);
            transform_torch(rts + 12 * c, pf, qf);
            REAL nn = norm3_torch(qn[0], qn[1], qn[2]), nf = norm3_torch(qf[0], qf[1], qf[2]);
            for (int j = 0; j < 3; ++j) { qn[j] = qn[j] / nn; qf[j] = qf[j] / nf; }
            REAL un[2], uf[2];
            int vn = project_torch(qn, &kc, un);
            int vf = project_torch(qf, &kc, uf);
            REAL dx = un[0] - uf[0], dy = un[1] - uf[1];
            REAL disp = r_sqrt(r_fma(dy, dy, dx * dx));
            const REAL* m = masks + (long)c * W * H;
            REAL mn = sample_mask(m, W, H, un[0], un[1]);
            REAL mf = sample_mask(m, W, H, uf[0], uf[1]);
            int best = (disp > max_disp) && ref_valid && vn && vf && (masks[(long)ref * W * H + i] >= (REAL)0.9f)
                       && (mn >= (REAL)0.9f) && (mf >= (REAL)0.9f);
            if (best) { max_disp = disp; sel = c; }
        }
        selected[i] = (int8_t)sel;
    }
}

/* Sphere sweep + matching cost for one reference (depth_estimation.py:141-175).
 * images: C x H x W x 3 (float [0,255], channel order as stored); selected: H*W;
 * candidates: N (1 / linspace(1/min, 1/max, N)); cost: N x H x W. */
void sso_sweep_cost(int W, int H, int C, const double* cams, int ref, const float* rts, const REAL* images,
                    const int8_t* selected, const REAL* candidates, int N, REAL* cost)
{
    torch_cam kr = make_torch_cam(cams + 6 * ref);
    const long P = (long)W * H;
    const REAL* refimg = images + (long)ref * P * 3;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < P; ++i) {
        REAL pu[3];
        unproject_torch((REAL)(i % W), (REAL)(i / W), &kr, pu);
        const int sel = selected[i];
        const REAL r0 = refimg[3 * i], r1 = refimg[3 * i + 1], r2 = refimg[3 * i + 2];
        torch_cam kc;
        if (sel >= 0) kc = make_torch_cam(cams + 6 * sel);
        for (int k = 0; k < N; ++k) {
            REAL s[3] = {0, 0, 0};
            if (sel >= 0) {
                REAL p[3] = {candidates[k] * pu[0], candidates[k] * pu[1], candidates[k] * pu[2]};
                REAL q[3], uv[2];
                transform_torch(rts + 12 * sel, p, q);
                project_torch(q, &kc, uv);
                /* normalisation (depth_estimation.py:160-161) and grid_sample's un-normalisation */
                REAL gx = ((uv[0] + (REAL)0.5) / (REAL)W) * 2 - 1;
                REAL gy = ((uv[1] + (REAL)0.5) / (REAL)H) * 2 - 1;
                REAL ix = ((gx + 1) * (REAL)W - 1) / 2;
                REAL iy = ((gy + 1) * (REAL)H - 1) / 2;
                REAL x0 = floor(ix), y0 = floor(iy), x1 = x0 + 1, y1 = y0 + 1;
                REAL ws[4] = {(x1 - ix) * (y1 - iy), (ix - x0) * (y1 - iy), (x1 - ix) * (iy - y0),
                              (ix - x0) * (iy - y0)};
                REAL xs[4] = {x0, x1, x0, x1}, ys[4] = {y0, y0, y1, y1};
                const REAL* img = images + (long)sel * P * 3;
                for (int t = 0; t < 4; ++t) {
                    if (xs[t] >= 0 && xs[t] < W && ys[t] >= 0 && ys[t] < H) {
                        const REAL* px = img + ((long)ys[t] * W + (long)xs[t]) * 3;
                        for (int ch = 0; ch < 3; ++ch) s[ch] = s[ch] + px[ch] * ws[t];
                    }
                }
            }
            REAL c = (r_abs(s[0] - r0) + r_abs(s[1] - r1)) + r_abs(s[2] - r2);
            cost[(long)k * P + i] = c > 500 ? 500 : c;
        }
    }
}

/* ---------------------------------------------------------------------------------------------
 * ISB filter (python/isb_filter.cu, python/isb_filter.py)
 * ------------------------------------------------------------------------------------------- */
#define ISB_EPS ((REAL)0.01f) /* isb_filter.cu:32 */

static inline REAL abs_sum3(const REAL a[3], const REAL b[3])
{
    return (r_abs(a[0] - b[0]) + r_abs(a[1] - b[1])) + r_abs(a[2] - b[2]);
}

/* guideDownsample2xKernel, isb_filter.cu:44-119 */
void sso_isb_down(const uint8_t* guide_in, const REAL* cost_in, int rows_in, int cols_in, uint8_t* guide_out,
                  REAL* cost_out, int rows_out, int cols_out, int N, REAL var_inv_i)
{
    const long pin = (long)rows_in * cols_in, pout = (long)rows_out * cols_out;
#pragma omp parallel for schedule(static)
    for (long o = 0; o < pout; ++o) {
        int x = (int)(o % cols_out), y = (int)(o / cols_out);
        int x2 = 2 * x, y2 = 2 * y;
        int px = x2 + 1 < cols_in ? x2 + 1 : cols_in - 1, py = y2 + 1 < rows_in ? y2 + 1 : rows_in - 1;
        int mx = x2 - 1 >= 0 ? x2 - 1 : 0, my = y2 - 1 >= 0 ? y2 - 1 : 0;
        const long idx[8] = {(long)my * cols_in + mx, (long)y2 * cols_in + mx, (long)py * cols_in + mx,
                             (long)py * cols_in + x2, (long)py * cols_in + px, (long)y2 * cols_in + px,
                             (long)my * cols_in + px, (long)my * cols_in + x2};
        const long ic = (long)y2 * cols_in + x2;
        REAL cur[3] = {guide_in[3 * ic], guide_in[3 * ic + 1], guide_in[3 * ic + 2]};
        REAL w[8] = {0.25f, 0.5f, 0.25f, 0.5f, 0.25f, 0.5f, 0.25f, 0.5f};
        REAL wsum = 1, g[3] = {cur[0], cur[1], cur[2]};
        for (int i = 0; i < 8; ++i) {
            REAL nb[3] = {guide_in[3 * idx[i]], guide_in[3 * idx[i] + 1], guide_in[3 * idx[i] + 2]};
            REAL d = abs_sum3(cur, nb);
            w[i] = w[i] * (r_exp(-d * d * var_inv_i) + ISB_EPS);
            wsum = wsum + w[i];
            for (int ch = 0; ch < 3; ++ch) g[ch] = g[ch] + nb[ch] * w[i];
        }
        REAL den = 1 / wsum;
        for (int ch = 0; ch < 3; ++ch) guide_out[3 * o + ch] = (uint8_t)(g[ch] * den);
        for (int z = 0; z < N; ++z) {
            const REAL* c = cost_in + (long)z * pin;
            REAL s = c[ic];
            for (int i = 0; i < 8; ++i) s = s + c[idx[i]] * w[i];
            cost_out[(long)z * pout + o] = s / wsum;
        }
    }
}

/* guideUpsample2xKernel, isb_filter.cu:132-329 (coarse level in, fine level in place) */
void sso_isb_up(const uint8_t* guide_in, const REAL* cost_in, int rows_in, int cols_in, uint8_t* guide_io,
                REAL* cost_io, int rows_io, int cols_io, int N, REAL weight_up, REAL weight_down, REAL var_inv_i)
{
    const long pin = (long)rows_in * cols_in, pio = (long)rows_io * cols_io;
#pragma omp parallel for schedule(static)
    for (long o = 0; o < pin; ++o) {
        int x = (int)(o % cols_in), y = (int)(o / cols_in);
        int mdx = x - 1 >= 0 ? x - 1 : 0, mdy = y - 1 >= 0 ? y - 1 : 0;
        int pdx = x + 1 < cols_in ? x + 1 : cols_in - 1, pdy = y + 1 < rows_in ? y + 1 : rows_in - 1;
        int x2 = 2 * x, y2 = 2 * y;
        int pux = x2 + 1 < cols_io ? x2 + 1 : cols_io - 1, puy = y2 + 1 < rows_io ? y2 + 1 : rows_io - 1;
        /* 3x3 coarse neighbourhood, [row][col] */
        const int rr[3] = {mdy, y, pdy}, cc[3] = {mdx, x, pdx};
        REAL gd[3][3][3];
        long cidx[3][3];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                cidx[a][b] = (long)rr[a] * cols_in + cc[b];
                for (int ch = 0; ch < 3; ++ch) gd[a][b][ch] = guide_in[3 * cidx[a][b] + ch];
            }
        /* tap lists of the four fine pixels (isb_filter.cu:155-208) */
        static const int t1[9][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 0}, {1, 1}, {1, 2}, {2, 0}, {2, 1}, {2, 2}};
        static const int t2[6][2] = {{1, 1}, {2, 1}, {1, 0}, {2, 0}, {1, 2}, {2, 2}};
        static const int t3[6][2] = {{1, 1}, {1, 2}, {0, 1}, {0, 2}, {2, 1}, {2, 2}};
        static const int t4[4][2] = {{1, 1}, {1, 2}, {2, 1}, {2, 2}};
        static const REAL b1[9] = {1, 1, 1, 1, 8, 1, 1, 1, 1}, b2[6] = {8, 8, 1, 1, 1, 1},
                          b3[6] = {8, 8, 1, 1, 1, 1}, b4[4] = {1, 1, 1, 1};
        const int (*taps[4])[2] = {t1, t2, t3, t4};
        const REAL* base[4] = {b1, b2, b3, b4};
        const int ntap[4] = {9, 6, 6, 4};
        const long fidx[4] = {(long)y2 * cols_io + x2, (long)puy * cols_io + x2, (long)y2 * cols_io + pux,
                              (long)puy * cols_io + pux};
        const int set[4] = {1, y2 != puy, x2 != pux, (y2 != puy) && (x2 != pux)};
        REAL w[4][9], inv[4];
        for (int f = 0; f < 4; ++f) {
            REAL up[3] = {guide_io[3 * fidx[f]], guide_io[3 * fidx[f] + 1], guide_io[3 * fidx[f] + 2]};
            REAL g[3] = {weight_up * up[0], weight_up * up[1], weight_up * up[2]};
            REAL wsum = weight_up;
            for (int i = 0; i < ntap[f]; ++i) {
                const REAL* nb = gd[taps[f][i][0]][taps[f][i][1]];
                REAL d = abs_sum3(nb, up);
                w[f][i] = base[f][i] * (weight_down * (r_exp(-d * d * var_inv_i) + ISB_EPS));
                for (int ch = 0; ch < 3; ++ch) g[ch] = g[ch] + nb[ch] * w[f][i];
                wsum = wsum + w[f][i];
            }
            inv[f] = 1 / wsum;
            if (set[f])
                for (int ch = 0; ch < 3; ++ch) guide_io[3 * fidx[f] + ch] = (uint8_t)(g[ch] * inv[f]);
        }
        for (int z = 0; z < N; ++z) {
            const REAL* c = cost_in + (long)z * pin;
            REAL* fc = cost_io + (long)z * pio;
            for (int f = 0; f < 4; ++f) {
                if (!set[f]) continue;
                REAL s = weight_up * fc[fidx[f]];
                for (int i = 0; i < ntap[f]; ++i) s = s + w[f][i] * c[cidx[taps[f][i][0]][taps[f][i][1]]];
                fc[fidx[f]] = s * inv[f];
            }
        }
    }
}

/* number of ISB scales, isb_filter.py:60 */
int sso_isb_scale_count(int cols, int rows)
{
    return (int)(fmin(log2((double)cols), log2((double)rows)) - 1);
}

/* ISB_Filter.apply, isb_filter.py:72-136: guide (rows x cols x 3) and cost (N x rows x cols) are
 * filtered in place; the pyramid levels are ceil(dim / 2^s) (isb_filter.py:62-70). */
void sso_isb_apply(uint8_t* guide, REAL* cost, int N, int rows, int cols, double sigma_i, double sigma_s)
{
    const int L = sso_isb_scale_count(cols, rows);
    if (L < 1) return;
    int r[64], c[64];
    uint8_t* g[64];
    REAL* k[64];
    for (int s = 0; s < L; ++s) {
        r[s] = (int)ceil(rows / pow(2.0, s));
        c[s] = (int)ceil(cols / pow(2.0, s));
        if (s == 0) { g[s] = guide; k[s] = cost; }
        else {
            g[s] = (uint8_t*)calloc((size_t)r[s] * c[s] * 3, 1);
            k[s] = (REAL*)calloc((size_t)N * r[s] * c[s], sizeof(REAL));
        }
    }
    const double vs = 1 / (2 * sigma_s * sigma_s), vi = 1 / (2 * sigma_i * sigma_i);
    const REAL var_inv_i = (REAL)(IS_F32 ? (double)(float)vi : vi);
    for (int s = 1; s < L; ++s)
        sso_isb_down(g[s - 1], k[s - 1], r[s - 1], c[s - 1], g[s], k[s], r[s], c[s], N, var_inv_i);
    for (int s = L - 2; s >= 0; --s) {
        double dist = pow(2.0, s) - 0.5;
        double wd = exp(-(dist * dist) * vs);
        double wu = 1 - wd;
        sso_isb_up(g[s + 1], k[s + 1], r[s + 1], c[s + 1], g[s], k[s], r[s], c[s], N, (REAL)wu, (REAL)wd, var_inv_i);
    }
    for (int s = 1; s < L; ++s) { free(g[s]); free(k[s]); }
}

/* Distance selection, depth_estimation.py:179-198: cost N x P -> distance P */
void sso_select_distance(const REAL* cost, int N, long P, const REAL* candidates, REAL* distance, int32_t* index)
{
    const REAL d0 = candidates[0], dl = candidates[N - 1];
    const REAL q = d0 / dl - 1;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < P; ++i) {
        REAL m = cost[i], M = cost[i];
        int idx = 0;
        for (int k = 1; k < N; ++k) {
            REAL c = cost[(long)k * P + i];
            if (c < m) { m = c; idx = k; }
            if (c > M) M = c;
        }
        REAL L = cost[(long)(idx - 1 < 0 ? 0 : idx - 1) * P + i];
        REAL R = cost[(long)(idx + 1 > N - 1 ? N - 1 : idx + 1) * P + i];
        REAL var = ((REAL)0.5 * (L - R)) / (((L + R) - 2 * m) + (REAL)1e-8f);
        if (!IS_F32) var = (0.5 * (L - R)) / (((L + R) - 2 * m) + 1e-8);
        var = var < (REAL)-0.5 ? (REAL)-0.5 : (var > (REAL)0.5 ? (REAL)0.5 : var);
        if (idx == N - 1 || idx == 0) var = 0;
        REAL sel = (REAL)idx + var;
        if (M == m) sel = (REAL)(N - 1);
        REAL d = d0 / ((q * sel) / (REAL)(N - 1) + 1);
        REAL eps = IS_F32 ? (REAL)1e-8f : (REAL)1e-8;
        if (r_abs(M - m) < eps) d = dl;
        distance[i] = d;
        if (index) index[i] = idx;
    }
}

/* ---------------------------------------------------------------------------------------------
 * Stitcher (python/stitcher.cu, python/stitcher.py).  Intrinsics follow the kernels' struct
 * (stitcher.cu:31-35): {fx*s, fy*s, cx*s, cy*s, xi, alpha} as float32 (vectorize_calibration,
 * stitcher.py:35-46).
 * ------------------------------------------------------------------------------------------- */

/* stitcher.cu:121-135 (no clamp of the square root's argument) */
static void unproject_cu(REAL u, REAL v, const float* k, REAL p[3])
{
    const REAL fx = k[0], fy = k[1], cx = k[2], cy = k[3], xi = k[4], al = k[5];
    REAL mx = (u - cx) / fx, my = (v - cy) / fy;
    REAL r2 = mx * mx + my * my;
    REAL mz = (1 - al * al * r2) / (al * r_sqrt(1 - (2 * al - 1) * r2) + 1 - al);
    REAL mz2 = mz * mz;
    REAL s = (mz * xi + r_sqrt(mz2 + (1 - xi * xi) * r2)) / (mz2 + r2);
    p[0] = mx * s; p[1] = my * s; p[2] = mz * s;
    p[2] = p[2] - xi;
}

/* stitcher.cu:140-168; valid (optional) is and-ed with the model's validity test */
static void project_cu(const REAL p[3], const float* k, REAL uv[2], int* valid)
{
    const REAL fx = k[0], fy = k[1], cx = k[2], cy = k[3], xi = k[4], al = k[5];
    REAL d1 = r_norm3(p[0], p[1], p[2]);
    REAL c = xi * d1 + p[2];
    REAL d2 = r_norm3(p[0], p[1], c);
    REAL nrm = al * d2 + (1 - al) * c;
    if (valid) {
        REAL w1 = al > (REAL)0.5 ? (1 - al) / al : al / (1 - al);
        REAL w2 = (w1 + xi) / r_sqrt(2 * w1 * xi + xi * xi + 1);
        *valid = *valid && (p[2] > -w2 * d1);
    }
    REAL den = 1 / nrm;
    uv[0] = (fx * p[0]) * den + cx;
    uv[1] = (fy * p[1]) * den + cy;
}

/* interpF (stitcher.cu:89-116): bilinear, no bounds check (callers clamp) */
static REAL interp_f(const REAL* s, REAL u, REAL v, int cols)
{
    int u1 = rd_int(u), v1 = rd_int(v), u2 = u1 + 1, v2 = v1 + 1;
    REAL u1f = (REAL)u1, u2f = (REAL)u2, v1f = (REAL)v1, v2f = (REAL)v2;
    REAL w1 = (u2f - u) * (v2f - v), w2 = (u2f - u) * (v - v1f), w3 = (u - u1f) * (v2f - v),
         w4 = (u - u1f) * (v - v1f);
    return w1 * s[(long)v1 * cols + u1] + w2 * s[(long)v2 * cols + u1] + w3 * s[(long)v1 * cols + u2]
           + w4 * s[(long)v2 * cols + u2];
}

/* createInpaintingWeightsKernel, stitcher.cu:212-272.  table: H x W x 2 bytes.  Offsets of a
 * slot that keeps weight 0 are undefined in the reference; here they are (0, 0). */
void sso_inpainting_table(int W, int H, const float* k, const float* t, double min_dist, double max_dist,
                          uint8_t* table)
{
    const REAL dmin = (REAL)(float)min_dist, dmax = (REAL)(float)max_dist;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)W * H; ++i) {
        REAL unit[3];
        unproject_cu((REAL)(i % W), (REAL)(i / W), k, unit);
        REAL pc[3] = {dmin * unit[0] - t[0], dmin * unit[1] - t[1], dmin * unit[2] - t[2]};
        REAL pf[3] = {dmax * unit[0] - t[0], dmax * unit[1] - t[1], dmax * unit[2] - t[2]};
        REAL uc[2], uf[2];
        project_cu(pc, k, uc, 0);
        project_cu(pf, k, uf, 0);
        REAL dx = uf[0] - uc[0], dy = uf[1] - uc[1];
        REAL den = 1 / r_hypot(dx, dy);
        dx = dx * den; dy = dy * den;
        int nx[2] = {0, 0}, ny[2] = {0, 0};
        REAL w[2] = {0, 0};
        for (int n = -1; n <= 1; ++n)
            for (int m = -1; m <= 1; ++m) {
                if (!(n || m)) continue;
                REAL pd = 1 / r_hypot((REAL)n, (REAL)m);
                REAL px = (REAL)n * pd, py = (REAL)m * pd;
                REAL wt = px * dx + py * dy;
                if (wt > w[1]) {
                    w[0] = w[1]; nx[0] = nx[1]; ny[0] = ny[1];
                    w[1] = wt; nx[1] = n; ny[1] = m;
                } else if (wt > w[0]) {
                    w[0] = wt; nx[0] = n; ny[0] = m;
                }
            }
        uint8_t q0 = (uint8_t)((uint8_t)(float)(w[0] * (REAL)255.f) & 240);
        uint8_t q1 = (uint8_t)((uint8_t)(float)(w[1] * (REAL)255.f) & 240);
        table[2 * i] = (uint8_t)(q0 + 4 * (uint8_t)(1 + ny[0]) + (uint8_t)(1 + nx[0]));
        table[2 * i + 1] = (uint8_t)(q1 + 4 * (uint8_t)(1 + ny[1]) + (uint8_t)(1 + nx[1]));
    }
}

/* Box filter used at stitcher init (stitcher.py:144-148, :162-164): mean over a
 * (2r+1)^2 window; outside the image the input is pad_value (1 for masks, 0 for weights). */
void sso_box_filter(const REAL* in, int H, int W, int radius, double pad_value, REAL* out)
{
    const REAL kw = IS_F32 ? (REAL)(1.0f / (float)((2 * radius + 1) * (2 * radius + 1)))
                           : (REAL)(1.0 / ((2 * radius + 1) * (2 * radius + 1)));
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)W * H; ++i) {
        int x = (int)(i % W), y = (int)(i / W);
        REAL s = 0;
        for (int dy = -radius; dy <= radius; ++dy)
            for (int dx = -radius; dx <= radius; ++dx) {
                int xx = x + dx, yy = y + dy;
                REAL v = (xx >= 0 && xx < W && yy >= 0 && yy < H) ? in[(long)yy * W + xx] : (REAL)pad_value;
                s = s + v * kw;
            }
        out[i] = s;
    }
}

/* createBlendingLutKernel, stitcher.cu:338-401.  masks: the box-filtered masks, R x H x W;
 * rots: R x 9 (inverse rotations); ts: R x 3; lut: R x Hp x Wp x 2; weights: R x Hp x Wp. */
void sso_blending_lut(int W, int H, int Wp, int Hp, int R, const float* ks, const float* rots, const float* ts,
                      const REAL* masks, double min_dist, double max_dist, REAL* lut, REAL* weights)
{
    const double PI = 3.14159265; /* stitcher.cu:325 */
    const REAL dmin = (REAL)(float)min_dist, dmax = (REAL)(float)max_dist;
    const long Q = (long)Wp * Hp;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < Q; ++i) {
        REAL px = (REAL)(i % Wp), py = (REAL)(i / Wp);
        REAL phi, theta;
        if (IS_F32) {
            phi = (REAL)((double)(float)(py + 0.5f) * PI / Hp - PI / 2.0);
            theta = (REAL)((double)(float)((px + 0.5f) * 2.f) * PI / Wp + PI);
        } else {
            phi = (py + 0.5) * PI / Hp - PI / 2.0;
            theta = (px + 0.5) * 2.0 * PI / Wp + PI;
        }
        REAL cp = r_cos(phi);
        REAL unit[3] = {cp * r_sin(theta), r_sin(phi), cp * r_cos(theta)};
        REAL bw[64], sum = 0;
        for (int r = 0; r < R; ++r) {
            const float* m = rots + 9 * r;
            REAL uf[3];
            for (int a = 0; a < 3; ++a) uf[a] = m[3 * a] * unit[0] + m[3 * a + 1] * unit[1] + m[3 * a + 2] * unit[2];
            int valid = 1;
            REAL uv[2];
            project_cu(uf, ks + 6 * r, uv, &valid);
            uv[0] = r_fmin(r_fmax(uv[0], (REAL)0.1f), (REAL)W - (REAL)1.1f);
            uv[1] = r_fmin(r_fmax(uv[1], (REAL)0.1f), (REAL)H - (REAL)1.1f);
            lut[((long)r * Q + i) * 2] = uv[0];
            lut[((long)r * Q + i) * 2 + 1] = uv[1];
            bw[r] = IS_F32 ? (REAL)1e-8f : (REAL)1e-8;
            const float* t = ts + 3 * r;
            REAL pn3[3] = {dmin * uf[0] - t[0], dmin * uf[1] - t[1], dmin * uf[2] - t[2]};
            REAL pf3[3] = {dmax * uf[0] - t[0], dmax * uf[1] - t[1], dmax * uf[2] - t[2]};
            REAL pn[2], pf[2];
            project_cu(pn3, ks + 6 * r, pn, &valid);
            pn[0] = r_fmin(r_fmax(pn[0], (REAL)0.1f), (REAL)W - (REAL)1.1f);
            pn[1] = (REAL)(r * H) + r_fmin(r_fmax(pn[1], (REAL)0.1f), (REAL)H - (REAL)1.1f);
            project_cu(pf3, ks + 6 * r, pf, &valid);
            pf[0] = r_fmin(r_fmax(pf[0], (REAL)0.1f), (REAL)W - (REAL)1.1f);
            pf[1] = (REAL)(r * H) + r_fmin(r_fmax(pf[1], (REAL)0.1f), (REAL)H - (REAL)1.1f);
            if (valid && interp_f(masks, pn[0], pn[1], W) > 0.99 && interp_f(masks, pf[0], pf[1], W) > 0.99) {
                REAL s = r_hypot(pf[0] - pn[0], pf[1] - pn[1]);
                double e = (double)(-s * s) / (1e-4 * H * W);
                bw[r] = r_exp((REAL)e);
            }
            sum = sum + bw[r];
        }
        for (int r = 0; r < R; ++r) weights[(long)r * Q + i] = bw[r] / sum;
    }
}

/* reprojectDistanceKernel, stitcher.cu:181-204, as the minimum over source pixels; out must be
 * pre-filled (the reference fills 1e8, stitcher.py:184). */
void sso_reproject(const REAL* dist_in, REAL* dist_out, int W, int H, const float* k, const float* t)
{
    const long P = (long)W * H;
    for (long i = 0; i < P; ++i) {
        REAL pt[3];
        unproject_cu((REAL)(i % W), (REAL)(i / W), k, pt);
        for (int a = 0; a < 3; ++a) pt[a] = dist_in[i] * pt[a] - t[a];
        REAL o[2];
        project_cu(pt, k, o, 0);
        REAL d = r_norm3(pt[0], pt[1], pt[2]);
        int32_t idx = (int32_t)((uint32_t)rn_int(o[1]) * (uint32_t)W + (uint32_t)rn_int(o[0]));
        if (idx < 0 || idx >= P) continue;
        if (d < dist_out[idx]) dist_out[idx] = d;
    }
}

/* inpaintKernel, stitcher.cu:283-323, one Jacobi step per iteration */
void sso_inpaint(REAL* dist, const uint8_t* table, int W, int H, double max_dist, int iterations)
{
    const long P = (long)W * H;
    REAL* prev = (REAL*)malloc(sizeof(REAL) * P);
    const double hole = max_dist + 0.1, ok = max_dist + (double)0.1f;
    for (int it = 0; it < iterations; ++it) {
        memcpy(prev, dist, sizeof(REAL) * P);
#pragma omp parallel for schedule(static)
        for (long i = 0; i < P; ++i) {
            if (!((double)prev[i] >= hole)) continue;
            int x = (int)(i % W), y = (int)(i / W);
            if (!(x < W - 1 && y < H - 1 && y >= 1 && x >= 1)) continue;
            uint8_t a = table[2 * i], b = table[2 * i + 1];
            int nx[2] = {x + (a & 3) - 1, x + (b & 3) - 1};
            int ny[2] = {y + ((a & 12) >> 2) - 1, y + ((b & 12) >> 2) - 1};
            /* an offset field of 3 (a step of 2) is never produced by the table kernel; such a
             * neighbour is ignored (the reference would read outside the 3x3 neighbourhood) */
            int ok0 = (a & 3) != 3 && (a & 12) != 12, ok1 = (b & 3) != 3 && (b & 12) != 12;
            REAL w[2] = {ok0 ? (REAL)(a & 240) : 0, ok1 ? (REAL)(b & 240) : 0};
            REAL val = 0, ws = 0;
            for (int s = 0; s < 2; ++s) {
                if (!(w[s] > 0)) continue;
                REAL sd = prev[(long)ny[s] * W + nx[s]];
                if ((double)sd <= ok) { val = val + w[s] * sd; ws = ws + w[s]; }
            }
            if (ws > 0) dist[i] = val / ws;
        }
    }
    free(prev);
}

/* mergeRGBDPanoramaKernel, stitcher.cu:423-473.  reproj, dists: R x H x W; images: R x Hs x Ws x 3
 * uint8; outputs: distance Hp x Wp, rgb Hp x Wp x 3. */
void sso_merge(const REAL* lut, const REAL* weights, const REAL* reproj, const REAL* dists, const uint8_t* images,
               int Hs, int Ws, const float* ts, const float* ks, int R, int W, int H, int Wp, int Hp,
               REAL* distance_pano, uint8_t* rgb_pano)
{
    const long Q = (long)Wp * Hp;
    const REAL ratio_x = IS_F32 ? (REAL)((float)Ws / (float)W) : (REAL)Ws / W;
    const REAL ratio_y = IS_F32 ? (REAL)((float)Hs / (float)H) : (REAL)Hs / H;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < Q; ++i) {
        REAL inv = 0, rgb[3] = {0, 0, 0};
        for (int r = 0; r < R; ++r) {
            REAL w = weights[(long)r * Q + i];
            REAL u = lut[((long)r * Q + i) * 2], v = lut[((long)r * Q + i) * 2 + 1];
            REAL vo = v + (REAL)(r * H);
            REAL rd = interp_f(reproj, u, vo, W);
            inv = inv + (w * 1) / rd;
            REAL dc = interp_f(dists, u, vo, W);
            dc = r_fmin(rd, dc);
            REAL pt[3];
            unproject_cu(u, v, ks + 6 * r, pt);
            for (int a = 0; a < 3; ++a) pt[a] = dc * pt[a] + ts[3 * r + a];
            REAL uv[2];
            project_cu(pt, ks + 6 * r, uv, 0);
            uv[0] = uv[0] * ratio_x;
            uv[1] = uv[1] * ratio_y;
            uv[0] = r_fmin(r_fmax(uv[0], (REAL)0.1f), (REAL)Ws - (REAL)1.1f);
            uv[1] = r_fmin(r_fmax(uv[1], (REAL)0.1f), (REAL)Hs - (REAL)1.1f);
            uv[1] = uv[1] + (REAL)(r * Hs);
            /* interp (stitcher.cu:56-83) on the stacked uint8 images */
            int u1 = rd_int(uv[0]), v1 = rd_int(uv[1]), u2 = u1 + 1, v2 = v1 + 1;
            REAL w1 = ((REAL)u2 - uv[0]) * ((REAL)v2 - uv[1]), w2 = ((REAL)u2 - uv[0]) * (uv[1] - (REAL)v1),
                 w3 = (uv[0] - (REAL)u1) * ((REAL)v2 - uv[1]), w4 = (uv[0] - (REAL)u1) * (uv[1] - (REAL)v1);
            const uint8_t* p1 = images + ((long)v1 * Ws + u1) * 3;
            const uint8_t* p2 = images + ((long)v2 * Ws + u1) * 3;
            const uint8_t* p3 = images + ((long)v1 * Ws + u2) * 3;
            const uint8_t* p4 = images + ((long)v2 * Ws + u2) * 3;
            for (int ch = 0; ch < 3; ++ch) {
                REAL s = (REAL)p1[ch] * w1 + (REAL)p2[ch] * w2 + (REAL)p3[ch] * w3 + (REAL)p4[ch] * w4;
                rgb[ch] = rgb[ch] + s * w;
            }
        }
        distance_pano[i] = 1 / inv;
        for (int ch = 0; ch < 3; ++ch) rgb_pano[3 * i + ch] = (uint8_t)(rgb[ch] > 255 ? 255 : rgb[ch]);
    }
}

/* ---------------------------------------------------------------------------------------------
 * ISB_Filter.apply as explicit linear operators on the cost (isb_filter.py:72-136): for a given
 * guide the filter is linear in the cost, with weights from the guide pyramid.  Exported for
 * the float64 autograd restatement of the differentiable sweep.
 *   down level s = 1..L-1, coarse pixel o:  c_s[o] = sum_t down_w[s][9o+t] c_{s-1}[down_idx[s][9o+t]]
 *   up step s = L-2..0, fine pixel p (level s):
 *       f_s[p] = up_own[s][p] c_s[p] + sum_t up_w[s][9p+t] f_{s+1}[up_idx[s][9p+t]]
 * with f_{L-1} = c_{L-1}.  Arrays are indexed by level; unused taps have weight 0.  The guide
 * pyramid is updated exactly as the filter updates it.
 * ------------------------------------------------------------------------------------------- */
void sso_isb_operators(const uint8_t* guide, int rows, int cols, double sigma_i, double sigma_s,
                       int32_t* const* down_idx, REAL* const* down_w, int32_t* const* up_idx, REAL* const* up_w,
                       REAL* const* up_own)
{
    const int L = sso_isb_scale_count(cols, rows);
    if (L < 2) return;
    int r[64], c[64];
    uint8_t* g[64];
    for (int s = 0; s < L; ++s) {
        r[s] = (int)ceil(rows / pow(2.0, s));
        c[s] = (int)ceil(cols / pow(2.0, s));
        g[s] = (uint8_t*)calloc((size_t)r[s] * c[s] * 3, 1);
    }
    memcpy(g[0], guide, (size_t)rows * cols * 3);
    const double vs = 1 / (2 * sigma_s * sigma_s), vi = 1 / (2 * sigma_i * sigma_i);
    const REAL var_inv_i = (REAL)(IS_F32 ? (double)(float)vi : vi);
    for (int s = 1; s < L; ++s) {
        const int ci = c[s - 1], ri = r[s - 1], co = c[s];
        const long pout = (long)r[s] * co;
        for (long o = 0; o < pout; ++o) {
            int x = (int)(o % co), y = (int)(o / co);
            int x2 = 2 * x, y2 = 2 * y;
            int px = x2 + 1 < ci ? x2 + 1 : ci - 1, py = y2 + 1 < ri ? y2 + 1 : ri - 1;
            int mx = x2 - 1 >= 0 ? x2 - 1 : 0, my = y2 - 1 >= 0 ? y2 - 1 : 0;
            const long idx[9] = {(long)y2 * ci + x2, (long)my * ci + mx, (long)y2 * ci + mx, (long)py * ci + mx,
                                 (long)py * ci + x2, (long)py * ci + px, (long)y2 * ci + px, (long)my * ci + px,
                                 (long)my * ci + x2};
            const uint8_t* gi = g[s - 1];
            REAL cur[3] = {gi[3 * idx[0]], gi[3 * idx[0] + 1], gi[3 * idx[0] + 2]};
            REAL w[9] = {1, 0.25f, 0.5f, 0.25f, 0.5f, 0.25f, 0.5f, 0.25f, 0.5f};
            REAL wsum = 1, gs[3] = {cur[0], cur[1], cur[2]};
            for (int t = 1; t < 9; ++t) {
                REAL nb[3] = {gi[3 * idx[t]], gi[3 * idx[t] + 1], gi[3 * idx[t] + 2]};
                REAL d = abs_sum3(cur, nb);
                w[t] = w[t] * (r_exp(-d * d * var_inv_i) + ISB_EPS);
                wsum = wsum + w[t];
                for (int ch = 0; ch < 3; ++ch) gs[ch] = gs[ch] + nb[ch] * w[t];
            }
            REAL den = 1 / wsum;
            for (int ch = 0; ch < 3; ++ch) g[s][3 * o + ch] = (uint8_t)(gs[ch] * den);
            for (int t = 0; t < 9; ++t) {
                down_idx[s][9 * o + t] = (int32_t)idx[t];
                down_w[s][9 * o + t] = w[t] / wsum;
            }
        }
    }
    static const int t1[9][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 0}, {1, 1}, {1, 2}, {2, 0}, {2, 1}, {2, 2}};
    static const int t2[6][2] = {{1, 1}, {2, 1}, {1, 0}, {2, 0}, {1, 2}, {2, 2}};
    static const int t3[6][2] = {{1, 1}, {1, 2}, {0, 1}, {0, 2}, {2, 1}, {2, 2}};
    static const int t4[4][2] = {{1, 1}, {1, 2}, {2, 1}, {2, 2}};
    static const REAL b1[9] = {1, 1, 1, 1, 8, 1, 1, 1, 1}, b2[6] = {8, 8, 1, 1, 1, 1},
                      b3[6] = {8, 8, 1, 1, 1, 1}, b4[4] = {1, 1, 1, 1};
    const int (*taps[4])[2] = {t1, t2, t3, t4};
    const REAL* base[4] = {b1, b2, b3, b4};
    const int ntap[4] = {9, 6, 6, 4};
    for (int s = L - 2; s >= 0; --s) {
        const double dist = pow(2.0, s) - 0.5;
        const double wd = exp(-(dist * dist) * vs);
        const REAL weight_down = (REAL)wd, weight_up = (REAL)(1 - wd);
        const int ci = c[s + 1], ri = r[s + 1], cio = c[s], rio = r[s];
        const long pf = (long)rio * cio;
        for (long p = 0; p < pf * 9; ++p) { up_idx[s][p] = 0; up_w[s][p] = 0; }
        uint8_t* gnew = (uint8_t*)malloc((size_t)pf * 3);
        memcpy(gnew, g[s], (size_t)pf * 3);
        for (long o = 0; o < (long)ri * ci; ++o) {
            int x = (int)(o % ci), y = (int)(o / ci);
            int mdx = x - 1 >= 0 ? x - 1 : 0, mdy = y - 1 >= 0 ? y - 1 : 0;
            int pdx = x + 1 < ci ? x + 1 : ci - 1, pdy = y + 1 < ri ? y + 1 : ri - 1;
            int x2 = 2 * x, y2 = 2 * y;
            int pux = x2 + 1 < cio ? x2 + 1 : cio - 1, puy = y2 + 1 < rio ? y2 + 1 : rio - 1;
            const int rr[3] = {mdy, y, pdy}, cc[3] = {mdx, x, pdx};
            const long fidx[4] = {(long)y2 * cio + x2, (long)puy * cio + x2, (long)y2 * cio + pux, (long)puy * cio + pux};
            const int set[4] = {1, y2 != puy, x2 != pux, (y2 != puy) && (x2 != pux)};
            for (int f = 0; f < 4; ++f) {
                const uint8_t* gf = g[s] + 3 * fidx[f];
                REAL up[3] = {gf[0], gf[1], gf[2]};
                REAL gs[3] = {weight_up * up[0], weight_up * up[1], weight_up * up[2]};
                REAL wsum = weight_up, w[9];
                long cidx[9];
                for (int i = 0; i < ntap[f]; ++i) {
                    const int a = taps[f][i][0], b = taps[f][i][1];
                    cidx[i] = (long)rr[a] * ci + cc[b];
                    const uint8_t* gc = g[s + 1] + 3 * cidx[i];
                    REAL nb[3] = {gc[0], gc[1], gc[2]};
                    REAL d = abs_sum3(nb, up);
                    w[i] = base[f][i] * (weight_down * (r_exp(-d * d * var_inv_i) + ISB_EPS));
                    for (int ch = 0; ch < 3; ++ch) gs[ch] = gs[ch] + nb[ch] * w[i];
                    wsum = wsum + w[i];
                }
                if (!set[f]) continue;
                REAL inv = 1 / wsum;
                for (int ch = 0; ch < 3; ++ch) gnew[3 * fidx[f] + ch] = (uint8_t)(gs[ch] * inv);
                up_own[s][fidx[f]] = weight_up * inv;
                for (int i = 0; i < ntap[f]; ++i) {
                    up_idx[s][9 * fidx[f] + i] = (int32_t)cidx[i];
                    up_w[s][9 * fidx[f] + i] = w[i] * inv;
                }
            }
        }
        memcpy(g[s], gnew, (size_t)pf * 3);
        free(gnew);
    }
    for (int s = 0; s < L; ++s) free(g[s]);
}
