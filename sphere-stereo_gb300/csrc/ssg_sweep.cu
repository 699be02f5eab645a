// Guide image, adaptive camera selection and the fused sphere sweep + matching cost.
//
// The sweep never materialises the point volume, the warped images or the sweeping volume of
// the reference (python/depth_estimation.py:147-175 builds [N,H,W,3] points, four [1,3,N,H,W]
// grid_sample outputs and a masked merge): each thread unprojects its reference pixel once,
// then for every candidate transforms the point into the pixel's selected camera, projects it,
// samples the source image bilinearly and writes the L1 cost.  The arithmetic is the
// reference's, operation by operation (see ssg_common.cuh), so the fp32 cost volume is
// bit-identical to the oracle's.
#include "ssg_common.cuh"

namespace ssg {

constexpr int kBlock = 256;

struct SweepParams {
    int cols, rows, ncam, ncand, reference;
    float colsf, rowsf, inv_cols, inv_rows;
    int cols_pow2, rows_pow2;
    TorchCam ref;
    TorchCam cams[SSG_MAX_CAMERAS];
    float rt[SSG_MAX_CAMERAS][12];
    const float* images[SSG_MAX_CAMERAS];
    float cand[SSG_MAX_CANDIDATES];
};

// grid_sample's un-normalisation of the reference's normalised coordinate
// ((uv + 0.5) / size) * 2 - 1 (depth_estimation.py:160-161): ((g + 1) * size - 1) / 2
__device__ __forceinline__ float to_sample_coord(float uv, float size, float inv_size, bool pow2)
{
    const float t = fadd(uv, 0.5f);
    const float q = pow2 ? fmul(t, inv_size) : fdiv(t, size);
    const float g = fsub(fmul(q, 2.0f), 1.0f);
    return fmul(fsub(fmul(fadd(g, 1.0f), size), 1.0f), 0.5f);
}

// torch grid_sample, bilinear, zero padding, on an HWC float32 image (corner order nw, ne, sw, se)
__device__ __forceinline__ void sample_rgb(const float* __restrict__ img, int cols, int rows, float ix, float iy,
                                           float s[3])
{
    const float x0 = floorf(ix), y0 = floorf(iy);
    const float x1 = fadd(x0, 1.0f), y1 = fadd(y0, 1.0f);
    const float wx0 = fsub(x1, ix), wx1 = fsub(ix, x0), wy0 = fsub(y1, iy), wy1 = fsub(iy, y0);
    const float w[4] = {fmul(wx0, wy0), fmul(wx1, wy0), fmul(wx0, wy1), fmul(wx1, wy1)};
    const float xs[4] = {x0, x1, x0, x1}, ys[4] = {y0, y0, y1, y1};
    s[0] = s[1] = s[2] = 0.0f;
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        if (xs[t] >= 0.0f && xs[t] < (float)cols && ys[t] >= 0.0f && ys[t] < (float)rows) {
            const float* q = img + 3 * ((int64_t)(int)ys[t] * cols + (int)xs[t]);
            s[0] = fadd(s[0], fmul(__ldg(q + 0), w[t]));
            s[1] = fadd(s[1], fmul(__ldg(q + 1), w[t]));
            s[2] = fadd(s[2], fmul(__ldg(q + 2), w[t]));
        }
    }
}

__global__ void __launch_bounds__(kBlock) sweep_cost_kernel(const __grid_constant__ SweepParams p,
                                                            const int8_t* __restrict__ selected,
                                                            float* __restrict__ cost)
{
    const int64_t P = (int64_t)p.cols * p.rows;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    const int x = (int)(i % p.cols), y = (int)(i / p.cols);
    float pu[3];
    unproject_torch((float)x, (float)y, p.ref, pu);
    const float* refimg = p.images[p.reference] + 3 * i;
    const float r0 = __ldg(refimg), r1 = __ldg(refimg + 1), r2 = __ldg(refimg + 2);
    const int sel = selected[i];
    if (sel < 0 || sel >= p.ncam) {
        // no camera: the sweeping volume stays zero (depth_estimation.py:150-152); a selection
        // outside [0, cameras) is treated the same way instead of indexing past the camera arrays
        float c = fadd(fadd(fabsf(r0), fabsf(r1)), fabsf(r2));
        c = c > 500.0f ? 500.0f : c;
        for (int k = 0; k < p.ncand; ++k) cost[(int64_t)k * P + i] = c;
        return;
    }
    const TorchCam cam = p.cams[sel];
    float rt[12];
#pragma unroll
    for (int j = 0; j < 12; ++j) rt[j] = p.rt[sel][j];
    const float* img = p.images[sel];
    for (int k = 0; k < p.ncand; ++k) {
        const float d = p.cand[k];
        const float pv[3] = {fmul(d, pu[0]), fmul(d, pu[1]), fmul(d, pu[2])};
        float q[3], uv[2], s[3];
        transform_torch(rt, pv, q);
        project_torch(q, cam, uv);
        const float ix = to_sample_coord(uv[0], p.colsf, p.inv_cols, p.cols_pow2);
        const float iy = to_sample_coord(uv[1], p.rowsf, p.inv_rows, p.rows_pow2);
        sample_rgb(img, p.cols, p.rows, ix, iy, s);
        float c = fadd(fadd(fabsf(fsub(s[0], r0)), fabsf(fsub(s[1], r1))), fabsf(fsub(s[2], r2)));
        c = c > 500.0f ? 500.0f : c;
        cost[(int64_t)k * P + i] = c;
    }
}

// grid_sample of a [1,1,H,W] mask at a projected pixel (depth_estimation.py:117-123)
__device__ __forceinline__ float sample_mask(const float* __restrict__ m, int cols, int rows, float u, float v,
                                             float colsf, float rowsf)
{
    const float gx = fsub(fmul(fdiv(fadd(u, 0.5f), colsf), 2.0f), 1.0f);
    const float gy = fsub(fmul(fdiv(fadd(v, 0.5f), rowsf), 2.0f), 1.0f);
    const float ix = fmul(fsub(fmul(fadd(gx, 1.0f), colsf), 1.0f), 0.5f);
    const float iy = fmul(fsub(fmul(fadd(gy, 1.0f), rowsf), 1.0f), 0.5f);
    const float x0 = floorf(ix), y0 = floorf(iy);
    const float x1 = fadd(x0, 1.0f), y1 = fadd(y0, 1.0f);
    const float w[4] = {fmul(fsub(x1, ix), fsub(y1, iy)), fmul(fsub(ix, x0), fsub(y1, iy)),
                        fmul(fsub(x1, ix), fsub(iy, y0)), fmul(fsub(ix, x0), fsub(iy, y0))};
    const float xs[4] = {x0, x1, x0, x1}, ys[4] = {y0, y0, y1, y1};
    float out = 0.0f;
#pragma unroll
    for (int t = 0; t < 4; ++t)
        if (xs[t] >= 0.0f && xs[t] < colsf && ys[t] >= 0.0f && ys[t] < rowsf)
            out = fadd(out, fmul(__ldg(m + (int64_t)(int)ys[t] * cols + (int)xs[t]), w[t]));
    return out;
}

struct SelectParams {
    int cols, rows, ncam, reference;
    float colsf, rowsf, dmin, dmax;
    TorchCam ref;
    TorchCam cams[SSG_MAX_CAMERAS];
    float rt[SSG_MAX_CAMERAS][12];
};

__global__ void __launch_bounds__(kBlock) select_camera_kernel(const __grid_constant__ SelectParams p,
                                                               const float* __restrict__ masks,
                                                               int8_t* __restrict__ selected)
{
    const int64_t P = (int64_t)p.cols * p.rows;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    float pu[3];
    const bool ref_valid = unproject_torch((float)(i % p.cols), (float)(i / p.cols), p.ref, pu);
    const bool ref_mask = masks[(int64_t)p.reference * P + i] >= 0.9f;
    float max_disp = 1.0f;
    int sel = -1;
    for (int c = 0; c < p.ncam; ++c) {
        const float pn[3] = {fmul(pu[0], p.dmin), fmul(pu[1], p.dmin), fmul(pu[2], p.dmin)};
        const float pf[3] = {fmul(pu[0], p.dmax), fmul(pu[1], p.dmax), fmul(pu[2], p.dmax)};
        float qn[3], qf[3];
        transform_torch(p.rt[c], pn, qn);
        transform_torch(p.rt[c], pf, qf);
        const float nn = norm3_torch(qn[0], qn[1], qn[2]), nf = norm3_torch(qf[0], qf[1], qf[2]);
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            qn[j] = fdiv(qn[j], nn);
            qf[j] = fdiv(qf[j], nf);
        }
        float un[2], uf[2];
        const bool vn = project_torch(qn, p.cams[c], un);
        const bool vf = project_torch(qf, p.cams[c], uf);
        const float dx = fsub(un[0], uf[0]), dy = fsub(un[1], uf[1]);
        const float disp = fsqrt(ffma(dy, dy, fmul(dx, dx)));
        const float* m = masks + (int64_t)c * P;
        const float mn = sample_mask(m, p.cols, p.rows, un[0], un[1], p.colsf, p.rowsf);
        const float mf = sample_mask(m, p.cols, p.rows, uf[0], uf[1], p.colsf, p.rowsf);
        if (disp > max_disp && ref_valid && vn && vf && ref_mask && mn >= 0.9f && mf >= 0.9f) {
            max_disp = disp;
            sel = c;
        }
    }
    selected[i] = (int8_t)sel;
}

// utils.py:144-155 + .type(torch.uint8)
__global__ void __launch_bounds__(kBlock) rgb_to_guide_kernel(const float* __restrict__ rgb, int64_t n,
                                                              uint8_t* __restrict__ guide)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float c0 = rgb[3 * i], c1 = rgb[3 * i + 1], c2 = rgb[3 * i + 2];
    float y = fadd(fadd(fadd(fmul(c0, 0.1826f), 16.0f), fmul(c1, 0.6142f)), fmul(c2, 0.062f));
    float cb = fadd(fsub(fsub(128.0f, fmul(c0, 0.1006f)), fmul(c1, 0.3386f)), fmul(c2, 0.4392f));
    float cr = fsub(fsub(fadd(fmul(c0, 0.4392f), 128.0f), fmul(c1, 0.3989f)), fmul(c2, 0.0403f));
    y = fminf(fmaxf(y, 16.0f), 235.0f);
    cb = fminf(fmaxf(cb, 16.0f), 240.0f);
    cr = fminf(fmaxf(cr, 16.0f), 240.0f);
    guide[3 * i] = (uint8_t)__float2uint_rz(y);
    guide[3 * i + 1] = (uint8_t)__float2uint_rz(cb);
    guide[3 * i + 2] = (uint8_t)__float2uint_rz(cr);
}

static bool is_pow2(int v) { return v > 0 && (v & (v - 1)) == 0; }

static int check_cameras(int camera_count, const ssg_camera* cameras, int reference, const float* poses)
{
    SSG_REQUIRE(camera_count >= 1 && camera_count <= SSG_MAX_CAMERAS, "camera_count %d outside [1, %d]",
                camera_count, SSG_MAX_CAMERAS);
    SSG_REQUIRE(cameras && poses, "cameras and relative_poses must not be NULL");
    SSG_REQUIRE(reference >= 0 && reference < camera_count, "reference %d outside [0, %d)", reference, camera_count);
    for (int c = 0; c < camera_count; ++c) {
        const ssg_camera& k = cameras[c];
        SSG_REQUIRE(std::isfinite(k.xi) && std::isfinite(k.alpha) && k.alpha > 0.0 && k.alpha <= 1.0,
                    "camera %d: xi must be finite and alpha in (0, 1]", c);
        SSG_REQUIRE(k.fx != 0.0f && k.fy != 0.0f, "camera %d: zero focal length", c);
    }
    return SSG_OK;
}

}  // namespace ssg

using namespace ssg;

extern "C" int ssg_rgb_to_guide(const float* d_rgb, int64_t pixels, uint8_t* d_guide, void* stream)
{
    SSG_REQUIRE(d_rgb && d_guide, "null pointer");
    SSG_REQUIRE(pixels >= 0, "negative pixel count");
    if (pixels == 0) return SSG_OK;
    rgb_to_guide_kernel<<<grid_1d(pixels, kBlock), kBlock, 0, as_stream(stream)>>>(d_rgb, pixels, d_guide);
    return launch_status("rgb_to_guide_kernel");
}

extern "C" int ssg_select_camera(int cols, int rows, int camera_count, const ssg_camera* cameras, int reference,
                                 const float* relative_poses, const float* d_masks, double min_dist, double max_dist,
                                 int8_t* d_selected, void* stream)
{
    SSG_REQUIRE(cols > 0 && rows > 0, "resolution must be positive");
    SSG_REQUIRE(d_masks && d_selected, "null device pointer");
    if (int e = check_cameras(camera_count, cameras, reference, relative_poses)) return e;
    SelectParams p{};
    p.cols = cols;
    p.rows = rows;
    p.ncam = camera_count;
    p.reference = reference;
    p.colsf = (float)cols;
    p.rowsf = (float)rows;
    p.dmin = (float)min_dist;
    p.dmax = (float)max_dist;
    p.ref = make_torch_cam(cameras[reference]);
    for (int c = 0; c < camera_count; ++c) {
        p.cams[c] = make_torch_cam(cameras[c]);
        for (int j = 0; j < 12; ++j) p.rt[c][j] = relative_poses[12 * c + j];
    }
    const int64_t P = (int64_t)cols * rows;
    select_camera_kernel<<<grid_1d(P, kBlock), kBlock, 0, as_stream(stream)>>>(p, d_masks, d_selected);
    return launch_status("select_camera_kernel");
}

extern "C" int ssg_sweep_cost(int cols, int rows, int camera_count, const ssg_camera* cameras, int reference,
                              const float* relative_poses, const float* const* d_images, const int8_t* d_selected,
                              const float* candidates, int candidate_count, float* d_cost, void* stream)
{
    SSG_REQUIRE(cols > 0 && rows > 0, "resolution must be positive");
    SSG_REQUIRE(d_images && d_selected && d_cost && candidates, "null pointer");
    SSG_REQUIRE(candidate_count >= 1 && candidate_count <= SSG_MAX_CANDIDATES, "candidate_count %d outside [1, %d]",
                candidate_count, SSG_MAX_CANDIDATES);
    if (int e = check_cameras(camera_count, cameras, reference, relative_poses)) return e;
    SweepParams p{};
    p.cols = cols;
    p.rows = rows;
    p.ncam = camera_count;
    p.ncand = candidate_count;
    p.reference = reference;
    p.colsf = (float)cols;
    p.rowsf = (float)rows;
    p.cols_pow2 = is_pow2(cols);
    p.rows_pow2 = is_pow2(rows);
    p.inv_cols = 1.0f / (float)cols;
    p.inv_rows = 1.0f / (float)rows;
    p.ref = make_torch_cam(cameras[reference]);
    for (int c = 0; c < camera_count; ++c) {
        SSG_REQUIRE(d_images[c], "image %d is NULL", c);
        p.cams[c] = make_torch_cam(cameras[c]);
        p.images[c] = d_images[c];
        for (int j = 0; j < 12; ++j) p.rt[c][j] = relative_poses[12 * c + j];
    }
    for (int k = 0; k < candidate_count; ++k) p.cand[k] = candidates[k];
    const int64_t P = (int64_t)cols * rows;
    sweep_cost_kernel<<<grid_1d(P, kBlock), kBlock, 0, as_stream(stream)>>>(p, d_selected, d_cost);
    return launch_status("sweep_cost_kernel");
}
