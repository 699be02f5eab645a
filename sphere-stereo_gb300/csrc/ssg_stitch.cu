// RGB-D panorama stitcher (python/stitcher.cu, python/stitcher.py).
//
// Differences from the reference's GPU code, all towards one deterministic result:
//  * reprojection is a z-buffer of atomicMin on the float bits (distances are non-negative), so
//    each target pixel gets the minimum distance in one launch (the reference runs a racy
//    compare-and-store twice, stitcher.py:185-192) and targets outside the map are dropped (the
//    reference's index is unchecked, stitcher.cu:198);
//  * inpainting is a sequence of Jacobi steps (every pixel reads the map as it was before the
//    step; the reference updates in place and its result depends on thread timing).  Up to 16
//    steps run per launch on a shared-memory tile with a 16-pixel halo, ping-ponging between
//    the map and a scratch map in global memory;
//  * a table entry whose two best weights stay 0 (outside the model's valid area) encodes the
//    offsets (0, 0); the reference leaves them uninitialised (stitcher.cu:231).
#include <atomic>
#include <cmath>
#include <cstring>

#include "ssg_common.cuh"
#include "ssg_uneven.cuh"

namespace ssg {

constexpr int kStitchBlock = 256;

// smallest float f with (double)f >= v, and largest float f with (double)f <= v
static float float_at_least(double v)
{
    float f = (float)v;
    while ((double)f < v) f = std::nextafter(f, INFINITY);
    while ((double)std::nextafter(f, -INFINITY) >= v) f = std::nextafter(f, -INFINITY);
    return f;
}
static float float_at_most(double v)
{
    float f = (float)v;
    while ((double)f > v) f = std::nextafter(f, -INFINITY);
    while ((double)std::nextafter(f, INFINITY) <= v) f = std::nextafter(f, INFINITY);
    return f;
}


// createInpaintingWeightsKernel, stitcher.cu:212-272
__global__ void __launch_bounds__(kStitchBlock) inpainting_table_kernel(int cols, int rows, Intr k, float tx,
                                                                        float ty, float tz, float dmin, float dmax,
                                                                        uint8_t* __restrict__ table)
{
    const int64_t P = (int64_t)cols * rows;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    float unit[3];
    unproject_cu((float)(i % cols), (float)(i / cols), k, unit);
    const float pc[3] = {fsub(fmul(dmin, unit[0]), tx), fsub(fmul(dmin, unit[1]), ty), fsub(fmul(dmin, unit[2]), tz)};
    const float pf[3] = {fsub(fmul(dmax, unit[0]), tx), fsub(fmul(dmax, unit[1]), ty), fsub(fmul(dmax, unit[2]), tz)};
    float uc[2], uf[2];
    project_cu(pc, k, uc, nullptr);
    project_cu(pf, k, uf, nullptr);
    float dx = fsub(uf[0], uc[0]), dy = fsub(uf[1], uc[1]);
    const float den = fdiv(1.0f, hypotf(dx, dy));
    dx = fmul(dx, den);
    dy = fmul(dy, den);
    int nx[2] = {0, 0}, ny[2] = {0, 0};
    float w[2] = {0.0f, 0.0f};
#pragma unroll
    for (int n = -1; n <= 1; ++n)
#pragma unroll
        for (int m = -1; m <= 1; ++m) {
            if (!(n || m)) continue;
            const float pd = fdiv(1.0f, hypotf((float)n, (float)m));
            const float wt = fadd(fmul(fmul((float)n, pd), dx), fmul(fmul((float)m, pd), dy));
            if (wt > w[1]) {
                w[0] = w[1];
                nx[0] = nx[1];
                ny[0] = ny[1];
                w[1] = wt;
                nx[1] = n;
                ny[1] = m;
            } else if (wt > w[0]) {
                w[0] = wt;
                nx[0] = n;
                ny[0] = m;
            }
        }
    const unsigned q0 = (__float2uint_rz(fmul(w[0], 255.0f)) & 0xFFu) & 240u;
    const unsigned q1 = (__float2uint_rz(fmul(w[1], 255.0f)) & 0xFFu) & 240u;
    table[2 * i] = (uint8_t)(q0 + 4u * (unsigned)(1 + ny[0]) + (unsigned)(1 + nx[0]));
    table[2 * i + 1] = (uint8_t)(q1 + 4u * (unsigned)(1 + ny[1]) + (unsigned)(1 + nx[1]));
}

// Box mean with constant padding, summed in row-major window order (stitcher.py:144-148, :162-163)
__global__ void __launch_bounds__(kStitchBlock) box_filter_kernel(const float* __restrict__ in, int rows, int cols,
                                                                  int radius, float pad, float kw,
                                                                  float* __restrict__ out)
{
    const int64_t P = (int64_t)cols * rows;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int plane = blockIdx.y;
    if (i >= P) return;
    const float* src = in + (int64_t)plane * P;
    const int x = (int)(i % cols), y = (int)(i / cols);
    float s = 0.0f;
    for (int dy = -radius; dy <= radius; ++dy) {
        const int yy = y + dy;
        const bool row_in = yy >= 0 && yy < rows;
        for (int dx = -radius; dx <= radius; ++dx) {
            const int xx = x + dx;
            const float v = (row_in && xx >= 0 && xx < cols) ? __ldg(src + (int64_t)yy * cols + xx) : pad;
            s = fadd(s, fmul(v, kw));
        }
    }
    out[(int64_t)plane * P + i] = s;
}

// The same box mean from a shared-memory tile: a block stages the products v * kw of its
// (kBoxX + 2r) x (kBoxY + 2r) input window once, then each thread sums the (2r + 1)^2 products of
// each of its kBoxK outputs in the same row-major window order (identical bits).  Threads of a
// warp take consecutive columns, so the tile reads are conflict-free.
constexpr int kBoxX = 64, kBoxY = 32, kBoxThreadsX = 32, kBoxThreadsY = 8;

__host__ __device__ constexpr int box_tile_floats(int radius)
{
    return (kBoxX + 2 * radius) * (kBoxY + 2 * radius);
}

__global__ void __launch_bounds__(kBoxThreadsX * kBoxThreadsY) box_filter_tiled_kernel(
    const float* __restrict__ in, int rows, int cols, int radius, float pad, float kw, float* __restrict__ out)
{
    extern __shared__ float tile[];
    const int64_t P = (int64_t)cols * rows;
    const int plane = blockIdx.z;
    const float* src = in + (int64_t)plane * P;
    const int x0 = blockIdx.x * kBoxX, y0 = blockIdx.y * kBoxY;
    const int tw = kBoxX + 2 * radius, th = kBoxY + 2 * radius;
    const float pad_product = fmul(pad, kw);
    for (int q = threadIdx.x; q < tw * th; q += blockDim.x) {
        const int lx = q % tw, ly = q / tw;
        const int xx = x0 - radius + lx, yy = y0 - radius + ly;
        tile[q] = (xx >= 0 && yy >= 0 && xx < cols && yy < rows) ? fmul(__ldg(src + (int64_t)yy * cols + xx), kw)
                                                                : pad_product;
    }
    __syncthreads();
    const int tx = threadIdx.x % kBoxThreadsX, ty = threadIdx.x / kBoxThreadsX;
    const int side = 2 * radius + 1;
    for (int m = 0; m < kBoxY / kBoxThreadsY; ++m) {
        const int ly = ty + m * kBoxThreadsY, y = y0 + ly;
        if (y >= rows) break;
#pragma unroll
        for (int k = 0; k < kBoxX / kBoxThreadsX; ++k) {
            const int lx = tx + k * kBoxThreadsX, x = x0 + lx;
            if (x >= cols) continue;
            float s = 0.0f;
            for (int dy = 0; dy < side; ++dy) {
                const float* row = tile + (ly + dy) * tw + lx;
                for (int dx = 0; dx < side; ++dx) s = fadd(s, row[dx]);
            }
            out[(int64_t)plane * P + (int64_t)y * cols + x] = s;
        }
    }
}

struct LutParams {
    int cols, rows, pano_cols, pano_rows, nref;
    float dmin, dmax;
    Intr k[SSG_MAX_REFERENCES];
    float rot[SSG_MAX_REFERENCES][9];
    float t[SSG_MAX_REFERENCES][3];
};

// createBlendingLutKernel, stitcher.cu:338-401
__global__ void __launch_bounds__(kStitchBlock) blending_lut_kernel(const __grid_constant__ LutParams p,
                                                                    const float* __restrict__ masks,
                                                                    float2* __restrict__ lut,
                                                                    float* __restrict__ weights)
{
    const int64_t Q = (int64_t)p.pano_cols * p.pano_rows;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Q) return;
    const double PI = 3.14159265;  // stitcher.cu:325, a double literal
    const float px = (float)(i % p.pano_cols), py = (float)(i / p.pano_cols);
    const float phi = (float)(__dsub_rn(__ddiv_rn(__dmul_rn((double)fadd(py, 0.5f), PI), (double)p.pano_rows), PI / 2.0));
    const float theta =
        (float)(__dadd_rn(__ddiv_rn(__dmul_rn((double)fmul(fadd(px, 0.5f), 2.0f), PI), (double)p.pano_cols), PI));
    const float cp = cosf(phi);
    const float unit[3] = {fmul(cp, sinf(theta)), sinf(phi), fmul(cp, cosf(theta))};
    const float colsm = fsub((float)p.cols, 1.1f), rowsm = fsub((float)p.rows, 1.1f);
    float bw[SSG_MAX_REFERENCES];
    float sum = 0.0f;
    for (int r = 0; r < p.nref; ++r) {
        const float* m = p.rot[r];
        float uf[3];
#pragma unroll
        for (int a = 0; a < 3; ++a)
            uf[a] = fadd(fadd(fmul(m[3 * a], unit[0]), fmul(m[3 * a + 1], unit[1])), fmul(m[3 * a + 2], unit[2]));
        bool valid = true;
        float uv[2];
        project_cu(uf, p.k[r], uv, &valid);
        uv[0] = fminf(fmaxf(uv[0], 0.1f), colsm);
        uv[1] = fminf(fmaxf(uv[1], 0.1f), rowsm);
        lut[(int64_t)r * Q + i] = make_float2(uv[0], uv[1]);
        bw[r] = 1e-8f;
        const float* t = p.t[r];
        const float pn3[3] = {fsub(fmul(p.dmin, uf[0]), t[0]), fsub(fmul(p.dmin, uf[1]), t[1]),
                              fsub(fmul(p.dmin, uf[2]), t[2])};
        const float pf3[3] = {fsub(fmul(p.dmax, uf[0]), t[0]), fsub(fmul(p.dmax, uf[1]), t[1]),
                              fsub(fmul(p.dmax, uf[2]), t[2])};
        float pn[2], pf[2];
        project_cu(pn3, p.k[r], pn, &valid);
        pn[0] = fminf(fmaxf(pn[0], 0.1f), colsm);
        pn[1] = fadd((float)(r * p.rows), fminf(fmaxf(pn[1], 0.1f), rowsm));
        project_cu(pf3, p.k[r], pf, &valid);
        pf[0] = fminf(fmaxf(pf[0], 0.1f), colsm);
        pf[1] = fadd((float)(r * p.rows), fminf(fmaxf(pf[1], 0.1f), rowsm));
        if (valid && (double)interp_f(masks, pn[0], pn[1], p.cols) > 0.99 &&
            (double)interp_f(masks, pf[0], pf[1], p.cols) > 0.99) {
            const float s = hypotf(fsub(pf[0], pn[0]), fsub(pf[1], pn[1]));
            const double e = __ddiv_rn((double)fmul(-s, s), 1e-4 * p.rows * p.cols);
            bw[r] = cw_expf((float)e);
        }
        sum = fadd(sum, bw[r]);
    }
    for (int r = 0; r < p.nref; ++r) weights[(int64_t)r * Q + i] = fdiv(bw[r], sum);
}

// python/stitcher.py:164: weights /= sum over references
__global__ void __launch_bounds__(kStitchBlock) normalize_weights_kernel(float* __restrict__ w, int nref, int64_t Q)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Q) return;
    float s = w[i];
    for (int r = 1; r < nref; ++r) s = fadd(s, w[(int64_t)r * Q + i]);
    for (int r = 0; r < nref; ++r) w[(int64_t)r * Q + i] = fdiv(w[(int64_t)r * Q + i], s);
}

// out[0, n) = v: four values per thread with one 16-byte store where out is 16-byte aligned
__global__ void __launch_bounds__(kStitchBlock) fill_kernel(float* __restrict__ out, int64_t n, float v)
{
    const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * 4;
    if (i + 4 <= n && ((uintptr_t)out & 15) == 0) {
        reinterpret_cast<float4*>(out + i)[0] = make_float4(v, v, v, v);
    } else {
        for (int64_t j = i; j < i + 4 && j < n; ++j) out[j] = v;
    }
}

static int fill_map(float* out, int64_t n, float v, cudaStream_t st)
{
    fill_kernel<<<grid_1d((n + 3) / 4, kStitchBlock), kStitchBlock, 0, st>>>(out, n, v);
    return launch_status("fill_kernel");
}

struct ReprojParams {
    int cols, rows, references;
    Intr k[SSG_MAX_REFERENCES];
    float t[SSG_MAX_REFERENCES][3];
};

// reprojectDistanceKernel, stitcher.cu:181-204, as a z-buffer on the float bits: pixel i of one
// map (din -> dout, P pixels), whose unit ray `ray` (unproject_cu of the pixel) is given
__device__ __forceinline__ void reproject_ray(const Intr& k, const float* t, const float (&ray)[3],
                                              const float* __restrict__ din, float* __restrict__ dout, int cols,
                                              int64_t P, int64_t i)
{
    const float d = din[i];
    float pt[3];
    pt[0] = fsub(fmul(d, ray[0]), t[0]);
    pt[1] = fsub(fmul(d, ray[1]), t[1]);
    pt[2] = fsub(fmul(d, ray[2]), t[2]);
    float o[2];
    project_cu(pt, k, o, nullptr);
    const float dist = norm3df(pt[0], pt[1], pt[2]);
    // __float2int_rn(y) * COLS + __float2int_rn(x) in 32-bit wrap-around arithmetic
    const int idx = (int)((unsigned)__float2int_rn(o[1]) * (unsigned)cols + (unsigned)__float2int_rn(o[0]));
    if (idx < 0 || (int64_t)idx >= P || !(dist >= 0.0f)) return;
    atomicMin(reinterpret_cast<int*>(dout) + idx, __float_as_int(dist));
}

__device__ __forceinline__ void pixel_ray(const Intr& k, int cols, int64_t i, float (&ray)[3])
{
    const int y = (int)i / cols;  // a map holds fewer than 2^31 pixels
    unproject_cu((float)((int)i - y * cols), (float)y, k, ray);
}

__device__ __forceinline__ void reproject_pixel(const Intr& k, const float* t, const float* __restrict__ din,
                                                float* __restrict__ dout, int cols, int64_t P, int64_t i)
{
    float ray[3];
    pixel_ray(k, cols, i, ray);
    reproject_ray(k, t, ray, din, dout, cols, P, i);
}

// blockIdx.y: instance (frame * references + reference slot) of contiguous maps.
__global__ void __launch_bounds__(kStitchBlock) reproject_kernel(const __grid_constant__ ReprojParams p,
                                                                 const float* __restrict__ din,
                                                                 float* __restrict__ dout)
{
    const int64_t P = (int64_t)p.cols * p.rows;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    const int slot = blockIdx.y % p.references;
    reproject_pixel(p.k[slot], p.t[slot], din + (int64_t)blockIdx.y * P, dout + (int64_t)blockIdx.y * P, p.cols, P, i);
}

// reproject_ray with fused multiply-adds and approximate square roots and reciprocal (the
// batched 16-bit path): the same steps, a relative error of a few 1e-7 in the position and the
// distance
__device__ __forceinline__ void reproject_ray_fast(const Intr& k, const float* t, const float (&ray)[3],
                                                   const float* __restrict__ din, float* __restrict__ dout, int cols,
                                                   int64_t P, int64_t i)
{
    const float d = din[i];
    const float pt[3] = {fmaf(d, ray[0], -t[0]), fmaf(d, ray[1], -t[1]), fmaf(d, ray[2], -t[2])};
    const float rxy = fmaf(pt[1], pt[1], pt[0] * pt[0]);
    const float d1 = sqrt_approx(fmaf(pt[2], pt[2], rxy));
    const float c = fmaf(k.xi, d1, pt[2]);
    const float d2 = sqrt_approx(fmaf(c, c, rxy));
    const float den = rcp_approx(fmaf(k.alpha, d2, (1.0f - k.alpha) * c));
    const float ox = fmaf(k.fx * pt[0], den, k.cx), oy = fmaf(k.fy * pt[1], den, k.cy);
    const int idx = (int)((unsigned)__float2int_rn(oy) * (unsigned)cols + (unsigned)__float2int_rn(ox));
    if (idx < 0 || (int64_t)idx >= P || !(d1 >= 0.0f)) return;
    atomicMin(reinterpret_cast<int*>(dout) + idx, __float_as_int(d1));
}

// The batch's maps of one reference slot share each pixel's ray: a thread unprojects its pixel
// once and reprojects it in every frame.  blockIdx.y: reference slot; instances frame * references
// + slot.  kFast: reproject_ray_fast.
template <bool kFast>
__global__ void __launch_bounds__(kStitchBlock) reproject_frames_kernel(const __grid_constant__ ReprojParams p,
                                                                        int frames, const float* __restrict__ din,
                                                                        float* __restrict__ dout)
{
    const int64_t P = (int64_t)p.cols * p.rows;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    const int slot = blockIdx.y;
    float ray[3];
    pixel_ray(p.k[slot], p.cols, i, ray);
    for (int f = 0; f < frames; ++f) {
        const int64_t inst = (int64_t)f * p.references + slot;
        if (kFast) reproject_ray_fast(p.k[slot], p.t[slot], ray, din + inst * P, dout + inst * P, p.cols, P, i);
        else reproject_ray(p.k[slot], p.t[slot], ray, din + inst * P, dout + inst * P, p.cols, P, i);
    }
}

// Tiled Jacobi inpainting: kTileW x kTileH outputs, a halo of kHalo >= steps pixels.
constexpr int kTileW = 64, kTileH = 32, kHalo = 16;
constexpr int kRegW = kTileW + 2 * kHalo, kRegH = kTileH + 2 * kHalo;
constexpr int kInpaintBlock = 512;
constexpr size_t kInpaintSmem =
    sizeof(float) * 2 * kRegW * kRegH + sizeof(uchar2) * kRegW * kRegH + sizeof(uint16_t) * kRegW * kRegH;

// One Jacobi step of inpaintKernel (stitcher.cu:283-323) at region cell j, reading `cur`.
__device__ __forceinline__ float inpaint_cell(const float* cur, const uchar2* tab, int j, float hole_at_least,
                                              float valid_at_most)
{
    const float v = cur[j];
    if (!(v >= hole_at_least)) return v;  // filled in an earlier step
    const uchar2 t = tab[j];
    const int n0 = j + ((t.x & 12) / 4 - 1) * kRegW + ((t.x & 3) - 1);
    const int n1 = j + ((t.y & 12) / 4 - 1) * kRegW + ((t.y & 3) - 1);
    // an offset field of 3 (a step of 2) never comes out of the table kernel; such a neighbour is
    // ignored instead of read outside the 3x3 neighbourhood
    const bool ok0 = (t.x & 3) != 3 && (t.x & 12) != 12, ok1 = (t.y & 3) != 3 && (t.y & 12) != 12;
    const float w0 = ok0 ? (float)(t.x & 240) : 0.0f, w1 = ok1 ? (float)(t.y & 240) : 0.0f;
    float val = 0.0f, ws = 0.0f;
    if (w0 > 0.0f) {
        const float sd = cur[n0];
        if (sd <= valid_at_most) {
            val = fadd(val, fmul(w0, sd));
            ws = fadd(ws, w0);
        }
    }
    if (w1 > 0.0f) {
        const float sd = cur[n1];
        if (sd <= valid_at_most) {
            val = fadd(val, fmul(w1, sd));
            ws = fadd(ws, w1);
        }
    }
    return ws > 0.0f ? fdiv(val, ws) : v;
}

// `steps` Jacobi steps on a 64 x 32 output tile from its region with a 16-pixel halo held in
// shared memory.  Only hole pixels change, and a pixel that is not a hole never becomes one, so
// the block lists the region's holes once and updates only those; a tile without holes copies
// its input through.
__global__ void __launch_bounds__(kInpaintBlock) inpaint_tile_kernel(const float* __restrict__ src,
                                                                     float* __restrict__ dst,
                                                                     const uchar2* __restrict__ table, int cols,
                                                                     int rows, int references, int steps,
                                                                     float hole_at_least, float valid_at_most)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int hole_count;
    // blockIdx.z: instance (frame * references + reference slot); tables are per slot
    const int64_t P = (int64_t)cols * rows;
    src += (int64_t)blockIdx.z * P;
    dst += (int64_t)blockIdx.z * P;
    table += (int64_t)(blockIdx.z % references) * P;
    float* buf0 = reinterpret_cast<float*>(smem);
    float* buf1 = buf0 + kRegW * kRegH;
    uchar2* tab = reinterpret_cast<uchar2*>(buf1 + kRegW * kRegH);
    uint16_t* holes = reinterpret_cast<uint16_t*>(tab + kRegW * kRegH);
    const int ox = blockIdx.x * kTileW - kHalo, oy = blockIdx.y * kTileH - kHalo;
    if (threadIdx.x == 0) hole_count = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    // kRegW * kRegH is a multiple of the block size: every warp runs whole iterations
    for (int j = threadIdx.x; j < kRegW * kRegH; j += blockDim.x) {
        const int lx = j % kRegW, ly = j / kRegW;
        const int x = ox + lx, y = oy + ly;
        const bool in = x >= 0 && x < cols && y >= 0 && y < rows;
        const int64_t g = (int64_t)y * cols + x;
        const float v = in ? src[g] : 0.0f;
        buf0[j] = v;
        buf1[j] = v;
        tab[j] = in ? table[g] : make_uchar2(0, 0);
        // hole test of stitcher.cu:287 and the interior test of :291; neighbours must lie inside
        // the region (pixels whose neighbours do not are farther than `steps` from the outputs)
        const bool hole = in && v >= hole_at_least && x >= 1 && y >= 1 && x < cols - 1 && y < rows - 1 && lx >= 1 &&
                          ly >= 1 && lx < kRegW - 1 && ly < kRegH - 1;
        const unsigned mask = __ballot_sync(0xffffffffu, hole);
        int base = 0;
        if (lane == 0 && mask) base = atomicAdd(&hole_count, __popc(mask));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (hole) holes[base + __popc(mask & ((1u << lane) - 1))] = (uint16_t)j;
    }
    __syncthreads();
    const int n = hole_count;
    float* cur = buf0;
    float* nxt = buf1;
    if (n > 0)
        for (int s = 0; s < steps; ++s) {
            for (int h = threadIdx.x; h < n; h += blockDim.x) {
                const int j = holes[h];
                nxt[j] = inpaint_cell(cur, tab, j, hole_at_least, valid_at_most);
            }
            __syncthreads();
            float* tmp = cur;
            cur = nxt;
            nxt = tmp;
        }
    for (int j = threadIdx.x; j < kTileW * kTileH; j += blockDim.x) {
        const int lx = kHalo + j % kTileW, ly = kHalo + j / kTileW;
        const int x = ox + lx, y = oy + ly;
        if (x < cols && y < rows) dst[(int64_t)y * cols + x] = cur[ly * kRegW + lx];
    }
}

// ---------------------------------------------------------------------------------------------
// Hole filling over lists of holes (the batched path), with the result of the Jacobi steps above.
// Only holes change, a filled hole keeps its value from then on, and a hole whose two table
// weights are 0 (outside the model's valid area) never changes.  Every pixel gets a one-byte
// stamp: 0 for a pixel that is not a hole, kUnfilled for a hole, s for a hole filled at step s.
// Step s reads a neighbour only when its stamp is below s, i.e. as it was before the step (a
// neighbour filled in the same step has stamp s and counts as a hole, as in a Jacobi step on a
// copy), and writes each filled hole's value and stamp in place: one map, no copy.
//   * Step 1 visits every fillable hole (listed by a scan).
//   * A hole that step 1 leaves open can only be filled at step s > 1 through a neighbour filled
//     at step s - 1 (a neighbour filled earlier would have filled it earlier), so step s visits the
//     holes that read a pixel filled at step s - 1: the work of a step is its frontier.  A claim
//     word per pixel (the last step that queued it) keeps a hole from being visited twice.
// ---------------------------------------------------------------------------------------------
constexpr uint8_t kUnfilled = 255;
constexpr int kMaxListIterations = 254;

struct HoleOffsets {
    int64_t n0, n1;
    float w0, w1;
};

// the two weighted neighbours a table entry encodes (stitcher.cu:297-316); a weight is 0 where
// the offset field is 3 (never written by the table kernel)
__device__ __forceinline__ HoleOffsets hole_offsets(uchar2 t, int64_t g, int cols)
{
    HoleOffsets h;
    h.n0 = g + ((t.x & 12) / 4 - 1) * (int64_t)cols + ((t.x & 3) - 1);
    h.n1 = g + ((t.y & 12) / 4 - 1) * (int64_t)cols + ((t.y & 3) - 1);
    const bool ok0 = (t.x & 3) != 3 && (t.x & 12) != 12, ok1 = (t.y & 3) != 3 && (t.y & 12) != 12;
    h.w0 = ok0 ? (float)(t.x & 240) : 0.0f;
    h.w1 = ok1 ? (float)(t.y & 240) : 0.0f;
    return h;
}

__device__ __forceinline__ bool fillable(uchar2 t)
{
    const HoleOffsets h = hole_offsets(t, 0, 1);
    return h.w0 > 0.0f || h.w1 > 0.0f;
}

// Loads of the data the hole steps change (map, stamps, lists, counts).  kL2: through L2 only
// (ld.global.cg), for the persistent launch whose phases read what other SMs wrote in an earlier
// phase of the same launch; otherwise ordinary loads (a launch boundary separates the steps).
template <bool kL2, typename T>
__device__ __forceinline__ T load_mutable(const T* p)
{
    if constexpr (kL2) return __ldcg(p);
    else return *p;
}

// Jacobi step `step` of hole g: fills it (value and stamp) when a usable neighbour exists
template <bool kL2 = false>
__device__ __forceinline__ bool fill_hole(float* __restrict__ map, uint8_t* __restrict__ stamp, int64_t g,
                                         const HoleOffsets& h, int step, float valid_at_most)
{
    float val = 0.0f, ws = 0.0f;
    if (h.w0 > 0.0f && load_mutable<kL2>(stamp + h.n0) < step) {
        const float sd = load_mutable<kL2>(map + h.n0);
        if (sd <= valid_at_most) {
            val = fadd(val, fmul(h.w0, sd));
            ws = fadd(ws, h.w0);
        }
    }
    if (h.w1 > 0.0f && load_mutable<kL2>(stamp + h.n1) < step) {
        const float sd = load_mutable<kL2>(map + h.n1);
        if (sd <= valid_at_most) {
            val = fadd(val, fmul(h.w1, sd));
            ws = fadd(ws, h.w1);
        }
    }
    if (!(ws > 0.0f)) return false;
    map[g] = fdiv(val, ws);
    stamp[g] = (uint8_t)step;
    return true;
}

// Appends `item` (where `take`) to the list counted by *count with one atomic per block: every
// thread of the block calls it (block-uniform control flow; blockDim.x == kStitchBlock).
__device__ __forceinline__ void block_append(bool take, int32_t item, int32_t* count, int32_t* list)
{
    __shared__ int warp_base[kStitchBlock / 32];
    __shared__ int block_base;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned mask = __ballot_sync(0xffffffffu, take);
    if (lane == 0) warp_base[warp] = __popc(mask);
    __syncthreads();
    if (threadIdx.x == 0) {
        int total = 0;
        for (int w = 0; w < kStitchBlock / 32; ++w) {
            const int n = warp_base[w];
            warp_base[w] = total;
            total += n;
        }
        block_base = total ? atomicAdd(count, total) : 0;
    }
    __syncthreads();
    if (take) list[block_base + warp_base[warp] + __popc(mask & ((1u << lane) - 1))] = item;
    __syncthreads();  // warp_base and block_base are reused by the next call
}

// Where a flat map pixel g lives: its map's size, its position in the map, its table entry.
struct MapPixel {
    int cols, rows, x, y;
    const uchar2* table;  // the map's inpainting table (entry of pixel (x, y): table[y * cols + x])
};

// `instances` maps of one size, tables per reference slot (the uniform batch); flat indices are
// below 2^31 (the hole lists hold them as int32), so positions come from 32-bit divisions by
// host-fixed divisors
struct UniformMaps {
    int cols, rows, references;
    const uchar2* tables;
    FastDiv by_map, by_cols, by_refs;
    UniformMaps(int c, int r, int refs, const uchar2* t)
        : cols(c), rows(r), references(refs), tables(t), by_map((uint32_t)c * (uint32_t)r), by_cols((uint32_t)c),
          by_refs((uint32_t)refs)
    {
    }
    __device__ __forceinline__ MapPixel at(int64_t g) const
    {
        const uint32_t P = (uint32_t)cols * (uint32_t)rows, gg = (uint32_t)g;
        const uint32_t inst = by_map.div(gg), j = gg - inst * P;
        const uint32_t y = by_cols.div(j), slot = inst - by_refs.div(inst) * (uint32_t)references;
        return MapPixel{cols, rows, (int)(j - y * (uint32_t)cols), (int)y, tables + (int64_t)slot * P};
    }
};

// Appends up to 32 items per thread (bit i of `take`: item first + i) to the list counted by
// *count, with one atomic per block; every thread of the block calls it (blockDim.x == kStitchBlock).
__device__ __forceinline__ void block_append_bits(uint32_t take, int64_t first, int32_t* count, int32_t* list)
{
    __shared__ int warp_base[kStitchBlock / 32];
    __shared__ int block_base;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int n = __popc(take);
    int incl = n;  // inclusive prefix over the warp's lanes
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += t;
    }
    if (lane == 31) warp_base[warp] = incl;
    __syncthreads();
    if (threadIdx.x == 0) {
        int total = 0;
        for (int w = 0; w < kStitchBlock / 32; ++w) {
            const int c = warp_base[w];
            warp_base[w] = total;
            total += c;
        }
        block_base = total ? atomicAdd(count, total) : 0;
    }
    __syncthreads();
    int at = block_base + warp_base[warp] + incl - n;
    while (take) {
        const int i = __ffs(take) - 1;
        take &= take - 1;
        list[at++] = (int32_t)(first + i);
    }
}

// Scan: stamps the map pixels of the flat index space, clears the claims of the holes (nothing
// reads the claim of a pixel that is not a hole) and lists the fillable holes in `list` (counted
// by *count).  kScanPixels consecutive pixels per thread: vector loads of the map and one vector
// store of their stamps when `vec` (map 16-byte and stamps 8-byte aligned, total a multiple of
// kScanPixels).
constexpr int kScanPixels = 8;

template <typename Maps>
__global__ void __launch_bounds__(kStitchBlock) hole_scan_wide_kernel(const Maps maps, int64_t total,
                                                                      const float* __restrict__ map,
                                                                      uint8_t* __restrict__ stamp,
                                                                      int32_t* __restrict__ claim,
                                                                      float hole_at_least, bool vec,
                                                                      int32_t* __restrict__ count,
                                                                      int32_t* __restrict__ list)
{
    const int64_t g0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * kScanPixels;
    uint32_t take = 0;
    if (g0 < total) {
        float v[kScanPixels];
        if (vec) {
            const float4 a = __ldg(reinterpret_cast<const float4*>(map + g0));
            const float4 b = __ldg(reinterpret_cast<const float4*>(map + g0) + 1);
            v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
            v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
        } else {
#pragma unroll
            for (int i = 0; i < kScanPixels; ++i) v[i] = g0 + i < total ? map[g0 + i] : 0.0f;
        }
        uint32_t st[2] = {0u, 0u};
#pragma unroll
        for (int i = 0; i < kScanPixels; ++i) {
            const int64_t g = g0 + i;
            const bool hole = g < total && v[i] >= hole_at_least;  // stitcher.cu:287
            if (hole) {
                st[i / 4] |= (uint32_t)kUnfilled << (8 * (i % 4));
                claim[g] = 0;
                const MapPixel m = maps.at(g);
                // interior test of stitcher.cu:291
                if (m.x >= 1 && m.y >= 1 && m.x < m.cols - 1 && m.y < m.rows - 1 &&
                    fillable(m.table[(int64_t)m.y * m.cols + m.x]))
                    take |= 1u << i;
            }
            if (!vec && g < total) stamp[g] = hole ? kUnfilled : 0;
        }
        if (vec) reinterpret_cast<uint2*>(stamp + g0)[0] = make_uint2(st[0], st[1]);
    }
    block_append_bits(take, g0, count, list);
}

// Step 1 on every listed hole; lists the holes it fills.  counts[3] rotate: counts[(s - 1) % 3]
// counts step s's input list, counts[s % 3] its output (zeroed by step s - 1 or the set-up), and
// step s zeroes counts[(s + 1) % 3].
template <bool kL2, typename Maps>
__device__ __forceinline__ void hole_first_step(const Maps& maps, float* __restrict__ map,
                                                uint8_t* __restrict__ stamp, int32_t* __restrict__ counts,
                                                const int32_t* __restrict__ list_in, int32_t* __restrict__ list_out,
                                                float valid_at_most)
{
    const int n = load_mutable<kL2>(counts);
    if (blockIdx.x == 0 && threadIdx.x == 0) counts[2] = 0;
    const int stride = gridDim.x * blockDim.x;
    // whole blocks iterate together (block_append is block-collective)
    for (int base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const int h = base + (int)threadIdx.x;
        bool filled = false;
        int32_t g = 0;
        if (h < n) {
            g = load_mutable<kL2>(list_in + h);
            const MapPixel m = maps.at(g);
            const uchar2 t = m.table[(int64_t)m.y * m.cols + m.x];
            filled = fill_hole<kL2>(map, stamp, g, hole_offsets(t, g, m.cols), 1, valid_at_most);
        }
        block_append(filled, g, counts + 1, list_out);
    }
}

// Step `step` >= 2: visits the open holes next to the pixels filled at step - 1 (list_in) that read
// one of them, fills those it can and lists them.  One thread per (filled pixel, neighbour): the
// frontier is short after the first steps, and a thread's work is a chain of dependent loads, so
// spreading the 8 neighbours over threads keeps a step's time near one chain's latency.  Returns
// the number of pixels filled at step - 1.
template <bool kL2, typename Maps>
__device__ __forceinline__ int hole_frontier_step(const Maps& maps, float* __restrict__ map,
                                                  uint8_t* __restrict__ stamp, int32_t* __restrict__ claim, int step,
                                                  int32_t* __restrict__ counts, const int32_t* __restrict__ list_in,
                                                  int32_t* __restrict__ list_out, float valid_at_most)
{
    const int n = load_mutable<kL2>(counts + (step - 1) % 3);
    if (blockIdx.x == 0 && threadIdx.x == 0) counts[(step + 1) % 3] = 0;
    const int64_t work = (int64_t)n * 8;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    // whole blocks iterate together (block_append is block-collective)
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < work; base += stride) {
        const int64_t h = base + threadIdx.x;
        bool filled = false;
        int64_t q = 0;
        if (h < work) {
            const int64_t p = load_mutable<kL2>(list_in + (h >> 3));
            const int k = (int)(h & 7);
            const int dx = k < 3 ? k - 1 : k == 3 ? -1 : k == 4 ? 1 : k - 6;  // the 8 neighbours
            const int dy = k < 3 ? -1 : k < 5 ? 0 : 1;
            const MapPixel m = maps.at(p);
            const int qx = m.x + dx, qy = m.y + dy;
            if (qx >= 1 && qy >= 1 && qx < m.cols - 1 && qy < m.rows - 1) {
                q = p + (int64_t)dy * m.cols + dx;
                if (load_mutable<kL2>(stamp + q) == kUnfilled) {
                    const HoleOffsets o = hole_offsets(m.table[(int64_t)qy * m.cols + qx], q, m.cols);
                    // q reads p, and no other thread has queued q for this step
                    filled = ((o.w0 > 0.0f && o.n0 == p) || (o.w1 > 0.0f && o.n1 == p)) &&
                             atomicMax(claim + q, step) < step &&
                             fill_hole<kL2>(map, stamp, q, o, step, valid_at_most);
                }
            }
        }
        block_append(filled, (int32_t)q, counts + step % 3, list_out);
    }
    return n;
}

// ---------------------------------------------------------------------------------------------
// The tail of the hole filling (the uniform batch): after the first steps, a step fills a few
// hundred holes per map, and a launch per step costs more than its work.  A hole only reads
// pixels of its own map, so the later steps of a map depend on nothing outside it: one block per
// map runs them all, separated by block barriers, with its frontier lists in its map's own region
// of the list arrays.  hole_tail_collect_kernel first gives each map the entries of the global
// list (the fills of step first - 1) that lie in it: region[0] is their count, region[1..] the
// pixels; hole_tail_kernel then runs steps first .. iterations with the same per-hole work as
// hole_frontier_step, so the results are those of the launches per step.
// ---------------------------------------------------------------------------------------------
constexpr int kTailBlock = 1024;

__global__ void __launch_bounds__(kStitchBlock) hole_tail_collect_kernel(int64_t map_pixels,
                                                                         const int32_t* __restrict__ count,
                                                                         const int32_t* __restrict__ list,
                                                                         int32_t* __restrict__ regions)
{
    __shared__ int n_map;
    const int64_t begin = (int64_t)blockIdx.x * map_pixels, end = begin + map_pixels;
    if (threadIdx.x == 0) n_map = 0;
    __syncthreads();
    const int n = *count;
    for (int h = threadIdx.x; h < n; h += blockDim.x) {
        const int32_t g = list[h];
        if (g >= begin && g < end) regions[begin + 1 + atomicAdd(&n_map, 1)] = g;
    }
    __syncthreads();
    if (threadIdx.x == 0) regions[begin] = n_map;
}

template <typename Maps>
__global__ void __launch_bounds__(kTailBlock) hole_tail_kernel(const Maps maps, int64_t map_pixels,
                                                               float* __restrict__ map, uint8_t* __restrict__ stamp,
                                                               int32_t* __restrict__ claim, int first, int iterations,
                                                               int32_t* __restrict__ regions_a,
                                                               int32_t* __restrict__ regions_b, float valid_at_most)
{
    __shared__ int n_cur, n_next;
    const int64_t begin = (int64_t)blockIdx.x * map_pixels;
    int32_t* cur = regions_a + begin + 1;  // region[0] holds the collected count
    int32_t* nxt = regions_b + begin + 1;
    if (threadIdx.x == 0) n_cur = regions_a[begin];
    __syncthreads();
    for (int step = first; step <= iterations; ++step) {
        const int nc = n_cur;  // the same value in every thread: the loop ends for the whole block
        if (nc == 0) break;
        if (threadIdx.x == 0) n_next = 0;
        __syncthreads();
        for (int64_t h = threadIdx.x; h < (int64_t)nc * 8; h += blockDim.x) {
            const int64_t p = cur[h >> 3];
            const int k = (int)(h & 7);
            const int dx = k < 3 ? k - 1 : k == 3 ? -1 : k == 4 ? 1 : k - 6;  // the 8 neighbours
            const int dy = k < 3 ? -1 : k < 5 ? 0 : 1;
            const MapPixel m = maps.at(p);
            const int qx = m.x + dx, qy = m.y + dy;
            if (qx >= 1 && qy >= 1 && qx < m.cols - 1 && qy < m.rows - 1) {
                const int64_t q = p + (int64_t)dy * m.cols + dx;
                if (stamp[q] == kUnfilled) {
                    const HoleOffsets o = hole_offsets(m.table[(int64_t)qy * m.cols + qx], q, m.cols);
                    // q reads p, and no other thread has taken q for this step
                    if (((o.w0 > 0.0f && o.n0 == p) || (o.w1 > 0.0f && o.n1 == p)) &&
                        atomicMax(claim + q, step) < step && fill_hole(map, stamp, q, o, step, valid_at_most))
                        nxt[atomicAdd(&n_next, 1)] = (int32_t)q;
                }
            }
        }
        __syncthreads();  // this step's fills are visible to the block before the next step reads them
        int32_t* t = cur;
        cur = nxt;
        nxt = t;
        if (threadIdx.x == 0) n_cur = n_next;
        __syncthreads();
    }
}

template <typename Maps>
__global__ void __launch_bounds__(kStitchBlock) hole_first_step_kernel(const Maps maps, float* __restrict__ map,
                                                                       uint8_t* __restrict__ stamp,
                                                                       int32_t* __restrict__ counts,
                                                                       const int32_t* __restrict__ list_in,
                                                                       int32_t* __restrict__ list_out,
                                                                       float valid_at_most)
{
    hole_first_step<false>(maps, map, stamp, counts, list_in, list_out, valid_at_most);
}

template <typename Maps>
__global__ void __launch_bounds__(kStitchBlock) hole_frontier_step_kernel(const Maps maps, float* __restrict__ map,
                                                                          uint8_t* __restrict__ stamp,
                                                                          int32_t* __restrict__ claim, int step,
                                                                          int32_t* __restrict__ counts,
                                                                          const int32_t* __restrict__ list_in,
                                                                          int32_t* __restrict__ list_out,
                                                                          float valid_at_most)
{
    hole_frontier_step<false>(maps, map, stamp, claim, step, counts, list_in, list_out, valid_at_most);
}

// ---------------------------------------------------------------------------------------------
// The hole-filling steps after the first in one cooperative launch: steps 2 .. iterations run as
// phases of a grid whose blocks are all resident (cudaLaunchCooperativeKernel guarantees it or
// refuses the launch), separated by grid-wide barriers.  After step 2 a step's frontier is
// a few hundred holes per map, so a launch per step costs more in launch gaps than in work; here
// a step costs one barrier.  Phases read what other SMs wrote in earlier phases through L2.
// Every barrier wait is bounded: a wait that runs out raises the launch's abort word (the other
// blocks then leave at their next barrier) and SSG_STATUS_BARRIER_TIMEOUT in the status word,
// and the maps are left partly filled.
// ---------------------------------------------------------------------------------------------
constexpr int kBarrierMaxPolls = 1 << 22;  // each poll sleeps ~0.1 us: a wait gives up after ~0.5 s

static __device__ uint32_t g_stitch_status;

// the launch's barrier words: the arrivals, the generation (advanced by the last arrival), abort
struct GridSync {
    uint32_t* count;
    uint32_t* generation;
    uint32_t* abort;
};

// true when every block of the grid arrived; false when the wait ran out or another block gave up
__device__ __forceinline__ bool grid_barrier(const GridSync& b)
{
    __shared__ int passed;
    __syncthreads();  // the block's writes of this phase precede its arrival
    if (threadIdx.x == 0) {
        const uint32_t gen = *reinterpret_cast<volatile uint32_t*>(b.generation);
        bool ok = true;
        __threadfence();
        if (atomicAdd(b.count, 1u) == gridDim.x - 1) {
            atomicExch(b.count, 0u);
            __threadfence();
            atomicAdd(b.generation, 1u);
        } else {
            for (int polls = 0; *reinterpret_cast<volatile uint32_t*>(b.generation) == gen; ++polls) {
                if (*reinterpret_cast<volatile uint32_t*>(b.abort) != 0u || polls >= kBarrierMaxPolls) {
                    ok = false;
                    break;
                }
                __nanosleep(100);
            }
        }
        if (!ok) {
            atomicExch(b.abort, 1u);
            atomicOr(&g_stitch_status, SSG_STATUS_BARRIER_TIMEOUT);
        }
        __threadfence();
        passed = ok;
    }
    __syncthreads();
    return passed != 0;
}

template <typename Maps>
__global__ void __launch_bounds__(kStitchBlock) hole_fill_persistent_kernel(
    const Maps maps, float* __restrict__ map, uint8_t* __restrict__ stamp, int32_t* __restrict__ claim,
    float valid_at_most, int iterations, int32_t* __restrict__ counts, int32_t* __restrict__ list0,
    int32_t* __restrict__ list1, const GridSync sync)
{
    for (int s = 2; s <= iterations; ++s) {
        if (s > 2 && !grid_barrier(sync)) return;
        int32_t* in = (s & 1) ? list0 : list1;  // step s reads lists[(s - 1) % 2], writes lists[s % 2]
        int32_t* out = (s & 1) ? list1 : list0;
        // every block reads the same count after the barrier: an empty frontier ends all of them
        if (hole_frontier_step<true>(maps, map, stamp, claim, s, counts, in, out, valid_at_most) == 0)
            return;
    }
}

uint32_t take_stitch_status(cudaError_t* err)
{
    uint32_t v = 0, zero = 0;
    *err = cudaMemcpyFromSymbol(&v, g_stitch_status, sizeof(uint32_t));
    if (*err == cudaSuccess) *err = cudaMemcpyToSymbol(g_stitch_status, &zero, sizeof(uint32_t));
    return v;
}

// blocks of a grid-stride launch: a few per SM
static int resident_grid(int per_sm)
{
    static std::atomic<int> sms[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152 * per_sm;
    int n = sms[dev].load();
    if (n == 0) {
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
        sms[dev].store(n);
    }
    return n * per_sm;
}

// The hole filling of `total` flat map pixels (see above): d_holes holds 3 rotating counts (+ 1),
// two lists and a claim word per pixel
// Blocks per SM of the cooperative hole filling on the current device (0: no cooperative launch)
template <typename Maps>
static int persistent_blocks_per_sm()
{
    static std::atomic<int> cached[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
    int n = cached[dev].load();
    if (n == 0) {
        int coop = 0, per_sm = 0;
        if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, hole_fill_persistent_kernel<Maps>, kStitchBlock,
                                                          0) != cudaSuccess)
            per_sm = 0;
        cudaGetLastError();
        n = per_sm > 0 ? per_sm : -1;
        cached[dev].store(n);
    }
    return n > 0 ? n : 0;
}

// tail_map_pixels: pixels of each map when all maps have one size (the uniform batch), enabling
// the per-map tail of the later steps; 0 otherwise
template <typename Maps>
static int inpaint_lists(const Maps& maps, int64_t total, float* d_map, uint8_t* d_stamps, int32_t* d_holes,
                         double max_dist, int iterations, cudaStream_t st, int64_t tail_map_pixels = 0)
{
    if (iterations == 0) return SSG_OK;
    const float hole = float_at_least(max_dist + 0.1);
    const float ok = float_at_most(max_dist + (double)0.1f);
    // header: 3 rotating counts and a spare, then the barrier words (arrivals, generation, abort)
    int32_t* counts = d_holes;
    int32_t* lists[2] = {d_holes + SSG_HOLE_SCRATCH_HEADER, d_holes + SSG_HOLE_SCRATCH_HEADER + total};
    int32_t* claims = d_holes + SSG_HOLE_SCRATCH_HEADER + 2 * total;
    const cudaError_t e = cudaMemsetAsync(counts, 0, SSG_HOLE_SCRATCH_HEADER * sizeof(int32_t), st);
    if (e != cudaSuccess) return fail(SSG_ERR_CUDA, "cudaMemsetAsync: %s", cudaGetErrorString(e));
    const bool vec = ((uintptr_t)d_map & 15) == 0 && ((uintptr_t)d_stamps & 7) == 0 && total % kScanPixels == 0;
    hole_scan_wide_kernel<Maps><<<grid_1d((total + kScanPixels - 1) / kScanPixels, kStitchBlock), kStitchBlock, 0,
                                  st>>>(maps, total, d_map, d_stamps, claims, hole, vec, counts, lists[0]);
    if (int err = launch_status("hole_scan_wide_kernel")) return err;
    const int grid = resident_grid(tuning(SSG_TUNE_HOLE_BLOCKS_PER_SM));
    hole_first_step_kernel<Maps><<<grid, kStitchBlock, 0, st>>>(maps, d_map, d_stamps, counts, lists[0], lists[1],
                                                                ok);
    if (int err = launch_status("hole_first_step_kernel")) return err;
    if (iterations == 1) return SSG_OK;
    const int per_sm = tuning(SSG_TUNE_HOLE_PERSISTENT) == 1 ? persistent_blocks_per_sm<Maps>() : 0;
    if (per_sm > 0) {
        // one block per SM: the barrier's arrivals are one atomic per block, and a step after the
        // first has a few thousand holes to visit
        const int pgrid = resident_grid(1);
        uint32_t* words = reinterpret_cast<uint32_t*>(d_holes + 4);
        const GridSync sync{words, words + 1, words + 2};
        void* args[] = {(void*)&maps, (void*)&d_map, (void*)&d_stamps, (void*)&claims, (void*)&ok, (void*)&iterations,
                        (void*)&counts, (void*)&lists[0], (void*)&lists[1], (void*)&sync};
        const cudaError_t le = cudaLaunchCooperativeKernel((const void*)hole_fill_persistent_kernel<Maps>,
                                                           dim3(pgrid), dim3(kStitchBlock), args, 0, st);
        if (le != cudaSuccess) return fail(SSG_ERR_CUDA, "hole_fill_persistent_kernel: %s", cudaGetErrorString(le));
        return SSG_OK;
    }
    // the uniform batch: a launch per step up to the tail, then one block per map for the rest
    const int first_tail = tail_map_pixels > 0 ? tuning(SSG_TUNE_HOLE_TAIL) : 0;
    const int last_launched = first_tail > 0 ? std::min(iterations, first_tail - 1) : iterations;
    for (int s = 2; s <= last_launched; ++s) {
        hole_frontier_step_kernel<Maps><<<grid, kStitchBlock, 0, st>>>(maps, d_map, d_stamps, claims, s, counts,
                                                                       lists[(s - 1) % 2], lists[s % 2], ok);
        if (int err = launch_status("hole_frontier_step_kernel")) return err;
    }
    if (first_tail > 0 && iterations >= first_tail) {
        const int maps_count = (int)(total / tail_map_pixels);
        // step first_tail - 1 listed its fills in lists[(first_tail - 1) % 2], counted by
        // counts[(first_tail - 1) % 3]; the tail's first regions go into the other array
        int32_t* in = lists[(first_tail - 1) % 2];
        int32_t* other = lists[first_tail % 2];
        hole_tail_collect_kernel<<<maps_count, kStitchBlock, 0, st>>>(tail_map_pixels,
                                                                      counts + (first_tail - 1) % 3, in, other);
        if (int err = launch_status("hole_tail_collect_kernel")) return err;
        hole_tail_kernel<Maps><<<maps_count, kTailBlock, 0, st>>>(maps, tail_map_pixels, d_map, d_stamps, claims,
                                                                  first_tail, iterations, other, in, ok);
        if (int err = launch_status("hole_tail_kernel")) return err;
    }
    return SSG_OK;
}

struct MergeParams {
    int cols, rows, pano_cols, pano_rows, nref, image_rows, image_cols;
    float ratio_x, ratio_y;
    int word_rows;  // the images start and end on 4-byte boundaries: texel pairs read as words
    int64_t image_frame;                // bytes of a frame's images
    // the image of a frame that reference r stitches.  The sample row is formed as in a stack of
    // the references' images (row + r x image_rows, in float as stitcher.cu forms it), and the
    // image pointer is moved by (image_slot[r] - r) images, so that the arithmetic does not depend
    // on where the images lie
    int image_slot[SSG_MAX_REFERENCES];
    Intr k[SSG_MAX_REFERENCES];
    float t[SSG_MAX_REFERENCES][3];
};

// interp (stitcher.cu:56-83) on uint8 RGB
__device__ __forceinline__ void interp_rgb(const uint8_t* __restrict__ img, float u, float v, int cols, float out[3])
{
    const int u1 = __float2int_rd(u), v1 = __float2int_rd(v), u2 = u1 + 1, v2 = v1 + 1;
    const float w1 = fmul(fsub((float)u2, u), fsub((float)v2, v)), w2 = fmul(fsub((float)u2, u), fsub(v, (float)v1));
    const float w3 = fmul(fsub(u, (float)u1), fsub((float)v2, v)), w4 = fmul(fsub(u, (float)u1), fsub(v, (float)v1));
    const uint8_t* p1 = img + 3 * ((int64_t)v1 * cols + u1);
    const uint8_t* p2 = img + 3 * ((int64_t)v2 * cols + u1);
    const uint8_t* p3 = img + 3 * ((int64_t)v1 * cols + u2);
    const uint8_t* p4 = img + 3 * ((int64_t)v2 * cols + u2);
#pragma unroll
    for (int ch = 0; ch < 3; ++ch)
        out[ch] = fadd(fadd(fadd(fmul((float)p1[ch], w1), fmul((float)p2[ch], w2)), fmul((float)p3[ch], w3)),
                       fmul((float)p4[ch], w4));
}

// Bilinear sample of a float map and of uint8 RGB (interpF, interp: stitcher.cu:56-116) in
// fused multiply-adds, for the batched 16-bit path's merge
__device__ __forceinline__ float interp_f_fast(const float* __restrict__ s, float u, float v, int cols)
{
    const float u1f = floorf(u), v1f = floorf(v);
    const int u1 = (int)u1f, v1 = (int)v1f;
    const float fu = u - u1f, fv = v - v1f;
    const float* r0 = s + (int64_t)v1 * cols + u1;
    const float p1 = __ldg(r0), p3 = __ldg(r0 + 1), p2 = __ldg(r0 + cols), p4 = __ldg(r0 + cols + 1);
    const float top = fmaf(fu, p3 - p1, p1), bot = fmaf(fu, p4 - p2, p2);
    return fmaf(fv, bot - top, top);
}

// The six bytes of two horizontally adjacent RGB texels from the aligned 32-bit words that hold
// them (two words, three when the pair starts at byte 3 of a word): lo = bytes 0..3 of the pair,
// hi = bytes 4, 5.  Only words holding one of the six bytes are read, so a buffer that starts
// and ends on 4-byte boundaries is never read outside.
__device__ __forceinline__ void texel_pair_words(const uint8_t* p, uint32_t& lo, uint32_t& hi)
{
    const uintptr_t a = reinterpret_cast<uintptr_t>(p);
    const uint32_t* w = reinterpret_cast<const uint32_t*>(a & ~(uintptr_t)3);
    const uint32_t s = (uint32_t)(a & 3) * 8;
    const uint32_t w0 = __ldg(w), w1 = __ldg(w + 1);
    const uint32_t w2 = s == 24 ? __ldg(w + 2) : 0u;
    lo = __funnelshift_r(w0, w1, s);
    hi = __funnelshift_r(w1, w2, s);
}

// words: the texel pairs are read with texel_pair_words (same values, fewer loads)
__device__ __forceinline__ void interp_rgb_fast(const uint8_t* __restrict__ img, float u, float v, int cols,
                                                float out[3], bool words = false)
{
    const float u1f = floorf(u), v1f = floorf(v);
    const int u1 = (int)u1f, v1 = (int)v1f;
    const float fu = u - u1f, fv = v - v1f;
    const uint8_t* p1 = img + 3 * ((int64_t)v1 * cols + u1);
    const uint8_t* p2 = p1 + 3 * (int64_t)cols;
    if (words) {
        uint32_t t0, t1, b0, b1;
        texel_pair_words(p1, t0, t1);
        texel_pair_words(p2, b0, b1);
        const uint32_t tr = __byte_perm(t0, t1, 0x0543), br = __byte_perm(b0, b1, 0x0543);  // right texels
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) {
            const float a = (float)((t0 >> (8 * ch)) & 0xFFu), b = (float)((tr >> (8 * ch)) & 0xFFu);
            const float c = (float)((b0 >> (8 * ch)) & 0xFFu), d = (float)((br >> (8 * ch)) & 0xFFu);
            const float top = fmaf(fu, b - a, a), bot = fmaf(fu, d - c, c);
            out[ch] = fmaf(fv, bot - top, top);
        }
        return;
    }
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
        const float a = p1[ch], b = p1[3 + ch], c = p2[ch], d = p2[3 + ch];
        const float top = fmaf(fu, b - a, a), bot = fmaf(fu, d - c, c);
        out[ch] = fmaf(fv, bot - top, top);
    }
}

// Double-sphere unprojection / projection of the stitcher (stitcher.cu:121-168) with
// approximate square roots and reciprocals
__device__ __forceinline__ void unproject_fast(float u, float v, const Intr& k, float p[3])
{
    const float mx = (u - k.cx) / k.fx, my = (v - k.cy) / k.fy;
    const float r2 = fmaf(my, my, mx * mx);
    const float mz = (1.0f - k.alpha * k.alpha * r2) *
                     rcp_approx(fmaf(k.alpha, sqrt_approx(1.0f - (2.0f * k.alpha - 1.0f) * r2), 1.0f - k.alpha));
    const float mz2 = mz * mz;
    const float s = fmaf(mz, k.xi, sqrt_approx(fmaf(1.0f - k.xi * k.xi, r2, mz2))) * rcp_approx(mz2 + r2);
    p[0] = mx * s;
    p[1] = my * s;
    p[2] = fmaf(mz, s, -k.xi);
}

__device__ __forceinline__ void project_fast(const float p[3], const Intr& k, float uv[2])
{
    const float rxy = fmaf(p[1], p[1], p[0] * p[0]);
    const float d1 = sqrt_approx(fmaf(p[2], p[2], rxy));
    const float c = fmaf(k.xi, d1, p[2]);
    const float d2 = sqrt_approx(fmaf(c, c, rxy));
    const float den = rcp_approx(fmaf(k.alpha, d2, (1.0f - k.alpha) * c));
    uv[0] = fmaf(k.fx * p[0], den, k.cx);
    uv[1] = fmaf(k.fy * p[1], den, k.cy);
}

// mergeRGBDPanoramaKernel, stitcher.cu:423-473
__global__ void __launch_bounds__(kStitchBlock) merge_kernel(const __grid_constant__ MergeParams p,
                                                             const float2* __restrict__ lut,
                                                             const float* __restrict__ weights,
                                                             const float* __restrict__ reproj,
                                                             const float* __restrict__ dists,
                                                             const uint8_t* __restrict__ images,
                                                             float* __restrict__ dist_pano,
                                                             uint8_t* __restrict__ rgb_pano)
{
    const int64_t Q = (int64_t)p.pano_cols * p.pano_rows;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Q) return;
    // blockIdx.y: frame of a batch of contiguous maps, images and panoramas
    const int64_t frame = blockIdx.y;
    reproj += frame * p.nref * (int64_t)p.cols * p.rows;
    dists += frame * p.nref * (int64_t)p.cols * p.rows;
    images += frame * p.image_frame;
    dist_pano += frame * Q;
    rgb_pano += frame * Q * 3;
    float inv = 0.0f, rgb[3] = {0.0f, 0.0f, 0.0f};
    const float colsm = fsub((float)p.image_cols, 1.1f), rowsm = fsub((float)p.image_rows, 1.1f);
    for (int r = 0; r < p.nref; ++r) {
        const float w = weights[(int64_t)r * Q + i];
        float2 uv = lut[(int64_t)r * Q + i];
        // the table kernel already clamps to [0.1, size - 1.1]; clamping again is exact for its
        // output and keeps any other table inside the maps
        uv.x = fminf(fmaxf(uv.x, 0.1f), fsub((float)p.cols, 1.1f));
        uv.y = fminf(fmaxf(uv.y, 0.1f), fsub((float)p.rows, 1.1f));
        const float vo = fadd(uv.y, (float)(r * p.rows));
        const float rd = interp_f(reproj, uv.x, vo, p.cols);
        inv = fadd(inv, fdiv(fmul(w, 1.0f), rd));
        float dc = interp_f(dists, uv.x, vo, p.cols);
        dc = fminf(rd, dc);
        float pt[3];
        unproject_cu(uv.x, uv.y, p.k[r], pt);
#pragma unroll
        for (int a = 0; a < 3; ++a) pt[a] = fadd(fmul(dc, pt[a]), p.t[r][a]);
        float o[2];
        project_cu(pt, p.k[r], o, nullptr);
        o[0] = fmul(o[0], p.ratio_x);
        o[1] = fmul(o[1], p.ratio_y);
        o[0] = fminf(fmaxf(o[0], 0.1f), colsm);
        o[1] = fminf(fmaxf(o[1], 0.1f), rowsm);
        o[1] = fadd(o[1], (float)(r * p.image_rows));
        float c[3];
        interp_rgb(images + (int64_t)(p.image_slot[r] - r) * p.image_rows * p.image_cols * 3, o[0], o[1],
                   p.image_cols, c);
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) rgb[ch] = fadd(rgb[ch], fmul(c[ch], w));
    }
    dist_pano[i] = fdiv(1.0f, inv);
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) rgb_pano[3 * i + ch] = (uint8_t)__float2uint_rz(fminf(rgb[ch], 255.0f));
}

// The approximate merge for a batch of frames of one rig: the blending table, the weights and the
// unprojected ray of each (panorama pixel, reference) are the same for every frame, so a thread
// reads and unprojects them once and applies them to kMergeFrames frames (blockIdx.y: group of
// frames; SSG_TUNE_MERGE_FRAMES), which also gives it that many independent gathers in flight.
template <int kMergeFrames>
__global__ void __launch_bounds__(kStitchBlock) merge_frames_kernel(const __grid_constant__ MergeParams p,
                                                                    int frames, const float2* __restrict__ lut,
                                                                    const float* __restrict__ weights,
                                                                    const float* __restrict__ reproj,
                                                                    const float* __restrict__ dists,
                                                                    const uint8_t* __restrict__ images,
                                                                    float* __restrict__ dist_pano,
                                                                    uint8_t* __restrict__ rgb_pano)
{
    const int64_t Q = (int64_t)p.pano_cols * p.pano_rows;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Q) return;
    const int f0 = blockIdx.y * kMergeFrames;
    const int nf = min(kMergeFrames, frames - f0);
    const int64_t map_frame = (int64_t)p.nref * p.cols * p.rows;
    const int64_t image_frame = p.image_frame;
    reproj += f0 * map_frame;
    dists += f0 * map_frame;
    images += f0 * image_frame;
    float inv[kMergeFrames], rgb[kMergeFrames][3];
#pragma unroll
    for (int f = 0; f < kMergeFrames; ++f) inv[f] = rgb[f][0] = rgb[f][1] = rgb[f][2] = 0.0f;
    const float colsm = fsub((float)p.image_cols, 1.1f), rowsm = fsub((float)p.image_rows, 1.1f);
    for (int r = 0; r < p.nref; ++r) {
        const float w = weights[(int64_t)r * Q + i];
        float2 uv = lut[(int64_t)r * Q + i];
        uv.x = fminf(fmaxf(uv.x, 0.1f), fsub((float)p.cols, 1.1f));
        uv.y = fminf(fmaxf(uv.y, 0.1f), fsub((float)p.rows, 1.1f));
        const float vo = fadd(uv.y, (float)(r * p.rows));
        float ray[3];
        unproject_fast(uv.x, uv.y, p.k[r], ray);
        // the bilinear taps of both maps are at the same place in every frame (interp_f_fast)
        const float u1f = floorf(uv.x), v1f = floorf(vo);
        const float fu = uv.x - u1f, fv = vo - v1f;
        const int64_t tap = (int64_t)(int)v1f * p.cols + (int)u1f;
#pragma unroll
        for (int f = 0; f < kMergeFrames; ++f) {
            if (f < nf) {
                const float* a = reproj + f * map_frame + tap;
                const float* b = dists + f * map_frame + tap;
                const float a1 = __ldg(a), a3 = __ldg(a + 1), a2 = __ldg(a + p.cols), a4 = __ldg(a + p.cols + 1);
                const float b1 = __ldg(b), b3 = __ldg(b + 1), b2 = __ldg(b + p.cols), b4 = __ldg(b + p.cols + 1);
                const float at = fmaf(fu, a3 - a1, a1), ab = fmaf(fu, a4 - a2, a2);
                const float bt = fmaf(fu, b3 - b1, b1), bb = fmaf(fu, b4 - b2, b2);
                const float rd = fmaf(fv, ab - at, at);
                inv[f] = fmaf(w, rcp_approx(rd), inv[f]);
                const float dc = fminf(rd, fmaf(fv, bb - bt, bt));
                float pt[3], o[2], c[3];
#pragma unroll
                for (int a = 0; a < 3; ++a) pt[a] = fmaf(dc, ray[a], p.t[r][a]);
                project_fast(pt, p.k[r], o);
                o[0] = fminf(fmaxf(fmul(o[0], p.ratio_x), 0.1f), colsm);
                o[1] = fadd(fminf(fmaxf(fmul(o[1], p.ratio_y), 0.1f), rowsm), (float)(r * p.image_rows));
                interp_rgb_fast(images + f * image_frame + (int64_t)(p.image_slot[r] - r) * p.image_rows *
                                                               p.image_cols * 3,
                                o[0], o[1], p.image_cols, c, p.word_rows != 0);
#pragma unroll
                for (int ch = 0; ch < 3; ++ch) rgb[f][ch] = fmaf(c[ch], w, rgb[f][ch]);
            }
        }
    }
#pragma unroll
    for (int f = 0; f < kMergeFrames; ++f) {
        if (f < nf) {
            const int64_t o = (int64_t)(f0 + f) * Q + i;
            dist_pano[o] = rcp_approx(inv[f]);
#pragma unroll
            for (int ch = 0; ch < 3; ++ch) rgb_pano[3 * o + ch] = (uint8_t)__float2uint_rz(fminf(rgb[f][ch], 255.0f));
        }
    }
}

// The tile kernel needs more than 48 KB of dynamic shared memory: opt in once per device.
static int enable_inpaint_smem()
{
    static std::atomic<uint64_t> done{0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return launch_status("cudaGetDevice");
    const uint64_t bit = 1ull << (dev & 63);
    if (done.load() & bit) return SSG_OK;
    const cudaError_t e =
        cudaFuncSetAttribute(inpaint_tile_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kInpaintSmem);
    if (e != cudaSuccess) return fail(SSG_ERR_CUDA, "cudaFuncSetAttribute(inpaint_tile_kernel): %s", cudaGetErrorString(e));
    done.fetch_or(bit);
    return SSG_OK;
}

static int check_intrinsics(const ssg_intrinsics* k, int n)
{
    SSG_REQUIRE(k, "intrinsics must not be NULL");
    for (int r = 0; r < n; ++r) {
        SSG_REQUIRE(std::isfinite(k[r].xi) && std::isfinite(k[r].alpha) && k[r].alpha > 0.0f && k[r].alpha <= 1.0f,
                    "intrinsics %d: xi must be finite and alpha in (0, 1]", r);
        SSG_REQUIRE(k[r].fx != 0.0f && k[r].fy != 0.0f, "intrinsics %d: zero focal length", r);
    }
    return SSG_OK;
}

}  // namespace ssg

using namespace ssg;

extern "C" int ssg_inpainting_table(int cols, int rows, const ssg_intrinsics* intrinsics, const float* translation,
                                    double min_dist, double max_dist, uint8_t* d_table, void* stream)
{
    SSG_REQUIRE(cols > 0 && rows > 0, "resolution must be positive");
    SSG_REQUIRE(translation && d_table, "null pointer");
    if (int e = check_intrinsics(intrinsics, 1)) return e;
    const int64_t P = (int64_t)cols * rows;
    inpainting_table_kernel<<<grid_1d(P, kStitchBlock), kStitchBlock, 0, as_stream(stream)>>>(
        cols, rows, to_intr(*intrinsics), translation[0], translation[1], translation[2], (float)min_dist,
        (float)max_dist, d_table);
    return launch_status("inpainting_table_kernel");
}

extern "C" int ssg_box_filter(const float* d_in, int planes, int rows, int cols, int radius, float pad_value,
                              float* d_out, void* stream)
{
    SSG_REQUIRE(d_in && d_out && d_in != d_out, "null or aliased pointers");
    SSG_REQUIRE(planes > 0 && planes <= 65535 && rows > 0 && cols > 0 && radius >= 0, "invalid sizes");
    const int64_t P = (int64_t)cols * rows;
    const int side = 2 * radius + 1;
    const float kw = 1.0f / (float)(side * side);
    const size_t smem = sizeof(float) * (size_t)box_tile_floats(radius);
    if (radius <= 64 && smem <= 48 * 1024) {
        const dim3 grid((unsigned)((cols + kBoxX - 1) / kBoxX), (unsigned)((rows + kBoxY - 1) / kBoxY), planes);
        SSG_REQUIRE(grid.y <= 65535, "maps of %d rows are too tall", rows);
        box_filter_tiled_kernel<<<grid, kBoxThreadsX * kBoxThreadsY, smem, as_stream(stream)>>>(
            d_in, rows, cols, radius, pad_value, kw, d_out);
        return launch_status("box_filter_tiled_kernel");
    }
    dim3 grid(grid_1d(P, kStitchBlock), planes);
    box_filter_kernel<<<grid, kStitchBlock, 0, as_stream(stream)>>>(d_in, rows, cols, radius, pad_value, kw, d_out);
    return launch_status("box_filter_kernel");
}

extern "C" int ssg_blending_lut(int cols, int rows, int pano_cols, int pano_rows, int reference_count,
                                const ssg_intrinsics* intrinsics, const float* rotations, const float* translations,
                                const float* d_masks, double min_dist, double max_dist, float* d_lut, float* d_weights,
                                void* stream)
{
    SSG_REQUIRE(cols > 0 && rows > 0 && pano_cols > 0 && pano_rows > 0, "resolutions must be positive");
    SSG_REQUIRE(reference_count >= 1 && reference_count <= SSG_MAX_REFERENCES, "reference_count %d outside [1, %d]",
                reference_count, SSG_MAX_REFERENCES);
    SSG_REQUIRE(rotations && translations && d_masks && d_lut && d_weights, "null pointer");
    if (int e = check_intrinsics(intrinsics, reference_count)) return e;
    LutParams p{};
    p.cols = cols;
    p.rows = rows;
    p.pano_cols = pano_cols;
    p.pano_rows = pano_rows;
    p.nref = reference_count;
    p.dmin = (float)min_dist;
    p.dmax = (float)max_dist;
    for (int r = 0; r < reference_count; ++r) {
        p.k[r] = to_intr(intrinsics[r]);
        std::memcpy(p.rot[r], rotations + 9 * r, sizeof(float) * 9);
        std::memcpy(p.t[r], translations + 3 * r, sizeof(float) * 3);
    }
    const int64_t Q = (int64_t)pano_cols * pano_rows;
    blending_lut_kernel<<<grid_1d(Q, kStitchBlock), kStitchBlock, 0, as_stream(stream)>>>(
        p, d_masks, reinterpret_cast<float2*>(d_lut), d_weights);
    return launch_status("blending_lut_kernel");
}

extern "C" int ssg_normalize_weights(float* d_weights, int reference_count, int64_t pixels, void* stream)
{
    SSG_REQUIRE(d_weights, "null pointer");
    SSG_REQUIRE(reference_count >= 1 && pixels >= 0, "invalid sizes");
    if (pixels == 0) return SSG_OK;
    normalize_weights_kernel<<<grid_1d(pixels, kStitchBlock), kStitchBlock, 0, as_stream(stream)>>>(
        d_weights, reference_count, pixels);
    return launch_status("normalize_weights_kernel");
}

extern "C" int ssg_reproject_distance(const float* d_distance_in, float* d_distance_out, int cols, int rows,
                                      const ssg_intrinsics* intrinsics, const float* translation, int fill,
                                      void* stream)
{
    SSG_REQUIRE(d_distance_in && d_distance_out && translation, "null pointer");
    SSG_REQUIRE(d_distance_in != d_distance_out, "input and output maps must differ");
    SSG_REQUIRE(cols > 0 && rows > 0 && (int64_t)cols * rows < ((int64_t)1 << 31), "resolution out of range");
    if (int e = check_intrinsics(intrinsics, 1)) return e;
    const int64_t P = (int64_t)cols * rows;
    if (fill) {
        if (int e = fill_map(d_distance_out, P, 1e8f, as_stream(stream))) return e;
    }
    ReprojParams p{};
    p.cols = cols;
    p.rows = rows;
    p.references = 1;
    p.k[0] = to_intr(*intrinsics);
    std::memcpy(p.t[0], translation, sizeof(float) * 3);
    reproject_kernel<<<grid_1d(P, kStitchBlock), kStitchBlock, 0, as_stream(stream)>>>(p, d_distance_in,
                                                                                       d_distance_out);
    return launch_status("reproject_kernel");
}

static int reproject_batch(const float* d_distance_in, float* d_distance_out, int cols, int rows, int instances,
                           int references, const ssg_intrinsics* intrinsics, const float* translations, int fill,
                           bool fast, void* stream)
{
    SSG_REQUIRE(d_distance_in && d_distance_out && translations, "null pointer");
    SSG_REQUIRE(d_distance_in != d_distance_out, "input and output maps must differ");
    SSG_REQUIRE(cols > 0 && rows > 0 && (int64_t)cols * rows < ((int64_t)1 << 31), "resolution out of range");
    SSG_REQUIRE(references >= 1 && references <= SSG_MAX_REFERENCES, "references out of range");
    SSG_REQUIRE(instances >= 1 && instances <= 65535 && instances % references == 0,
                "instances must be a positive multiple of references");
    if (int e = check_intrinsics(intrinsics, references)) return e;
    const int64_t P = (int64_t)cols * rows;
    if (fill) {
        if (int e = fill_map(d_distance_out, P * instances, 1e8f, as_stream(stream))) return e;
    }
    ReprojParams p{};
    p.cols = cols;
    p.rows = rows;
    p.references = references;
    for (int r = 0; r < references; ++r) {
        p.k[r] = to_intr(intrinsics[r]);
        std::memcpy(p.t[r], translations + 3 * r, sizeof(float) * 3);
    }
    dim3 grid(grid_1d(P, kStitchBlock), references);
    if (fast)
        reproject_frames_kernel<true><<<grid, kStitchBlock, 0, as_stream(stream)>>>(p, instances / references,
                                                                                   d_distance_in, d_distance_out);
    else
        reproject_frames_kernel<false><<<grid, kStitchBlock, 0, as_stream(stream)>>>(p, instances / references,
                                                                                    d_distance_in, d_distance_out);
    return launch_status("reproject_frames_kernel");
}

extern "C" int ssg_reproject_distance_batch(const float* d_distance_in, float* d_distance_out, int cols, int rows,
                                            int instances, int references, const ssg_intrinsics* intrinsics,
                                            const float* translations, int fill, void* stream)
{
    return reproject_batch(d_distance_in, d_distance_out, cols, rows, instances, references, intrinsics,
                           translations, fill, false, stream);
}

extern "C" int ssg_reproject_distance_batch_approx(const float* d_distance_in, float* d_distance_out, int cols,
                                                   int rows, int instances, int references,
                                                   const ssg_intrinsics* intrinsics, const float* translations,
                                                   int fill, void* stream)
{
    return reproject_batch(d_distance_in, d_distance_out, cols, rows, instances, references, intrinsics,
                           translations, fill, true, stream);
}

extern "C" int ssg_inpaint(float* d_distance, const uint8_t* d_table, float* d_scratch, int cols, int rows,
                           double max_dist, int iterations, void* stream)
{
    return ssg_inpaint_batch(d_distance, d_table, d_scratch, cols, rows, 1, 1, max_dist, iterations, stream);
}

extern "C" int ssg_inpaint_batch(float* d_distance, const uint8_t* d_tables, float* d_scratch, int cols, int rows,
                                 int instances, int references, double max_dist, int iterations, void* stream)
{
    const uint8_t* d_table = d_tables;
    SSG_REQUIRE(d_distance && d_table && d_scratch && d_distance != d_scratch, "null or aliased pointer");
    SSG_REQUIRE(cols > 0 && rows > 0 && iterations >= 0, "invalid sizes");
    SSG_REQUIRE(references >= 1 && instances >= 1 && instances <= 65535 && instances % references == 0,
                "instances must be a positive multiple of references");
    if (int e = enable_inpaint_smem()) return e;
    // hole: distance >= MAX_DIST + 0.1 (double, stitcher.cu:287); usable neighbour:
    // distance <= MAX_DIST + 0.1f (stitcher.cu:311)
    const float hole = float_at_least(max_dist + 0.1);
    const float ok = float_at_most(max_dist + (double)0.1f);
    dim3 grid((cols + kTileW - 1) / kTileW, (rows + kTileH - 1) / kTileH, instances);
    float* a = d_distance;
    float* b = d_scratch;
    for (int done = 0; done < iterations;) {
        const int steps = iterations - done < kHalo ? iterations - done : kHalo;
        inpaint_tile_kernel<<<grid, kInpaintBlock, kInpaintSmem, as_stream(stream)>>>(
            a, b, reinterpret_cast<const uchar2*>(d_table), cols, rows, references, steps, hole, ok);
        if (int e = launch_status("inpaint_tile_kernel")) return e;
        float* t = a;
        a = b;
        b = t;
        done += steps;
    }
    if (a != d_distance) {
        cudaError_t e = cudaMemcpyAsync(d_distance, a, sizeof(float) * (size_t)cols * rows * instances,
                                        cudaMemcpyDeviceToDevice, as_stream(stream));
        if (e != cudaSuccess) return fail(SSG_ERR_CUDA, "cudaMemcpyAsync: %s", cudaGetErrorString(e));
    }
    return SSG_OK;
}

namespace ssg {

// ---------------------------------------------------------------------------------------------
// Stitch of an uneven batch: every job has its own rig, map and panorama sizes; its maps are
// concatenated job by job (StitchJob::map_begin).
// ---------------------------------------------------------------------------------------------
struct JobMaps {
    const StitchJob* jobs;
    int n;
    __device__ __forceinline__ MapPixel at(int64_t g) const
    {
        int lo = 0, hi = n - 1;  // the last job whose maps begin at or before g
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (jobs[mid].map_begin <= g) lo = mid;
            else hi = mid - 1;
        }
        const StitchJob& J = jobs[lo];
        const int64_t P = (int64_t)J.cols * J.rows, off = g - J.map_begin, slot = off / P, j = off - slot * P;
        return MapPixel{J.cols, J.rows, (int)(j % J.cols), (int)(j / J.cols),
                        reinterpret_cast<const uchar2*>(J.tables) + slot * P};
    }
};

// blockIdx.y: job * max_references + reference slot
__global__ void __launch_bounds__(kStitchBlock) reproject_uneven_kernel(const StitchJob* __restrict__ jobs,
                                                                        int max_references)
{
    const StitchJob& J = jobs[blockIdx.y / max_references];
    const int slot = blockIdx.y % max_references;
    const int64_t P = (int64_t)J.cols * J.rows;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= J.references || i >= P) return;
    // the uniform batch's arithmetic (reproject_frames_kernel<true>)
    float ray[3];
    pixel_ray(J.k[slot], J.cols, i, ray);
    reproject_ray_fast(J.k[slot], J.t[slot], ray, J.distance + slot * P, J.reprojected + slot * P, J.cols, P, i);
}

// the approximate merge (merge_frames_kernel's arithmetic) of one job's panorama; blockIdx.y: job
__global__ void __launch_bounds__(kStitchBlock) merge_uneven_kernel(const StitchJob* __restrict__ jobs)
{
    const StitchJob& J = jobs[blockIdx.y];
    const int64_t Q = (int64_t)J.pano_cols * J.pano_rows;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Q) return;
    const int cols = J.cols, rows = J.rows;
    float inv = 0.0f, rgb[3] = {0.0f, 0.0f, 0.0f};
    const float colsm = fsub((float)J.image_cols, 1.1f), rowsm = fsub((float)J.image_rows, 1.1f);
    for (int r = 0; r < J.references; ++r) {
        const float w = J.weights[(int64_t)r * Q + i];
        float2 uv = J.lut[(int64_t)r * Q + i];
        uv.x = fminf(fmaxf(uv.x, 0.1f), fsub((float)cols, 1.1f));
        uv.y = fminf(fmaxf(uv.y, 0.1f), fsub((float)rows, 1.1f));
        const float vo = fadd(uv.y, (float)(r * rows));
        float ray[3], pt[3], o[2], c[3];
        unproject_fast(uv.x, uv.y, J.k[r], ray);
        const float rd = interp_f_fast(J.reprojected, uv.x, vo, cols);
        inv = fmaf(w, rcp_approx(rd), inv);
        const float dc = fminf(rd, interp_f_fast(J.distance, uv.x, vo, cols));
#pragma unroll
        for (int a = 0; a < 3; ++a) pt[a] = fmaf(dc, ray[a], J.t[r][a]);
        project_fast(pt, J.k[r], o);
        o[0] = fminf(fmaxf(fmul(o[0], J.ratio_x), 0.1f), colsm);
        o[1] = fadd(fminf(fmaxf(fmul(o[1], J.ratio_y), 0.1f), rowsm), (float)(r * J.image_rows));
        interp_rgb_fast(J.images, o[0], o[1], J.image_cols, c, J.word_rows != 0);
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) rgb[ch] = fmaf(c[ch], w, rgb[ch]);
    }
    J.pano_distance[i] = rcp_approx(inv);
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) J.rgb[3 * i + ch] = (uint8_t)__float2uint_rz(fminf(rgb[ch], 255.0f));
}

int launch_stitch_uneven(const StitchJob* d_jobs, int jobs, float* d_maps, int64_t total_map_pixels,
                         int max_map_pixels, int max_pano_pixels, int max_references, double max_dist,
                         int iterations, uint8_t* d_stamps, int32_t* d_holes, cudaStream_t st)
{
    SSG_REQUIRE(iterations >= 0 && iterations <= kMaxListIterations, "iterations %d outside [0, %d]", iterations,
                kMaxListIterations);
    SSG_REQUIRE(total_map_pixels < ((int64_t)1 << 31), "too many map pixels");
    if (int e = fill_map(d_maps, total_map_pixels, 1e8f, st)) return e;
    reproject_uneven_kernel<<<dim3(grid_1d(max_map_pixels, kStitchBlock), jobs * max_references), kStitchBlock, 0,
                              st>>>(d_jobs, max_references);
    if (int e = launch_status("reproject_uneven_kernel")) return e;
    if (int e = inpaint_lists(JobMaps{d_jobs, jobs}, total_map_pixels, d_maps, d_stamps, d_holes, max_dist,
                              iterations, st))
        return e;
    merge_uneven_kernel<<<dim3(grid_1d(max_pano_pixels, kStitchBlock), jobs), kStitchBlock, 0, st>>>(d_jobs);
    return launch_status("merge_uneven_kernel");
}

}  // namespace ssg

extern "C" int ssg_inpaint_holes_batch(float* d_distance, const uint8_t* d_tables, uint8_t* d_stamps,
                                       int32_t* d_holes, int cols, int rows, int instances, int references,
                                       double max_dist, int iterations, void* stream)
{
    SSG_REQUIRE(d_distance && d_tables && d_stamps && d_holes, "null pointer");
    SSG_REQUIRE(cols > 0 && rows > 0, "invalid sizes");
    SSG_REQUIRE(iterations >= 0 && iterations <= kMaxListIterations, "iterations %d outside [0, %d]", iterations,
                kMaxListIterations);
    SSG_REQUIRE(references >= 1 && instances >= 1 && instances <= 65535 && instances % references == 0,
                "instances must be a positive multiple of references");
    SSG_REQUIRE((int64_t)cols * rows * instances < ((int64_t)1 << 31), "%d maps of %dx%d pixels are too many",
                instances, cols, rows);
    const UniformMaps maps(cols, rows, references, reinterpret_cast<const uchar2*>(d_tables));
    return inpaint_lists(maps, (int64_t)cols * rows * instances, d_distance, d_stamps, d_holes, max_dist, iterations,
                         as_stream(stream), (int64_t)cols * rows);
}

extern "C" int ssg_merge_panorama(const float* d_lut, const float* d_weights, const float* d_reprojected,
                                  const float* d_distances, const uint8_t* d_images, int image_rows, int image_cols,
                                  const float* translations, const ssg_intrinsics* intrinsics, int reference_count,
                                  int cols, int rows, int pano_cols, int pano_rows, float* d_distance_panorama,
                                  uint8_t* d_rgb_panorama, void* stream)
{
    return ssg_merge_panorama_batch(d_lut, d_weights, d_reprojected, d_distances, d_images, image_rows, image_cols,
                                    translations, intrinsics, reference_count, cols, rows, pano_cols, pano_rows, 1,
                                    d_distance_panorama, d_rgb_panorama, stream);
}

template <bool kFast>
// image_count images of image_rows x image_cols x 3 bytes per frame in d_images; reference r
// stitches image image_slots[r] (nullptr: image r, image_count = reference_count)
static int merge_batch(const float* d_lut, const float* d_weights, const float* d_reprojected,
                       const float* d_distances, const uint8_t* d_images, int image_rows, int image_cols,
                       const float* translations, const ssg_intrinsics* intrinsics, int reference_count, int cols,
                       int rows, int pano_cols, int pano_rows, int frames, float* d_distance_panorama,
                       uint8_t* d_rgb_panorama, void* stream, int image_count = 0, const int* image_slots = nullptr)
{
    SSG_REQUIRE(frames >= 1 && frames <= 65535, "frames out of range");
    SSG_REQUIRE(d_lut && d_weights && d_reprojected && d_distances && d_images && translations &&
                    d_distance_panorama && d_rgb_panorama,
                "null pointer");
    SSG_REQUIRE(cols > 1 && rows > 1 && pano_cols > 0 && pano_rows > 0 && image_rows > 1 && image_cols > 1,
                "invalid sizes");
    SSG_REQUIRE(reference_count >= 1 && reference_count <= SSG_MAX_REFERENCES, "reference_count %d outside [1, %d]",
                reference_count, SSG_MAX_REFERENCES);
    if (int e = check_intrinsics(intrinsics, reference_count)) return e;
    if (!image_slots) image_count = reference_count;
    SSG_REQUIRE(image_count >= 1 && image_count <= SSG_MAX_CAMERAS, "image_count %d outside [1, %d]", image_count,
                SSG_MAX_CAMERAS);
    MergeParams p{};
    for (int r = 0; r < reference_count; ++r) {
        p.image_slot[r] = image_slots ? image_slots[r] : r;
        SSG_REQUIRE(p.image_slot[r] >= 0 && p.image_slot[r] < image_count, "image slot %d of reference %d outside [0, %d)",
                    p.image_slot[r], r, image_count);
    }
    p.image_frame = (int64_t)image_count * image_rows * image_cols * 3;
    p.cols = cols;
    p.rows = rows;
    p.pano_cols = pano_cols;
    p.pano_rows = pano_rows;
    p.nref = reference_count;
    p.image_rows = image_rows;
    p.image_cols = image_cols;
    p.ratio_x = (float)image_cols / (float)cols;
    p.ratio_y = (float)image_rows / (float)rows;
    for (int r = 0; r < reference_count; ++r) {
        p.k[r] = to_intr(intrinsics[r]);
        std::memcpy(p.t[r], translations + 3 * r, sizeof(float) * 3);
    }
    const int64_t Q = (int64_t)pano_cols * pano_rows;
    dim3 grid(grid_1d(Q, kStitchBlock), frames);
    // every image starts and ends on a 4-byte boundary when the buffer does and an image's bytes are
    // a multiple of 4
    p.word_rows = ((uintptr_t)d_images & 3) == 0 && (((int64_t)image_rows * image_cols * 3) & 3) == 0;
    if constexpr (kFast) {
        const int group = tuning(SSG_TUNE_MERGE_FRAMES);
        const dim3 fgrid(grid_1d(Q, kStitchBlock), (frames + group - 1) / group);
        const float2* lut = reinterpret_cast<const float2*>(d_lut);
        if (group == 2)
            merge_frames_kernel<2><<<fgrid, kStitchBlock, 0, as_stream(stream)>>>(
                p, frames, lut, d_weights, d_reprojected, d_distances, d_images, d_distance_panorama, d_rgb_panorama);
        else if (group == 8)
            merge_frames_kernel<8><<<fgrid, kStitchBlock, 0, as_stream(stream)>>>(
                p, frames, lut, d_weights, d_reprojected, d_distances, d_images, d_distance_panorama, d_rgb_panorama);
        else
            merge_frames_kernel<4><<<fgrid, kStitchBlock, 0, as_stream(stream)>>>(
                p, frames, lut, d_weights, d_reprojected, d_distances, d_images, d_distance_panorama, d_rgb_panorama);
        return launch_status("merge_frames_kernel");
    } else {
        merge_kernel<<<grid, kStitchBlock, 0, as_stream(stream)>>>(
            p, reinterpret_cast<const float2*>(d_lut), d_weights, d_reprojected, d_distances, d_images,
            d_distance_panorama, d_rgb_panorama);
        return launch_status("merge_kernel");
    }
}

extern "C" int ssg_merge_panorama_batch(const float* d_lut, const float* d_weights, const float* d_reprojected,
                                        const float* d_distances, const uint8_t* d_images, int image_rows,
                                        int image_cols, const float* translations, const ssg_intrinsics* intrinsics,
                                        int reference_count, int cols, int rows, int pano_cols, int pano_rows,
                                        int frames, float* d_distance_panorama, uint8_t* d_rgb_panorama, void* stream)
{
    return merge_batch<false>(d_lut, d_weights, d_reprojected, d_distances, d_images, image_rows, image_cols,
                              translations, intrinsics, reference_count, cols, rows, pano_cols, pano_rows, frames,
                              d_distance_panorama, d_rgb_panorama, stream);
}

extern "C" int ssg_merge_panorama_batch_approx_images(const float* d_lut, const float* d_weights,
                                                      const float* d_reprojected, const float* d_distances,
                                                      const uint8_t* d_images, int image_count,
                                                      const int* image_slots, int image_rows, int image_cols,
                                                      const float* translations, const ssg_intrinsics* intrinsics,
                                                      int reference_count, int cols, int rows, int pano_cols,
                                                      int pano_rows, int frames, float* d_distance_panorama,
                                                      uint8_t* d_rgb_panorama, void* stream)
{
    SSG_REQUIRE(image_slots, "null image_slots");
    return merge_batch<true>(d_lut, d_weights, d_reprojected, d_distances, d_images, image_rows, image_cols,
                             translations, intrinsics, reference_count, cols, rows, pano_cols, pano_rows, frames,
                             d_distance_panorama, d_rgb_panorama, stream, image_count, image_slots);
}

extern "C" int ssg_merge_panorama_batch_approx(const float* d_lut, const float* d_weights,
                                               const float* d_reprojected, const float* d_distances,
                                               const uint8_t* d_images, int image_rows, int image_cols,
                                               const float* translations, const ssg_intrinsics* intrinsics,
                                               int reference_count, int cols, int rows, int pano_cols,
                                               int pano_rows, int frames, float* d_distance_panorama,
                                               uint8_t* d_rgb_panorama, void* stream)
{
    return merge_batch<true>(d_lut, d_weights, d_reprojected, d_distances, d_images, image_rows, image_cols,
                             translations, intrinsics, reference_count, cols, rows, pano_cols, pano_rows, frames,
                             d_distance_panorama, d_rgb_panorama, stream);
}

// ---------------------------------------------------------------------------------------------
// Hole filling without any device allocation by the caller.
//
// ssg_inpaint alternates between the caller's map and a caller-owned scratch map.  Some callers
// cannot allocate device memory for that scratch: a plugin inside a host application whose own
// memory manager owns the device heap, or a hard real-time loop where cudaMalloc may synchronise
// the device and stall it.  For them ssg_inpaint_noalloc keeps the scratch in this fixed array,
// part of the library image: every GPU that loads the library holds these 4 MiB until the
// process exits.  Maps up to kNoAllocMaxPixels pixels are accepted.
// ---------------------------------------------------------------------------------------------
namespace ssg {
constexpr int64_t kNoAllocMaxPixels = int64_t(1) << 20;  // 4 MiB of float32, e.g. 1024 x 1024
static __device__ __align__(256) float g_noalloc_scratch[kNoAllocMaxPixels];

// Device address of g_noalloc_scratch on the current device, looked up once per device (host
// code only sees a host-side stand-in for the symbol, never its device address).  Kept for the
// life of the process: a cudaDeviceReset after the first call would leave it stale (documented
// as unsupported at the entry point).
static int noalloc_scratch_address(float** out)
{
    static std::atomic<float*> cached[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(SSG_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= 64) return fail(SSG_ERR_UNSUPPORTED, "device ordinal %d beyond 63", dev);
    float* p = cached[dev].load();
    if (!p) {
        e = cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_noalloc_scratch);
        if (e != cudaSuccess) return fail(SSG_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
        cached[dev].store(p);
    }
    *out = p;
    return SSG_OK;
}
}  // namespace ssg

extern "C" int ssg_inpaint_noalloc(float* d_distance, const uint8_t* d_table, int cols, int rows, double max_dist,
                                   int iterations, void* stream)
{
    SSG_REQUIRE(d_distance && d_table, "null pointer");
    SSG_REQUIRE(cols > 0 && rows > 0 && iterations >= 0, "invalid sizes");
    if ((int64_t)cols * rows > kNoAllocMaxPixels)
        return fail(SSG_ERR_UNSUPPORTED,
                    "ssg_inpaint_noalloc: a %d x %d map has %lld pixels, more than the %lld of its built-in scratch; "
                    "use ssg_inpaint with a caller-allocated scratch map",
                    cols, rows, (long long)cols * rows, (long long)kNoAllocMaxPixels);
    float* scratch = nullptr;
    if (int e = noalloc_scratch_address(&scratch)) return e;
    if (int e = enable_inpaint_smem()) return e;
    // every pass writes every pixel of its destination, so nothing left in the scratch by an
    // earlier call is read
    const float hole = float_at_least(max_dist + 0.1);
    const float ok = float_at_most(max_dist + (double)0.1f);
    dim3 grid((cols + kTileW - 1) / kTileW, (rows + kTileH - 1) / kTileH, 1);
    float* a = d_distance;
    float* b = scratch;
    for (int done = 0; done < iterations;) {
        const int steps = iterations - done < kHalo ? iterations - done : kHalo;
        inpaint_tile_kernel<<<grid, kInpaintBlock, kInpaintSmem, as_stream(stream)>>>(
            a, b, reinterpret_cast<const uchar2*>(d_table), cols, rows, 1, steps, hole, ok);
        if (int e = launch_status("inpaint_tile_kernel")) return e;
        float* t = a;
        a = b;
        b = t;
        done += steps;
    }
    if (a != d_distance) {
        cudaError_t e = cudaMemcpyAsync(d_distance, a, sizeof(float) * (size_t)cols * rows, cudaMemcpyDeviceToDevice,
                                        as_stream(stream));
        if (e != cudaSuccess) return fail(SSG_ERR_CUDA, "cudaMemcpyAsync: %s", cudaGetErrorString(e));
    }
    return SSG_OK;
}
