// Batched sweep + cost (python/depth_estimation.py:141-175) for many (frame, reference) instances
// per launch, with 16-bit output in the chunked layout of ssg_cells.cuh.
//
// A batch is `instances` independent (frame, reference camera) pairs of one rig; blockIdx.y is the
// instance, so a whole batch is one launch.  One thread per pixel of the reference camera walks
// the candidates in order, projects each candidate point into the pixel's selected camera,
// samples it bilinearly from float4 texels (16-byte loads) and writes 8 candidates at a time as
// one 16-byte cell.  Level-0 storage is __half (fp16) or unorm16 (q = round(c * 65535 / 500);
// costs are clamped to [0, 500]); the arithmetic is fp32.  The fp32 kernels of ssg_sweep.cu are
// the ones that reproduce the reference bit for bit; this sweep projects with approximate square
// roots and reciprocal, a change far below the 16-bit rounding of its output.
#include <cmath>

#include "ssg_cells.cuh"

namespace ssg {

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

// ---------------------------------------------------------------------------------------------
// Image staging.  The sweep reads each bilinear sample as two 16-byte loads, one per image row:
// a staged entry holds two horizontally adjacent texels as fp16 RGB ([R0 G0 B0 R1 G1 B1 0 0],
// texels x - 1 and x of entry x).  fp16 holds every 8-bit value exactly, so for images made from
// 8-bit data (all of the reference's inputs before resizing) the samples are the float32 ones;
// other float inputs are rounded to fp16 (a relative 2^-11).  Entries form planes of
// (rows + 2) x (cols + 2) with a border of zeros, so that every tap of a sample whose top-left
// tap lies in [-1, cols - 1] x [-1, rows - 1] is a plain load and the border supplies
// grid_sample's zero padding; the border rows and the last column are never written (the caller
// zeroes the buffer once).  The guide of every reference camera (rgb2yCbCr + uint8 cast) is
// written in the same pass, from the float values.
// ---------------------------------------------------------------------------------------------
struct StageParams {
    int cameras, references, cols, rows;
    int ref_slot[SSG_MAX_CAMERAS];  // reference slot of each camera, -1 if not a reference
};

__device__ __forceinline__ float texel_value(float v) { return v; }
__device__ __forceinline__ float texel_value(uint8_t v) { return (float)v; }

__device__ __forceinline__ uint32_t half_bits(float v) { return (uint32_t)__half_as_ushort(__float2half_rn(v)); }

template <typename Tin>
__global__ void __launch_bounds__(kBatchBlock) stage_images_kernel(const __grid_constant__ StageParams p,
                                                                  const Tin* __restrict__ images,
                                                                  uint4* __restrict__ staged,
                                                                  uint8_t* __restrict__ guides)
{
    const int64_t P = (int64_t)p.cols * p.rows;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;  // entry (y, e), e in [0, cols]
    if (i >= (int64_t)p.rows * (p.cols + 1)) return;
    const int inst = blockIdx.y;  // frame * cameras + camera
    const int frame = inst / p.cameras, cam = inst % p.cameras;
    const int y = (int)(i / (p.cols + 1)), e = (int)(i % (p.cols + 1));
    const Tin* row = images + ((int64_t)inst * P + (int64_t)y * p.cols) * 3;
    float lo[3] = {0.0f, 0.0f, 0.0f}, hi[3] = {0.0f, 0.0f, 0.0f};
    if (e >= 1)
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) lo[ch] = texel_value(row[3 * (e - 1) + ch]);
    if (e < p.cols)
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) hi[ch] = texel_value(row[3 * e + ch]);
    const int64_t plane = (int64_t)(p.cols + 2) * (p.rows + 2);
    staged[(int64_t)inst * plane + (int64_t)(y + 1) * (p.cols + 2) + e] =
        make_uint4(half_bits(lo[0]) | (half_bits(lo[1]) << 16), half_bits(lo[2]) | (half_bits(hi[0]) << 16),
                   half_bits(hi[1]) | (half_bits(hi[2]) << 16), 0u);
    const int slot = p.ref_slot[cam];
    if (slot >= 0 && e < p.cols) {
        // utils.py:144-155, the arithmetic of ssg_rgb_to_guide, for pixel (e, y)
        const float c0 = hi[0], c1 = hi[1], c2 = hi[2];
        float yy = fadd(fadd(fadd(fmul(c0, 0.1826f), 16.0f), fmul(c1, 0.6142f)), fmul(c2, 0.062f));
        float cb = fadd(fsub(fsub(128.0f, fmul(c0, 0.1006f)), fmul(c1, 0.3386f)), fmul(c2, 0.4392f));
        float cr = fsub(fsub(fadd(fmul(c0, 0.4392f), 128.0f), fmul(c1, 0.3989f)), fmul(c2, 0.0403f));
        uint8_t* g = guides + (((int64_t)frame * p.references + slot) * P + (int64_t)y * p.cols + e) * 3;
        g[0] = (uint8_t)__float2uint_rz(fminf(fmaxf(yy, 16.0f), 235.0f));
        g[1] = (uint8_t)__float2uint_rz(fminf(fmaxf(cb, 16.0f), 240.0f));
        g[2] = (uint8_t)__float2uint_rz(fminf(fmaxf(cr, 16.0f), 240.0f));
    }
}

// the two texels of an entry as float RGB
__device__ __forceinline__ void unpack_entry(uint4 q, float lo[3], float hi[3])
{
    const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&q.x));
    const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&q.y));
    const float2 c = __half22float2(*reinterpret_cast<const __half2*>(&q.z));
    lo[0] = a.x; lo[1] = a.y; lo[2] = b.x;
    hi[0] = b.y; hi[1] = c.x; hi[2] = c.y;
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
    float cand[SSG_MAX_CANDIDATES];  // padded to whole chunks with the last candidate
};

// Double-sphere projection (utils.py:75-94) with approximate square roots and reciprocal: a
// relative error of a few 1e-7 in the sample position, well below the 16-bit rounding of the
// cost it feeds.
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

// Bilinear sample with zero padding (torch grid_sample, align_corners=False, taps nw, ne, sw,
// se) from a bordered plane of texel pairs; `img` points at the entry of texels (-1, 0), (0, 0),
// `pitch` = cols + 2.
__device__ __forceinline__ void fast_sample(const uint4* __restrict__ img, int pitch, int cols, int rows, float ix,
                                            float iy, float& s0, float& s1, float& s2)
{
    const float x0 = floorf(ix), y0 = floorf(iy);
    // saturating conversions (NaN converts to 0 and is rejected by the x0 == x0 tests)
    const int xi = __float2int_rz(x0), yi = __float2int_rz(y0);
    s0 = s1 = s2 = 0.0f;
    // all four taps outside (or a NaN coordinate): zero.  -1 <= xi <= cols - 1 as one unsigned test
    if (!((unsigned)xi + 1u <= (unsigned)cols && (unsigned)yi + 1u <= (unsigned)rows && x0 == x0 && y0 == y0)) return;
    const uint4* t = img + yi * pitch + xi + 1;  // entry of texels (xi, yi), (xi + 1, yi)
    float a[3], b[3], c[3], d[3];
    unpack_entry(__ldg(t), a, b);
    unpack_entry(__ldg(t + pitch), c, d);
    const float fx = ix - x0, fy = iy - y0;
    const float gx = 1.0f - fx, gy = 1.0f - fy;
    const float wa = gx * gy, wb = fx * gy, wc = gx * fy, wd = fx * fy;
    s0 = fmaf(d[0], wd, fmaf(c[0], wc, fmaf(b[0], wb, a[0] * wa)));
    s1 = fmaf(d[1], wd, fmaf(c[1], wc, fmaf(b[1], wb, a[1] * wa)));
    s2 = fmaf(d[2], wd, fmaf(c[2], wc, fmaf(b[2], wb, a[2] * wa)));
}

template <typename T>
__global__ void __launch_bounds__(kBatchBlock) sweep_batch_kernel(const __grid_constant__ FastSweepParams p,
                                                                const uint4* __restrict__ staged,
                                                                const int8_t* __restrict__ selected,
                                                                T* __restrict__ cost)
{
    const int cols = p.cols, rows = p.rows, pitch = cols + 2;
    const int P = cols * rows;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    const int inst = blockIdx.y;  // frame * references + slot
    const int frame = inst / p.references, slot = inst % p.references;
    const int plane = pitch * (rows + 2);
    const uint4* frame_img = staged + (int64_t)frame * p.cameras * plane + pitch;  // row 0, entry 0 of camera 0
    const int x = i % cols, y = i / cols;
    float rp[3], unused[3];
    unpack_entry(__ldg(frame_img + (int64_t)p.ref_index[slot] * plane + y * pitch + x + 1), rp, unused);
    T* out = cost + (int64_t)inst * p.chunks * P * 8 + (int64_t)i * 8;
    const int64_t chunk_stride = (int64_t)P * 8;
    const int sel = selected[(int64_t)slot * P + i];
    if (sel < 0 || sel >= p.cameras) {
        // no camera sees the point: grid_sample of an all-zero image (depth_estimation.py:166)
        float c = fminf(fabsf(rp[0]) + fabsf(rp[1]) + fabsf(rp[2]), 500.0f);
        float cc[8] = {c, c, c, c, c, c, c, c};
        const uint4 v = Cell<T>::pack(cc);
        for (int ch = 0; ch < p.chunks; ++ch) reinterpret_cast<uint4*>(out + ch * chunk_stride)[0] = v;
        return;
    }
    float pu[3];
    unproject_torch((float)x, (float)y, p.ref_cam[slot], pu);
    const float* m = p.pose[slot][sel];
    // p_cam = R (d u) + t = d (R u) + t
    const float ax = fmaf(m[2], pu[2], fmaf(m[1], pu[1], m[0] * pu[0]));
    const float ay = fmaf(m[6], pu[2], fmaf(m[5], pu[1], m[4] * pu[0]));
    const float az = fmaf(m[10], pu[2], fmaf(m[9], pu[1], m[8] * pu[0]));
    const float tx = m[3], ty = m[7], tz = m[11];
    const FastCam k = p.cam[sel];
    const uint4* img = frame_img + (int64_t)sel * plane;
    for (int ch = 0; ch < p.chunks; ++ch) {
        uint32_t packed[4];
#pragma unroll
        for (int j = 0; j < 8; j += 2) {
            float c2[2];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int kk = ch * 8 + j + h;
                const float d = p.cand[kk];
                float u, v, s0, s1, s2;
                fast_project(fmaf(d, ax, tx), fmaf(d, ay, ty), fmaf(d, az, tz), k, u, v);
                fast_sample(img, pitch, cols, rows, u, v, s0, s1, s2);
                c2[h] = fminf(fabsf(s0 - rp[0]) + fabsf(s1 - rp[1]) + fabsf(s2 - rp[2]), 500.0f);
            }
            packed[j / 2] = Cell<T>::pack2(c2[0], c2[1]);
        }
        reinterpret_cast<uint4*>(out + ch * chunk_stride)[0] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
    }
}

static int check_storage(int storage)
{
    SSG_REQUIRE(storage == SSG_STORAGE_F16 || storage == SSG_STORAGE_UNORM16, "unknown cost storage %d", storage);
    return SSG_OK;
}

static int chunks_of(int n) { return (n + 7) / 8; }

}  // namespace ssg

using namespace ssg;

using namespace ssg;

static int staged_plane_fits(int cols, int rows)
{
    SSG_REQUIRE(cols > 0 && rows > 0, "resolution must be positive");
    SSG_REQUIRE((int64_t)(cols + 2) * (rows + 2) < ((int64_t)1 << 31), "images of %dx%d pixels are too large", cols,
                rows);
    return SSG_OK;
}

template <typename Tin>
static int stage_images(const Tin* d_images, int frames, int cameras, int cols, int rows,
                        const int* reference_cameras, int references, float* d_staged, uint8_t* d_guides,
                        void* stream)
{
    SSG_REQUIRE(d_images && d_staged && d_guides && reference_cameras, "null pointer");
    SSG_REQUIRE(frames >= 1 && frames <= 65535 / SSG_MAX_CAMERAS, "frames %d outside [1, %d]", frames,
                65535 / SSG_MAX_CAMERAS);
    SSG_REQUIRE(cameras >= 1 && cameras <= SSG_MAX_CAMERAS && references >= 1 && references <= SSG_MAX_REFERENCES,
                "camera or reference count out of range");
    if (int e = staged_plane_fits(cols, rows)) return e;
    SSG_REQUIRE(((uintptr_t)d_staged & 15) == 0, "staged images must be 16-byte aligned");
    StageParams p{};
    p.cameras = cameras;
    p.references = references;
    p.cols = cols;
    p.rows = rows;
    for (int c = 0; c < SSG_MAX_CAMERAS; ++c) p.ref_slot[c] = -1;
    for (int r = 0; r < references; ++r) {
        SSG_REQUIRE(reference_cameras[r] >= 0 && reference_cameras[r] < cameras, "reference camera out of range");
        p.ref_slot[reference_cameras[r]] = r;
    }
    dim3 grid(grid_1d((int64_t)(cols + 1) * rows, kBatchBlock), frames * cameras);
    stage_images_kernel<Tin><<<grid, kBatchBlock, 0, as_stream(stream)>>>(p, d_images,
                                                                         reinterpret_cast<uint4*>(d_staged), d_guides);
    return launch_status("stage_images_kernel");
}

extern "C" int ssg_stage_images(const float* d_images, int frames, int cameras, int cols, int rows,
                                const int* reference_cameras, int references, float* d_staged, uint8_t* d_guides,
                                void* stream)
{
    return stage_images(d_images, frames, cameras, cols, rows, reference_cameras, references, d_staged, d_guides,
                        stream);
}

extern "C" int ssg_stage_images_u8(const uint8_t* d_images, int frames, int cameras, int cols, int rows,
                                   const int* reference_cameras, int references, float* d_staged, uint8_t* d_guides,
                                   void* stream)
{
    return stage_images(d_images, frames, cameras, cols, rows, reference_cameras, references, d_staged, d_guides,
                        stream);
}

extern "C" int ssg_sweep_cost_batch(int cols, int rows, int frames, int camera_count, const ssg_camera* cameras,
                                    int references, const int* reference_cameras, const float* relative_poses,
                                    const float* d_staged, const int8_t* d_selected, const float* candidates,
                                    int candidate_count, int storage, void* d_cost, void* stream)
{
    if (int e = staged_plane_fits(cols, rows)) return e;
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
    for (int k = 0; k < 8 * p.chunks; ++k) p.cand[k] = candidates[k < candidate_count ? k : candidate_count - 1];
    const int64_t P = (int64_t)cols * rows;
    dim3 grid(grid_1d(P, kBatchBlock), frames * references);
    const uint4* staged = reinterpret_cast<const uint4*>(d_staged);
    if (storage == SSG_STORAGE_F16)
        sweep_batch_kernel<__half><<<grid, kBatchBlock, 0, as_stream(stream)>>>(p, staged, d_selected,
                                                                              static_cast<__half*>(d_cost));
    else
        sweep_batch_kernel<uint16_t><<<grid, kBatchBlock, 0, as_stream(stream)>>>(p, staged, d_selected,
                                                                                static_cast<uint16_t*>(d_cost));
    return launch_status("sweep_batch_kernel");
}
