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
#include "ssg_uneven.cuh"

namespace ssg {


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
// written in the same pass, from the float values, as one 32-bit word per pixel (Y, Cb, Cr, 0).
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
        // one 32-bit word per pixel: bytes (Y, Cb, Cr, 0)
        const uint32_t g0 = __float2uint_rz(fminf(fmaxf(yy, 16.0f), 235.0f));
        const uint32_t g1 = __float2uint_rz(fminf(fmaxf(cb, 16.0f), 240.0f));
        const uint32_t g2 = __float2uint_rz(fminf(fmaxf(cr, 16.0f), 240.0f));
        reinterpret_cast<uint32_t*>(guides)[((int64_t)frame * p.references + slot) * P + (int64_t)y * p.cols + e] =
            g0 | (g1 << 8) | (g2 << 16);
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

struct FastSweepParams {
    int cols, rows, cameras, references, ncand, chunks;
    TorchCam ref_cam[SSG_MAX_REFERENCES];
    int ref_index[SSG_MAX_REFERENCES];
    FastCam cam[SSG_MAX_CAMERAS];
    float pose[SSG_MAX_REFERENCES][SSG_MAX_CAMERAS][12];  // reference -> camera, rows 0..2
    alignas(8) float cand[SSG_MAX_CANDIDATES];  // padded to whole chunks with the last candidate
};

// Double-sphere projection (utils.py:75-94) of two points with approximate square roots and
// reciprocal: a relative error of a few 1e-7 in the sample position, well below the 16-bit
// rounding of the cost it feeds.
__device__ __forceinline__ void project_pair(float2 x, float2 y, float2 z, const FastCam& k, float2& u, float2& v)
{
    const float2 rxy = fma2(y, y, mul2(x, x));
    const float2 s1 = fma2(z, z, rxy);
    const float2 d1 = make_float2(sqrt_approx(s1.x), sqrt_approx(s1.y));
    const float2 c = fma2(splat(k.xi), d1, z);
    const float2 s2 = fma2(c, c, rxy);
    const float2 d2 = make_float2(sqrt_approx(s2.x), sqrt_approx(s2.y));
    const float2 n = fma2(splat(k.alpha), d2, mul2(splat(k.one_minus_alpha), c));
    const float2 inv = make_float2(rcp_approx(n.x), rcp_approx(n.y));
    u = fma2(mul2(splat(k.fx), x), inv, splat(k.cx));
    v = fma2(mul2(splat(k.fy), y), inv, splat(k.cy));
}

// Bilinear samples with zero padding (torch grid_sample, align_corners=False, taps nw, ne, sw,
// se) at two positions, from a bordered plane of texel pairs; `img` points at the entry of texels
// (-1, 0), (0, 0), `pitch` = cols + 2.  The coordinates are clamped to [-1, cols] x [-1, rows]
// (a NaN to -1): a sample whose four taps all lie outside the image then reads border zeros, or
// has weight 0 on its in-image taps, so it is exactly 0 as grid_sample's, without a branch.  The
// bottom tap row is clamped to the last border row for a sample at row `rows` (its weight is 0).
__device__ __forceinline__ void sample_pair(const uint4* __restrict__ img, int pitch, float colsf, float rowsf,
                                            int rows, float2 ix, float2 iy, float (&s)[2][3])
{
    ix = make_float2(fminf(fmaxf(ix.x, -1.0f), colsf), fminf(fmaxf(ix.y, -1.0f), colsf));
    iy = make_float2(fminf(fmaxf(iy.x, -1.0f), rowsf), fminf(fmaxf(iy.y, -1.0f), rowsf));
    const float2 x0 = make_float2(floorf(ix.x), floorf(ix.y)), y0 = make_float2(floorf(iy.x), floorf(iy.y));
    const float2 fx = add2(ix, make_float2(-x0.x, -x0.y)), fy = add2(iy, make_float2(-y0.x, -y0.y));
    const float2 gx = add2(splat(1.0f), make_float2(-fx.x, -fx.y)), gy = add2(splat(1.0f), make_float2(-fy.x, -fy.y));
    // weights of the taps of both samples: (nw, ne, sw, se)
    const float2 wa = mul2(gx, gy), wb = mul2(fx, gy), wc = mul2(gx, fy), wd = mul2(fx, fy);
    float t[2][4][3];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int xi = (int)(h ? x0.y : x0.x), yi = (int)(h ? y0.y : y0.x);
        const uint4* top = img + yi * pitch + xi + 1;  // entry of texels (xi, yi), (xi + 1, yi)
        const uint4* bot = img + min(yi + 1, rows) * pitch + xi + 1;
        unpack_entry(__ldg(top), t[h][0], t[h][1]);
        unpack_entry(__ldg(bot), t[h][2], t[h][3]);
    }
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
        float2 v = mul2(wa, make_float2(t[0][0][ch], t[1][0][ch]));
        v = fma2(wb, make_float2(t[0][1][ch], t[1][1][ch]), v);
        v = fma2(wc, make_float2(t[0][2][ch], t[1][2][ch]), v);
        v = fma2(wd, make_float2(t[0][3][ch], t[1][3][ch]), v);
        s[0][ch] = v.x;
        s[1][ch] = v.y;
    }
}

// Sweep + cost of one reference pixel (x, y) over all candidates, into its cells (`out`, chunk
// stride `chunk_stride`).  `V` gives the instance's constants: ref_cam(), cam(c), pose(c) (12
// floats), cand(k) (pairs are read as float2) and cameras(), chunks().  `frame_img` points at row
// 0, entry 0 of the frame's camera 0 plane; planes are `plane` entries apart.
template <typename T, typename V>
__device__ __forceinline__ void sweep_pixel(const V& view, const uint4* __restrict__ frame_img, int plane,
                                            int ref_camera, int cols, int rows, int x, int y, int sel,
                                            T* __restrict__ out, int64_t chunk_stride)
{
    const int pitch = cols + 2;
    float rp[3], unused[3];
    unpack_entry(__ldg(frame_img + (int64_t)ref_camera * plane + y * pitch + x + 1), rp, unused);
    const int chunks = view.chunks();
    if (sel < 0 || sel >= view.cameras()) {
        // no camera sees the point: grid_sample of an all-zero image (depth_estimation.py:166)
        float c = fminf(fabsf(rp[0]) + fabsf(rp[1]) + fabsf(rp[2]), 500.0f);
        float cc[8] = {c, c, c, c, c, c, c, c};
        const uint4 v = Cell<T>::pack(cc);
        for (int ch = 0; ch < chunks; ++ch) reinterpret_cast<uint4*>(out + ch * chunk_stride)[0] = v;
        return;
    }
    float pu[3];
    unproject_torch((float)x, (float)y, view.ref_cam(), pu);
    float m[12];
#pragma unroll
    for (int j = 0; j < 12; ++j) m[j] = view.pose(sel, j);
    // p_cam = R (d u) + t = d (R u) + t
    const float2 ax = splat(fmaf(m[2], pu[2], fmaf(m[1], pu[1], m[0] * pu[0])));
    const float2 ay = splat(fmaf(m[6], pu[2], fmaf(m[5], pu[1], m[4] * pu[0])));
    const float2 az = splat(fmaf(m[10], pu[2], fmaf(m[9], pu[1], m[8] * pu[0])));
    const float2 tx = splat(m[3]), ty = splat(m[7]), tz = splat(m[11]);
    const FastCam k = view.cam(sel);
    const uint4* img = frame_img + (int64_t)sel * plane;
    const float colsf = (float)cols, rowsf = (float)rows;
    for (int ch = 0; ch < chunks; ++ch) {
        uint32_t packed[4];
#pragma unroll
        for (int j = 0; j < 8; j += 2) {
            const float2 d = view.cand2(ch * 8 + j);
            float2 u, v;
            project_pair(fma2(d, ax, tx), fma2(d, ay, ty), fma2(d, az, tz), k, u, v);
            float s[2][3];
            sample_pair(img, pitch, colsf, rowsf, rows, u, v, s);
            float c2[2];
#pragma unroll
            for (int h = 0; h < 2; ++h)
                c2[h] = fminf(fabsf(s[h][0] - rp[0]) + fabsf(s[h][1] - rp[1]) + fabsf(s[h][2] - rp[2]), 500.0f);
            packed[j / 2] = Cell<T>::pack2(c2[0], c2[1]);
        }
        reinterpret_cast<uint4*>(out + ch * chunk_stride)[0] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
    }
}

// the constants of one reference slot of a uniform batch (kernel parameters)
struct UniformView {
    const FastSweepParams& p;
    int slot;
    __device__ __forceinline__ int chunks() const { return p.chunks; }
    __device__ __forceinline__ int cameras() const { return p.cameras; }
    __device__ __forceinline__ const TorchCam& ref_cam() const { return p.ref_cam[slot]; }
    __device__ __forceinline__ float pose(int c, int j) const { return p.pose[slot][c][j]; }
    __device__ __forceinline__ FastCam cam(int c) const { return p.cam[c]; }
    __device__ __forceinline__ float2 cand2(int k) const { return *reinterpret_cast<const float2*>(&p.cand[k]); }
};

// Block shapes of the sweep (SSG_TUNE_SWEEP_VARIANT): threads per block and blocks per SM, which
// bounds the registers (64, 80, 64)
template <int V>
struct SweepShape;
template <>
struct SweepShape<0> {
    static constexpr int threads = 256, blocks = 4;
};
template <>
struct SweepShape<1> {
    static constexpr int threads = 256, blocks = 3;
};
template <>
struct SweepShape<2> {
    static constexpr int threads = 128, blocks = 8;
};

template <typename T, int V>
__global__ void __launch_bounds__(SweepShape<V>::threads, SweepShape<V>::blocks)
    sweep_batch_kernel(const __grid_constant__ FastSweepParams p,
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
    T* out = cost + (int64_t)inst * p.chunks * P * 8 + (int64_t)i * 8;
    sweep_pixel<T>(UniformView{p, slot}, frame_img, plane, p.ref_index[slot], cols, rows, i % cols, i / cols,
                   selected[(int64_t)slot * P + i], out, (int64_t)P * 8);
}

// the constants of one instance of an uneven batch (device memory)
struct InstView {
    const SweepInst* I;
    __device__ __forceinline__ int chunks() const { return I->chunks; }
    __device__ __forceinline__ int cameras() const { return I->cameras; }
    __device__ __forceinline__ const TorchCam& ref_cam() const { return I->ref_cam; }
    __device__ __forceinline__ float pose(int c, int j) const { return __ldg(&I->pose[c][j]); }
    __device__ __forceinline__ FastCam cam(int c) const { return I->cam[c]; }
    __device__ __forceinline__ float2 cand2(int k) const { return __ldg(reinterpret_cast<const float2*>(&I->cand[k])); }
};

// Persistent sweep over an uneven batch: each block takes work items (`span` consecutive tiles of
// kSweepTile reference pixels, in the instances' order) from a queue (*counter, zeroed before the
// launch) until the batch is done; each tile belongs to one instance.
template <typename T, int V>
__global__ void __launch_bounds__(SweepShape<V>::threads, SweepShape<V>::blocks)
    sweep_uneven_kernel(const SweepInst* __restrict__ insts, int instances, int total_tiles, int span,
                        int* __restrict__ counter)
{
    __shared__ int s_item;
    __shared__ int s_inst[4];
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
        __syncthreads();
        const int first = s_item * span;
        if (threadIdx.x < span && first + (int)threadIdx.x < total_tiles) {
            const int t = first + threadIdx.x;
            int lo = 0, hi = instances - 1;  // the last instance whose tiles begin at or before t
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (insts[mid].tile_begin <= t) lo = mid;
                else hi = mid - 1;
            }
            s_inst[threadIdx.x] = lo;
        }
        __syncthreads();
        if (first >= total_tiles) return;
        for (int u = 0; u < span && first + u < total_tiles; ++u) {
            const SweepInst* I = insts + s_inst[u];
            const int cols = I->cols, rows = I->rows, P = cols * rows;
            const int plane = (cols + 2) * (rows + 2);
            for (int j = threadIdx.x; j < kSweepTile; j += blockDim.x) {
                const int i = (first + u - I->tile_begin) * kSweepTile + j;
                if (i < P) {
                    T* out = static_cast<T*>(I->cost) + (int64_t)i * 8;
                    sweep_pixel<T>(InstView{I}, I->staged, plane, I->ref_camera, cols, rows, i % cols, i / cols,
                                   I->selected[i], out, (int64_t)P * 8);
                }
            }
        }
        __syncthreads();  // s_item and s_inst are rewritten by the next take
    }
}

template <typename T, int V>
static void launch_sweep_uneven_shape(const SweepInst* d_insts, int instances, int total_tiles, int span,
                                      int* d_counter, int sms, cudaStream_t st)
{
    sweep_uneven_kernel<T, V><<<sms * SweepShape<V>::blocks, SweepShape<V>::threads, 0, st>>>(
        d_insts, instances, total_tiles, span, d_counter);
}

template <typename T>
static void launch_sweep_uneven_t(const SweepInst* d_insts, int instances, int total_tiles, int span,
                                  int* d_counter, int sms, cudaStream_t st)
{
    switch (tuning(SSG_TUNE_SWEEP_VARIANT)) {
        case 1: launch_sweep_uneven_shape<T, 1>(d_insts, instances, total_tiles, span, d_counter, sms, st); break;
        case 2: launch_sweep_uneven_shape<T, 2>(d_insts, instances, total_tiles, span, d_counter, sms, st); break;
        default: launch_sweep_uneven_shape<T, 0>(d_insts, instances, total_tiles, span, d_counter, sms, st); break;
    }
}

int launch_sweep_uneven(const SweepInst* d_insts, int instances, int total_tiles, int storage, int* d_counter,
                        cudaStream_t st)
{
    const cudaError_t e = cudaMemsetAsync(d_counter, 0, sizeof(int), st);
    if (e != cudaSuccess) return fail(SSG_ERR_CUDA, "cudaMemsetAsync: %s", cudaGetErrorString(e));
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int span = tuning(SSG_TUNE_UNEVEN_SPAN);  // 1, 2 or 4 (<= the 4 entries of s_inst)
    if (storage == SSG_STORAGE_F16)
        launch_sweep_uneven_t<__half>(d_insts, instances, total_tiles, span, d_counter, sms, st);
    else
        launch_sweep_uneven_t<uint16_t>(d_insts, instances, total_tiles, span, d_counter, sms, st);
    return launch_status("sweep_uneven_kernel");
}

template <typename T, int V>
static void launch_sweep_shape(const FastSweepParams& p, const uint4* staged, const int8_t* selected, T* cost,
                               int64_t P, int instances, cudaStream_t st)
{
    constexpr int threads = SweepShape<V>::threads;
    const dim3 grid(grid_1d(P, threads), instances);
    sweep_batch_kernel<T, V><<<grid, threads, 0, st>>>(p, staged, selected, cost);
}

template <typename T>
static void launch_sweep(const FastSweepParams& p, const uint4* staged, const int8_t* selected, T* cost, int64_t P,
                         int instances, cudaStream_t st)
{
    switch (tuning(SSG_TUNE_SWEEP_VARIANT)) {
        case 1: launch_sweep_shape<T, 1>(p, staged, selected, cost, P, instances, st); break;
        case 2: launch_sweep_shape<T, 2>(p, staged, selected, cost, P, instances, st); break;
        default: launch_sweep_shape<T, 0>(p, staged, selected, cost, P, instances, st); break;
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
    SSG_REQUIRE(((uintptr_t)d_staged & 15) == 0 && ((uintptr_t)d_guides & 3) == 0,
                "staged images must be 16-byte and guides 4-byte aligned");
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
    const uint4* staged = reinterpret_cast<const uint4*>(d_staged);
    if (storage == SSG_STORAGE_F16)
        launch_sweep<__half>(p, staged, d_selected, static_cast<__half*>(d_cost), P, frames * references,
                             as_stream(stream));
    else
        launch_sweep<uint16_t>(p, staged, d_selected, static_cast<uint16_t*>(d_cost), P, frames * references,
                               as_stream(stream));
    return launch_status("sweep_batch_kernel");
}
