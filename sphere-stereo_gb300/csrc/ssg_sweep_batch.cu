// Batched sweep + cost (python/depth_estimation.py:141-175) for many (frame, reference) instances
// per launch, with 16-bit output in the chunked layout of ssg_cells.cuh.
//
// A batch is `instances` independent (frame, reference camera) pairs of one rig; blockIdx.y is the
// instance, so a whole batch is one launch.  One thread per pixel of the reference camera walks
// the candidates in order, projects each candidate point into the pixel's selected camera,
// samples it bilinearly (one 16-byte load of the 2 x 2 footprint) and writes 8 candidates at a
// time as one 16-byte cell.  Level-0 storage is __half (fp16) or unorm16 (q = round(c * 65535 / 500);
// costs are clamped to [0, 500]); the arithmetic is fp32.  The fp32 kernels of ssg_sweep.cu are
// the ones that reproduce the reference bit for bit; this sweep projects with approximate square
// roots and reciprocal, a change far below the 16-bit rounding of its output.
#include <algorithm>
#include <atomic>
#include <cmath>

#include "ssg_cells.cuh"
#include "ssg_resize.cuh"
#include "ssg_uneven.cuh"

namespace ssg {


// ---------------------------------------------------------------------------------------------
// Image staging.  The sweep's samples are bilinear, so what it reads per sample is a 2 x 2
// footprint of texels.  A staged entry holds one whole footprint as 8-bit RGB in 16 bytes, one
// 32-bit word per channel: word c of entry (j, i) holds channel c of texels (x0, y0), (x0 + 1, y0),
// (x0, y0 + 1), (x0 + 1, y0 + 1) (bytes 0..3) with (x0, y0) = (i - 1, j - 1); texels outside the
// image are 0 (grid_sample's zero padding).  Entries form planes of (rows + 2) x (cols + 2), one
// per (frame, camera), covering every footprint whose top-left tap lies in [-1, cols] x
// [-1, rows]; every entry is written.  A sample is one 16-byte load, and a channel's bilinear
// blend is two 16-bit x 8-bit dot products.
//
// 8 bits hold decoded images exactly (python/utils.py:157-205 decodes 8-bit files and converts
// them to float32); a linear resize makes fractional values.  Float inputs are therefore checked
// while staging: a plane with a value that is not an integer in [0, 255] gets its flag set
// (plane_flags[plane] = 1), and the sweep samples that plane from the float images themselves.  The guide of every
// reference camera (rgb2yCbCr + uint8 cast) is written in the same pass, from the float values,
// as one 32-bit word per pixel (Y, Cb, Cr, 0).
// ---------------------------------------------------------------------------------------------
struct StageParams {
    int cameras, references, cols, rows;
    int ref_slot[SSG_MAX_CAMERAS];  // reference slot of each camera, -1 if not a reference
};

constexpr int kStageTileX = 64, kStageTileY = 16;                         // entries per block
constexpr int kStageTexX = kStageTileX + 1, kStageTexY = kStageTileY + 1;  // texels they cover

__device__ __forceinline__ float texel_value(float v) { return v; }
__device__ __forceinline__ float texel_value(uint8_t v) { return (float)v; }

// How a plane's values are staged (plane_flags: the largest class over the plane):
//   0: integers in [0, 255]: one byte per value (the high plane);
//   1: values in [0, 65535 / 256] with fractions (a linear resize makes them): 8.8 fixed point,
//      q = round(256 v), high byte in the high plane and low byte in the low plane (a value moves
//      by at most 1/512);
//   2: anything else (negative, larger, NaN): the sweep samples the float images.
constexpr int kPlaneBytes = 0, kPlaneFixed = 1, kPlaneFloats = 2;
constexpr float kFixedMax = 65535.0f / 256.0f;

__device__ __forceinline__ int value_class(float v)
{
    if (v >= 0.0f && v <= 255.0f && v == rintf(v)) return kPlaneBytes;
    return v >= 0.0f && v <= kFixedMax ? kPlaneFixed : kPlaneFloats;
}
__device__ __forceinline__ int value_class(uint8_t) { return kPlaneBytes; }

// the 8.8 fixed-point code of a value of class 0 or 1 (0 for class 2)
__device__ __forceinline__ uint32_t fixed_code(float v, int cls)
{
    return cls == kPlaneFloats ? 0u : __float2uint_rn(v * 256.0f);
}
__device__ __forceinline__ uint32_t fixed_code(uint8_t v, int) { return (uint32_t)v << 8; }

// byte c of three codes' high (kLow = false) or low bytes, packed as one word (byte 3 zero)
template <bool kLow>
__device__ __forceinline__ uint32_t code_bytes(uint32_t q0, uint32_t q1, uint32_t q2)
{
    const int sh = kLow ? 0 : 8;
    return ((q0 >> sh) & 255u) | (((q1 >> sh) & 255u) << 8) | (((q2 >> sh) & 255u) << 16);
}

// The texels of a tile, read from images at the matching resolution: texel (x, y) of the image
// is three consecutive values (a warp reads 384 contiguous bytes per channel load).
template <typename Tin>
struct ImageTexels {
    const Tin* img;
    int cols;
    __device__ __forceinline__ void get(int x, int y, int, int, Tin (&v)[3]) const
    {
        const int64_t o = ((int64_t)y * cols + x) * 3;
        v[0] = img[o];
        v[1] = img[o + 1];
        v[2] = img[o + 2];
    }
};

// The texels of a tile resized from 8-bit source images (the linear resize of ssg_prep.cu, u8 ->
// float32, with its taps and its separately rounded products and sums).  `win` holds the tile's
// source window as floats (one per byte); for each texel column, `cw` gives the window offsets of
// its two source texels' first bytes and their weights (1 - f, f), and for each texel row, `rw`
// the window offsets of its two source rows and their weights: four floats, one 16-byte shared
// load each.  An exact 2x reduction averages the four taps instead.
struct TapOffsets {
    int o0, o1;
    float w0, w1;
};

struct ResizedTexels {
    const float* win;
    const TapOffsets* cw;
    const TapOffsets* rw;
    int area2;
    __device__ __forceinline__ void get(int, int, int lx, int ly, float (&v)[3]) const
    {
        const TapOffsets tx = cw[lx], ty = rw[ly];
        const float* r0 = win + ty.o0;
        const float* r1 = win + ty.o1;
        const int a = tx.o0, b = tx.o1;
        if (area2) {
#pragma unroll
            for (int c = 0; c < 3; ++c)
                v[c] = __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(r0[a + c], r0[b + c]), r1[a + c]), r1[b + c]), 0.25f);
        } else {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float h0 = __fadd_rn(__fmul_rn(r0[a + c], tx.w0), __fmul_rn(r0[b + c], tx.w1));
                const float h1 = __fadd_rn(__fmul_rn(r1[a + c], tx.w0), __fmul_rn(r1[b + c], tx.w1));
                v[c] = __fadd_rn(__fmul_rn(h0, ty.w0), __fmul_rn(h1, ty.w1));
            }
        }
    }
};

// One block: a kStageTileX x kStageTileY tile of entries from shared-memory tiles of texels.
// Each thread converts whole texels (from `src`), classifies them and, for the texels that are
// pixels of this tile, writes their guide word; then each thread assembles entries from the
// shared tiles.  inst: frame * cameras + camera; its entries start at staged[2 * inst * plane]:
// 16-byte entries of high bytes for 8-bit inputs, 32-byte entries (high words x, y, z and low
// word x, then low words y, z) for float inputs.
template <typename Tin, typename Src>
__device__ __forceinline__ void stage_tile(const StageParams& p, const Src& src, int inst, int i0, int j0,
                                           uint4* __restrict__ staged, uint32_t* __restrict__ guides,
                                           int* __restrict__ plane_flags)
{
    constexpr bool kLowPlane = sizeof(Tin) == 4;  // 8-bit inputs have no fractions
    __shared__ uint32_t tex[kStageTexY][kStageTexX];                      // high bytes, byte 3 zero
    __shared__ uint32_t tex_low[kLowPlane ? kStageTexY : 1][kStageTexX];  // low bytes
    __shared__ int block_class;
    const int pitch = p.cols + 2;
    const int64_t P = (int64_t)p.cols * p.rows, plane = (int64_t)pitch * (p.rows + 2);
    const int frame = inst / p.cameras, cam = inst % p.cameras;
    const int slot = p.ref_slot[cam];
    uint32_t* guide = slot >= 0 ? guides + ((int64_t)frame * p.references + slot) * P : nullptr;
    if (threadIdx.x == 0) block_class = 0;
    // texel (x, y), x in [i0 - 1, i0 + kStageTileX - 1], y in [j0 - 1, j0 + kStageTileY - 1]: the
    // entries' top-left taps and their right / lower neighbours.  The top-left taps are the
    // pixels whose guide words this block writes.
    int cls = 0;
    for (int t = threadIdx.x; t < kStageTexY * kStageTexX; t += blockDim.x) {
        const int ly = t / kStageTexX, lx = t % kStageTexX;
        const int x = i0 - 1 + lx, y = j0 - 1 + ly;
        uint32_t q0 = 0, q1 = 0, q2 = 0;
        if (x >= 0 && y >= 0 && x < p.cols && y < p.rows) {
            const int64_t o = (int64_t)y * p.cols + x;
            Tin r[3];
            src.get(x, y, lx, ly, r);
            const int k0 = value_class(r[0]), k1 = value_class(r[1]), k2 = value_class(r[2]);
            cls = max(cls, max(k0, max(k1, k2)));
            q0 = fixed_code(r[0], k0);
            q1 = fixed_code(r[1], k1);
            q2 = fixed_code(r[2], k2);
            if (guide && lx < kStageTileX && ly < kStageTileY) {
                // utils.py:144-155, the arithmetic of ssg_rgb_to_guide, from the input values
                const float c0 = texel_value(r[0]), c1 = texel_value(r[1]), c2 = texel_value(r[2]);
                const float yy = fadd(fadd(fadd(fmul(c0, 0.1826f), 16.0f), fmul(c1, 0.6142f)), fmul(c2, 0.062f));
                const float cb = fadd(fsub(fsub(128.0f, fmul(c0, 0.1006f)), fmul(c1, 0.3386f)), fmul(c2, 0.4392f));
                const float cr = fsub(fsub(fadd(fmul(c0, 0.4392f), 128.0f), fmul(c1, 0.3989f)), fmul(c2, 0.0403f));
                // one 32-bit word per pixel: bytes (Y, Cb, Cr, 0)
                const uint32_t g0 = __float2uint_rz(fminf(fmaxf(yy, 16.0f), 235.0f));
                const uint32_t g1 = __float2uint_rz(fminf(fmaxf(cb, 16.0f), 240.0f));
                const uint32_t g2 = __float2uint_rz(fminf(fmaxf(cr, 16.0f), 240.0f));
                guide[o] = g0 | (g1 << 8) | (g2 << 16);
            }
        }
        tex[ly][lx] = code_bytes<false>(q0, q1, q2);
        if constexpr (kLowPlane) tex_low[ly][lx] = code_bytes<true>(q0, q1, q2);
    }
    __syncthreads();  // block_class is cleared before any thread raises it
    if (cls) atomicMax(&block_class, cls);
    __syncthreads();
    if (threadIdx.x == 0 && block_class) atomicMax(plane_flags + inst, block_class);
    uint4* out = staged + (int64_t)(2 * inst) * plane;
    for (int e = threadIdx.x; e < kStageTileX * kStageTileY; e += blockDim.x) {
        const int li = e % kStageTileX, lj = e / kStageTileX;
        const int i = i0 + li, j = j0 + lj;
        if (i >= pitch || j >= p.rows + 2) continue;
        uint32_t word[2][3];
#pragma unroll
        for (int h = 0; h < (kLowPlane ? 2 : 1); ++h) {
            const uint32_t(*tx)[kStageTexX] = h ? tex_low : tex;
            const uint32_t t00 = tx[lj][li], t10 = tx[lj][li + 1];
            const uint32_t t01 = tx[lj + 1][li], t11 = tx[lj + 1][li + 1];
#pragma unroll
            for (int ch = 0; ch < 3; ++ch) {
                const uint32_t sel = (uint32_t)ch | ((uint32_t)(4 + ch) << 4);
                word[h][ch] = __byte_perm(__byte_perm(t00, t10, sel), __byte_perm(t01, t11, sel), 0x5410);
            }
        }
        const int64_t at = (int64_t)j * pitch + i;
        if constexpr (kLowPlane) {
            // a 32-byte entry, one 256-bit store: high words x, y, z, low word x | low words y, z
            const unsigned long long w0 = word[0][0] | (unsigned long long)word[0][1] << 32,
                                     w1 = word[0][2] | (unsigned long long)word[1][0] << 32,
                                     w2 = word[1][1] | (unsigned long long)word[1][2] << 32;
            asm volatile("st.global.v4.b64 [%0], {%1, %2, %3, %4};" ::"l"(out + 2 * at), "l"(w0), "l"(w1), "l"(w2),
                         "l"(0ull)
                         : "memory");
        } else {
            out[at] = make_uint4(word[0][0], word[0][1], word[0][2], 0u);
        }
    }
}

// the tile of entries of block blockIdx.x, for images of cols x rows pixels
__device__ __forceinline__ void stage_tile_origin(const StageParams& p, int& i0, int& j0)
{
    const int tiles_x = (p.cols + 2 + kStageTileX - 1) / kStageTileX;
    i0 = (blockIdx.x % tiles_x) * kStageTileX;
    j0 = (blockIdx.x / tiles_x) * kStageTileY;
}

// blockIdx.y: frame * cameras + camera, images at the matching resolution
template <typename Tin>
__global__ void __launch_bounds__(kBatchBlock) stage_images_kernel(const __grid_constant__ StageParams p,
                                                                  const Tin* __restrict__ images,
                                                                  uint4* __restrict__ staged,
                                                                  uint32_t* __restrict__ guides,
                                                                  int* __restrict__ plane_flags)
{
    int i0, j0;
    stage_tile_origin(p, i0, j0);
    const int inst = blockIdx.y;
    const ImageTexels<Tin> src{images + (int64_t)inst * p.cols * p.rows * 3, p.cols};
    stage_tile<Tin>(p, src, inst, i0, j0, staged, guides, plane_flags);
}

// The same staging from 8-bit source images of any size, resized to the matching resolution on
// the way (ssg_stage_images_resized).  The block first forms its texel columns' and rows' taps,
// then copies the source window they cover (rows rtap[0].s0 .. rtap[last].s1, columns
// ctap[0].s0 .. ctap[last].s1; `win_rows` x `row_floats` floats of dynamic shared memory, sized on
// the host for the largest window of any tile) with aligned 32-bit loads, one float per byte.
// Each image's bytes start 4-byte aligned and end on a word boundary (checked on the host), so
// every word read lies inside its image.
__global__ void __launch_bounds__(kBatchBlock) stage_resized_kernel(const __grid_constant__ StageParams p,
                                                                    const __grid_constant__ ResizeParams rp,
                                                                    const uint8_t* __restrict__ images,
                                                                    int row_floats, uint4* __restrict__ staged,
                                                                    uint32_t* __restrict__ guides,
                                                                    int* __restrict__ plane_flags)
{
    extern __shared__ __align__(16) float win[];
    __shared__ Tap ctap[kStageTexX], rtap[kStageTexY];
    __shared__ __align__(16) TapOffsets cw[kStageTexX], rw[kStageTexY];
    int i0, j0;
    stage_tile_origin(p, i0, j0);
    const int inst = blockIdx.y;
    const int t = threadIdx.x;
    if (t < kStageTexX) ctap[t] = column_tap(rp, min(max(i0 - 1 + t, 0), p.cols - 1));
    else if (t < kStageTexX + kStageTexY)
        rtap[t - kStageTexX] = row_tap(rp, min(max(j0 - 1 + t - kStageTexX, 0), p.rows - 1));
    __syncthreads();
    const int r_min = rtap[0].s0, r_max = rtap[kStageTexY - 1].s1;
    const int c_min = ctap[0].s0, c_max = ctap[kStageTexX - 1].s1;
    // byte offset of source byte 3 (r src_cols + c) within its 32-bit word; only the low two bits
    // of the (wrapping) 32-bit product matter
    const uint32_t row_bytes = 3u * (uint32_t)rp.src_cols;
    if (t < kStageTexX) {
        const Tap tx = ctap[t];
        cw[t] = TapOffsets{3 * (tx.s0 - c_min), 3 * (tx.s1 - c_min), __fsub_rn(1.0f, tx.f), tx.f};
    } else if (t < kStageTexX + kStageTexY) {
        const Tap ty = rtap[t - kStageTexX];
        const uint32_t lead = 3u * (uint32_t)c_min;
        const int o0 = (ty.s0 - r_min) * row_floats + (int)(((uint32_t)ty.s0 * row_bytes + lead) & 3u);
        const int o1 = (ty.s1 - r_min) * row_floats + (int)(((uint32_t)ty.s1 * row_bytes + lead) & 3u);
        rw[t - kStageTexX] = TapOffsets{o0, o1, __fsub_rn(1.0f, ty.f), ty.f};
    }
    // the window: rows r_min..r_max, each from the word holding byte 3 c_min to the one holding
    // byte 3 c_max + 2, one float per byte
    const int64_t image_bytes = (int64_t)rp.src_cols * rp.src_rows * 3;
    const uint32_t* words = reinterpret_cast<const uint32_t*>(images + (int64_t)inst * image_bytes);
    const int row_words = row_floats / 4;
    for (int k = t; k < (r_max - r_min + 1) * row_words; k += blockDim.x) {
        const int wr = k / row_words, q = k % row_words;
        const int64_t b0 = ((int64_t)(r_min + wr) * rp.src_cols + c_min) * 3;
        const int64_t b1 = b0 + 3 * (int64_t)(c_max - c_min + 1);
        const int64_t w = (b0 >> 2) + q;
        if (w < (b1 + 3) >> 2) {
            const uint32_t v = __ldg(words + w);
            reinterpret_cast<float4*>(win + wr * row_floats)[q] =
                make_float4((float)(v & 255u), (float)((v >> 8) & 255u), (float)((v >> 16) & 255u), (float)(v >> 24));
        }
    }
    __syncthreads();
    const ResizedTexels src{win, cw, rw, rp.area2};
    stage_tile<float>(p, src, inst, i0, j0, staged, guides, plane_flags);
}

// ---------------------------------------------------------------------------------------------
// Column-sweep staging: the same entries, guides and plane classes as stage_tile, with no shared
// tile and no block barrier.  A warp walks down a strip of 32 texel columns, x = ib - 1 + lane,
// over kColRows + 1 texel rows (the first a halo); at each texel row y it forms its texel's codes,
// takes its right neighbour's from lane + 1 (one shuffle per plane) and, with the previous row's
// kept in registers, writes the entry of row y for lanes 0..30 (entry ib + lane).  Strips overlap
// by one texel column; the guide of pixel (x, y) is written by the lane for which x is not the
// halo column (lanes 1..31) and for the rows that are not the halo row.
// ---------------------------------------------------------------------------------------------
constexpr int kColStrip = 31;  // entry columns per strip (32 lanes: 32 texel columns)
constexpr int kColRows = 31;   // entry rows per warp (32 texel rows with the halo)
constexpr int kColWarps = 8;   // warps per block

// the three codes of a texel as words of high and low bytes (byte 3 zero; the codes are 16-bit)
__device__ __forceinline__ void pack_codes(uint32_t q0, uint32_t q1, uint32_t q2, uint32_t& hi, uint32_t& lo)
{
    const uint32_t q01 = __byte_perm(q0, q1, 0x5410);
    hi = __byte_perm(q01, q2, 0x6531);
    lo = __byte_perm(q01, q2, 0x6420);
}

// texels of images at the matching resolution: three consecutive values
template <typename Tin>
struct ColumnImage {
    const Tin* img;
    int cols;
    __device__ __forceinline__ void rows(int, int, int) {}
    __device__ __forceinline__ void get(int x, int y, int, Tin (&v)[3])
    {
        const int64_t o = ((int64_t)y * cols + x) * 3;
        v[0] = __ldg(img + o);
        v[1] = __ldg(img + o + 1);
        v[2] = __ldg(img + o + 2);
    }
};

// a byte of a word as a float: 2^23 + b assembled in the bits, minus 2^23 (exact)
__device__ __forceinline__ float byte_float(uint32_t w, int k)
{
    return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7440u | (uint32_t)k)) - 8388608.0f;
}

// Texels resized from 8-bit source images (ssg_prep.cu's u8 -> float32 linear resize: its taps and
// its separately rounded products and sums).  Each lane forms its column's taps once; the row taps
// of the warp's texel rows are formed one per lane and shuffled to the warp row by row (rows()).
// The last two source rows read (values of the lane's two source texels, three channels each)
// are kept, so a source row shared by consecutive texel rows is read once.  (Reading the next
// row's source texels one row ahead was measured slower: 80 registers instead of 64.)
struct ColumnResized {
    const uint8_t* img;  // this image's bytes (4-byte aligned, a multiple of 4 bytes long)
    int src_cols, area2;
    Tap tx;
    float a0, a1;
    Tap ty;                // the current row's taps (rows())
    int lane_s0, lane_s1;  // the row taps of texel row y0 + lane, y0 the warp's first texel row
    float lane_f;
    int ra = -1, rb = -1;
    float va[6], vb[6];
    __device__ __forceinline__ void init(const ResizeParams& rp, int x, int y0, int cols, int rows)
    {
        tx = column_tap(rp, min(max(x, 0), cols - 1));
        a0 = __fsub_rn(1.0f, tx.f);
        a1 = tx.f;
        const int lane = threadIdx.x & 31;
        const Tap t = row_tap(rp, min(max(y0 + lane, 0), rows - 1));
        lane_s0 = t.s0;
        lane_s1 = t.s1;
        lane_f = t.f;
    }
    // every lane, texel row y0 + k.  Lanes 0 and 31 also ask L2 for the first and the last
    // source texel of the warp's segment of the bottom source row of texel row k + 3 (about 38
    // texels, 114 bytes, one or two lines), so that the first read of a source row finds it there
    __device__ __forceinline__ void rows(int k, int, int)
    {
        ty.s0 = __shfl_sync(0xFFFFFFFFu, lane_s0, k);
        ty.s1 = __shfl_sync(0xFFFFFFFFu, lane_s1, k);
        ty.f = __shfl_sync(0xFFFFFFFFu, lane_f, k);
        const int ahead = __shfl_sync(0xFFFFFFFFu, lane_s1, min(k + 3, 31));
        const int lane = threadIdx.x & 31;
        if (lane == 0 || lane == 31) {
            const uint8_t* p = img + ((int64_t)ahead * src_cols + tx.s0) * 3;  // a byte of the image
            asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
        }
    }
    // the lane's two source texels of source row r
    __device__ __forceinline__ void load_row(int r, float (&v)[6]) const
    {
        const uint32_t* words = reinterpret_cast<const uint32_t*>(img);
        const int64_t b = ((int64_t)r * src_cols + tx.s0) * 3;
        const int64_t w = b >> 2;
        const int off = (int)(b & 3);
        const bool pair = tx.s1 != tx.s0;
        const int last = off + (pair ? 5 : 2);  // the last byte, counted from word w
        const uint32_t w0 = __ldg(words + w);
        const uint32_t w1 = last >= 4 ? __ldg(words + w + 1) : 0u;
        const uint32_t w2 = last >= 8 ? __ldg(words + w + 2) : 0u;
        const uint32_t lo = __funnelshift_r(w0, w1, 8 * off), hi = __funnelshift_r(w1, w2, 8 * off);
        v[0] = byte_float(lo, 0);
        v[1] = byte_float(lo, 1);
        v[2] = byte_float(lo, 2);
        if (pair) {
            v[3] = byte_float(lo, 3);
            v[4] = byte_float(hi, 0);
            v[5] = byte_float(hi, 1);
        } else {
            v[3] = v[0];
            v[4] = v[1];
            v[5] = v[2];
        }
    }
    __device__ __forceinline__ void get(int, int, int, float (&out)[3])
    {
        float top[6], bot[6];
        // rows only advance: the new top row is one of the kept rows or a new one, the bottom row too
        if (ty.s0 == rb) {
#pragma unroll
            for (int i = 0; i < 6; ++i) top[i] = vb[i];
        } else if (ty.s0 == ra) {
#pragma unroll
            for (int i = 0; i < 6; ++i) top[i] = va[i];
        } else {
            load_row(ty.s0, top);
        }
        if (ty.s1 == ty.s0) {
#pragma unroll
            for (int i = 0; i < 6; ++i) bot[i] = top[i];
        } else if (ty.s1 == rb) {
#pragma unroll
            for (int i = 0; i < 6; ++i) bot[i] = vb[i];
        } else {
            load_row(ty.s1, bot);
        }
        ra = ty.s0;
        rb = ty.s1;
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            va[i] = top[i];
            vb[i] = bot[i];
        }
        if (area2) {
#pragma unroll
            for (int c = 0; c < 3; ++c)
                out[c] = __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(top[c], top[3 + c]), bot[c]), bot[3 + c]), 0.25f);
        } else {
            const float b0 = __fsub_rn(1.0f, ty.f), b1 = ty.f;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float h0 = __fadd_rn(__fmul_rn(top[c], a0), __fmul_rn(top[3 + c], a1));
                const float h1 = __fadd_rn(__fmul_rn(bot[c], a0), __fmul_rn(bot[3 + c], a1));
                out[c] = __fadd_rn(__fmul_rn(h0, b0), __fmul_rn(h1, b1));
            }
        }
    }
};

// One warp's strip.  Src: ColumnImage<Tin> or ColumnResized (Tin = float), initialised for the
// lane's column; inst: frame * cameras + camera.
template <typename Tin, typename Src>
__device__ __forceinline__ void stage_strip(const StageParams& p, Src& src, int inst, int ib, int jb,
                                            uint4* __restrict__ staged, uint32_t* __restrict__ guides,
                                            int* __restrict__ plane_flags)
{
    constexpr bool kLowPlane = sizeof(Tin) == 4;
    const int lane = threadIdx.x & 31;
    const int pitch = p.cols + 2;
    const int64_t P = (int64_t)p.cols * p.rows, plane = (int64_t)pitch * (p.rows + 2);
    const int frame = inst / p.cameras, cam = inst % p.cameras;
    const int slot = p.ref_slot[cam];
    uint32_t* guide = slot >= 0 ? guides + ((int64_t)frame * p.references + slot) * P : nullptr;
    uint4* out = staged + (int64_t)(2 * inst) * plane;
    const int x = ib - 1 + lane;
    const bool col_in = x >= 0 && x < p.cols;
    const int i = ib + lane;  // this lane's entry column
    const bool writes = lane < kColStrip && i < pitch;
    int cls = 0;
    uint32_t up_hi = 0, up_lo = 0, up_hi_r = 0, up_lo_r = 0;  // the previous texel row's words
    const int y_end = min(jb + kColRows, p.rows + 2);
    for (int y = jb - 1, k = 0; y < y_end; ++y, ++k) {
        src.rows(k, y, p.rows);
        uint32_t hi = 0, lo = 0;
        if (col_in && y >= 0 && y < p.rows) {
            Tin r[3];
            src.get(x, y, k, r);
            const int k0 = value_class(r[0]), k1 = value_class(r[1]), k2 = value_class(r[2]);
            cls = max(cls, max(k0, max(k1, k2)));
            pack_codes(fixed_code(r[0], k0), fixed_code(r[1], k1), fixed_code(r[2], k2), hi, lo);
            if (guide && lane > 0 && y >= jb) {
                // utils.py:144-155, the arithmetic of ssg_rgb_to_guide, from the input values
                const float c0 = texel_value(r[0]), c1 = texel_value(r[1]), c2 = texel_value(r[2]);
                const float yy = fadd(fadd(fadd(fmul(c0, 0.1826f), 16.0f), fmul(c1, 0.6142f)), fmul(c2, 0.062f));
                const float cb = fadd(fsub(fsub(128.0f, fmul(c0, 0.1006f)), fmul(c1, 0.3386f)), fmul(c2, 0.4392f));
                const float cr = fsub(fsub(fadd(fmul(c0, 0.4392f), 128.0f), fmul(c1, 0.3989f)), fmul(c2, 0.0403f));
                const uint32_t g0 = __float2uint_rz(fminf(fmaxf(yy, 16.0f), 235.0f));
                const uint32_t g1 = __float2uint_rz(fminf(fmaxf(cb, 16.0f), 240.0f));
                const uint32_t g2 = __float2uint_rz(fminf(fmaxf(cr, 16.0f), 240.0f));
                guide[(int64_t)y * p.cols + x] = g0 | (g1 << 8) | (g2 << 16);
            }
        }
        const uint32_t hi_r = __shfl_down_sync(0xFFFFFFFFu, hi, 1);
        const uint32_t lo_r = kLowPlane ? __shfl_down_sync(0xFFFFFFFFu, lo, 1) : 0u;
        if (y >= jb && writes) {
            // entry (i, y): taps (x, y - 1), (x + 1, y - 1), (x, y), (x + 1, y) as bytes 0..3
            uint32_t word[2][3];
#pragma unroll
            for (int ch = 0; ch < 3; ++ch) {
                const uint32_t sel = (uint32_t)ch | ((uint32_t)(4 + ch) << 4);
                word[0][ch] = __byte_perm(__byte_perm(up_hi, up_hi_r, sel), __byte_perm(hi, hi_r, sel), 0x5410);
                if constexpr (kLowPlane)
                    word[1][ch] = __byte_perm(__byte_perm(up_lo, up_lo_r, sel), __byte_perm(lo, lo_r, sel), 0x5410);
            }
            const int64_t at = (int64_t)y * pitch + i;
            if constexpr (kLowPlane) {
                const unsigned long long w0 = word[0][0] | (unsigned long long)word[0][1] << 32,
                                         w1 = word[0][2] | (unsigned long long)word[1][0] << 32,
                                         w2 = word[1][1] | (unsigned long long)word[1][2] << 32;
                asm volatile("st.global.v4.b64 [%0], {%1, %2, %3, %4};" ::"l"(out + 2 * at), "l"(w0), "l"(w1),
                             "l"(w2), "l"(0ull)
                             : "memory");
            } else {
                out[at] = make_uint4(word[0][0], word[0][1], word[0][2], 0u);
            }
        }
        up_hi = hi;
        up_lo = lo;
        up_hi_r = hi_r;
        up_lo_r = lo_r;
    }
    cls = __reduce_max_sync(0xFFFFFFFFu, cls);
    if (lane == 0 && cls) atomicMax(plane_flags + inst, cls);
}

// the strip of warp w of an image: strips of kColStrip entry columns by kColRows entry rows
__device__ __forceinline__ bool strip_origin(const StageParams& p, int& ib, int& jb)
{
    const int strips_x = (p.cols + 2 + kColStrip - 1) / kColStrip;
    const int strips = strips_x * ((p.rows + 2 + kColRows - 1) / kColRows);
    const int w = blockIdx.x * kColWarps + (int)(threadIdx.x >> 5);
    if (w >= strips) return false;
    ib = (w % strips_x) * kColStrip;
    jb = (w / strips_x) * kColRows;
    return true;
}

template <typename Tin>
__global__ void __launch_bounds__(kColWarps * 32) stage_columns_kernel(const __grid_constant__ StageParams p,
                                                                      const Tin* __restrict__ images,
                                                                      uint4* __restrict__ staged,
                                                                      uint32_t* __restrict__ guides,
                                                                      int* __restrict__ plane_flags)
{
    int ib, jb;
    if (!strip_origin(p, ib, jb)) return;  // whole warps
    const int inst = blockIdx.y;
    ColumnImage<Tin> src{images + (int64_t)inst * p.cols * p.rows * 3, p.cols};
    stage_strip<Tin>(p, src, inst, ib, jb, staged, guides, plane_flags);
}

__global__ void __launch_bounds__(kColWarps * 32) stage_resized_columns_kernel(const __grid_constant__ StageParams p,
                                                                              const __grid_constant__ ResizeParams rp,
                                                                              const uint8_t* __restrict__ images,
                                                                              uint4* __restrict__ staged,
                                                                              uint32_t* __restrict__ guides,
                                                                              int* __restrict__ plane_flags)
{
    int ib, jb;
    if (!strip_origin(p, ib, jb)) return;  // whole warps
    const int inst = blockIdx.y;
    ColumnResized src;
    src.img = images + (int64_t)inst * rp.src_cols * rp.src_rows * 3;
    src.src_cols = rp.src_cols;
    src.area2 = rp.area2;
    src.init(rp, ib - 1 + (int)(threadIdx.x & 31), jb - 1, p.cols, p.rows);
    stage_strip<float>(p, src, inst, ib, jb, staged, guides, plane_flags);
}

static dim3 column_grid(int cols, int rows, int images)
{
    const int64_t strips =
        (int64_t)((cols + 2 + kColStrip - 1) / kColStrip) * ((rows + 2 + kColRows - 1) / kColRows);
    return dim3((unsigned)((strips + kColWarps - 1) / kColWarps), (unsigned)images);
}

// channel c (0..2) of texel k (0: nw, 1: ne, 2: sw, 3: se) of an entry
__device__ __forceinline__ float entry_texel(const uint4& q, int c, int k)
{
    const uint32_t w = c == 0 ? q.x : c == 1 ? q.y : q.z;
    return (float)((w >> (8 * k)) & 0xFFu);
}

// the same footprint from the float images (a plane whose values are not all 8-bit integers)
__device__ __forceinline__ void float_footprint(const float* __restrict__ img, int cols, int rows, int x0, int y0,
                                                float (&t)[4][3])
{
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int x = x0 + (k & 1), y = y0 + (k >> 1);
        const bool in = x >= 0 && y >= 0 && x < cols && y < rows;
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) t[k][ch] = in ? __ldg(img + ((int64_t)y * cols + x) * 3 + ch) : 0.0f;
    }
}

// ---------------------------------------------------------------------------------------------
// Sweep + cost, batched, 16-bit output
// ---------------------------------------------------------------------------------------------

struct FastSweepParams {
    int cols, rows, cameras, references, ncand, chunks;
    int entry_words;  // 16-byte words per staged entry: 1 (8-bit inputs) or 2 (8.8 fixed point)
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
// se) at two positions of one camera plane.  The coordinates are clamped to [-1, cols] x
// [-1, rows] (a NaN to -1): a sample whose four taps all lie outside the image then reads a
// footprint of zeros, or has weight 0 on its in-image taps, so it is exactly 0 as grid_sample's,
// without a branch.  The tap weights of both samples are returned as (nw, ne, sw, se) = (wa, wb,
// wc, wd), the top-left taps as x0, y0.
__device__ __forceinline__ void bilinear_pair(int cols, int rows, float2 ix, float2 iy, float2& x0, float2& y0,
                                              float2& wa, float2& wb, float2& wc, float2& wd)
{
    const float colsf = (float)cols, rowsf = (float)rows;
    ix = make_float2(fminf(fmaxf(ix.x, -1.0f), colsf), fminf(fmaxf(ix.y, -1.0f), colsf));
    iy = make_float2(fminf(fmaxf(iy.x, -1.0f), rowsf), fminf(fmaxf(iy.y, -1.0f), rowsf));
    x0 = make_float2(floorf(ix.x), floorf(ix.y));
    y0 = make_float2(floorf(iy.x), floorf(iy.y));
    const float2 fx = add2(ix, make_float2(-x0.x, -x0.y)), fy = add2(iy, make_float2(-y0.x, -y0.y));
    const float2 gx = add2(splat(1.0f), make_float2(-fx.x, -fx.y)), gy = add2(splat(1.0f), make_float2(-fy.x, -fy.y));
    wa = mul2(gx, gy);
    wb = mul2(fx, gy);
    wc = mul2(gx, fy);
    wd = mul2(fx, fy);
}

// Samples of a plane whose values are not all 8-bit integers, from its float image.
__device__ __forceinline__ void sample_pair_floats(const float* __restrict__ floats, int cols, int rows, float2 ix,
                                                   float2 iy, float (&s)[2][3])
{
    float2 x0, y0, wa, wb, wc, wd;
    bilinear_pair(cols, rows, ix, iy, x0, y0, wa, wb, wc, wd);
    float t[2][4][3];
#pragma unroll
    for (int h = 0; h < 2; ++h) float_footprint(floats, cols, rows, (int)(h ? x0.y : x0.x), (int)(h ? y0.y : y0.x), t[h]);
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

// Samples of a staged plane from its footprints (`entries`), in units of 1/65535: the weights
// are 16-bit fractions of 65535 (a rounding of at most 1/131070 each: a sample moves by at most
// 4 * 255 / 131070 < 0.008), each channel blended by two dot products of two 16-bit weights
// with two 8-bit taps.  w * 65535 + 1.5 * 2^23 has round(w * 65535) in the low 16 bits of its
// representation (one fused multiply-add per weight, for both samples).  Entries are kStride
// 16-byte words apart (2: the 32-byte entries of float inputs).  kFixed: the entries hold 8.8
// fixed-point codes, low bytes in word 3 and the second half.  A low byte weighs 1/256 of a high
// one, so the low bytes are blended by one 4-way byte dot product with the high bytes of the
// 16-bit weights (floor(w * 65535 / 256), within 1 of w * 65535 / 256): the result is again in
// units of 1/65535, below the exact low-byte blend by less than 4 * 255 units (0.016 of a grey
// level), on top of the high bytes' rounding above.
// One 32-byte footprint entry in one 256-bit load (sm_100 and later; `p` 32-byte aligned, which
// the entry points check for the staged planes of float inputs)
__device__ __forceinline__ void load_entry32(const uint4* p, uint4& q, uint4& r)
{
    unsigned long long a, b, c, d;
    asm("ld.global.nc.v4.b64 {%0, %1, %2, %3}, [%4];" : "=l"(a), "=l"(b), "=l"(c), "=l"(d) : "l"(p));
    q = make_uint4((uint32_t)a, (uint32_t)(a >> 32), (uint32_t)b, (uint32_t)(b >> 32));
    r = make_uint4((uint32_t)c, (uint32_t)(c >> 32), (uint32_t)d, (uint32_t)(d >> 32));
}

template <bool kFixed, int kStride>
__device__ __forceinline__ void sample_pair_codes(const uint4* __restrict__ entries, int cols, int rows, float2 ix,
                                                  float2 iy, uint32_t (&s)[2][3])
{
    static_assert(!kFixed || kStride == 2, "fixed-point codes are staged in 32-byte entries");
    // bilinear_pair's clamp, floors and weights, the floors formed on the FMA pipe: the clamped
    // coordinate plus 2^23 + 1, rounded down, is exactly floor + 1 + 2^23 (the sum lies in
    // [2^23, 2^24), where floats are the integers), so its bits hold floor + 1 and subtracting
    // 2^23 + 1 gives the floor itself
    const float colsf = (float)cols, rowsf = (float)rows;
    ix = make_float2(fminf(fmaxf(ix.x, -1.0f), colsf), fminf(fmaxf(ix.y, -1.0f), colsf));
    iy = make_float2(fminf(fmaxf(iy.x, -1.0f), rowsf), fminf(fmaxf(iy.y, -1.0f), rowsf));
    const float2 tx = add2_rd(ix, splat(8388609.0f)), ty = add2_rd(iy, splat(8388609.0f));
    const float2 x0 = add2(tx, splat(-8388609.0f)), y0 = add2(ty, splat(-8388609.0f));
    const float2 fx = add2(ix, make_float2(-x0.x, -x0.y)), fy = add2(iy, make_float2(-y0.x, -y0.y));
    const float2 gx = add2(splat(1.0f), make_float2(-fx.x, -fx.y)), gy = add2(splat(1.0f), make_float2(-fy.x, -fy.y));
    const float2 wa = mul2(gx, gy), wb = mul2(fx, gy), wc = mul2(gx, fy), wd = mul2(fx, fy);
    const float2 scale = splat(65535.0f), magic = splat(12582912.0f);
    const float2 qa = fma2(wa, scale, magic), qb = fma2(wb, scale, magic), qc = fma2(wc, scale, magic),
                 qd = fma2(wd, scale, magic);
    // entry index (y0 + 1) * pitch + x0 + 1 from the bits of tx, ty (0x4B000000 + floor + 1 each),
    // in wrapping 32-bit arithmetic: the offsets cancel and the index fits
    const uint32_t pitch = (uint32_t)cols + 2u, bias = 0x4B000000u * (pitch + 1u);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const uint32_t top = __byte_perm(__float_as_uint(h ? qa.y : qa.x), __float_as_uint(h ? qb.y : qb.x), 0x5410);
        const uint32_t bot = __byte_perm(__float_as_uint(h ? qc.y : qc.x), __float_as_uint(h ? qd.y : qd.x), 0x5410);
        const uint32_t idx = __float_as_uint(h ? ty.y : ty.x) * pitch + __float_as_uint(h ? tx.y : tx.x) - bias;
        uint4 q, r;
        if constexpr (kFixed) load_entry32(entries + kStride * idx, q, r);  // both halves of the entry
        else q = __ldg(entries + kStride * idx);
        s[h][0] = __dp2a_hi(bot, q.x, __dp2a_lo(top, q.x, 0u));
        s[h][1] = __dp2a_hi(bot, q.y, __dp2a_lo(top, q.y, 0u));
        s[h][2] = __dp2a_hi(bot, q.z, __dp2a_lo(top, q.z, 0u));
        if constexpr (kFixed) {
            const uint32_t w8 = __byte_perm(top, bot, 0x7531);  // high bytes of the weights nw, ne, sw, se
            s[h][0] = __dp4a(w8, q.w, s[h][0]);
            s[h][1] = __dp4a(w8, r.x, s[h][1]);
            s[h][2] = __dp4a(w8, r.y, s[h][2]);
        }
    }
}

// The candidate loop of one pixel: points d (R u) + t, projected and sampled in pairs, costs
// written 8 candidates per cell.  kMode (the plane classes, kPlane*): kPlaneFloats samples the
// float image with the reference's arithmetic against the float reference texels `rp`; otherwise
// the cost sum_c |sample_c - ref_c| is formed in units of 1/65535 with integer absolute
// differences against `rq` (the reference texels in those units).
template <typename T, int kMode, int kStride, typename V>
__device__ __forceinline__ void sweep_candidates_body(const V& view, const uint4* __restrict__ entries,
                                                      const float* __restrict__ floats, int cols,
                                                      int rows, float2 ax, float2 ay, float2 az, float2 tx, float2 ty,
                                                      float2 tz, const FastCam& k, const float (&rp)[3],
                                                      const uint32_t (&rq)[3], T* __restrict__ out,
                                                      int64_t chunk_stride)
{
    const int chunks = view.chunks();
    for (int ch = 0; ch < chunks; ++ch) {
        uint32_t packed[4];
#pragma unroll
        for (int j = 0; j < 8; j += 2) {
            const float2 d = view.cand2(ch * 8 + j);
            float2 u, v;
            project_pair(fma2(d, ax, tx), fma2(d, ay, ty), fma2(d, az, tz), k, u, v);
            float c2[2];
            if constexpr (kMode == kPlaneFloats) {
                float s[2][3];
                sample_pair_floats(floats, cols, rows, u, v, s);
#pragma unroll
                for (int h = 0; h < 2; ++h)
                    c2[h] = fminf(fabsf(s[h][0] - rp[0]) + fabsf(s[h][1] - rp[1]) + fabsf(s[h][2] - rp[2]), 500.0f);
            } else {
                uint32_t s[2][3];
                sample_pair_codes<kMode == kPlaneFixed, kStride>(entries, cols, rows, u, v, s);
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const uint32_t sad = __usad(s[h][2], rq[2], __usad(s[h][1], rq[1], __usad(s[h][0], rq[0], 0u)));
                    c2[h] = (float)min(sad, 500u * 65535u);
                }
                const float2 c = mul2(make_float2(c2[0], c2[1]), splat(1.0f / 65535.0f));
                c2[0] = c.x;
                c2[1] = c.y;
            }
            packed[j / 2] = Cell<T>::pack2(c2[0], c2[1]);
        }
        reinterpret_cast<uint4*>(out + ch * chunk_stride)[0] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
    }
}

// the rarer plane classes, kept out of line so that their registers do not weigh on the 8-bit path
template <typename T, int kMode, int kStride, typename V>
__device__ __noinline__ void sweep_candidates_outlined(const V view, const uint4* __restrict__ entries,
                                                       const float* __restrict__ floats, int cols, int rows, float2 ax,
                                                       float2 ay, float2 az, float2 tx, float2 ty, float2 tz,
                                                       const FastCam k, float r0, float r1, float r2, uint32_t q0,
                                                       uint32_t q1, uint32_t q2, T* __restrict__ out,
                                                       int64_t chunk_stride)
{
    const float rp[3] = {r0, r1, r2};
    const uint32_t rq[3] = {q0, q1, q2};
    sweep_candidates_body<T, kMode, kStride>(view, entries, floats, cols, rows, ax, ay, az, tx, ty, tz, k, rp, rq, out,
                                             chunk_stride);
}

// Sweep + cost of one reference pixel (x, y) over all candidates, into its cells (`out`, chunk
// stride `chunk_stride`).  `V` gives the instance's constants: ref_cam(), cam(c), pose(c) (12
// floats), cand(k) (pairs are read as float2), cameras(), chunks() and entry_words() (16-byte
// words per entry: 1 for 8-bit inputs, 2 for the 32-byte entries of float or resized inputs).
// `frame_entries` / `frame_floats` point at the frame's camera-0 footprints (camera c's at 2 c
// `plane` 16-byte words) / float image (cols x rows x 3 floats apart; NULL when the frame was
// staged from 8-bit images, resized or not), `flags` at the frame's per-camera plane classes.  The
// pixel takes the path of the larger class of its reference and selected planes.
template <typename T, typename V>
__device__ __forceinline__ void sweep_pixel(const V& view, const uint4* __restrict__ frame_entries,
                                            const float* __restrict__ frame_floats, const int* __restrict__ flags,
                                            int plane, int ref_camera, int cols, int rows, int x, int y, int sel,
                                            T* __restrict__ out, int64_t chunk_stride)
{
    const int pitch = cols + 2;
    const int64_t P = (int64_t)cols * rows;
    const bool seen = sel >= 0 && sel < view.cameras();
    const int stride = view.entry_words();  // 16-byte words per entry: 2 for 32-byte entries
    // 16-byte entries hold 8-bit texels only (a plane flagged otherwise was not staged in them)
    const int mode = stride == 1 ? kPlaneBytes : max(__ldg(flags + ref_camera), seen ? __ldg(flags + sel) : 0);
    float rp[3];
    uint32_t rq[3];
    if (mode == kPlaneFloats && frame_floats) {
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) rp[ch] = __ldg(frame_floats + (ref_camera * P + (int64_t)y * cols + x) * 3 + ch);
    } else {
        // the footprint of top-left tap (x, y): its nw texels (byte 0 of each word) are the pixel's
        const int64_t at = (int64_t)(2 * ref_camera) * plane + (int64_t)stride * ((y + 1) * pitch + x + 1);
        const uint4 q = __ldg(frame_entries + at);
        const uint32_t hw[3] = {q.x, q.y, q.z};
        if (mode == kPlaneFixed) {
            const uint4 r = __ldg(frame_entries + at + 1);
            const uint32_t lw[3] = {q.w, r.x, r.y};
#pragma unroll
            for (int ch = 0; ch < 3; ++ch) {
                const uint32_t code = (hw[ch] & 0xFFu) << 8 | (lw[ch] & 0xFFu);
                rp[ch] = (float)code * (1.0f / 256.0f);
                rq[ch] = (code * 65535u + 128u) >> 8;
            }
        } else {
#pragma unroll
            for (int ch = 0; ch < 3; ++ch) {
                rp[ch] = (float)(hw[ch] & 0xFFu);
                rq[ch] = (hw[ch] & 0xFFu) * 65535u;
            }
        }
    }
    const int chunks = view.chunks();
    if (!seen) {
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
    const uint4* entries = frame_entries + (int64_t)(2 * sel) * plane;
    const float* floats = frame_floats ? frame_floats + sel * P * 3 : nullptr;
    if (mode == kPlaneFloats && floats)
        sweep_candidates_outlined<T, kPlaneFloats, 2>(view, entries, floats, cols, rows, ax, ay, az, tx, ty, tz, k,
                                                      rp[0], rp[1], rp[2], rq[0], rq[1], rq[2], out, chunk_stride);
    else if (mode == kPlaneFixed)
        sweep_candidates_outlined<T, kPlaneFixed, 2>(view, entries, floats, cols, rows, ax, ay, az, tx, ty, tz, k,
                                                     rp[0], rp[1], rp[2], rq[0], rq[1], rq[2], out, chunk_stride);
    else if (stride == 2)
        sweep_candidates_outlined<T, kPlaneBytes, 2>(view, entries, floats, cols, rows, ax, ay, az, tx, ty, tz, k,
                                                     rp[0], rp[1], rp[2], rq[0], rq[1], rq[2], out, chunk_stride);
    else
        sweep_candidates_body<T, kPlaneBytes, 1>(view, entries, floats, cols, rows, ax, ay, az, tx, ty, tz, k, rp, rq,
                                                 out, chunk_stride);
}

// the constants of one reference slot of a uniform batch (kernel parameters)
struct UniformView {
    const FastSweepParams& p;
    int slot;
    __device__ __forceinline__ int chunks() const { return p.chunks; }
    __device__ __forceinline__ int cameras() const { return p.cameras; }
    __device__ __forceinline__ int entry_words() const { return p.entry_words; }
    __device__ __forceinline__ const TorchCam& ref_cam() const { return p.ref_cam[slot]; }
    __device__ __forceinline__ float pose(int c, int j) const { return p.pose[slot][c][j]; }
    __device__ __forceinline__ FastCam cam(int c) const { return p.cam[c]; }
    __device__ __forceinline__ float2 cand2(int k) const { return *reinterpret_cast<const float2*>(&p.cand[k]); }
};

// Block shapes of the sweep (SSG_TUNE_SWEEP_VARIANT): threads per block and blocks per SM, which
// bounds the registers (64, 80, 64, 72)
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
template <>
struct SweepShape<3> {
    static constexpr int threads = 128, blocks = 7;
};

template <typename T, int V>
__global__ void __launch_bounds__(SweepShape<V>::threads, SweepShape<V>::blocks)
    sweep_batch_kernel(const __grid_constant__ FastSweepParams p, const uint4* __restrict__ staged,
                       const float* __restrict__ floats, const int* __restrict__ plane_flags,
                       const int8_t* __restrict__ selected, T* __restrict__ cost, int tiles_x, int tile_w)
{
    const int cols = p.cols, rows = p.rows, pitch = cols + 2;
    const int P = cols * rows;
    int i;
    if (tiles_x > 0) {
        // a block covers tile_w x (threads / tile_w) pixels: the samples of neighbouring rows fall
        // on neighbouring footprints, which the block's warps then share through L1
        const int x = (blockIdx.x % tiles_x) * tile_w + (int)threadIdx.x % tile_w;
        const int y = (blockIdx.x / tiles_x) * (SweepShape<V>::threads / tile_w) + (int)threadIdx.x / tile_w;
        if (x >= cols || y >= rows) return;
        i = y * cols + x;
    } else {
        i = blockIdx.x * blockDim.x + threadIdx.x;  // a block covers consecutive pixels of a row
        if (i >= P) return;
    }
    const int inst = blockIdx.y;  // frame * references + slot
    const int frame = inst / p.references, slot = inst % p.references;
    const int plane = pitch * (rows + 2);
    T* out = cost + (int64_t)inst * p.chunks * P * 8 + (int64_t)i * 8;
    sweep_pixel<T>(UniformView{p, slot}, staged + (int64_t)frame * p.cameras * 2 * plane,
                   floats ? floats + (int64_t)frame * p.cameras * P * 3 : nullptr, plane_flags + frame * p.cameras,
                   plane, p.ref_index[slot], cols, rows, i % cols, i / cols, selected[(int64_t)slot * P + i], out,
                   (int64_t)P * 8);
}

// the constants of one instance of an uneven batch (device memory)
struct InstView {
    const SweepInst* I;
    __device__ __forceinline__ int chunks() const { return I->chunks; }
    __device__ __forceinline__ int cameras() const { return I->cameras; }
    __device__ __forceinline__ int entry_words() const { return I->floats ? 2 : 1; }
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
                    sweep_pixel<T>(InstView{I}, I->staged, I->floats, I->plane_flags, plane, I->ref_camera, cols,
                                   rows, i % cols, i / cols, I->selected[i], out, (int64_t)P * 8);
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
        case 3: launch_sweep_uneven_shape<T, 3>(d_insts, instances, total_tiles, span, d_counter, sms, st); break;
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
static void launch_sweep_shape(const FastSweepParams& p, const uint4* staged, const float* floats, const int* flags,
                               const int8_t* selected, T* cost, int64_t P, int instances, cudaStream_t st)
{
    constexpr int threads = SweepShape<V>::threads;
    const int tile_w = tuning(SSG_TUNE_SWEEP_TILES);  // 0: rows; else the tile width
    if (tile_w > 0) {
        const int th = threads / tile_w;
        const int tiles_x = (p.cols + tile_w - 1) / tile_w, tiles_y = (p.rows + th - 1) / th;
        sweep_batch_kernel<T, V><<<dim3((unsigned)(tiles_x * tiles_y), instances), threads, 0, st>>>(
            p, staged, floats, flags, selected, cost, tiles_x, tile_w);
    } else {
        const dim3 grid(grid_1d(P, threads), instances);
        sweep_batch_kernel<T, V><<<grid, threads, 0, st>>>(p, staged, floats, flags, selected, cost, 0, 0);
    }
}

template <typename T>
static void launch_sweep(const FastSweepParams& p, const uint4* staged, const float* floats, const int* flags,
                         const int8_t* selected, T* cost, int64_t P, int instances, cudaStream_t st)
{
    switch (tuning(SSG_TUNE_SWEEP_VARIANT)) {
        case 1: launch_sweep_shape<T, 1>(p, staged, floats, flags, selected, cost, P, instances, st); break;
        case 2: launch_sweep_shape<T, 2>(p, staged, floats, flags, selected, cost, P, instances, st); break;
        case 3: launch_sweep_shape<T, 3>(p, staged, floats, flags, selected, cost, P, instances, st); break;
        default: launch_sweep_shape<T, 0>(p, staged, floats, flags, selected, cost, P, instances, st); break;
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

// the sweep forms entry offsets in float (exact below 2^24 entries a plane)
static int staged_plane_fits(int cols, int rows)
{
    SSG_REQUIRE(cols > 0 && rows > 0, "resolution must be positive");
    if ((int64_t)(cols + 2) * (rows + 2) >= ((int64_t)1 << 24))
        return fail(SSG_ERR_UNSUPPORTED, "images of %dx%d pixels exceed the batched sweep's 2^24-entry planes", cols,
                    rows);
    return SSG_OK;
}

template <typename Tin>
static int stage_images(const Tin* d_images, int frames, int cameras, int cols, int rows,
                        const int* reference_cameras, int references, float* d_staged, uint8_t* d_guides,
                        int32_t* d_plane_flags, void* stream)
{
    SSG_REQUIRE(d_images && d_staged && d_guides && d_plane_flags && reference_cameras, "null pointer");
    SSG_REQUIRE(frames >= 1 && frames <= 65535 / SSG_MAX_CAMERAS, "frames %d outside [1, %d]", frames,
                65535 / SSG_MAX_CAMERAS);
    SSG_REQUIRE(cameras >= 1 && cameras <= SSG_MAX_CAMERAS && references >= 1 && references <= SSG_MAX_REFERENCES,
                "camera or reference count out of range");
    if (int e = staged_plane_fits(cols, rows)) return e;
    SSG_REQUIRE(((uintptr_t)d_staged & 15) == 0 && ((uintptr_t)d_guides & 3) == 0,
                "staged images must be 16-byte and guides 4-byte aligned");
    SSG_REQUIRE(sizeof(Tin) == 1 || ((uintptr_t)d_staged & 31) == 0,
                "the staged planes of float images (32-byte entries) must be 32-byte aligned");
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
    const cudaError_t e = cudaMemsetAsync(d_plane_flags, 0, sizeof(int32_t) * frames * cameras, as_stream(stream));
    if (e != cudaSuccess) return fail(SSG_ERR_CUDA, "cudaMemsetAsync: %s", cudaGetErrorString(e));
    const int64_t tiles = (int64_t)((cols + 2 + kStageTileX - 1) / kStageTileX) *
                          ((rows + 2 + kStageTileY - 1) / kStageTileY);
    SSG_REQUIRE(tiles < ((int64_t)1 << 31), "images of %dx%d pixels are too large", cols, rows);
    if (tuning(SSG_TUNE_STAGE_COLUMNS) == 1) {
        stage_columns_kernel<Tin><<<column_grid(cols, rows, frames * cameras), kColWarps * 32, 0, as_stream(stream)>>>(
            p, d_images, reinterpret_cast<uint4*>(d_staged), reinterpret_cast<uint32_t*>(d_guides), d_plane_flags);
        return launch_status("stage_columns_kernel");
    }
    dim3 grid((unsigned)tiles, frames * cameras);
    stage_images_kernel<Tin><<<grid, kBatchBlock, 0, as_stream(stream)>>>(
        p, d_images, reinterpret_cast<uint4*>(d_staged), reinterpret_cast<uint32_t*>(d_guides), d_plane_flags);
    return launch_status("stage_images_kernel");
}

// float32 -> uint8 truncation (the reference's float -> uint8 copy of the images to stitch,
// python/depth_estimation.py:239-240): 16 values per thread, four 16-byte loads and one store
template <bool kAligned>
__global__ void __launch_bounds__(kBatchBlock) convert_u8_kernel(const float* __restrict__ src,
                                                                 uint8_t* __restrict__ dst, int64_t n)
{
    const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * 16;
    if (kAligned && i + 16 <= n) {
        uint32_t w[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float4 v = __ldg(reinterpret_cast<const float4*>(src + i) + q);
            w[q] = __float2uint_rz(v.x) | (__float2uint_rz(v.y) << 8) | (__float2uint_rz(v.z) << 16) |
                   (__float2uint_rz(v.w) << 24);
        }
        reinterpret_cast<uint4*>(dst + i)[0] = make_uint4(w[0], w[1], w[2], w[3]);
    } else {
        for (int64_t k = i; k < n; ++k) dst[k] = (uint8_t)__float2uint_rz(src[k]);
    }
}

extern "C" int ssg_convert_u8(const float* d_src, uint8_t* d_dst, int64_t count, void* stream)
{
    SSG_REQUIRE(d_src && d_dst, "null pointer");
    SSG_REQUIRE(count >= 0, "negative count");
    if (count == 0) return SSG_OK;
    const int grid = grid_1d((count + 15) / 16, kBatchBlock);
    if (((uintptr_t)d_src & 15) == 0 && ((uintptr_t)d_dst & 15) == 0)
        convert_u8_kernel<true><<<grid, kBatchBlock, 0, as_stream(stream)>>>(d_src, d_dst, count);
    else
        convert_u8_kernel<false><<<grid, kBatchBlock, 0, as_stream(stream)>>>(d_src, d_dst, count);
    return launch_status("convert_u8_kernel");
}

extern "C" int ssg_stage_images(const float* d_images, int frames, int cameras, int cols, int rows,
                                const int* reference_cameras, int references, float* d_staged, uint8_t* d_guides,
                                int32_t* d_plane_flags, void* stream)
{
    return stage_images(d_images, frames, cameras, cols, rows, reference_cameras, references, d_staged, d_guides,
                        d_plane_flags, stream);
}

extern "C" int ssg_stage_images_u8(const uint8_t* d_images, int frames, int cameras, int cols, int rows,
                                   const int* reference_cameras, int references, float* d_staged, uint8_t* d_guides,
                                   int32_t* d_plane_flags, void* stream)
{
    return stage_images(d_images, frames, cameras, cols, rows, reference_cameras, references, d_staged, d_guides,
                        d_plane_flags, stream);
}

extern "C" int ssg_stage_images_resized(const uint8_t* d_images, int src_cols, int src_rows, int frames,
                                        int cameras, int cols, int rows, const int* reference_cameras,
                                        int references, float* d_staged, uint8_t* d_guides, int32_t* d_plane_flags,
                                        void* stream)
{
    SSG_REQUIRE(d_images && d_staged && d_guides && d_plane_flags && reference_cameras, "null pointer");
    SSG_REQUIRE(src_cols >= 1 && src_rows >= 1, "empty source images");
    SSG_REQUIRE(frames >= 1 && frames <= 65535 / SSG_MAX_CAMERAS, "frames %d outside [1, %d]", frames,
                65535 / SSG_MAX_CAMERAS);
    SSG_REQUIRE(cameras >= 1 && cameras <= SSG_MAX_CAMERAS && references >= 1 && references <= SSG_MAX_REFERENCES,
                "camera or reference count out of range");
    if (int e = staged_plane_fits(cols, rows)) return e;
    SSG_REQUIRE(((uintptr_t)d_staged & 31) == 0 && ((uintptr_t)d_guides & 3) == 0,
                "staged planes must be 32-byte and guides 4-byte aligned");
    if (((uintptr_t)d_images & 3) != 0 || ((int64_t)src_cols * src_rows) % 4 != 0)
        return fail(SSG_ERR_UNSUPPORTED,
                    "source images must start on 4-byte boundaries with a pixel count divisible by 4 (%dx%d): "
                    "resize with ssg_resize_linear and stage the result",
                    src_cols, src_rows);
    SSG_REQUIRE((int64_t)src_cols * src_rows * 3 < ((int64_t)1 << 40), "source images too large");
    const ResizeParams rp = make_resize_params(src_cols, src_rows, cols, rows, 3);
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
    if (tuning(SSG_TUNE_STAGE_COLUMNS) == 1) {
        const cudaError_t e = cudaMemsetAsync(d_plane_flags, 0, sizeof(int32_t) * frames * cameras, as_stream(stream));
        if (e != cudaSuccess) return fail(SSG_ERR_CUDA, "cudaMemsetAsync: %s", cudaGetErrorString(e));
        stage_resized_columns_kernel<<<column_grid(cols, rows, frames * cameras), kColWarps * 32, 0,
                                       as_stream(stream)>>>(p, rp, d_images, reinterpret_cast<uint4*>(d_staged),
                                                            reinterpret_cast<uint32_t*>(d_guides), d_plane_flags);
        return launch_status("stage_resized_columns_kernel");
    }
    // the largest source window of any tile: texel columns [i0 - 1, i0 + kStageTileX - 1] and
    // rows [j0 - 1, j0 + kStageTileY - 1] clamped into the image, taps as the kernel forms them
    int win_cols = 0, win_rows = 0;
    for (int i0 = 0; i0 < cols + 2; i0 += kStageTileX) {
        const int a = std::min(std::max(i0 - 1, 0), cols - 1), b = std::min(i0 + kStageTileX - 1, cols - 1);
        win_cols = std::max(win_cols, column_tap(rp, b).s1 - column_tap(rp, a).s0 + 1);
    }
    for (int j0 = 0; j0 < rows + 2; j0 += kStageTileY) {
        const int a = std::min(std::max(j0 - 1, 0), rows - 1), b = std::min(j0 + kStageTileY - 1, rows - 1);
        win_rows = std::max(win_rows, row_tap(rp, b).s1 - row_tap(rp, a).s0 + 1);
    }
    // a window row starts at byte offset 0..3 of its first word: ceil((3 + 3 cols) / 4) words
    const int row_floats = 4 * ((3 * win_cols + 6) / 4 + 1);
    const int64_t smem = (int64_t)win_rows * row_floats * (int64_t)sizeof(float);
    constexpr int64_t kMaxWindow = 160 * 1024;
    if (smem > kMaxWindow)
        return fail(SSG_ERR_UNSUPPORTED,
                    "a tile's source window (%d x %d texels) exceeds %lld bytes of shared memory: resize with "
                    "ssg_resize_linear and stage the result",
                    win_cols, win_rows, (long long)kMaxWindow);
    if (smem > 48 * 1024) {
        // above the default limit the kernel opts in, once per device and size
        static std::atomic<int64_t> opted[64];
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return fail(SSG_ERR_CUDA, "cudaGetDevice");
        if (opted[dev].load() < smem) {
            const cudaError_t e =
                cudaFuncSetAttribute(stage_resized_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return fail(SSG_ERR_CUDA, "cudaFuncSetAttribute: %s", cudaGetErrorString(e));
            opted[dev].store(smem);
        }
    }
    const cudaError_t e = cudaMemsetAsync(d_plane_flags, 0, sizeof(int32_t) * frames * cameras, as_stream(stream));
    if (e != cudaSuccess) return fail(SSG_ERR_CUDA, "cudaMemsetAsync: %s", cudaGetErrorString(e));
    const int64_t tiles = (int64_t)((cols + 2 + kStageTileX - 1) / kStageTileX) *
                          ((rows + 2 + kStageTileY - 1) / kStageTileY);
    SSG_REQUIRE(tiles < ((int64_t)1 << 31), "images of %dx%d pixels are too large", cols, rows);
    stage_resized_kernel<<<dim3((unsigned)tiles, frames * cameras), kBatchBlock, (size_t)smem, as_stream(stream)>>>(
        p, rp, d_images, row_floats, reinterpret_cast<uint4*>(d_staged), reinterpret_cast<uint32_t*>(d_guides),
        d_plane_flags);
    return launch_status("stage_resized_kernel");
}

extern "C" int ssg_sweep_cost_batch(int cols, int rows, int frames, int camera_count, const ssg_camera* cameras,
                                    int references, const int* reference_cameras, const float* relative_poses,
                                    const float* d_staged, const float* d_images, const int32_t* d_plane_flags,
                                    const int8_t* d_selected, const float* candidates, int candidate_count,
                                    int storage, void* d_cost, void* stream)
{
    return ssg_sweep_cost_batch_entries(cols, rows, frames, camera_count, cameras, references, reference_cameras,
                                        relative_poses, d_staged, d_images ? 32 : 16, d_images, d_plane_flags,
                                        d_selected, candidates, candidate_count, storage, d_cost, stream);
}

extern "C" int ssg_sweep_cost_batch_entries(int cols, int rows, int frames, int camera_count,
                                            const ssg_camera* cameras, int references, const int* reference_cameras,
                                            const float* relative_poses, const float* d_staged, int entry_bytes,
                                            const float* d_images, const int32_t* d_plane_flags,
                                            const int8_t* d_selected, const float* candidates, int candidate_count,
                                            int storage, void* d_cost, void* stream)
{
    if (int e = staged_plane_fits(cols, rows)) return e;
    SSG_REQUIRE(entry_bytes == 16 || entry_bytes == 32, "entry_bytes %d is neither 16 nor 32", entry_bytes);
    SSG_REQUIRE(!d_images || entry_bytes == 32, "float images are staged in 32-byte entries");
    SSG_REQUIRE(cameras && reference_cameras && relative_poses && d_staged && d_plane_flags && d_selected &&
                    candidates && d_cost,
                "null pointer");
    SSG_REQUIRE(camera_count >= 1 && camera_count <= SSG_MAX_CAMERAS, "camera_count out of range");
    SSG_REQUIRE(references >= 1 && references <= SSG_MAX_REFERENCES, "references out of range");
    SSG_REQUIRE(frames >= 1 && frames * references <= 65535, "frames out of range");
    SSG_REQUIRE(candidate_count >= 1 && candidate_count <= SSG_MAX_CANDIDATES, "candidate_count %d outside [1, %d]",
                candidate_count, SSG_MAX_CANDIDATES);
    SSG_REQUIRE(((uintptr_t)d_staged & 15) == 0 && ((uintptr_t)d_cost & 15) == 0, "buffers must be 16-byte aligned");
    SSG_REQUIRE(entry_bytes == 16 || ((uintptr_t)d_staged & 31) == 0,
                "staged planes of 32-byte entries must be 32-byte aligned");
    if (int e = check_storage(storage)) return e;
    FastSweepParams p{};
    p.cols = cols;
    p.rows = rows;
    p.entry_words = entry_bytes / 16;
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
        launch_sweep<__half>(p, staged, d_images, d_plane_flags, d_selected, static_cast<__half*>(d_cost), P,
                             frames * references, as_stream(stream));
    else
        launch_sweep<uint16_t>(p, staged, d_images, d_plane_flags, d_selected, static_cast<uint16_t*>(d_cost), P,
                               frames * references, as_stream(stream));
    return launch_status("sweep_batch_kernel");
}
