// Input preparation on the GPU: the linear resize the reference applies to every decoded image
// before the estimator (python/utils.py:198-201, cv2.resize(image, size, cv2.INTER_AREA) -- the
// third positional argument of cv2.resize is `dst`, so the interpolation in effect is the
// default, INTER_LINEAR).
//
// The taps are ssg_resize.cuh's.  Arithmetic:
//   - float pixels: h = S[sx] * (1 - fx) + S[sx + 1] * fx per row, then h0 * (1 - fy) + h1 * fy,
//     each product and sum rounded separately;
//   - uint8 pixels to uint8 (the ground-truth resize of the evaluation): 11-bit fixed-point
//     weights w0 = round(2048 (1 - f)) (saturated), w1 = 2048 - w0, integer sums, result
//     (v + 2^21) >> 22;
//   - an exact 2x reduction on both axes is an area average (OpenCV switches to INTER_AREA
//     there): floats (a + b + c + d) * 0.25, bytes (a + b + c + d + 2) >> 2.
// cv2 is not available here, so these statements are not pinned against OpenCV's own outputs.
#include <cmath>

#include "ssg_common.cuh"
#include "ssg_resize.cuh"

namespace ssg {

__device__ __forceinline__ float in_value(const float* s, int64_t i) { return __ldg(s + i); }
__device__ __forceinline__ float in_value(const uint8_t* s, int64_t i) { return (float)__ldg(s + i); }

__device__ __forceinline__ int fixed_weight(float f)
{
    const float w = __fmul_rn(__fsub_rn(1.0f, f), 2048.0f);
    return min(max(__float2int_rn(w), -32768), 32767);
}

// One block per kTileX x kTileY destination pixels of one image (blockIdx.z): the tile's column
// and row taps are formed once (in double, as OpenCV forms its tables) into shared memory, then
// one thread per destination pixel (all channels) blends.
constexpr int kTileX = 32, kTileY = 8;

template <typename Tin, typename Tout>
__global__ void __launch_bounds__(kTileX * kTileY) resize_linear_kernel(const __grid_constant__ ResizeParams p,
                                                                        const Tin* __restrict__ src,
                                                                        Tout* __restrict__ dst)
{
    __shared__ Tap cols_tap[kTileX], rows_tap[kTileY];
    const int x0 = blockIdx.x * kTileX, y0 = blockIdx.y * kTileY;
    const int C = p.channels;
    src += (int64_t)blockIdx.z * p.src_cols * p.src_rows * C;
    dst += (int64_t)blockIdx.z * p.dst_cols * p.dst_rows * C;
    if (!p.area2) {
        if (threadIdx.x < kTileX) cols_tap[threadIdx.x] = column_tap(p, min(x0 + (int)threadIdx.x, p.dst_cols - 1));
        else if (threadIdx.x < kTileX + kTileY)
            rows_tap[threadIdx.x - kTileX] = row_tap(p, min(y0 + (int)threadIdx.x - kTileX, p.dst_rows - 1));
        __syncthreads();
    }
    const int dx = x0 + (int)(threadIdx.x % kTileX), dy = y0 + (int)(threadIdx.x / kTileX);
    if (dx >= p.dst_cols || dy >= p.dst_rows) return;
    dst += ((int64_t)dy * p.dst_cols + dx) * C;
    if (p.area2) {
        const int64_t r0 = (int64_t)(2 * dy) * p.src_cols, r1 = r0 + p.src_cols;
        for (int c = 0; c < C; ++c) {
            const int64_t a = (r0 + 2 * dx) * C + c, b = a + C, d0 = (r1 + 2 * dx) * C + c, d1 = d0 + C;
            if constexpr (sizeof(Tout) == 1) {
                const int s = (int)__ldg(src + a) + __ldg(src + b) + __ldg(src + d0) + __ldg(src + d1);
                dst[c] = (Tout)((s + 2) >> 2);
            } else {
                const float s = __fadd_rn(__fadd_rn(__fadd_rn(in_value(src, a), in_value(src, b)), in_value(src, d0)),
                                          in_value(src, d1));
                dst[c] = __fmul_rn(s, 0.25f);
            }
        }
        return;
    }
    const Tap tx = cols_tap[threadIdx.x % kTileX], ty = rows_tap[threadIdx.x / kTileX];
    const int64_t r0 = (int64_t)ty.s0 * p.src_cols, r1 = (int64_t)ty.s1 * p.src_cols;
    if constexpr (sizeof(Tout) == 1) {
        const int a0 = fixed_weight(tx.f), a1 = 2048 - a0, b0 = fixed_weight(ty.f), b1 = 2048 - b0;
        for (int c = 0; c < C; ++c) {
            const int h0 = (int)__ldg(src + (r0 + tx.s0) * C + c) * a0 + (int)__ldg(src + (r0 + tx.s1) * C + c) * a1;
            const int h1 = (int)__ldg(src + (r1 + tx.s0) * C + c) * a0 + (int)__ldg(src + (r1 + tx.s1) * C + c) * a1;
            const int v = (h0 * b0 + h1 * b1 + (1 << 21)) >> 22;
            dst[c] = (Tout)min(max(v, 0), 255);
        }
    } else {
        const float a0 = __fsub_rn(1.0f, tx.f), a1 = tx.f, b0 = __fsub_rn(1.0f, ty.f), b1 = ty.f;
        for (int c = 0; c < C; ++c) {
            const float h0 = __fadd_rn(__fmul_rn(in_value(src, (r0 + tx.s0) * C + c), a0),
                                       __fmul_rn(in_value(src, (r0 + tx.s1) * C + c), a1));
            const float h1 = __fadd_rn(__fmul_rn(in_value(src, (r1 + tx.s0) * C + c), a0),
                                       __fmul_rn(in_value(src, (r1 + tx.s1) * C + c), a1));
            dst[c] = __fadd_rn(__fmul_rn(h0, b0), __fmul_rn(h1, b1));
        }
    }
}

}  // namespace ssg

using namespace ssg;

extern "C" int ssg_resize_linear(const void* d_src, int src_type, int src_cols, int src_rows, int channels,
                                 void* d_dst, int dst_type, int dst_cols, int dst_rows, int images, void* stream)
{
    SSG_REQUIRE(d_src && d_dst, "null pointer");
    SSG_REQUIRE(src_cols >= 1 && src_rows >= 1 && dst_cols >= 1 && dst_rows >= 1, "empty image");
    SSG_REQUIRE(channels >= 1 && channels <= 4, "channels %d outside [1, 4]", channels);
    SSG_REQUIRE(images >= 1 && images <= 65535, "images %d outside [1, 65535]", images);
    SSG_REQUIRE((int64_t)src_cols * src_rows * channels < ((int64_t)1 << 40) &&
                    (int64_t)dst_cols * dst_rows < ((int64_t)1 << 31) * 256,
                "images too large");
    SSG_REQUIRE((src_type == SSG_PIXEL_U8 || src_type == SSG_PIXEL_F32) &&
                    (dst_type == SSG_PIXEL_F32 || (dst_type == SSG_PIXEL_U8 && src_type == SSG_PIXEL_U8)),
                "unsupported pixel types %d -> %d (u8 -> f32, f32 -> f32, u8 -> u8)", src_type, dst_type);
    const ResizeParams p = make_resize_params(src_cols, src_rows, dst_cols, dst_rows, channels);
    const dim3 grid((unsigned)((dst_cols + kTileX - 1) / kTileX), (unsigned)((dst_rows + kTileY - 1) / kTileY),
                    (unsigned)images);
    SSG_REQUIRE(grid.y <= 65535, "destination of %d rows is too tall", dst_rows);
    cudaStream_t st = as_stream(stream);
    constexpr int kThreads = kTileX * kTileY;
    if (src_type == SSG_PIXEL_F32)
        resize_linear_kernel<float, float>
            <<<grid, kThreads, 0, st>>>(p, static_cast<const float*>(d_src), static_cast<float*>(d_dst));
    else if (dst_type == SSG_PIXEL_F32)
        resize_linear_kernel<uint8_t, float>
            <<<grid, kThreads, 0, st>>>(p, static_cast<const uint8_t*>(d_src), static_cast<float*>(d_dst));
    else
        resize_linear_kernel<uint8_t, uint8_t>
            <<<grid, kThreads, 0, st>>>(p, static_cast<const uint8_t*>(d_src), static_cast<uint8_t*>(d_dst));
    return launch_status("resize_linear_kernel");
}
