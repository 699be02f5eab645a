// Evaluation of RGB-D panoramas against ground truth (python/utils.py:206-250): PSNR and SSIM of
// the colour panorama, MAE, RMSE and bad-pixel ratios of the inverse-distance panorama, for a
// batch of frames, as device reductions.
//
// The metrics follow scikit-image's published definitions as the reference calls them
// (structural_similarity(gt, est, multichannel=True) and peak_signal_noise_ratio(gt, est) on
// float32 images in [0, 1]) and numpy's element-wise arithmetic:
//   - colour values x = u8 / 255 in float32;
//   - PSNR: mse = mean over all values of the float32 square of the float32 difference, summed in
//     float64; psnr = 10 log10(1 / mse) (data range 1: float images with no negative value);
//   - SSIM per channel on float64 values: 7x7 uniform windows, sample covariances (49 / 48),
//     data range 2 (the float dtype's range -1..1), C1 = (0.01 * 2)^2, C2 = (0.03 * 2)^2, the
//     map cropped by 3 pixels on each side and averaged; the mean over the 3 channels;
//   - err = |est - gt| in float32; MAE = sum(err) / n, RMSE = sqrt(sum(err * err) / n) with the
//     float32 products summed in float64; bad-pixel ratio = 100 * count(err > t) / n, t rounded to
//     float32 as numpy compares a float32 array with a Python float.
// Sums are taken per block in a fixed order and reduced in a fixed order, so results do not
// depend on scheduling.
#include "ssg_common.cuh"

namespace ssg {

constexpr int kEvalBlocks = 304;  // blocks per frame: two per SM
constexpr int kEvalThreads = 256;
constexpr int kSsimTileX = 32, kSsimTileY = 8, kSsimWin = 7, kSsimHalf = 3;
constexpr int kSsimInX = kSsimTileX + kSsimWin - 1, kSsimInY = kSsimTileY + kSsimWin - 1;

struct EvalParams {
    int cols, rows, frames, thresholds;
    float threshold[SSG_EVAL_MAX_THRESHOLDS];
};

// slots of a block's partial sums
enum { kSlotSq = 0, kSlotErr = 1, kSlotErr2 = 2, kSlotSsim = 3, kSlotBad = 4 };

__device__ __forceinline__ int eval_slots(const EvalParams& p) { return kSlotBad + p.thresholds; }

// fixed-order sum of one value per thread of the block (thread 0 returns it)
__device__ __forceinline__ double block_sum(double v, double* sh)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();  // sh is free
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[w];
    return s;
}

__device__ __forceinline__ float unit_value(uint8_t v) { return __fdiv_rn((float)v, 255.0f); }

// Per-pixel sums: squared colour differences, inverse-distance errors and bad-pixel counts.
// blockIdx.y: frame.
__global__ void __launch_bounds__(kEvalThreads) eval_pointwise_kernel(const __grid_constant__ EvalParams p,
                                                                      const uint8_t* __restrict__ rgb,
                                                                      const uint8_t* __restrict__ gt_rgb,
                                                                      const float* __restrict__ inv,
                                                                      const float* __restrict__ gt_inv,
                                                                      double* __restrict__ partials)
{
    __shared__ double sh[kEvalThreads / 32];
    const int64_t n = (int64_t)p.cols * p.rows;
    const int frame = blockIdx.y;
    rgb += (int64_t)frame * n * 3;
    gt_rgb += (int64_t)frame * n * 3;
    inv += (int64_t)frame * n;
    gt_inv += (int64_t)frame * n;
    double sq = 0.0, err = 0.0, err2 = 0.0;
    double bad[SSG_EVAL_MAX_THRESHOLDS];
#pragma unroll
    for (int k = 0; k < SSG_EVAL_MAX_THRESHOLDS; ++k) bad[k] = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) {
            const float d = __fsub_rn(unit_value(__ldg(gt_rgb + i * 3 + ch)), unit_value(__ldg(rgb + i * 3 + ch)));
            sq += (double)__fmul_rn(d, d);
        }
        const float e = fabsf(__fsub_rn(__ldg(inv + i), __ldg(gt_inv + i)));
        err += (double)e;
        err2 += (double)__fmul_rn(e, e);
#pragma unroll
        for (int k = 0; k < SSG_EVAL_MAX_THRESHOLDS; ++k)
            if (k < p.thresholds && e > p.threshold[k]) bad[k] += 1.0;
    }
    double* out = partials + ((int64_t)frame * gridDim.x + blockIdx.x) * eval_slots(p);
    double s = block_sum(sq, sh);
    if (threadIdx.x == 0) out[kSlotSq] = s;
    s = block_sum(err, sh);
    if (threadIdx.x == 0) out[kSlotErr] = s;
    s = block_sum(err2, sh);
    if (threadIdx.x == 0) out[kSlotErr2] = s;
#pragma unroll
    for (int k = 0; k < SSG_EVAL_MAX_THRESHOLDS; ++k) {
        if (k >= p.thresholds) break;
        s = block_sum(bad[k], sh);
        if (threadIdx.x == 0) out[kSlotBad + k] = s;
    }
}

// SSIM map sums over the cropped region [3, rows - 3) x [3, cols - 3), all three channels:
// tiles of kSsimTileX x kSsimTileY map pixels, each with its 6-pixel halo staged in shared memory
// and the five window sums formed by rows, then by columns.  blockIdx.y: frame.
__global__ void __launch_bounds__(kEvalThreads) eval_ssim_kernel(const __grid_constant__ EvalParams p,
                                                                 const uint8_t* __restrict__ rgb,
                                                                 const uint8_t* __restrict__ gt_rgb,
                                                                 double* __restrict__ partials)
{
    __shared__ double sx[kSsimInY][kSsimInX], sy[kSsimInY][kSsimInX];
    __shared__ double hs[5][kSsimInY][kSsimTileX];  // row sums of x, y, xx, yy, xy
    __shared__ double sh[kEvalThreads / 32];
    const int64_t n = (int64_t)p.cols * p.rows;
    const int frame = blockIdx.y;
    rgb += (int64_t)frame * n * 3;
    gt_rgb += (int64_t)frame * n * 3;
    const int out_cols = p.cols - 2 * kSsimHalf, out_rows = p.rows - 2 * kSsimHalf;
    const int tiles_x = (out_cols + kSsimTileX - 1) / kSsimTileX;
    const int tiles = tiles_x * ((out_rows + kSsimTileY - 1) / kSsimTileY);
    constexpr double kNp = kSsimWin * kSsimWin, kCovNorm = kNp / (kNp - 1.0);
    constexpr double kC1 = (0.01 * 2.0) * (0.01 * 2.0), kC2 = (0.03 * 2.0) * (0.03 * 2.0);
    const int tx = threadIdx.x % kSsimTileX, ty = threadIdx.x / kSsimTileX;
    double acc = 0.0;
    for (int t = blockIdx.x; t < tiles; t += gridDim.x) {
        // map pixel (x, y) is image pixel (x + 3, y + 3); its window covers image x .. x + 6
        const int x0 = (t % tiles_x) * kSsimTileX, y0 = (t / tiles_x) * kSsimTileY;
        for (int ch = 0; ch < 3; ++ch) {
            __syncthreads();  // the previous tile's sums are consumed
            for (int q = threadIdx.x; q < kSsimInX * kSsimInY; q += blockDim.x) {
                const int lx = q % kSsimInX, ly = q / kSsimInX;
                const int x = min(x0 + lx, p.cols - 1), y = min(y0 + ly, p.rows - 1);
                const int64_t o = ((int64_t)y * p.cols + x) * 3 + ch;
                sx[ly][lx] = (double)unit_value(__ldg(gt_rgb + o));
                sy[ly][lx] = (double)unit_value(__ldg(rgb + o));
            }
            __syncthreads();
            for (int q = threadIdx.x; q < kSsimInY * kSsimTileX; q += blockDim.x) {
                const int lx = q % kSsimTileX, ly = q / kSsimTileX;
                double a = 0.0, b = 0.0, aa = 0.0, bb = 0.0, ab = 0.0;
#pragma unroll
                for (int k = 0; k < kSsimWin; ++k) {
                    const double u = sx[ly][lx + k], v = sy[ly][lx + k];
                    a += u;
                    b += v;
                    aa += u * u;
                    bb += v * v;
                    ab += u * v;
                }
                hs[0][ly][lx] = a;
                hs[1][ly][lx] = b;
                hs[2][ly][lx] = aa;
                hs[3][ly][lx] = bb;
                hs[4][ly][lx] = ab;
            }
            __syncthreads();
            if (x0 + tx < out_cols && y0 + ty < out_rows) {
                double m[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
#pragma unroll
                for (int k = 0; k < kSsimWin; ++k)
#pragma unroll
                    for (int j = 0; j < 5; ++j) m[j] += hs[j][ty + k][tx];
#pragma unroll
                for (int j = 0; j < 5; ++j) m[j] /= kNp;
                const double ux = m[0], uy = m[1];
                const double vx = kCovNorm * (m[2] - ux * ux), vy = kCovNorm * (m[3] - uy * uy);
                const double vxy = kCovNorm * (m[4] - ux * uy);
                const double a1 = 2.0 * ux * uy + kC1, a2 = 2.0 * vxy + kC2;
                const double b1 = ux * ux + uy * uy + kC1, b2 = vx + vy + kC2;
                acc += (a1 * a2) / (b1 * b2);
            }
        }
    }
    const double s = block_sum(acc, sh);
    if (threadIdx.x == 0) partials[((int64_t)frame * gridDim.x + blockIdx.x) * eval_slots(p) + kSlotSsim] = s;
}

// One block per frame: the blocks' partial sums in block order, then the metrics.
__global__ void __launch_bounds__(kEvalThreads) eval_finish_kernel(const __grid_constant__ EvalParams p, int blocks,
                                                                   const double* __restrict__ partials,
                                                                   double* __restrict__ out)
{
    __shared__ double sh[kEvalThreads / 32];
    const int frame = blockIdx.x, slots = eval_slots(p);
    const double n = (double)p.cols * p.rows;
    const double map_n = (double)(p.cols - 2 * kSsimHalf) * (p.rows - 2 * kSsimHalf);
    double* o = out + (int64_t)frame * (SSG_EVAL_FIXED_METRICS + p.thresholds);
    for (int slot = 0; slot < slots; ++slot) {
        double v = 0.0;
        for (int b = threadIdx.x; b < blocks; b += blockDim.x) v += partials[((int64_t)frame * blocks + b) * slots + slot];
        const double s = block_sum(v, sh);
        if (threadIdx.x == 0) {
            if (slot == kSlotSq) o[0] = 10.0 * log10(1.0 / (s / (3.0 * n)));
            else if (slot == kSlotSsim) o[1] = s / (3.0 * map_n);
            else if (slot == kSlotErr) o[2] = s / n;
            else if (slot == kSlotErr2) o[3] = sqrt(s / n);
            else o[SSG_EVAL_FIXED_METRICS + slot - kSlotBad] = 100.0 * s / n;
        }
    }
}

}  // namespace ssg

using namespace ssg;

extern "C" size_t ssg_eval_scratch_bytes(int frames, int threshold_count)
{
    if (frames < 1 || threshold_count < 0 || threshold_count > SSG_EVAL_MAX_THRESHOLDS) return 0;
    return sizeof(double) * (size_t)frames * kEvalBlocks * (kSlotBad + threshold_count);
}

extern "C" int ssg_eval_panoramas(int cols, int rows, int frames, const uint8_t* d_rgb, const uint8_t* d_gt_rgb,
                                  const float* d_inv_distance, const float* d_gt_inv_distance, const float* thresholds,
                                  int threshold_count, void* d_scratch, double* d_metrics, void* stream)
{
    SSG_REQUIRE(d_rgb && d_gt_rgb && d_inv_distance && d_gt_inv_distance && d_scratch && d_metrics, "null pointer");
    SSG_REQUIRE(cols >= 2 * kSsimHalf + 1 && rows >= 2 * kSsimHalf + 1,
                "panoramas of %dx%d are smaller than the 7x7 SSIM window", cols, rows);
    SSG_REQUIRE((int64_t)cols * rows * 3 < ((int64_t)1 << 40), "panoramas of %dx%d are too large", cols, rows);
    SSG_REQUIRE(frames >= 1 && frames <= 65535, "frames %d outside [1, 65535]", frames);
    SSG_REQUIRE(threshold_count >= 0 && threshold_count <= SSG_EVAL_MAX_THRESHOLDS,
                "threshold_count %d outside [0, %d]", threshold_count, SSG_EVAL_MAX_THRESHOLDS);
    SSG_REQUIRE(threshold_count == 0 || thresholds, "null thresholds");
    SSG_REQUIRE(((uintptr_t)d_scratch & 7) == 0 && ((uintptr_t)d_metrics & 7) == 0,
                "scratch and metrics must be 8-byte aligned");
    EvalParams p{};
    p.cols = cols;
    p.rows = rows;
    p.frames = frames;
    p.thresholds = threshold_count;
    for (int k = 0; k < threshold_count; ++k) p.threshold[k] = thresholds[k];
    cudaStream_t st = as_stream(stream);
    double* partials = static_cast<double*>(d_scratch);
    const dim3 grid(kEvalBlocks, frames);
    eval_pointwise_kernel<<<grid, kEvalThreads, 0, st>>>(p, d_rgb, d_gt_rgb, d_inv_distance, d_gt_inv_distance,
                                                         partials);
    if (int e = launch_status("eval_pointwise_kernel")) return e;
    eval_ssim_kernel<<<grid, kEvalThreads, 0, st>>>(p, d_rgb, d_gt_rgb, partials);
    if (int e = launch_status("eval_ssim_kernel")) return e;
    eval_finish_kernel<<<frames, kEvalThreads, 0, st>>>(p, kEvalBlocks, partials, d_metrics);
    return launch_status("eval_finish_kernel");
}
