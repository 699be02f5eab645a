// The linear resize's source taps (python/utils.py:198-201: cv2.resize, INTER_LINEAR in effect),
// shared by the resize kernel (ssg_prep.cu) and the staging that resizes while it stages
// (ssg_sweep_batch.cu), so that both form the same taps and weights.
//
// Restated from OpenCV's published linear resize:
//   - source coordinate of destination column dx: fx = float((dx + 0.5) * scale_x - 0.5) in
//     double, scale_x = 1 / (dst_cols / src_cols); sx = floor(fx), fx -= sx; sx < 0 gives
//     (sx, fx) = (0, 0) and sx >= src_cols - 1 gives (src_cols - 1, 0) (the second tap then has
//     weight 0); rows the same way, except that the row weights are kept and the rows clamped to
//     [0, src_rows - 1];
//   - an exact 2x reduction on both axes is an area average (taps 2 d and 2 d + 1).
#pragma once

#include <cmath>

namespace ssg {

struct ResizeParams {
    int src_cols, src_rows, dst_cols, dst_rows, channels;
    double scale_x, scale_y;
    int area2;  // exact 2x reduction on both axes
};

inline ResizeParams make_resize_params(int src_cols, int src_rows, int dst_cols, int dst_rows, int channels)
{
    ResizeParams p{};
    p.src_cols = src_cols;
    p.src_rows = src_rows;
    p.dst_cols = dst_cols;
    p.dst_rows = dst_rows;
    p.channels = channels;
    p.scale_x = 1.0 / ((double)dst_cols / src_cols);
    p.scale_y = 1.0 / ((double)dst_rows / src_rows);
    p.area2 = src_cols == 2 * dst_cols && src_rows == 2 * dst_rows;
    return p;
}

struct Tap {
    int s0, s1;
    float f;  // weight of s1
};

__host__ __device__ __forceinline__ Tap column_tap(const ResizeParams& p, int dx)
{
    if (p.area2) return Tap{2 * dx, 2 * dx + 1, 0.5f};
    float fx = (float)((dx + 0.5) * p.scale_x - 0.5);
    int sx = (int)floorf(fx);
    fx -= (float)sx;
    if (sx < 0) fx = 0.0f, sx = 0;
    if (sx >= p.src_cols - 1) fx = 0.0f, sx = p.src_cols - 1;
    return Tap{sx, sx + 1 < p.src_cols ? sx + 1 : p.src_cols - 1, fx};
}

__host__ __device__ __forceinline__ Tap row_tap(const ResizeParams& p, int dy)
{
    if (p.area2) return Tap{2 * dy, 2 * dy + 1, 0.5f};
    float fy = (float)((dy + 0.5) * p.scale_y - 0.5);
    const int sy = (int)floorf(fy);
    fy -= (float)sy;
    const int last = p.src_rows - 1;
    const int s0 = sy < 0 ? 0 : (sy > last ? last : sy), s1 = sy + 1 < 0 ? 0 : (sy + 1 > last ? last : sy + 1);
    return Tap{s0, s1, fy};
}

}  // namespace ssg
