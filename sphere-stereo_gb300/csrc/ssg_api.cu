// Library-wide plumbing of the C ABI: per-thread error messages, version, limits, and the
// host-side derivation of the torch-form camera constants.
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "ssg_common.cuh"

namespace ssg {

static thread_local char g_error[512] = "";

void clear_error() { g_error[0] = '\0'; }

int fail(int code, const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_error, sizeof(g_error), fmt, ap);
    va_end(ap);
    return code;
}

int launch_status(const char* what)
{
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(SSG_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return SSG_OK;
}

TorchCam make_torch_cam(const ssg_camera& c)
{
    // python/utils.py:57-94: Python-float expressions of xi and alpha are evaluated in double and
    // rounded to float32 when they meet a float32 tensor.
    const double xi = c.xi, al = c.alpha;
    TorchCam k;
    k.fx = c.fx;
    k.fy = c.fy;
    k.cx = c.cx;
    k.cy = c.cy;
    k.xi = (float)xi;
    k.alpha = (float)al;
    k.alpha2 = (float)(al * al);
    k.k1 = (float)(2 * al - 1);
    k.one_minus_xi2 = (float)(1 - xi * xi);
    k.one_minus_alpha = (float)(1 - al);
    const double w1 = al > 0.5 ? (1 - al) / al : al / (1 - al);
    const double w2 = (w1 + xi) / std::sqrt(2 * w1 * xi + xi * xi + 1);
    k.minus_w2 = (float)(-w2);
    return k;
}

// ---------------------------------------------------------------------------------------------
// Launch-shape knobs (chosen by the Python autotuner): process-wide, read when a launch is
// enqueued, so a CUDA graph keeps the values it was captured with.
// ---------------------------------------------------------------------------------------------
namespace {
struct Knob {
    const int* values;
    int count;
    std::atomic<int> value;
};
constexpr int kOnOff[] = {0, 1};
constexpr int kSweepVariants[] = {0, 1, 2, 3};
constexpr int kHoleBlocks[] = {2, 4, 8};
constexpr int kMergeFramesValues[] = {2, 4, 8};
constexpr int kUnevenSpans[] = {1, 2, 4};
constexpr int kIsbUpBlocks[] = {2, 3};
constexpr int kSweepTiles[] = {0, 16, 32};
constexpr int kHoleTail[] = {0, 3, 4, 6, 8};
constexpr int kIsbTail[] = {0, 256, 1024, 4096};
constexpr int kPostTail[] = {0, 1024, 4096, 16384};
Knob g_knobs[] = {
    {kSweepVariants, 4, {0}},      // SSG_TUNE_SWEEP_VARIANT
    {kHoleBlocks, 3, {4}},         // SSG_TUNE_HOLE_BLOCKS_PER_SM
    {kMergeFramesValues, 3, {4}},  // SSG_TUNE_MERGE_FRAMES
    {kUnevenSpans, 3, {1}},        // SSG_TUNE_UNEVEN_SPAN
    {kIsbUpBlocks, 2, {2}},        // SSG_TUNE_ISB_UP_BLOCKS
    {kIsbUpBlocks, 2, {2}},        // SSG_TUNE_ISB_SELECT_BLOCKS
    {kOnOff, 2, {0}},              // SSG_TUNE_ISB_TILE_TMA
    {kOnOff, 2, {0}},              // SSG_TUNE_TMA_WITHHOLD
    {kOnOff, 2, {0}},              // SSG_TUNE_HOLE_PERSISTENT
    {kSweepTiles, 3, {16}},        // SSG_TUNE_SWEEP_TILES
    {kHoleTail, 5, {8}},           // SSG_TUNE_HOLE_TAIL
    {kOnOff, 2, {1}},              // SSG_TUNE_SELECT_WHOLE
    {kOnOff, 2, {0}},              // SSG_TUNE_UP_WHOLE
    {kIsbTail, 4, {1024}},         // SSG_TUNE_ISB_TAIL
    {kPostTail, 4, {4096}},        // SSG_TUNE_POST_TAIL
    {kOnOff, 2, {1}},              // SSG_TUNE_STAGE_COLUMNS
};
constexpr int kKnobCount = sizeof(g_knobs) / sizeof(g_knobs[0]);
}  // namespace

int tuning(int knob) { return g_knobs[knob].value.load(std::memory_order_relaxed); }

}  // namespace ssg

extern "C" {

int ssg_tuning_set(int knob, int value)
{
    SSG_REQUIRE(knob >= 0 && knob < ssg::kKnobCount, "unknown tuning knob %d", knob);
    ssg::Knob& k = ssg::g_knobs[knob];
    for (int i = 0; i < k.count; ++i)
        if (k.values[i] == value) {
            k.value.store(value);
            return SSG_OK;
        }
    return ssg::fail(SSG_ERR_INVALID_ARGUMENT, "value %d is not a choice of tuning knob %d", value, knob);
}

int ssg_tuning_get(int knob)
{
    if (knob < 0 || knob >= ssg::kKnobCount) return -1;
    return ssg::tuning(knob);
}

int ssg_tuning_choices(int knob, int32_t* values, int capacity)
{
    if (knob < 0 || knob >= ssg::kKnobCount) return 0;
    const ssg::Knob& k = ssg::g_knobs[knob];
    for (int i = 0; i < k.count && i < capacity && values; ++i) values[i] = k.values[i];
    return k.count;
}

const char* ssg_last_error(void) { return ssg::g_error; }

int ssg_version(void) { return 100; }

void ssg_limits(int32_t* out4)
{
    if (!out4) return;
    out4[0] = SSG_MAX_CAMERAS;
    out4[1] = SSG_MAX_CANDIDATES;
    out4[2] = SSG_MAX_REFERENCES;
    out4[3] = SSG_MAX_LEVELS;
}

}  // extern "C"
