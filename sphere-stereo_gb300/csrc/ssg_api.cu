// Library-wide plumbing of the C ABI: per-thread error messages, version, limits, and the
// host-side derivation of the torch-form camera constants.
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

}  // namespace ssg

extern "C" {

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
