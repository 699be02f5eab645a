// Shared device helpers of the sphere_stereo_gb300 kernels: error plumbing, IEEE-exact
// arithmetic, the double-sphere camera model in the two forms the reference uses, and the
// exponential used by the ISB filter.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/sphere_stereo_gb300.h"

namespace ssg {

// ---------------------------------------------------------------------------------------------
// Error plumbing (ssg_api.cu)
// ---------------------------------------------------------------------------------------------
int fail(int code, const char* fmt, ...);
int launch_status(const char* what);  // cudaGetLastError() -> SSG_OK / SSG_ERR_CUDA
void clear_error();

#define SSG_REQUIRE(cond, ...)                                                          \
    do {                                                                                \
        if (!(cond)) return ::ssg::fail(SSG_ERR_INVALID_ARGUMENT, __VA_ARGS__);         \
    } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

int tuning(int knob);  // current value of an SSG_TUNE_* knob (ssg_api.cu)

// ---------------------------------------------------------------------------------------------
// IEEE round-to-nearest arithmetic that the compiler never contracts into FMAs.  The exact
// (fp32) kernels use these so that every operation is the one the reference performs, in the
// reference's order; the oracle performs the same operations.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float ffma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float fsqrt(float a) { return __fsqrt_rn(a); }

// The hardware's approximate square root and reciprocal (PTX sqrt.approx / rcp.approx, a few ulp):
// used only by the batched 16-bit path, whose outputs are compared within tolerances.
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

// Exponential by Cody-Waite range reduction and a degree-7 Taylor polynomial (W. J. Cody and
// W. Waite, "Software Manual for the Elementary Functions", 1980): x = n ln2 + r with
// |r| <= ln2 / 2, e^r by Horner's scheme in fused multiply-adds, then scaling by 2^n.  Every
// step is an IEEE operation, so oracle/sphere_oracle.c reproduces it bit for bit on the host.
// Accuracy: within 2 ulp of the exact value for normal results (checked in the tests against
// libm).  Results below 2^-126 are rounded once, to the nearest subnormal.
__host__ __device__ __forceinline__ float scale_by_pow2(float p, int n)
{
    // p in [0.7, 1.5); 2^n assembled from exponent bits, split in two steps below 2^-125.
    if (n > 127) return p * 1.7014118e38f * 2.0f;  // overflow to inf as the product rounds
    if (n >= -125) {
        union { int32_t i; float f; } s;
        s.i = (n + 127) << 23;
        return p * s.f;
    }
    if (n < -152) return 0.0f;
    union { int32_t i; float f; } a, b;
    a.i = (n + 100 + 127) << 23;  // 2^(n+100), normal
    b.i = (-100 + 127) << 23;     // 2^-100
    return (p * a.f) * b.f;       // first product exact, second rounds once
}

#ifdef __CUDACC__
__device__ __forceinline__ float cw_expf(float x)
{
    if (!(x == x)) return x;
    if (x > 88.8f) return __int_as_float(0x7f800000);
    if (x < -104.0f) return 0.0f;
    const float n = rintf(__fmul_rn(x, 1.44269504088896341f));
    // ln2 = LN2_HI + LN2_LO, LN2_HI with 16 significant bits so n * LN2_HI is exact
    float r = __fmaf_rn(n, -0.693145751953125f, x);
    r = __fmaf_rn(n, -1.42860682030941723e-06f, r);
    float p = 1.98412698e-04f;                 // 1/7!
    p = __fmaf_rn(p, r, 1.38888889e-03f);      // 1/6!
    p = __fmaf_rn(p, r, 8.33333333e-03f);      // 1/5!
    p = __fmaf_rn(p, r, 4.16666667e-02f);      // 1/4!
    p = __fmaf_rn(p, r, 1.66666667e-01f);      // 1/3!
    p = __fmaf_rn(p, r, 0.5f);                 // 1/2!
    p = __fmaf_rn(p, r, 1.0f);
    p = __fmaf_rn(p, r, 1.0f);
    return scale_by_pow2(p, (int)n);
}
#endif

// ---------------------------------------------------------------------------------------------
// Double-sphere model, torch form (python/utils.py:57-94): the constants that torch derives
// from the calibration's Python floats, rounded to float32 exactly where torch rounds them.
// ---------------------------------------------------------------------------------------------
struct TorchCam {
    float fx, fy, cx, cy;
    float xi, alpha, alpha2, k1, one_minus_xi2, one_minus_alpha, minus_w2;
};

TorchCam make_torch_cam(const ssg_camera& c);  // ssg_api.cu

#ifdef __CUDACC__
// utils.py:57-73; returns the validity flag of utils.py:72
__device__ __forceinline__ bool unproject_torch(float u, float v, const TorchCam& k, float p[3])
{
    const float mx = fdiv(fsub(u, k.cx), k.fx);
    const float my = fdiv(fsub(v, k.cy), k.fy);
    const float r2 = fadd(fmul(mx, mx), fmul(my, my));
    const float disc = fsub(1.0f, fmul(k.k1, r2));
    const float mz = fdiv(fsub(1.0f, fmul(k.alpha2, r2)),
                          fsub(fadd(fmul(k.alpha, fsqrt(disc > 0.0f ? disc : 0.0f)), 1.0f), k.alpha));
    const float mz2 = fmul(mz, mz);
    const float s = fdiv(fadd(fmul(mz, k.xi), fsqrt(fadd(mz2, fmul(k.one_minus_xi2, r2)))), fadd(mz2, r2));
    p[0] = fmul(s, mx);
    p[1] = fmul(s, my);
    p[2] = fsub(fmul(s, mz), k.xi);
    return disc >= 0.0f;
}

// torch.norm(., dim=-1) of a 3-vector on the reference's CPU kernels: fma(z, z, fma(y, y, x*x))
__device__ __forceinline__ float norm3_torch(float x, float y, float z)
{
    return fsqrt(ffma(z, z, ffma(y, y, fmul(x, x))));
}

// utils.py:75-94; returns the validity flag of utils.py:92
__device__ __forceinline__ bool project_torch(const float p[3], const TorchCam& k, float uv[2])
{
    const float d1 = norm3_torch(p[0], p[1], p[2]);
    const float c = fadd(fmul(k.xi, d1), p[2]);
    const float d2 = norm3_torch(p[0], p[1], c);
    const float nrm = fadd(fmul(k.alpha, d2), fmul(k.one_minus_alpha, c));
    uv[0] = fadd(fdiv(fmul(k.fx, p[0]), nrm), k.cx);
    uv[1] = fadd(fdiv(fmul(k.fy, p[1]), nrm), k.cy);
    return p[2] > fmul(k.minus_w2, d1);
}

// [p, 1] @ rt.T as the reference's CPU matmul evaluates it (fma chain over x, y, z, then + t)
__device__ __forceinline__ void transform_torch(const float* rt, const float p[3], float q[3])
{
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        float acc = fmul(p[0], rt[4 * i + 0]);
        acc = ffma(p[1], rt[4 * i + 1], acc);
        acc = ffma(p[2], rt[4 * i + 2], acc);
        q[i] = fadd(acc, rt[4 * i + 3]);
    }
}

// ---------------------------------------------------------------------------------------------
// Double-sphere model, stitcher-kernel form (python/stitcher.cu:121-168), float32 intrinsics.
// ---------------------------------------------------------------------------------------------
struct Intr {
    float fx, fy, cx, cy, xi, alpha;
};

__device__ __forceinline__ void unproject_cu(float u, float v, const Intr& k, float p[3])
{
    const float mx = fdiv(fsub(u, k.cx), k.fx);
    const float my = fdiv(fsub(v, k.cy), k.fy);
    const float r2 = fadd(fmul(mx, mx), fmul(my, my));
    const float mz = fdiv(fsub(1.0f, fmul(fmul(k.alpha, k.alpha), r2)),
                          fsub(fadd(fmul(k.alpha, fsqrt(fsub(1.0f, fmul(fsub(fmul(2.0f, k.alpha), 1.0f), r2)))), 1.0f),
                               k.alpha));
    const float mz2 = fmul(mz, mz);
    const float s = fdiv(fadd(fmul(mz, k.xi), fsqrt(fadd(mz2, fmul(fsub(1.0f, fmul(k.xi, k.xi)), r2)))),
                         fadd(mz2, r2));
    p[0] = fmul(mx, s);
    p[1] = fmul(my, s);
    p[2] = fsub(fmul(mz, s), k.xi);
}

// stitcher.cu:140-168; `valid` is and-ed with the model's validity test when non-null
__device__ __forceinline__ void project_cu(const float p[3], const Intr& k, float uv[2], bool* valid)
{
    const float d1 = norm3df(p[0], p[1], p[2]);
    const float c = fadd(fmul(k.xi, d1), p[2]);
    const float d2 = norm3df(p[0], p[1], c);
    const float nrm = fadd(fmul(k.alpha, d2), fmul(fsub(1.0f, k.alpha), c));
    if (valid) {
        const float w1 = k.alpha > 0.5f ? fdiv(fsub(1.0f, k.alpha), k.alpha) : fdiv(k.alpha, fsub(1.0f, k.alpha));
        const float w2 = fdiv(fadd(w1, k.xi),
                              fsqrt(fadd(fadd(fmul(fmul(2.0f, w1), k.xi), fmul(k.xi, k.xi)), 1.0f)));
        *valid = *valid && (p[2] > fmul(-w2, d1));
    }
    const float den = fdiv(1.0f, nrm);
    uv[0] = fadd(fmul(fmul(k.fx, p[0]), den), k.cx);
    uv[1] = fadd(fmul(fmul(k.fy, p[1]), den), k.cy);
}

// interpF (stitcher.cu:89-116): bilinear, no bounds check (callers clamp coordinates)
__device__ __forceinline__ float interp_f(const float* __restrict__ s, float u, float v, int cols)
{
    const int u1 = __float2int_rd(u), v1 = __float2int_rd(v), u2 = u1 + 1, v2 = v1 + 1;
    const float u1f = (float)u1, u2f = (float)u2, v1f = (float)v1, v2f = (float)v2;
    const float w1 = fmul(fsub(u2f, u), fsub(v2f, v)), w2 = fmul(fsub(u2f, u), fsub(v, v1f));
    const float w3 = fmul(fsub(u, u1f), fsub(v2f, v)), w4 = fmul(fsub(u, u1f), fsub(v, v1f));
    const float p1 = __ldg(s + (int64_t)v1 * cols + u1), p2 = __ldg(s + (int64_t)v2 * cols + u1);
    const float p3 = __ldg(s + (int64_t)v1 * cols + u2), p4 = __ldg(s + (int64_t)v2 * cols + u2);
    return fadd(fadd(fadd(fmul(w1, p1), fmul(w2, p2)), fmul(w3, p3)), fmul(w4, p4));
}
#endif  // __CUDACC__

inline Intr to_intr(const ssg_intrinsics& k) { return Intr{k.fx, k.fy, k.cx, k.cy, k.xi, k.alpha}; }

inline int grid_1d(int64_t n, int block) { return (int)((n + block - 1) / block); }

// Division of n < 2^31 by a divisor fixed on the host, by a multiply-high and a shift
// (T. Granlund and P. L. Montgomery, "Division by invariant integers using multiplication",
// PLDI 1994): with s = floor(log2 d) and m = floor(2^(32+s) / d) + 1 (below 2^32 when d is not a
// power of two), floor(n * m / 2^(32+s)) = floor(n / d) whenever n * (m - 2^(32+s) / d) * d <
// 2^(32+s), which holds for every n < 2^31 because 2^(32+s) / d > 2^31.  Powers of two shift.
struct FastDiv {
    uint32_t m = 0;
    int s = 0;
    FastDiv() = default;
    explicit FastDiv(uint32_t d)
    {
        while ((2u << s) <= d && s < 31) ++s;  // s = floor(log2 d)
        m = (d & (d - 1)) ? (uint32_t)((((uint64_t)1) << (32 + s)) / d + 1) : 0u;
    }
    __host__ __device__ __forceinline__ uint32_t div(uint32_t n) const
    {
#ifdef __CUDA_ARCH__
        return m ? __umulhi(n, m) >> s : n >> s;
#else
        return m ? (uint32_t)(((uint64_t)n * m) >> 32) >> s : n >> s;
#endif
    }
};

}  // namespace ssg
