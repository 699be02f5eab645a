// Cost cells of the batched path: 8 consecutive candidates of one pixel in 16 bytes (fp16 or
// unorm16) or 32 bytes (float32), the unit of every load and store of the chunked layout
// [chunks][pixels][8]; and single-candidate cells of the reference's planar layout.
#pragma once

#include <cuda_fp16.h>

#include "ssg_common.cuh"

namespace ssg {

constexpr int kBatchBlock = 256;

// Double-sphere camera of the batched sweep (utils.py:75-94 constants in float32)
struct FastCam {
    float fx, fy, cx, cy, xi, alpha, one_minus_alpha;
};

// Packed pairs of fp32 values: one Blackwell instruction performs a rounded-to-nearest operation
// on both halves (two candidates of one pixel), which halves the issue slots of the batched
// kernels' arithmetic.
__device__ __forceinline__ float2 splat(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
// a + b rounded toward minus infinity, two lanes in one instruction
__device__ __forceinline__ float2 add2_rd(float2 a, float2 b)
{
    unsigned long long ra, rb, rd;
    asm("mov.b64 %0, {%1, %2};" : "=l"(ra) : "f"(a.x), "f"(a.y));
    asm("mov.b64 %0, {%1, %2};" : "=l"(rb) : "f"(b.x), "f"(b.y));
    asm("add.rm.f32x2 %0, %1, %2;" : "=l"(rd) : "l"(ra), "l"(rb));
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(rd));
    return r;
}
constexpr float kUnormScale = 65535.0f / 500.0f;
constexpr float kUnormInv = 500.0f / 65535.0f;

// 8 costs <-> one 16-byte cell
template <typename T>
struct Cell;

template <>
struct Cell<__half> {
    __device__ static __forceinline__ void unpack(uint4 v, float c[8])
    {
        const __half2* h = reinterpret_cast<const __half2*>(&v);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const float2 f = __half22float2(h[i]);
            c[2 * i] = f.x;
            c[2 * i + 1] = f.y;
        }
    }
    __device__ static __forceinline__ uint32_t pack2(float a, float b)
    {
        const __half2 h = __floats2half2_rn(a, b);
        return *reinterpret_cast<const uint32_t*>(&h);
    }
    __device__ static __forceinline__ uint4 pack(const float c[8])
    {
        uint4 v;
        __half2* h = reinterpret_cast<__half2*>(&v);
#pragma unroll
        for (int i = 0; i < 4; ++i) h[i] = __floats2half2_rn(c[2 * i], c[2 * i + 1]);
        return v;
    }
};

template <>
struct Cell<uint16_t> {
    __device__ static __forceinline__ void unpack(uint4 v, float c[8])
    {
        const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            c[2 * i] = (float)(w[i] & 0xFFFFu) * kUnormInv;
            c[2 * i + 1] = (float)(w[i] >> 16) * kUnormInv;
        }
    }
    __device__ static __forceinline__ uint32_t q(float c)
    {
        return (uint32_t)__float2uint_rn(fminf(fmaxf(c, 0.0f), 500.0f) * kUnormScale);
    }
    __device__ static __forceinline__ uint32_t pack2(float a, float b) { return q(a) | (q(b) << 16); }
    __device__ static __forceinline__ uint4 pack(const float c[8])
    {
        return make_uint4(q(c[0]) | (q(c[1]) << 16), q(c[2]) | (q(c[3]) << 16), q(c[4]) | (q(c[5]) << 16),
                          q(c[6]) | (q(c[7]) << 16));
    }
};

template <>
struct Cell<float> {};

__device__ __forceinline__ uint4 ldg16(const void* p) { return __ldg(reinterpret_cast<const uint4*>(p)); }

// A float32 cell (32 bytes) in one 256-bit access (sm_100 and later).  The address is 32-byte
// aligned: every entry point that passes float32 chunked levels checks their base pointers, and
// cells lie at multiples of 32 bytes from them.
__device__ __forceinline__ void ldg256(const float* p, float v[8])
{
    unsigned long long a, b, c, d;
    asm("ld.global.nc.v4.b64 {%0, %1, %2, %3}, [%4];" : "=l"(a), "=l"(b), "=l"(c), "=l"(d) : "l"(p));
    const unsigned long long w[4] = {a, b, c, d};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        v[2 * i] = __uint_as_float((uint32_t)w[i]);
        v[2 * i + 1] = __uint_as_float((uint32_t)(w[i] >> 32));
    }
}
__device__ __forceinline__ void stg256(float* p, const float v[8])
{
    unsigned long long w[4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
        w[i] = (unsigned long long)__float_as_uint(v[2 * i]) |
               ((unsigned long long)__float_as_uint(v[2 * i + 1]) << 32);
    asm volatile("st.global.v4.b64 [%0], {%1, %2, %3, %4};" ::"l"(p), "l"(w[0]), "l"(w[1]), "l"(w[2]), "l"(w[3])
                 : "memory");
}

// 8 consecutive candidates of one cell, any storage type
template <typename T>
__device__ __forceinline__ void load8(const T* __restrict__ p, float v[8])
{
    Cell<T>::unpack(ldg16(p), v);
}
template <>
__device__ __forceinline__ void load8<float>(const float* __restrict__ p, float v[8])
{
    ldg256(p, v);
}
template <typename T>
__device__ __forceinline__ void store8(T* p, const float v[8])
{
    reinterpret_cast<uint4*>(p)[0] = Cell<T>::pack(v);
}
template <>
__device__ __forceinline__ void store8<float>(float* p, const float v[8])
{
    stg256(p, v);
}

// Cells of W candidates: W = 8 for the chunked layout [chunks][pixels][8] of the batched path,
// W = 1 for the planar layout [candidates][pixels] (chunks = candidates) of the reference.
template <int W, typename T>
struct CellIO;
template <typename T>
struct CellIO<8, T> {
    __device__ static __forceinline__ void load(const T* p, float v[8]) { load8<T>(p, v); }
    __device__ static __forceinline__ void store(T* p, const float v[8]) { store8<T>(p, v); }
};
template <>
struct CellIO<1, float> {
    __device__ static __forceinline__ void load(const float* p, float v[1]) { v[0] = __ldg(p); }
    __device__ static __forceinline__ void store(float* p, const float v[1]) { p[0] = v[0]; }
};

}  // namespace ssg
