/*
 * Test infrastructure (oracle pinning only; never linked into the product library).
 *
 * Host-C++ stand-ins for the CUDA built-ins used by the reference kernels
 * python/isb_filter.cu, python/stitcher.cu and python/vec_utils.cuh, so that those sources,
 * read where they lie, compile with g++ into a host library (oracle/_ref/) that runs the
 * reference's own kernel bodies on the CPU.  Each stand-in follows the GPU semantics the
 * kernels rely on:
 *   - __float2int_rd / __float2int_rn: round down / to nearest even, NaN -> 0, saturating
 *     (PTX cvt.rmi / cvt.rni .s32.f32);
 *   - min / max on floats: fminf / fmaxf (CUDA's device overloads), so a NaN operand yields the
 *     other operand;
 *   - __expf: libm expf (the GPU's fast approximation is not reproduced; see the oracle header);
 *   - norm3df: the correctly rounded Euclidean norm, computed in double;
 *   - int2 is zero-initialised by default (see below).
 * blockIdx / threadIdx / blockDim are thread-local globals set by the launch harness.
 */
#pragma once
#include <math.h>
#include <climits>
#include <cstdint>

struct float2 { float x, y; };
struct float3 { float x, y, z; };
// zero default initialisers: the reference declares `int2 neighbours[2];` without initialising
// it (stitcher.cu:231) and encodes it when no neighbour gets a weight; this build reads zeros
// there, the value the library's table kernel writes.
struct int2 { int x = 0, y = 0; };
struct uchar2 { unsigned char x, y; };
struct uchar3 { unsigned char x, y, z; };
struct dim3 { unsigned int x, y, z; };

static inline float2 make_float2(float x, float y) { return float2{x, y}; }
static inline float3 make_float3(float x, float y, float z) { return float3{x, y, z}; }
static inline int2 make_int2(int x, int y) { return int2{x, y}; }
static inline uchar2 make_uchar2(unsigned char x, unsigned char y) { return uchar2{x, y}; }
static inline uchar3 make_uchar3(unsigned char x, unsigned char y, unsigned char z) { return uchar3{x, y, z}; }

#define __global__
#define __device__

extern thread_local dim3 blockIdx;
extern thread_local dim3 threadIdx;
extern thread_local dim3 blockDim;

static inline int refcuda_saturate_int(double v)
{
    if (v != v) return 0;
    if (v >= 2147483647.0) return INT_MAX;
    if (v <= -2147483648.0) return INT_MIN;
    return (int)v;
}
static inline int __float2int_rd(float x) { return refcuda_saturate_int(floor((double)x)); }
static inline int __float2int_rn(float x) { return refcuda_saturate_int(nearbyint((double)x)); }
#define __expf(x) expf(x)
static inline float norm3df(float a, float b, float c)
{
    return (float)sqrt((double)a * a + (double)b * b + (double)c * c);
}
static inline float min(float a, float b) { return fminf(a, b); }
static inline float max(float a, float b) { return fmaxf(a, b); }
