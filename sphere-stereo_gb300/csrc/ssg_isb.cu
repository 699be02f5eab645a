// ISB multiscale edge-aware cost filter (python/isb_filter.cu, python/isb_filter.py) and the
// distance selection of python/depth_estimation.py:179-198, for one cost volume in the reference's
// planar layout [candidates][rows][cols] and for batches of volumes in the chunked layout of
// ssg_cells.cuh.
//
// Both layouts run the same kernels, templated on the cell width W (1 = planar, 8 = chunked):
//   - downsampling: one thread per coarse pixel; its 3x3 range weights are computed once from the
//     uint8 guides and shared by all candidates;
//   - upsampling: one thread per fine pixel, with the coarse neighbourhood of a block staged in
//     shared memory per chunk of candidates;
//   - the last upsampling step can be fused with the selection, so that the filtered level-0
//     volume is never written.
// Guides, range weights and cost sums use the reference's arithmetic in its order
// (ssg_isb_common.cuh), so both layouts give the same bits; the batched path differs from the
// reference only by the 16-bit rounding of its level-0 volume.
#include <atomic>
#include <cmath>
#include <cstring>
#include <mutex>
#include <type_traits>

#include "ssg_cells.cuh"
#include "ssg_isb_common.cuh"
#include "ssg_tma.cuh"
#include "ssg_uneven.cuh"

namespace ssg {

// ---------------------------------------------------------------------------------------------
// Range-weight tables: one per distinct var_inv_i, evaluated once by a kernel with the same
// device function as the per-block tables, so the values are the same bits.
// ---------------------------------------------------------------------------------------------
constexpr int kRangeTableSlots = 64;
__device__ float g_range_tables[kRangeTableSlots][kRangeLutStride];

__global__ void range_table_kernel(float* __restrict__ table, float var_inv_i)
{
    for (int d = threadIdx.x; d < kRangeLutStride; d += blockDim.x)
        table[d] = d < kRangeLutSize ? range_weight((float)d, var_inv_i) : 0.0f;
}

// a one-thread launch rather than a memset of the symbol: no host-side symbol lookup, which is
// not allowed while the stream is being captured into a graph
__global__ void clear_tma_abort_kernel() { g_tma_abort = 0u; }

cudaError_t clear_tma_abort(cudaStream_t st)
{
    clear_tma_abort_kernel<<<1, 1, 0, st>>>();
    return cudaGetLastError();
}

bool encode_tensor_map(CUtensorMap* map, const void* base, int rank, const uint64_t* dims, const uint64_t* strides,
                       const uint32_t* box)
{
    static PFN_cuTensorMapEncodeTiled_v12000 encode = [] {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            fn = nullptr;
        }
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }();
    if (!encode || ((uintptr_t)base & 15) != 0 || rank < 1 || rank > 5) return false;
    cuuint64_t gdim[5], gstride[4];
    cuuint32_t bdim[5], estride[5];
    for (int i = 0; i < rank; ++i) {
        gdim[i] = dims[i];
        bdim[i] = box[i];
        estride[i] = 1;
        if (i + 1 < rank) {
            if (strides[i] % 16 != 0) return false;
            gstride[i] = strides[i];
        }
    }
    return encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, (cuuint32_t)rank, const_cast<void*>(base), gdim, gstride, bdim,
                  estride, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

const float* range_table(float var_inv_i, cudaStream_t stream)
{
    struct Device {
        uint32_t key[kRangeTableSlots];
        int used = 0;
        float* base = nullptr;
    };
    constexpr int kMaxDevices = 64;
    static std::mutex mutex;
    static Device devices[kMaxDevices];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return nullptr;
    }
    uint32_t key;
    std::memcpy(&key, &var_inv_i, sizeof key);
    std::lock_guard<std::mutex> lock(mutex);
    Device& D = devices[dev];
    for (int s = 0; s < D.used; ++s)
        if (D.key[s] == key) return D.base + (int64_t)s * kRangeLutStride;
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(stream, &capture) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (capture != cudaStreamCaptureStatusNone || D.used == kRangeTableSlots) return nullptr;
    if (!D.base) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_range_tables) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        D.base = static_cast<float*>(p);
    }
    float* table = D.base + (int64_t)D.used * kRangeLutStride;
    range_table_kernel<<<1, kBatchBlock, 0, stream>>>(table, var_inv_i);
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(stream) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    D.key[D.used++] = key;
    return table;
}

// ---------------------------------------------------------------------------------------------
// ISB filter on the chunked layout. Guides and range weights come from the same device functions
// as the fp32 path (ssg_isb_common.cuh), so the guide pyramid is bit-identical to it: the uint8
// truncation of the filtered guide turns a one-ulp change of a weight into a step of one grey
// level on a sizeable share of coarse pixels, which then moves the argmin. The costs are summed
// in the fp32 path's order as well; the level-0 rounding is the only difference.
// ---------------------------------------------------------------------------------------------

// Downsampling, one thread per coarse pixel; level 0 (any storage) or a float32 level in,
// float32 out.
// One coarse pixel o of a level: pointers are the instance's own; `lut` is the block's filled
// range table.
// W float32 costs through L2 (ld.global.cg): for cells written earlier in the same launch, which
// the read-only path does not see
template <int W>
__device__ __forceinline__ void load_coherent(const float* p, float* v)
{
    if constexpr (W == 1) {
        v[0] = __ldcg(p);
    } else {
        static_assert(W == 8, "cells of 1 or 8 candidates");
        const float4 a = __ldcg(reinterpret_cast<const float4*>(p)), b = __ldcg(reinterpret_cast<const float4*>(p) + 1);
        v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w, v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w;
    }
}

// kCoherent: the costs are read through L2 (with GL = G4C for the guides), for a launch that runs
// several levels one after the other
template <int W, typename Tin, typename GL, bool kCoherent = false>
__device__ __forceinline__ void isb_down_pixel(const uint8_t* __restrict__ guide_in, const Tin* __restrict__ cost_in,
                                               uint8_t* __restrict__ guide_out, float* __restrict__ cost_out,
                                               const LevelGeom& g, int chunks, int o, const float* lut)
{
    static_assert(!kCoherent || std::is_same<Tin, float>::value, "coherent reads are of float32 levels");
    const int64_t pin = (int64_t)g.rows_in * g.cols_in, pout = (int64_t)g.rows_out * g.cols_out;
    DownTapsT<int> t;
    const int y = o / g.cols_out;  // 32-bit: a level holds fewer than 2^31 pixels
    down_weights<int, LutRange, GL>(guide_in, g.rows_in, g.cols_in, o - y * g.cols_out, y, LutRange{lut}, guide_out,
                                    o, t);
    // the chunked (16-bit) path sums with fused multiply-adds and scales by the reciprocal; the
    // planar path keeps the reference's separate products and its division
    constexpr bool kFast = W == 8;
    const float rsum = kFast ? __frcp_rn(t.wsum) : 0.0f;
    for (int c = 0; c < chunks; ++c) {
        const Tin* src = cost_in + (int64_t)c * pin * W;
        float acc[W];
        if constexpr (kCoherent) load_coherent<W>(reinterpret_cast<const float*>(src) + (int64_t)t.centre * W, acc);
        else CellIO<W, Tin>::load(src + (int64_t)t.centre * W, acc);
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            float v[W];
            if constexpr (kCoherent) load_coherent<W>(reinterpret_cast<const float*>(src) + (int64_t)t.idx[i] * W, v);
            else CellIO<W, Tin>::load(src + (int64_t)t.idx[i] * W, v);
#pragma unroll
            for (int j = 0; j < W; ++j) acc[j] = kFast ? fmaf(v[j], t.w[i], acc[j]) : fadd(acc[j], fmul(v[j], t.w[i]));
        }
#pragma unroll
        for (int j = 0; j < W; ++j) acc[j] = kFast ? acc[j] * rsum : fdiv(acc[j], t.wsum);
        CellIO<W, float>::store(cost_out + ((int64_t)c * pout + o) * W, acc);
    }
}

// Downsampling, one thread per coarse pixel; level 0 (any storage) or a float32 level in,
// float32 out.  blockIdx.y: instance of contiguous levels; GL: the guides' layout.
template <int W, typename Tin, typename GL>
__global__ void __launch_bounds__(kBatchBlock) isb_down_kernel(const uint8_t* __restrict__ guide_in,
                                                                   const Tin* __restrict__ cost_in,
                                                                   uint8_t* __restrict__ guide_out,
                                                                   float* __restrict__ cost_out, LevelGeom g,
                                                                   int chunks, float var_inv_i,
                                                                   const float* __restrict__ table)
{
    __shared__ __align__(16) float lut[kRangeLutStride];
    load_range_lut(lut, table, var_inv_i);
    __syncthreads();
    const int64_t pin = (int64_t)g.rows_in * g.cols_in, pout = (int64_t)g.rows_out * g.cols_out;
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= pout) return;
    const int inst = blockIdx.y;
    isb_down_pixel<W, Tin, GL>(guide_in + (int64_t)inst * pin * GL::bytes, cost_in + (int64_t)inst * chunks * pin * W,
                               guide_out + (int64_t)inst * pout * GL::bytes, cost_out + (int64_t)inst * chunks * pout * W,
                               g, chunks, (int)o, lut);
}

// ---------------------------------------------------------------------------------------------
// Upsampling.  A coarse pixel (x, y) owns four fine pixels F = 0 (2x, 2y), 1 (2x, 2y + 1),
// 2 (2x + 1, 2y), 3 (2x + 1, 2y + 1), each filtered from its own list of the coarse 3x3 taps
// (UpTaps<F>: 9, 6, 6 and 4 taps).  A thread takes two of them, so that every thread has about
// the same work and shares its tap loads between its two pixels: kind 0 takes F = 0 and 3
// (13 taps, 9 distinct), kind 1 takes F = 1 and 2 (12 taps, 8 distinct).  A block of 256 threads
// covers kUpTileX = 128 coarse pixels of one coarse row: warps 0-3 are kind 0, warps 4-7 kind 1,
// so every warp follows one tap list.  The coarse costs of the block's 3 x (kUpTileX + 2)
// neighbourhood, edge-clamped as the taps are, are staged per chunk of candidates in shared
// memory with cp.async, double-buffered: each coarse cell is read from memory once per block,
// and the next chunk streams in while this one is filtered.  Candidates are processed in parts
// of 4 (W = 8) or 1 (W = 1) to bound the registers that hold the taps.
// ---------------------------------------------------------------------------------------------
constexpr int kUpTileX = kBatchBlock / 2;
constexpr int kUpTileCols = kUpTileX + 2;

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem));
}
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_one() { asm volatile("cp.async.wait_group 1;\n" ::); }

// A chunk's tile: [part][row 0..2][col 0..kUpTileCols-1][E floats], parts of E = 4 candidates
// (W = 8, two parts) or of one candidate (W = 1).  A part starts on a 128-byte boundary (the
// alignment of a TMA destination).
template <int W>
struct UpTile {
    static constexpr int parts = W == 8 ? 2 : 1;
    static constexpr int E = W == 8 ? 4 : 1;
    static constexpr int part_floats = (3 * kUpTileCols * E + 31) / 32 * 32;
    static constexpr int floats = parts * part_floats;
    static constexpr uint32_t part_bytes = 3 * kUpTileCols * E * sizeof(float);  // one TMA box
};

template <int W>
__device__ __forceinline__ void load_tile_async(float* __restrict__ buf, const float* __restrict__ chunk,
                                                int rows_in, int cols_in, int x0, int y)
{
    constexpr int cells = 3 * kUpTileCols;
    for (int e = threadIdx.x; e < UpTile<W>::parts * cells; e += blockDim.x) {
        const int part = e / cells, rc = e % cells;
        const int row = rc / kUpTileCols, col = rc % kUpTileCols;
        const int gx = min(max(x0 - 1 + col, 0), cols_in - 1), gy = min(max(y - 1 + row, 0), rows_in - 1);
        const float* src = chunk + ((int64_t)gy * cols_in + gx) * W + part * 4;
        float* dst = buf + part * UpTile<W>::part_floats + rc * UpTile<W>::E;
        if constexpr (W == 8)
            cp_async16(dst, src);
        else
            cp_async4(dst, src);
    }
}

// The TMA form of load_tile_async (W = 8): one box of 4 floats x kUpTileCols x 3 rows per part,
// issued by thread 0 on `bar`.  The box starts at column x0 - 1 and row y - 1, possibly outside
// the level: those cells arrive as zeros and tma_clamp_edges replaces them afterwards.
// c3: the chunk's plane (instance * chunks + chunk) of the level's tensor map.
// withhold: the barrier is armed but no copy is issued, so that its wait runs out (the tests of
// the timeout path; SSG_TUNE_TMA_WITHHOLD).  Returns whether copies were issued.
__device__ __forceinline__ bool load_tile_tma(float* __restrict__ buf, const CUtensorMap* map, int x0, int y, int c3,
                                              uint64_t* bar, bool withhold = false)
{
    mbar_arrive_expect_tx(bar, 2 * UpTile<8>::part_bytes);
    if (withhold) return false;
#pragma unroll
    for (int part = 0; part < 2; ++part) tma_load_4d(buf + part * UpTile<8>::part_floats, map, 4 * part, x0 - 1, y - 1, c3, bar);
    return true;
}

// A block whose tile wait ran out: thread 0 waits (bounded, without the early-out) for the copies
// it issued that have not been seen to land, for chunk c (buffer c & 1) and chunk c + 1, so that
// no copy writes the block's shared memory after it exits.
__device__ __forceinline__ void tma_drain(uint64_t* bar, uint32_t in_flight, int c)
{
#pragma unroll
    for (int k = c; k <= c + 1; ++k)
        if (in_flight & (1u << (k & 1))) mbar_wait(&bar[k & 1], (uint32_t)(k >> 1) & 1u, kTmaMaxPolls, false);
}

// Edge clamping of a TMA tile: cells whose column or row lies outside the level take the value of
// the clamped cell, as load_tile_async's addresses do.  Block-uniform; the caller synchronises
// the block before and after.
__device__ __forceinline__ void tma_clamp_edges(float* __restrict__ buf, int rows_in, int cols_in, int x0, int y)
{
    const bool left = x0 == 0, right = x0 - 1 + kUpTileCols > cols_in, top = y == 0, bottom = y + 1 >= rows_in;
    if (!(left || right || top || bottom)) return;
    constexpr int cells = 3 * kUpTileCols;
    for (int e = threadIdx.x; e < 2 * cells; e += blockDim.x) {
        const int part = e / cells, rc = e % cells;
        const int row = rc / kUpTileCols, col = rc % kUpTileCols;
        const int gx = x0 - 1 + col, gy = y - 1 + row;
        const int cx = min(max(gx, 0), cols_in - 1), cy = min(max(gy, 0), rows_in - 1);
        if (cx == gx && cy == gy) continue;
        // the source is a cell inside the level (never itself a target)
        const int src = (cy - (y - 1)) * kUpTileCols + (cx - (x0 - 1));
        float* p = buf + part * UpTile<8>::part_floats;
        reinterpret_cast<float4*>(p)[rc] = reinterpret_cast<const float4*>(p)[src];
    }
}

// One fine cell held in registers as loaded (prefetched a chunk ahead), read out in parts of E
// candidates; and the store of a float32 part.
template <int W, typename T>
struct RawCell;
template <>
struct RawCell<8, __half> {
    uint4 q;
    __device__ __forceinline__ void load(const __half* cell) { q = __ldg(reinterpret_cast<const uint4*>(cell)); }
    __device__ __forceinline__ void part(int p, float v[4]) const
    {
        const uint32_t lo = p == 0 ? q.x : q.z, hi = p == 0 ? q.y : q.w;
        const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&lo));
        const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&hi));
        v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
    }
};
template <>
struct RawCell<8, uint16_t> {
    uint4 q;
    __device__ __forceinline__ void load(const uint16_t* cell) { q = __ldg(reinterpret_cast<const uint4*>(cell)); }
    __device__ __forceinline__ void part(int p, float v[4]) const
    {
        const uint32_t lo = p == 0 ? q.x : q.z, hi = p == 0 ? q.y : q.w;
        v[0] = (float)(lo & 0xFFFFu) * kUnormInv;
        v[1] = (float)(lo >> 16) * kUnormInv;
        v[2] = (float)(hi & 0xFFFFu) * kUnormInv;
        v[3] = (float)(hi >> 16) * kUnormInv;
    }
};
template <>
struct RawCell<8, float> {
    float c[8];
    __device__ __forceinline__ void load(const float* cell) { ldg256(cell, c); }
    __device__ __forceinline__ void part(int p, float v[4]) const
    {
        v[0] = p == 0 ? c[0] : c[4];
        v[1] = p == 0 ? c[1] : c[5];
        v[2] = p == 0 ? c[2] : c[6];
        v[3] = p == 0 ? c[3] : c[7];
    }
};
template <>
struct RawCell<1, float> {
    float a;
    __device__ __forceinline__ void load(const float* cell) { a = __ldg(cell); }
    __device__ __forceinline__ void part(int, float v[1]) const { v[0] = a; }
};

template <int E>
__device__ __forceinline__ void store_part(float* cell, int p, const float v[E])
{
    if constexpr (E == 4)
        reinterpret_cast<float4*>(cell + 4 * p)[0] = make_float4(v[0], v[1], v[2], v[3]);
    else
        cell[0] = v[0];
}

template <int F>
__device__ __forceinline__ constexpr bool uses_tap(int t)
{
    for (int i = 0; i < UpTaps<F>::n; ++i)
        if (UpTaps<F>::tap(i) == t) return true;
    return false;
}

template <int F, typename GL>
__device__ __forceinline__ float fine_weights_padded(const typename GL::Pix (&gd)[9], const typename GL::Pix& up,
                                                     float weight_up, float weight_down, const LutRange& range,
                                                     float (&w)[9], float g[3])
{
    float wf[UpTaps<F>::n];
    const float inv = fine_weights<F, LutRange, GL>(gd, up, weight_up, weight_down, range, wf, g);
#pragma unroll
    for (int i = 0; i < 9; ++i) w[i] = i < UpTaps<F>::n ? wf[i < UpTaps<F>::n ? i : 0] : 0.0f;
    return inv;
}

// filtered costs of fine pixel F from the staged taps: the arithmetic and order of up_costs, or
// (kFast, the chunked 16-bit path) the same sum with fused multiply-adds; kPacked: two candidates
// at a time (the same bits; taken by the steps that store their cells, the selecting step keeps
// the scalar form, which leaves its three-block build fewer spilled registers)
template <int F, int E, bool kFast, bool kPacked = true>
__device__ __forceinline__ void filter_part(const float (&tap)[9][E], const float (&w)[9], float inv, float weight_up,
                                            float acc[E])
{
    if constexpr (kFast && kPacked && E % 2 == 0) {
        // two candidates per packed f32x2 operation: each lane rounds as the scalar form does
        float2 pair[E / 2];
#pragma unroll
        for (int j = 0; j < E / 2; ++j) pair[j] = mul2(splat(weight_up), make_float2(acc[2 * j], acc[2 * j + 1]));
#pragma unroll
        for (int i = 0; i < UpTaps<F>::n; ++i) {
            const float* t = tap[UpTaps<F>::tap(i)];
#pragma unroll
            for (int j = 0; j < E / 2; ++j) pair[j] = fma2(splat(w[i]), make_float2(t[2 * j], t[2 * j + 1]), pair[j]);
        }
#pragma unroll
        for (int j = 0; j < E / 2; ++j) {
            pair[j] = mul2(pair[j], splat(inv));
            acc[2 * j] = pair[j].x;
            acc[2 * j + 1] = pair[j].y;
        }
        return;
    }
#pragma unroll
    for (int e = 0; e < E; ++e) acc[e] = fmul(weight_up, acc[e]);
#pragma unroll
    for (int i = 0; i < UpTaps<F>::n; ++i)
#pragma unroll
        for (int e = 0; e < E; ++e)
            acc[e] = kFast ? fmaf(w[i], tap[UpTaps<F>::tap(i)][e], acc[e])
                           : fadd(acc[e], fmul(w[i], tap[UpTaps<F>::tap(i)][e]));
#pragma unroll
    for (int e = 0; e < E; ++e) acc[e] = fmul(acc[e], inv);
}


// State of one fine pixel of a thread
struct FinePixel {
    float w[9];
    float inv;
    int index;  // fine pixel index in its level
    bool active;
};

template <int F, bool kWriteGuide, typename GL>
__device__ __forceinline__ void fine_setup(const typename GL::Pix (&gd)[9], const uint8_t* __restrict__ guide_io,
                                           const LevelGeom& g, int x, int y, bool coarse_ok, float weight_up,
                                           float weight_down, const LutRange& range, FinePixel& px)
{
    const int fx = 2 * x + (F >= 2 ? 1 : 0), fy = 2 * y + (F & 1);
    // a fine pixel outside the level is the clamped duplicate of another one and is skipped
    px.active = coarse_ok && fx < g.cols_out && fy < g.rows_out;
    // an inactive pixel reads pixel 0 with zero weights (the selecting step filters it without a
    // branch and drops the result)
    px.index = px.active ? fy * g.cols_out + fx : 0;
    px.inv = 0.0f;
    if (!px.active) {
#pragma unroll
        for (int i = 0; i < 9; ++i) px.w[i] = 0.0f;
        return;
    }
    float gsum[3];
    const typename GL::Pix up = GL::load(guide_io, px.index);
    px.inv = fine_weights_padded<F, GL>(gd, up, weight_up, weight_down, range, px.w, gsum);
    if (kWriteGuide) {
        uint32_t v[3];
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) v[ch] = __float2uint_rz(fmul(gsum[ch], px.inv));
        GL::store(const_cast<uint8_t*>(guide_io), px.index, v);
    }
}

// filter one part of fine pixel F and select or store it
template <int F, int W, typename Tf, bool kSelect>
__device__ __forceinline__ void up_part(const float (&tap)[9][UpTile<W>::E], const FinePixel& px,
                                        const RawCell<W, Tf>& raw, int part, int k0, bool full, int ncand,
                                        float weight_up, Tf* __restrict__ fine_chunk, Selector& s, float* kept)
{
    constexpr int E = UpTile<W>::E;
    float acc[E];
    raw.part(part, acc);
    filter_part<F, E, W == 8, !kSelect>(tap, px.w, px.inv, weight_up, acc);
    if constexpr (kSelect) {
        if (full) {
#pragma unroll
            for (int e = 0; e < E; ++e) s.push(k0 + e, acc[e]);
        } else {
#pragma unroll
            for (int e = 0; e < E; ++e)
                if (k0 + e < ncand) s.push(k0 + e, acc[e]);
        }
    } else if constexpr (W == 8) {
        // kept for the store of the whole cell after both parts
#pragma unroll
        for (int e = 0; e < E; ++e) kept[part * E + e] = acc[e];
    } else {
        store_part<E>(reinterpret_cast<float*>(fine_chunk + (int64_t)px.index * W), part, acc);
    }
}

// one chunk for the two fine pixels FA, FB of a thread, from their prefetched fine cells
template <int FA, int FB, int W, typename Tf, bool kSelect>
__device__ __forceinline__ void up_chunk(const float* __restrict__ buf, int lx, Tf* __restrict__ fine_chunk, int c,
                                         int ncand, float weight_up, const FinePixel& pa, const FinePixel& pb,
                                         const RawCell<W, Tf>& ra, const RawCell<W, Tf>& rb, Selector& sa,
                                         Selector& sb)
{
    constexpr int E = UpTile<W>::E;
    const bool full = (c + 1) * W <= ncand;
    float kept_a[W], kept_b[W];  // the non-selecting chunked step's filtered cells
#pragma unroll
    for (int part = 0; part < UpTile<W>::parts; ++part) {
        float tap[9][E];
#pragma unroll
        for (int t = 0; t < 9; ++t) {
            if (uses_tap<FA>(t) || uses_tap<FB>(t)) {
                const int cell = (t / 3) * kUpTileCols + lx + t % 3;
                const float* pb = buf + part * UpTile<W>::part_floats;
                if constexpr (E == 4) {
                    const float4 q = reinterpret_cast<const float4*>(pb)[cell];
                    tap[t][0] = q.x; tap[t][1] = q.y; tap[t][2] = q.z; tap[t][3] = q.w;
                } else {
                    tap[t][0] = pb[cell];
                }
            } else {
#pragma unroll
                for (int e = 0; e < E; ++e) tap[t][e] = 0.0f;
            }
        }
        const int k0 = c * W + part * E;
        if (kSelect || pa.active)
            up_part<FA, W, Tf, kSelect>(tap, pa, ra, part, k0, full, ncand, weight_up, fine_chunk, sa, kept_a);
        if (kSelect || pb.active)
            up_part<FB, W, Tf, kSelect>(tap, pb, rb, part, k0, full, ncand, weight_up, fine_chunk, sb, kept_b);
    }
    if constexpr (!kSelect && W == 8) {
        // one 256-bit store per fine cell (float32 levels, 32-byte aligned)
        if (pa.active) stg256(reinterpret_cast<float*>(fine_chunk + (int64_t)pa.index * W), kept_a);
        if (pb.active) stg256(reinterpret_cast<float*>(fine_chunk + (int64_t)pb.index * W), kept_b);
    }
}

// Shared memory of one upsampling block
template <int W>
struct UpShared {
    __align__(128) float tile[2][UpTile<W>::floats];
    __align__(16) float lut[kRangeLutStride];
    uint64_t bar[2];  // TMA completion of the two tile buffers
};

// One block of an upsampling step: coarse pixels x0 .. x0 + kUpTileX - 1 of coarse row y, their
// fine pixels.  Pointers are the instance's own (so.distance / so.index / so.distance2 included);
// sh.lut is filled with the level's range weights and the block synchronised before the call.
// kSelect = false: coarse float32 -> fine float32 in place (and the fine guides);
// kSelect = true: the last step, fine level-0 costs of type Tf in, the selection out.
// kWriteGuide: the filtered fine guide is formed and written (kGuideDefault: always except by
// the chunked selecting step, whose guide nothing reads; the planar one writes it as the
// reference's filter does).
template <int W, typename Tf, bool kSelect, typename GL, bool kWriteGuide, bool kTma = false>
__device__ __forceinline__ void isb_up_block(const uint8_t* __restrict__ guide_in, const float* __restrict__ cost_in,
                                             uint8_t* __restrict__ guide_io, Tf* __restrict__ cost_fine,
                                             const LevelGeom& g, int chunks, int ncand, float weight_up,
                                             float weight_down, const SelectOut& so, int x0, int y, UpShared<W>& sh,
                                             const CUtensorMap* tmap = nullptr, int plane0 = 0, bool withhold = false)
{
    static_assert(!kTma || W == 8, "TMA tiles are for the chunked layout");
    const int64_t pin = (int64_t)g.rows_in * g.cols_in, pio = (int64_t)g.rows_out * g.cols_out;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int kind = warp >> 2;  // warp-uniform
    const int lx = (warp & 3) * 32 + lane, x = x0 + lx;
    const bool coarse_ok = x < g.cols_in;
    const LutRange range{sh.lut};
    FinePixel pa, pb;
    {
        int ci[9];
        typename GL::Pix gd[9];
        if (coarse_ok) coarse_neighbourhood<int, GL>(guide_in, g.rows_in, g.cols_in, x, y, ci, gd);
        if (kind == 0) {
            fine_setup<0, kWriteGuide, GL>(gd, guide_io, g, x, y, coarse_ok, weight_up, weight_down, range, pa);
            fine_setup<3, kWriteGuide, GL>(gd, guide_io, g, x, y, coarse_ok, weight_up, weight_down, range, pb);
        } else {
            fine_setup<1, kWriteGuide, GL>(gd, guide_io, g, x, y, coarse_ok, weight_up, weight_down, range, pa);
            fine_setup<2, kWriteGuide, GL>(gd, guide_io, g, x, y, coarse_ok, weight_up, weight_down, range, pb);
        }
    }
    Selector sa, sb;
    uint32_t in_flight = 0;  // thread 0, TMA: bit b set while a copy into sh.tile[b] has not been seen to land
    if constexpr (kTma) {
        // the coarse tiles come by TMA (plane0 + c: the chunk's plane of the level's tensor map)
        if (threadIdx.x == 0) {
            mbar_init(&sh.bar[0], 1);
            mbar_init(&sh.bar[1], 1);
            mbar_init_fence();
        }
        __syncthreads();
        if (threadIdx.x == 0 && load_tile_tma(sh.tile[0], tmap, x0, y, plane0, &sh.bar[0], withhold)) in_flight = 1u;
    } else {
        load_tile_async<W>(sh.tile[0], cost_in, g.rows_in, g.cols_in, x0, y);
        cp_async_commit();
    }
    // fine cells are read once, from memory: prefetched a chunk ahead of their use
    RawCell<W, Tf> ra, rb;
    if (kSelect || pa.active) ra.load(cost_fine + (int64_t)pa.index * W);
    if (kSelect || pb.active) rb.load(cost_fine + (int64_t)pb.index * W);
    for (int c = 0; c < chunks; ++c) {
        if constexpr (kTma) {
            if (threadIdx.x == 0 && c + 1 < chunks &&
                load_tile_tma(sh.tile[(c + 1) & 1], tmap, x0, y, plane0 + c + 1, &sh.bar[(c + 1) & 1], withhold))
                in_flight |= 1u << ((c + 1) & 1);
        } else {
            if (c + 1 < chunks)
                load_tile_async<W>(sh.tile[(c + 1) & 1], cost_in + (int64_t)(c + 1) * pin * W, g.rows_in, g.cols_in,
                                   x0, y);
            cp_async_commit();
        }
        RawCell<W, Tf> na = ra, nb = rb;
        if (c + 1 < chunks) {
            const Tf* next = cost_fine + (int64_t)(c + 1) * pio * W;
            if (kSelect || pa.active) na.load(next + (int64_t)pa.index * W);
            if (kSelect || pb.active) nb.load(next + (int64_t)pb.index * W);
        }
        if constexpr (kTma) {
            // this chunk's tile has landed, for every thread of the block; else the block stops
            // here and writes nothing more (the chunks before it are written, the selection not)
            const bool landed =
                mbar_wait(&sh.bar[c & 1], (uint32_t)(c >> 1) & 1u, withhold ? kTmaShortPolls : kTmaMaxPolls);
            if (!__syncthreads_and(landed)) {
                if (threadIdx.x == 0) tma_drain(sh.bar, in_flight, c);
                return;
            }
            if (threadIdx.x == 0) in_flight &= ~(1u << (c & 1));
            tma_clamp_edges(sh.tile[c & 1], g.rows_in, g.cols_in, x0, y);
        } else {
            cp_async_wait_one();  // this chunk's tile has landed
        }
        __syncthreads();
        Tf* fine_chunk = cost_fine + (int64_t)c * pio * W;
        if (kind == 0)
            up_chunk<0, 3, W, Tf, kSelect>(sh.tile[c & 1], lx, fine_chunk, c, ncand, weight_up, pa, pb, ra, rb, sa, sb);
        else
            up_chunk<1, 2, W, Tf, kSelect>(sh.tile[c & 1], lx, fine_chunk, c, ncand, weight_up, pa, pb, ra, rb, sa, sb);
        // the edge writes of this buffer (generic proxy) are ordered before the TMA copy that
        // refills it two chunks on; the block's reads are, by the barrier
        if constexpr (kTma)
            if (x0 == 0 || x0 - 1 + kUpTileCols > g.cols_in || y == 0 || y + 1 >= g.rows_in) fence_proxy_async();
        __syncthreads();  // the tile is refilled two chunks on
        ra = na;
        rb = nb;
    }
    if constexpr (kSelect) {
        if (pa.active) {
            const float d = select_from(sa, ncand, so.d0, so.dl, so.q);
            so.distance[pa.index] = d;
            if (so.distance2) so.distance2[pa.index] = d;
            if (so.index) so.index[pa.index] = sa.idx;
        }
        if (pb.active) {
            const float d = select_from(sb, ncand, so.d0, so.dl, so.q);
            so.distance[pb.index] = d;
            if (so.distance2) so.distance2[pb.index] = d;
            if (so.index) so.index[pb.index] = sb.idx;
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Chunked upsampling with every chunk's tile staged at once (SSG_TUNE_SELECT_WHOLE for the level
// fused with the selection, SSG_TUNE_UP_WHOLE for the coarse levels; volumes of at most
// kWholeChunks chunks): the block copies the coarse neighbourhood of all its candidates with
// cp.async, waits once, and filters every chunk without a block barrier between chunks.  The
// threads, fine pixels, tile layout and arithmetic are those of isb_up_block<8, Tf, kSelect>
// (same bits); the tiles live in dynamic shared memory (12.5 KB per chunk).
// ---------------------------------------------------------------------------------------------
constexpr int kWholeChunks = 4;

template <typename Tf, bool kSelect, int kBlocks>
__global__ void __launch_bounds__(kBatchBlock, kBlocks) isb_up_whole_kernel(
    const uint8_t* __restrict__ guide_in, const float* __restrict__ cost_in, uint8_t* __restrict__ guide_fine,
    Tf* __restrict__ cost_fine, LevelGeom g, int chunks, int ncand, float weight_up, float weight_down,
    float var_inv_i, const float* __restrict__ table, SelectOut so)
{
    extern __shared__ __align__(128) float whole_smem[];
    float* lut = whole_smem;                          // kRangeLutStride floats (a multiple of 32)
    float* tiles = whole_smem + kRangeLutStride;      // chunks x UpTile<8>::floats, 128-byte aligned
    const int64_t pin = (int64_t)g.rows_in * g.cols_in, pio = (int64_t)g.rows_out * g.cols_out;
    const int inst = blockIdx.z;
    guide_in += (int64_t)inst * pin * G4::bytes;
    cost_in += (int64_t)inst * chunks * pin * 8;
    guide_fine += (int64_t)inst * pio * G4::bytes;
    cost_fine += (int64_t)inst * chunks * pio * 8;
    const int x0 = blockIdx.x * kUpTileX, y = blockIdx.y;
    // the whole neighbourhood streams in while the range table and the weights are formed
    for (int c = 0; c < chunks; ++c)
        load_tile_async<8>(tiles + c * UpTile<8>::floats, cost_in + (int64_t)c * pin * 8, g.rows_in, g.cols_in, x0, y);
    cp_async_commit();
    load_range_lut(lut, table, var_inv_i);
    __syncthreads();  // the range table is filled
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int kind = warp >> 2;  // warp-uniform
    const int lx = (warp & 3) * 32 + lane, x = x0 + lx;
    const bool coarse_ok = x < g.cols_in;
    const LutRange range{lut};
    FinePixel pa, pb;
    {
        int ci[9];
        G4::Pix gd[9];
        if (coarse_ok) coarse_neighbourhood<int, G4>(guide_in, g.rows_in, g.cols_in, x, y, ci, gd);
        // the coarse levels form the filtered fine guide; the selecting level's is never read
        constexpr bool kG = !kSelect;
        if (kind == 0) {
            fine_setup<0, kG, G4>(gd, guide_fine, g, x, y, coarse_ok, weight_up, weight_down, range, pa);
            fine_setup<3, kG, G4>(gd, guide_fine, g, x, y, coarse_ok, weight_up, weight_down, range, pb);
        } else {
            fine_setup<1, kG, G4>(gd, guide_fine, g, x, y, coarse_ok, weight_up, weight_down, range, pa);
            fine_setup<2, kG, G4>(gd, guide_fine, g, x, y, coarse_ok, weight_up, weight_down, range, pb);
        }
    }
    Selector sa, sb;
    RawCell<8, Tf> ra, rb;
    if (kSelect || pa.active) ra.load(cost_fine + (int64_t)pa.index * 8);
    if (kSelect || pb.active) rb.load(cost_fine + (int64_t)pb.index * 8);
    asm volatile("cp.async.wait_all;\n" ::);
    __syncthreads();  // every chunk's tile has landed
    for (int c = 0; c < chunks; ++c) {
        RawCell<8, Tf> na = ra, nb = rb;  // the next chunk's fine cells, a chunk ahead
        if (c + 1 < chunks) {
            const Tf* next = cost_fine + (int64_t)(c + 1) * pio * 8;
            if (kSelect || pa.active) na.load(next + (int64_t)pa.index * 8);
            if (kSelect || pb.active) nb.load(next + (int64_t)pb.index * 8);
        }
        const float* buf = tiles + c * UpTile<8>::floats;
        Tf* fine_chunk = cost_fine + (int64_t)c * pio * 8;
        if (kind == 0)
            up_chunk<0, 3, 8, Tf, kSelect>(buf, lx, fine_chunk, c, ncand, weight_up, pa, pb, ra, rb, sa, sb);
        else
            up_chunk<1, 2, 8, Tf, kSelect>(buf, lx, fine_chunk, c, ncand, weight_up, pa, pb, ra, rb, sa, sb);
        ra = na;
        rb = nb;
    }
    if constexpr (!kSelect) return;
    so.distance += (int64_t)inst * pio;
    if (so.distance2) so.distance2 += (int64_t)inst * pio;
    if (so.index) so.index += (int64_t)inst * pio;
    if (pa.active) {
        const float d = select_from(sa, ncand, so.d0, so.dl, so.q);
        so.distance[pa.index] = d;
        if (so.distance2) so.distance2[pa.index] = d;
        if (so.index) so.index[pa.index] = sa.idx;
    }
    if (pb.active) {
        const float d = select_from(sb, ncand, so.d0, so.dl, so.q);
        so.distance[pb.index] = d;
        if (so.distance2) so.distance2[pb.index] = d;
        if (so.index) so.index[pb.index] = sb.idx;
    }
}

template <typename Tf, bool kSelect, int kBlocks>
static cudaError_t launch_up_whole(dim3 grid, cudaStream_t st, const uint8_t* gi, const float* ci, uint8_t* gio, Tf* cf,
                                   const LevelGeom& g, int chunks, int ncand, float wu, float wd, float var_inv_i,
                                   const float* table, const SelectOut& so)
{
    const size_t bytes = sizeof(float) * (kRangeLutStride + (size_t)kWholeChunks * UpTile<8>::floats);
    static std::atomic<int> opted[64] = {};  // per device: the opt-in above 48 KB is set once
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < 64 && !opted[dev].load()) {
        const cudaError_t e = cudaFuncSetAttribute(isb_up_whole_kernel<Tf, kSelect, kBlocks>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
        if (e != cudaSuccess) return e;
        opted[dev].store(1);
    }
    const size_t used = sizeof(float) * (kRangeLutStride + (size_t)chunks * UpTile<8>::floats);
    isb_up_whole_kernel<Tf, kSelect, kBlocks><<<grid, kBatchBlock, used, st>>>(gi, ci, gio, cf, g, chunks, ncand, wu,
                                                                               wd, var_inv_i, table, so);
    return cudaSuccess;
}

// ---------------------------------------------------------------------------------------------
// Single-candidate upsampling (W = 1: planar one-candidate volumes and the distance post-filter).
// One thread per coarse pixel filters its four fine pixels: the 3x3 coarse guides and values are
// read once (neighbouring threads share them through L1) and each fine pixel's weights are formed
// once for its one value, with the same device functions and order as the chunked kernels.  No
// shared tile or barrier besides the range table.  Blocks of kUp1X x kUp1Y coarse pixels.
// ---------------------------------------------------------------------------------------------
constexpr int kUp1X = 32, kUp1Y = 8;

template <int F, typename GL, bool kWriteGuide, bool kCoherent = false>
__device__ __forceinline__ void up1_fine(const typename GL::Pix (&gd)[9], const float (&cv)[9],
                                         uint8_t* __restrict__ guide_io, float* __restrict__ cost_io,
                                         const LevelGeom& g, int x, int y, float weight_up, float weight_down,
                                         const LutRange& range)
{
    const int fx = 2 * x + (F >= 2 ? 1 : 0), fy = 2 * y + (F & 1);
    if (fx >= g.cols_out || fy >= g.rows_out) return;  // the clamped duplicate of another pixel
    const int index = fy * g.cols_out + fx;
    const typename GL::Pix up = GL::load(guide_io, index);
    float w[UpTaps<F>::n], gsum[3];
    const float inv = fine_weights<F, LutRange, GL>(gd, up, weight_up, weight_down, range, w, gsum);
    float acc = fmul(weight_up, kCoherent ? __ldcg(cost_io + index) : __ldg(cost_io + index));
#pragma unroll
    for (int i = 0; i < UpTaps<F>::n; ++i) acc = fadd(acc, fmul(w[i], cv[UpTaps<F>::tap(i)]));
    cost_io[index] = fmul(acc, inv);
    if (kWriteGuide) {
        uint32_t v[3];
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) v[ch] = __float2uint_rz(fmul(gsum[ch], inv));
        GL::store(guide_io, index, v);
    }
}

// coarse pixel (x, y) of one instance's level pair; `lut` is the block's filled range table
template <typename GL, bool kWriteGuide, bool kCoherent = false>
__device__ __forceinline__ void isb_up1_pixel(const uint8_t* __restrict__ guide_in, const float* __restrict__ cost_in,
                                              uint8_t* __restrict__ guide_io, float* __restrict__ cost_io,
                                              const LevelGeom& g, float weight_up, float weight_down, int x, int y,
                                              const float* lut)
{
    int ci[9];
    typename GL::Pix gd[9];
    coarse_neighbourhood<int, GL>(guide_in, g.rows_in, g.cols_in, x, y, ci, gd);
    float cv[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) cv[k] = kCoherent ? __ldcg(cost_in + ci[k]) : __ldg(cost_in + ci[k]);
    const LutRange range{lut};
    up1_fine<0, GL, kWriteGuide, kCoherent>(gd, cv, guide_io, cost_io, g, x, y, weight_up, weight_down, range);
    up1_fine<1, GL, kWriteGuide, kCoherent>(gd, cv, guide_io, cost_io, g, x, y, weight_up, weight_down, range);
    up1_fine<2, GL, kWriteGuide, kCoherent>(gd, cv, guide_io, cost_io, g, x, y, weight_up, weight_down, range);
    up1_fine<3, GL, kWriteGuide, kCoherent>(gd, cv, guide_io, cost_io, g, x, y, weight_up, weight_down, range);
}

// ---------------------------------------------------------------------------------------------
// Pyramid tails.  The small levels of a pyramid hold too little work to fill the GPU, and one
// launch per step costs more than the step: one launch runs every step from level `first` down
// to the coarsest level and back, one block per instance, the steps separated by block barriers.
// Each step calls the per-pixel functions of the per-level kernels (the same arithmetic, so the
// same bits), reading through L2 what earlier steps of the launch wrote.
// ---------------------------------------------------------------------------------------------

// chunked upsampling of coarse pixel (x, y): its four fine pixels, every chunk, with the per-
// element arithmetic of up_part (whole 8-candidate cells instead of halves; the candidates are
// independent)
template <int F>
__device__ __forceinline__ void up8_fine(const float (&tap)[9][8], const FinePixel& px, float weight_up,
                                         float* __restrict__ fine_chunk)
{
    if (!px.active) return;
    float acc[8];
    load_coherent<8>(fine_chunk + (int64_t)px.index * 8, acc);
    filter_part<F, 8, true>(tap, px.w, px.inv, weight_up, acc);
    stg256(fine_chunk + (int64_t)px.index * 8, acc);
}

__device__ __forceinline__ void isb_up8_pixel(const uint8_t* __restrict__ guide_in, const float* __restrict__ cost_in,
                                              uint8_t* __restrict__ guide_io, float* __restrict__ cost_io,
                                              const LevelGeom& g, int chunks, float weight_up, float weight_down,
                                              int x, int y, const float* lut)
{
    const int64_t pin = (int64_t)g.rows_in * g.cols_in, pio = (int64_t)g.rows_out * g.cols_out;
    int ci[9];
    G4C::Pix gd[9];
    coarse_neighbourhood<int, G4C>(guide_in, g.rows_in, g.cols_in, x, y, ci, gd);
    const LutRange range{lut};
    FinePixel px[4];
    fine_setup<0, true, G4C>(gd, guide_io, g, x, y, true, weight_up, weight_down, range, px[0]);
    fine_setup<1, true, G4C>(gd, guide_io, g, x, y, true, weight_up, weight_down, range, px[1]);
    fine_setup<2, true, G4C>(gd, guide_io, g, x, y, true, weight_up, weight_down, range, px[2]);
    fine_setup<3, true, G4C>(gd, guide_io, g, x, y, true, weight_up, weight_down, range, px[3]);
    for (int c = 0; c < chunks; ++c) {
        const float* coarse = cost_in + (int64_t)c * pin * 8;
        float* fine = cost_io + (int64_t)c * pio * 8;
        float tap[9][8];
#pragma unroll
        for (int t = 0; t < 9; ++t) load_coherent<8>(coarse + (int64_t)ci[t] * 8, tap[t]);
        up8_fine<0>(tap, px[0], weight_up, fine);
        up8_fine<1>(tap, px[1], weight_up, fine);
        up8_fine<2>(tap, px[2], weight_up, fine);
        up8_fine<3>(tap, px[3], weight_up, fine);
    }
}

// Levels of a tail: level s of instance 0 (instance i at + i x its pixels x 4 guide bytes and
// + i x chunks x its pixels x W floats)
struct TailParams {
    int levels, first, chunks;
    int rows[SSG_MAX_LEVELS], cols[SSG_MAX_LEVELS];
    uint8_t* guides[SSG_MAX_LEVELS];
    float* costs[SSG_MAX_LEVELS];
    float weight_up[SSG_MAX_LEVELS], weight_down[SSG_MAX_LEVELS];
};

template <int W>
constexpr int kTailThreads = W == 8 ? 256 : 512;

// blockIdx.x: instance.  Down steps first -> first + 1 ... levels - 2 -> levels - 1, then up steps
// levels - 1 -> levels - 2 ... first + 1 -> first (W = 1: one value per pixel, isb_up1_pixel; W = 8:
// the chunked layout, isb_up8_pixel).  The up steps form the filtered fine guides.
template <int W>
__global__ void __launch_bounds__(kTailThreads<W>) isb_tail_kernel(const __grid_constant__ TailParams T,
                                                                   float var_inv_i, const float* __restrict__ table)
{
    __shared__ __align__(16) float lut[kRangeLutStride];
    load_range_lut(lut, table, var_inv_i);
    __syncthreads();
    const int64_t inst = blockIdx.x;
    for (int s = T.first + 1; s < T.levels; ++s) {
        const LevelGeom g{T.rows[s - 1], T.cols[s - 1], T.rows[s], T.cols[s]};
        const int64_t pin = (int64_t)g.rows_in * g.cols_in, pout = (int64_t)g.rows_out * g.cols_out;
        const uint8_t* gi = T.guides[s - 1] + inst * pin * 4;
        const float* ci = T.costs[s - 1] + inst * T.chunks * pin * W;
        uint8_t* go = T.guides[s] + inst * pout * 4;
        float* co = T.costs[s] + inst * T.chunks * pout * W;
        for (int o = threadIdx.x; o < pout; o += blockDim.x)
            isb_down_pixel<W, float, G4C, true>(gi, ci, go, co, g, T.chunks, o, lut);
        __syncthreads();
    }
    for (int s = T.levels - 2; s >= T.first; --s) {
        const LevelGeom g{T.rows[s + 1], T.cols[s + 1], T.rows[s], T.cols[s]};
        const int64_t pc = (int64_t)g.rows_in * g.cols_in, pf = (int64_t)g.rows_out * g.cols_out;
        const uint8_t* gi = T.guides[s + 1] + inst * pc * 4;
        const float* ci = T.costs[s + 1] + inst * T.chunks * pc * W;
        uint8_t* gio = T.guides[s] + inst * pf * 4;
        float* cio = T.costs[s] + inst * T.chunks * pf * W;
        for (int k = threadIdx.x; k < pc; k += blockDim.x) {
            const int y = k / g.cols_in, x = k - y * g.cols_in;
            if constexpr (W == 1)
                isb_up1_pixel<G4C, true, true>(gi, ci, gio, cio, g, T.weight_up[s], T.weight_down[s], x, y, lut);
            else
                isb_up8_pixel(gi, ci, gio, cio, g, T.chunks, T.weight_up[s], T.weight_down[s], x, y, lut);
        }
        __syncthreads();
    }
}

// blockIdx.z: instance of contiguous levels
template <typename GL, bool kWriteGuide>
__global__ void __launch_bounds__(kUp1X * kUp1Y) isb_up1_kernel(const uint8_t* __restrict__ guide_in,
                                                                const float* __restrict__ cost_in,
                                                                uint8_t* __restrict__ guide_io,
                                                                float* __restrict__ cost_io, LevelGeom g,
                                                                float weight_up, float weight_down, float var_inv_i,
                                                                const float* __restrict__ table)
{
    __shared__ __align__(16) float lut[kRangeLutStride];
    load_range_lut(lut, table, var_inv_i);
    __syncthreads();
    const int x = blockIdx.x * kUp1X + (threadIdx.x % kUp1X), y = blockIdx.y * kUp1Y + (threadIdx.x / kUp1X);
    if (x >= g.cols_in || y >= g.rows_in) return;
    const int64_t pin = (int64_t)g.rows_in * g.cols_in, pio = (int64_t)g.rows_out * g.cols_out;
    const int inst = blockIdx.z;
    isb_up1_pixel<GL, kWriteGuide>(guide_in + inst * pin * GL::bytes, cost_in + inst * pin,
                                   guide_io + inst * pio * GL::bytes, cost_io + inst * pio, g, weight_up, weight_down,
                                   x, y, lut);
}

static dim3 up1_grid(int cols_in, int rows_in, int instances)
{
    return dim3((unsigned)((cols_in + kUp1X - 1) / kUp1X), (unsigned)((rows_in + kUp1Y - 1) / kUp1Y),
                (unsigned)instances);
}

template <int W, bool kSelect>
constexpr bool kGuideDefault = !kSelect || W == 1;

// blockIdx.z: instance of contiguous levels.  kBlocks: blocks per SM the registers are bounded
// for (3 for the single-candidate filter; 2 or 3 for the chunked volumes, SSG_TUNE_ISB_UP_BLOCKS and
// SSG_TUNE_ISB_SELECT_BLOCKS:
// 3 spills a few of the taps' registers for more resident warps).
template <int W, typename Tf, bool kSelect, typename GL, int kBlocks = (W == 1 ? 3 : 2),
          bool kWriteGuide = kGuideDefault<W, kSelect>, bool kTma = false>
__global__ void __launch_bounds__(kBatchBlock, kBlocks) isb_up_kernel(const uint8_t* __restrict__ guide_in,
                                                            const float* __restrict__ cost_in,
                                                            uint8_t* __restrict__ guide_io,
                                                            Tf* __restrict__ cost_fine, LevelGeom g, int chunks,
                                                            int ncand, float weight_up, float weight_down,
                                                            float var_inv_i, const float* __restrict__ table,
                                                            SelectOut so, const __grid_constant__ CUtensorMap tmap,
                                                            bool withhold)
{
    __shared__ UpShared<W> sh;
    load_range_lut(sh.lut, table, var_inv_i);
    __syncthreads();  // the range table is filled
    const int64_t pin = (int64_t)g.rows_in * g.cols_in, pio = (int64_t)g.rows_out * g.cols_out;
    const int inst = blockIdx.z;
    if (kSelect) {
        so.distance += (int64_t)inst * pio;
        if (so.distance2) so.distance2 += (int64_t)inst * pio;
        if (so.index) so.index += (int64_t)inst * pio;
    }
    isb_up_block<W, Tf, kSelect, GL, kWriteGuide, kTma>(guide_in + (int64_t)inst * pin * GL::bytes,
                                     cost_in + (int64_t)inst * chunks * pin * W,
                                     guide_io + (int64_t)inst * pio * GL::bytes,
                                     cost_fine + (int64_t)inst * chunks * pio * W, g, chunks, ncand, weight_up,
                                     weight_down, so, blockIdx.x * kUpTileX, blockIdx.y, sh, &tmap, inst * chunks,
                                     withhold);
}

// Selection from an unfiltered level-0 volume (pyramids of fewer than two levels, or the
// reference's own select_distance on a filtered planar volume)
template <int W, typename T>
__global__ void __launch_bounds__(kBatchBlock) select_kernel(const T* __restrict__ cost, int64_t P, int chunks,
                                                            int ncand, float d0, float dl, float q,
                                                            float* __restrict__ distance,
                                                            int32_t* __restrict__ index)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P) return;
    const int inst = blockIdx.y;
    cost += (int64_t)inst * chunks * P * W;
    Selector s;
    for (int c = 0; c < chunks; ++c) {
        float v[W];
        CellIO<W, T>::load(cost + ((int64_t)c * P + i) * W, v);
#pragma unroll
        for (int j = 0; j < W; ++j)
            if (c * W + j < ncand) s.push(c * W + j, v[j]);
    }
    distance[(int64_t)inst * P + i] = select_from(s, ncand, d0, dl, q);
    if (index) index[(int64_t)inst * P + i] = s.idx;
}

// ---------------------------------------------------------------------------------------------
// Uneven batches: one launch per filter step over the instances that have the step, each block
// reading its instance's LevelDesc (blockIdx.y / blockIdx.z); blocks beyond an instance's level
// size return before touching shared memory.
// ---------------------------------------------------------------------------------------------
template <int W, typename Tin>
__global__ void __launch_bounds__(kBatchBlock) isb_down_uneven_kernel(const LevelDesc* __restrict__ descs)
{
    const LevelDesc& d = descs[blockIdx.y];
    const LevelGeom g = d.g;
    const int64_t pout = (int64_t)g.rows_out * g.cols_out;
    if ((int64_t)blockIdx.x * blockDim.x >= pout) return;
    __shared__ __align__(16) float lut[kRangeLutStride];
    load_range_lut(lut, d.lut, d.var_inv_i);
    __syncthreads();
    const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= pout) return;
    isb_down_pixel<W, Tin, G4>(d.guide_in, static_cast<const Tin*>(d.cost_in), d.guide_out,
                               static_cast<float*>(d.cost_out), g, d.chunks, (int)o, lut);
}

template <int W, typename Tf, bool kSelect, int kBlocks = (W == 1 ? 3 : 2),
          bool kWriteGuide = kGuideDefault<W, kSelect>>
__global__ void __launch_bounds__(kBatchBlock, kBlocks) isb_up_uneven_kernel(const LevelDesc* __restrict__ descs)
{
    const LevelDesc& d = descs[blockIdx.z];
    const LevelGeom g = d.g;
    const int x0 = blockIdx.x * kUpTileX, y = blockIdx.y;
    if (x0 >= g.cols_in || y >= g.rows_in) return;
    __shared__ UpShared<W> sh;
    load_range_lut(sh.lut, d.lut, d.var_inv_i);
    __syncthreads();
    isb_up_block<W, Tf, kSelect, G4, kWriteGuide>(d.guide_in, static_cast<const float*>(d.cost_in), d.guide_out,
                                     static_cast<Tf*>(d.cost_out), g, d.chunks, d.ncand, d.weight_up, d.weight_down,
                                     d.so, x0, y, sh);
}

int launch_down_uneven(const LevelDesc* d_descs, int count, int max_rows_out, int max_cols_out, int width,
                       int storage_in, cudaStream_t st)
{
    SSG_REQUIRE(count >= 1 && count <= 65535, "instances out of range");
    const dim3 grid(grid_1d((int64_t)max_rows_out * max_cols_out, kBatchBlock), count);
    if (width == 1)
        isb_down_uneven_kernel<1, float><<<grid, kBatchBlock, 0, st>>>(d_descs);
    else if (storage_in == SSG_STORAGE_F16)
        isb_down_uneven_kernel<8, __half><<<grid, kBatchBlock, 0, st>>>(d_descs);
    else if (storage_in == SSG_STORAGE_UNORM16)
        isb_down_uneven_kernel<8, uint16_t><<<grid, kBatchBlock, 0, st>>>(d_descs);
    else
        isb_down_uneven_kernel<8, float><<<grid, kBatchBlock, 0, st>>>(d_descs);
    return launch_status("isb_down_uneven_kernel");
}

template <bool kWriteGuide>
__global__ void __launch_bounds__(kUp1X * kUp1Y) isb_up1_uneven_kernel(const LevelDesc* __restrict__ descs)
{
    const LevelDesc& d = descs[blockIdx.z];
    const LevelGeom g = d.g;
    const int x = blockIdx.x * kUp1X + (threadIdx.x % kUp1X), y = blockIdx.y * kUp1Y + (threadIdx.x / kUp1X);
    if ((int)(blockIdx.x * kUp1X) >= g.cols_in || (int)(blockIdx.y * kUp1Y) >= g.rows_in) return;
    __shared__ __align__(16) float lut[kRangeLutStride];
    load_range_lut(lut, d.lut, d.var_inv_i);
    __syncthreads();
    if (x >= g.cols_in || y >= g.rows_in) return;
    isb_up1_pixel<G4, kWriteGuide>(d.guide_in, static_cast<const float*>(d.cost_in), d.guide_out,
                                   static_cast<float*>(d.cost_out), g, d.weight_up, d.weight_down, x, y, lut);
}

int launch_up_uneven(const LevelDesc* d_descs, int count, int max_rows_in, int max_cols_in, int width,
                     int storage_fine, bool select, bool guide, cudaStream_t st)
{
    if (width == 1 && !select) {
        SSG_REQUIRE(count >= 1 && count <= 65535, "sizes out of range");
        const dim3 grid = up1_grid(max_cols_in, max_rows_in, count);
        if (guide) isb_up1_uneven_kernel<true><<<grid, kUp1X * kUp1Y, 0, st>>>(d_descs);
        else isb_up1_uneven_kernel<false><<<grid, kUp1X * kUp1Y, 0, st>>>(d_descs);
        return launch_status("isb_up1_uneven_kernel");
    }
    SSG_REQUIRE(count >= 1 && count <= 65535 && max_rows_in <= 65535, "sizes out of range");
    const dim3 grid((unsigned)((max_cols_in + kUpTileX - 1) / kUpTileX), (unsigned)max_rows_in, (unsigned)count);
    const bool three = tuning(select ? SSG_TUNE_ISB_SELECT_BLOCKS : SSG_TUNE_ISB_UP_BLOCKS) == 3;
    if (!select)
        three ? isb_up_uneven_kernel<8, float, false, 3><<<grid, kBatchBlock, 0, st>>>(d_descs)
              : isb_up_uneven_kernel<8, float, false, 2><<<grid, kBatchBlock, 0, st>>>(d_descs);
    else if (storage_fine == SSG_STORAGE_F16)
        three ? isb_up_uneven_kernel<8, __half, true, 3><<<grid, kBatchBlock, 0, st>>>(d_descs)
              : isb_up_uneven_kernel<8, __half, true, 2><<<grid, kBatchBlock, 0, st>>>(d_descs);
    else
        three ? isb_up_uneven_kernel<8, uint16_t, true, 3><<<grid, kBatchBlock, 0, st>>>(d_descs)
              : isb_up_uneven_kernel<8, uint16_t, true, 2><<<grid, kBatchBlock, 0, st>>>(d_descs);
    return launch_status("isb_up_uneven_kernel");
}

static int chunks_of(int n) { return (n + 7) / 8; }

// blocks of kUpTileX coarse pixels of one coarse row, per instance
static dim3 up_grid(int cols_in, int rows_in, int instances)
{
    return dim3((unsigned)((cols_in + kUpTileX - 1) / kUpTileX), (unsigned)rows_in, (unsigned)instances);
}

int level_rows(int rows, int s) { return (int)std::ceil(rows / std::pow(2.0, s)); }

// python/isb_filter.py:87-88, :110-112 in double, rounded to float32 as cupy.float32 does
Levels isb_constants(int level_count, double sigma_i, double sigma_s)
{
    Levels l{};
    const double vs = 1 / (2 * sigma_s * sigma_s), vi = 1 / (2 * sigma_i * sigma_i);
    l.var_inv_i = (float)vi;
    for (int s = 0; s + 1 < level_count; ++s) {
        const double dist = std::pow(2.0, s) - 0.5;
        const double wd = std::exp(-(dist * dist) * vs);
        l.weight_down[s] = (float)wd;
        l.weight_up[s] = (float)(1 - wd);
    }
    return l;
}

// (candidates[0] / candidates[-1] - 1) in float32, depth_estimation.py:195-196
SelectOut select_constants(const float* candidates, int ncand, float* distance, int32_t* index)
{
    const float d0 = candidates[0], dl = candidates[ncand - 1];
    return SelectOut{d0, dl, d0 / dl - 1.0f, distance, index, nullptr};
}

// chunked cost levels are read and written in whole cells: 16-byte cells of 16-bit levels,
// 32-byte cells (one 256-bit access) of float32 levels
static int check_aligned(const void* p, int bytes, const char* what)
{
    SSG_REQUIRE(((uintptr_t)p & (uintptr_t)(bytes - 1)) == 0, "%s must be %d-byte aligned", what, bytes);
    return SSG_OK;
}
static int check_cells(const void* p, int storage, const char* what)
{
    return check_aligned(p, storage == SSG_STORAGE_F32 ? 32 : 16, what);
}

static int check_levels(int rows_in, int cols_in, int rows_out, int cols_out)
{
    SSG_REQUIRE(rows_in > 0 && cols_in > 0 && rows_out > 0 && cols_out > 0, "sizes must be positive");
    SSG_REQUIRE((int64_t)rows_in * cols_in < ((int64_t)1 << 31) && rows_in <= 65535 && rows_out <= 65535,
                "a level of %dx%d pixels is too large", rows_in, cols_in);
    SSG_REQUIRE(2 * (rows_out - 1) < rows_in && 2 * (cols_out - 1) < cols_in && (rows_in + 1) / 2 <= rows_out &&
                    (cols_in + 1) / 2 <= cols_out,
                "level %dx%d is not the 2x downsampling of %dx%d", rows_out, cols_out, rows_in, cols_in);
    return SSG_OK;
}

// --- launches shared by both layouts ---------------------------------------------------------
template <int W, typename Tin, typename GL>
static int launch_down(const uint8_t* gi, const Tin* ci, int ri, int cl_i, uint8_t* go, float* co, int ro, int cl_o,
                       int chunks, int instances, float var_inv_i, cudaStream_t st)
{
    const LevelGeom g{ri, cl_i, ro, cl_o};
    const dim3 grid(grid_1d((int64_t)ro * cl_o, kBatchBlock), instances);
    isb_down_kernel<W, Tin, GL><<<grid, kBatchBlock, 0, st>>>(gi, ci, go, co, g, chunks, var_inv_i,
                                                              range_table(var_inv_i, st));
    return launch_status("isb_down_kernel");
}

// guide = false: the single-candidate step does not form the filtered fine guide
template <int W, typename Tf, bool kSelect, typename GL>
static int launch_up(const uint8_t* gi, const float* ci, int rc, int cc, uint8_t* gio, Tf* cf, int rf, int cf_cols,
                     int chunks, int ncand, int instances, float wu, float wd, float var_inv_i, const SelectOut& so,
                     cudaStream_t st, bool guide = true)
{
    const LevelGeom g{rc, cc, rf, cf_cols};
    const float* table = range_table(var_inv_i, st);
    if constexpr (W == 1 && !kSelect) {
        if (chunks == 1) {
            if (guide)
                isb_up1_kernel<GL, true><<<up1_grid(cc, rc, instances), kUp1X * kUp1Y, 0, st>>>(
                    gi, ci, gio, cf, g, wu, wd, var_inv_i, table);
            else
                isb_up1_kernel<GL, false><<<up1_grid(cc, rc, instances), kUp1X * kUp1Y, 0, st>>>(
                    gi, ci, gio, cf, g, wu, wd, var_inv_i, table);
            return launch_status("isb_up1_kernel");
        }
    }
    CUtensorMap map;
    std::memset(&map, 0, sizeof map);
    const dim3 grid = up_grid(cc, rc, instances);
    if constexpr (W == 8 && std::is_same<GL, G4>::value) {
        if (tuning(kSelect ? SSG_TUNE_SELECT_WHOLE : SSG_TUNE_UP_WHOLE) == 1 && tuning(SSG_TUNE_ISB_TILE_TMA) == 0 &&
            chunks <= kWholeChunks) {
            const bool three = tuning(kSelect ? SSG_TUNE_ISB_SELECT_BLOCKS : SSG_TUNE_ISB_UP_BLOCKS) == 3;
            const cudaError_t e =
                three ? launch_up_whole<Tf, kSelect, 3>(grid, st, gi, ci, gio, cf, g, chunks, ncand, wu, wd, var_inv_i,
                                                        table, so)
                      : launch_up_whole<Tf, kSelect, 2>(grid, st, gi, ci, gio, cf, g, chunks, ncand, wu, wd, var_inv_i,
                                                        table, so);
            if (e != cudaSuccess) return fail(SSG_ERR_CUDA, "isb_up_whole_kernel: %s", cudaGetErrorString(e));
            return launch_status(kSelect ? "isb_up_whole_kernel<select>" : "isb_up_whole_kernel");
        }
    }
    if constexpr (W == 8) {
        // the coarse level of every instance as one tensor [planes][rows][cols][8 floats], plane =
        // instance * chunks + chunk, read in boxes of 4 floats x kUpTileCols x 3 rows
        const uint64_t dims[4] = {8, (uint64_t)cc, (uint64_t)rc, (uint64_t)chunks * (uint64_t)instances};
        const uint64_t strides[3] = {32, 32ull * cc, 32ull * cc * rc};
        const uint32_t box[4] = {4, (uint32_t)kUpTileCols, 3, 1};
        const bool tma = tuning(SSG_TUNE_ISB_TILE_TMA) == 1 && encode_tensor_map(&map, ci, 4, dims, strides, box);
        const bool three = tuning(kSelect ? SSG_TUNE_ISB_SELECT_BLOCKS : SSG_TUNE_ISB_UP_BLOCKS) == 3;
        const bool withhold = tma && tuning(SSG_TUNE_TMA_WITHHOLD) == 1;
        constexpr bool kG = kGuideDefault<W, kSelect>;
        if (tma) {
            const cudaError_t e = clear_tma_abort(st);
            if (e != cudaSuccess) return fail(SSG_ERR_CUDA, "clearing the TMA abort word: %s", cudaGetErrorString(e));
        }
        if (tma && three)
            isb_up_kernel<W, Tf, kSelect, GL, 3, kG, true><<<grid, kBatchBlock, 0, st>>>(
                gi, ci, gio, cf, g, chunks, ncand, wu, wd, var_inv_i, table, so, map, withhold);
        else if (tma)
            isb_up_kernel<W, Tf, kSelect, GL, 2, kG, true><<<grid, kBatchBlock, 0, st>>>(
                gi, ci, gio, cf, g, chunks, ncand, wu, wd, var_inv_i, table, so, map, withhold);
        else if (three)
            isb_up_kernel<W, Tf, kSelect, GL, 3><<<grid, kBatchBlock, 0, st>>>(gi, ci, gio, cf, g, chunks, ncand, wu,
                                                                              wd, var_inv_i, table, so, map, false);
        else
            isb_up_kernel<W, Tf, kSelect, GL><<<grid, kBatchBlock, 0, st>>>(gi, ci, gio, cf, g, chunks, ncand, wu, wd,
                                                                           var_inv_i, table, so, map, false);
    } else {
        isb_up_kernel<W, Tf, kSelect, GL><<<grid, kBatchBlock, 0, st>>>(gi, ci, gio, cf, g, chunks, ncand, wu, wd,
                                                                       var_inv_i, table, so, map, false);
    }
    return launch_status(kSelect ? "isb_up_kernel<select>" : "isb_up_kernel");
}

// The first level of a pyramid's fused tail: the first level s >= 1 of at most `max_pixels`
// pixels, provided the tail then has a step (s <= levels - 2); otherwise `levels` (no tail).
static int tail_first(int rows, int cols, int levels, int max_pixels)
{
    if (max_pixels <= 0) return levels;
    for (int s = 1; s + 2 <= levels; ++s)
        if ((int64_t)level_rows(rows, s) * level_rows(cols, s) <= max_pixels) return s;
    return levels;
}

template <int W>
static int launch_tail(uint8_t* const* guides, float* const* costs, int levels, int first, int rows, int cols,
                       int chunks, int instances, const float* weight_up, const float* weight_down, float var_inv_i,
                       cudaStream_t st)
{
    TailParams T{};
    T.levels = levels;
    T.first = first;
    T.chunks = chunks;
    for (int s = 0; s < levels; ++s) {
        T.rows[s] = level_rows(rows, s);
        T.cols[s] = level_rows(cols, s);
        T.guides[s] = guides[s];
        T.costs[s] = costs[s];
        if (s + 1 < levels) {
            T.weight_up[s] = weight_up[s];
            T.weight_down[s] = weight_down[s];
        }
    }
    isb_tail_kernel<W><<<instances, kTailThreads<W>, 0, st>>>(T, var_inv_i, range_table(var_inv_i, st));
    return launch_status("isb_tail_kernel");
}

// the whole filter on planar levels (W = 1, chunks = candidates): python/isb_filter.py:72-136
template <typename GL>
static int apply_planar(uint8_t* const* d_guides, float* const* d_costs, int level_count, int rows, int cols,
                        int candidate_count, int instances, double sigma_i, double sigma_s, cudaStream_t st,
                        int flags = 0)
{
    const Levels c = isb_constants(level_count, sigma_i, sigma_s);
    for (int s = 1; s < level_count; ++s)
        if (int e = check_levels(level_rows(rows, s - 1), level_rows(cols, s - 1), level_rows(rows, s),
                                 level_rows(cols, s)))
            return e;
    // the batched single-candidate filter (the distance post-filter) runs its small levels as one
    // fused tail (SSG_TUNE_POST_TAIL: the largest first level, in pixels; 0 = none)
    const int first = std::is_same<GL, G4>::value && candidate_count == 1
                          ? tail_first(rows, cols, level_count, tuning(SSG_TUNE_POST_TAIL))
                          : level_count;
    for (int s = 1; s < level_count && s <= first; ++s) {
        const int ri = level_rows(rows, s - 1), ci = level_rows(cols, s - 1), ro = level_rows(rows, s),
                  co = level_rows(cols, s);
        if (int e = launch_down<1, float, GL>(d_guides[s - 1], d_costs[s - 1], ri, ci, d_guides[s], d_costs[s], ro,
                                              co, candidate_count, instances, c.var_inv_i, st))
            return e;
    }
    if (first < level_count)
        if (int e = launch_tail<1>(d_guides, d_costs, level_count, first, rows, cols, 1, instances, c.weight_up,
                                   c.weight_down, c.var_inv_i, st))
            return e;
    for (int s = (first < level_count ? first : level_count - 1) - 1; s >= 0; --s) {
        const int rc = level_rows(rows, s + 1), cc = level_rows(cols, s + 1), rf = level_rows(rows, s),
                  cf = level_rows(cols, s);
        if (int e = launch_up<1, float, false, GL>(d_guides[s + 1], d_costs[s + 1], rc, cc, d_guides[s], d_costs[s],
                                                   rf, cf, candidate_count, candidate_count, instances,
                                                   c.weight_up[s], c.weight_down[s], c.var_inv_i, SelectOut{}, st,
                                                   s > 0 || !(flags & SSG_ISB_SKIP_FINE_GUIDE)))
            return e;
    }
    return SSG_OK;
}

static int check_apply_args(uint8_t* const* d_guides, float* const* d_costs, int level_count, int rows, int cols,
                            int candidate_count, double sigma_i, double sigma_s)
{
    SSG_REQUIRE(d_guides && d_costs, "null level arrays");
    const int expected = cols > 0 && rows > 0 ? (int)(std::fmin(std::log2((double)cols), std::log2((double)rows)) - 1) : 0;
    SSG_REQUIRE(level_count == expected, "level_count %d differs from the pyramid of a %dx%d image (%d)", level_count,
                cols, rows, expected);
    SSG_REQUIRE(level_count <= SSG_MAX_LEVELS, "too many levels");
    SSG_REQUIRE(candidate_count >= 1 && candidate_count <= 65535, "candidate_count out of range");
    SSG_REQUIRE(sigma_i > 0 && sigma_s > 0, "sigmas must be positive");
    for (int s = 0; s < level_count; ++s) SSG_REQUIRE(d_guides[s] && d_costs[s], "level %d is NULL", s);
    return SSG_OK;
}

}  // namespace ssg

using namespace ssg;

// ---------------------------------------------------------------------------------------------
// One planar volume, the reference's layout (python/isb_filter.py, depth_estimation.py:179-198)
// ---------------------------------------------------------------------------------------------
extern "C" int ssg_isb_level_count(int cols, int rows)
{
    if (cols <= 0 || rows <= 0) return 0;
    return (int)(std::fmin(std::log2((double)cols), std::log2((double)rows)) - 1);
}

extern "C" int ssg_isb_downsample(const uint8_t* d_guide_in, const float* d_cost_in, int rows_in, int cols_in,
                                  uint8_t* d_guide_out, float* d_cost_out, int rows_out, int cols_out,
                                  int candidate_count, float var_inv_i, void* stream)
{
    SSG_REQUIRE(d_guide_in && d_cost_in && d_guide_out && d_cost_out, "null device pointer");
    if (int e = check_levels(rows_in, cols_in, rows_out, cols_out)) return e;
    SSG_REQUIRE(candidate_count >= 1, "candidate_count must be positive");
    return launch_down<1, float, G3>(d_guide_in, d_cost_in, rows_in, cols_in, d_guide_out, d_cost_out, rows_out, cols_out,
                                 candidate_count, 1, var_inv_i, as_stream(stream));
}

extern "C" int ssg_isb_upsample(const uint8_t* d_guide_in, const float* d_cost_in, int rows_in, int cols_in,
                                uint8_t* d_guide_inout, float* d_cost_inout, int rows_inout, int cols_inout,
                                int candidate_count, float weight_up, float weight_down, float var_inv_i,
                                void* stream)
{
    SSG_REQUIRE(d_guide_in && d_cost_in && d_guide_inout && d_cost_inout, "null device pointer");
    if (int e = check_levels(rows_inout, cols_inout, rows_in, cols_in)) return e;
    SSG_REQUIRE(candidate_count >= 1, "candidate_count must be positive");
    return launch_up<1, float, false, G3>(d_guide_in, d_cost_in, rows_in, cols_in, d_guide_inout, d_cost_inout,
                                      rows_inout, cols_inout, candidate_count, candidate_count, 1, weight_up,
                                      weight_down, var_inv_i, SelectOut{}, as_stream(stream));
}

extern "C" int ssg_isb_apply(uint8_t* const* d_guides, float* const* d_costs, int level_count, int rows, int cols,
                             int candidate_count, double sigma_i, double sigma_s, void* stream)
{
    if (int e = check_apply_args(d_guides, d_costs, level_count, rows, cols, candidate_count, sigma_i, sigma_s))
        return e;
    return apply_planar<G3>(d_guides, d_costs, level_count, rows, cols, candidate_count, 1, sigma_i, sigma_s,
                        as_stream(stream));
}

extern "C" int ssg_isb_apply_batch(uint8_t* const* d_guides, float* const* d_costs, int level_count, int rows,
                                   int cols, int candidate_count, int instances, double sigma_i, double sigma_s,
                                   int flags, void* stream)
{
    if (int e = check_apply_args(d_guides, d_costs, level_count, rows, cols, candidate_count, sigma_i, sigma_s))
        return e;
    SSG_REQUIRE(instances >= 1 && instances <= 65535, "instances out of range");
    SSG_REQUIRE((flags & ~SSG_ISB_SKIP_FINE_GUIDE) == 0, "unknown flags 0x%x", flags);
    return apply_planar<G4>(d_guides, d_costs, level_count, rows, cols, candidate_count, instances, sigma_i, sigma_s,
                        as_stream(stream), flags);
}

extern "C" int ssg_select_distance(const float* d_cost, int candidate_count, int64_t pixels, const float* candidates,
                                   float* d_distance, int32_t* d_index, void* stream)
{
    SSG_REQUIRE(d_cost && d_distance && candidates, "null pointer");
    SSG_REQUIRE(candidate_count >= 1, "candidate_count must be positive");
    SSG_REQUIRE(pixels >= 0, "negative pixel count");
    if (pixels == 0) return SSG_OK;
    const SelectOut so = select_constants(candidates, candidate_count, d_distance, d_index);
    select_kernel<1, float><<<dim3(grid_1d(pixels, kBatchBlock), 1), kBatchBlock, 0, as_stream(stream)>>>(
        d_cost, pixels, candidate_count, candidate_count, so.d0, so.dl, so.q, d_distance, d_index);
    return launch_status("select_kernel");
}

extern "C" int ssg_isb_upsample_select(const uint8_t* d_guide_in, const float* d_cost_in, int rows_in, int cols_in,
                                       uint8_t* d_guide_inout, const float* d_cost_fine, int rows_fine, int cols_fine,
                                       int candidate_count, float weight_up, float weight_down, float var_inv_i,
                                       const float* candidates, float* d_distance, int32_t* d_index, void* stream)
{
    SSG_REQUIRE(d_guide_in && d_cost_in && d_guide_inout && d_cost_fine && d_distance && candidates,
                "null pointer");
    if (int e = check_levels(rows_fine, cols_fine, rows_in, cols_in)) return e;
    SSG_REQUIRE(candidate_count >= 1, "candidate_count must be positive");
    const SelectOut so = select_constants(candidates, candidate_count, d_distance, d_index);
    return launch_up<1, float, true, G3>(d_guide_in, d_cost_in, rows_in, cols_in, d_guide_inout,
                                     const_cast<float*>(d_cost_fine), rows_fine, cols_fine, candidate_count,
                                     candidate_count, 1, weight_up, weight_down, var_inv_i, so, as_stream(stream));
}

// ---------------------------------------------------------------------------------------------
// Batches of chunked volumes (the batched path)
// ---------------------------------------------------------------------------------------------
extern "C" int ssg_isb_downsample_batch(const uint8_t* d_guide_in, const void* d_cost_in, int rows_in, int cols_in,
                                        uint8_t* d_guide_out, void* d_cost_out, int rows_out, int cols_out,
                                        int candidate_count, int instances, int storage, float var_inv_i,
                                        void* stream)
{
    SSG_REQUIRE(d_guide_in && d_cost_in && d_guide_out && d_cost_out, "null pointer");
    if (int e = check_levels(rows_in, cols_in, rows_out, cols_out)) return e;
    SSG_REQUIRE(storage == SSG_STORAGE_F16 || storage == SSG_STORAGE_UNORM16 || storage == SSG_STORAGE_F32,
                "unknown input storage %d", storage);
    SSG_REQUIRE(candidate_count >= 1 && candidate_count <= SSG_MAX_CANDIDATES, "candidate_count out of range");
    SSG_REQUIRE(instances >= 1 && instances <= 65535, "instances out of range");
    if (int e = check_cells(d_cost_in, storage, "d_cost_in")) return e;
    if (int e = check_cells(d_cost_out, SSG_STORAGE_F32, "d_cost_out")) return e;
    const int chunks = chunks_of(candidate_count);
    float* out = static_cast<float*>(d_cost_out);
    cudaStream_t st = as_stream(stream);
    if (storage == SSG_STORAGE_F16)
        return launch_down<8, __half, G4>(d_guide_in, static_cast<const __half*>(d_cost_in), rows_in, cols_in, d_guide_out,
                                      out, rows_out, cols_out, chunks, instances, var_inv_i, st);
    if (storage == SSG_STORAGE_UNORM16)
        return launch_down<8, uint16_t, G4>(d_guide_in, static_cast<const uint16_t*>(d_cost_in), rows_in, cols_in,
                                        d_guide_out, out, rows_out, cols_out, chunks, instances, var_inv_i, st);
    return launch_down<8, float, G4>(d_guide_in, static_cast<const float*>(d_cost_in), rows_in, cols_in, d_guide_out, out,
                                 rows_out, cols_out, chunks, instances, var_inv_i, st);
}

extern "C" int ssg_isb_upsample_batch(const uint8_t* d_guide_in, const void* d_cost_in, int rows_in, int cols_in,
                                      uint8_t* d_guide_inout, void* d_cost_inout, int rows_inout, int cols_inout,
                                      int candidate_count, int instances, int storage, float weight_up,
                                      float weight_down, float var_inv_i, void* stream)
{
    SSG_REQUIRE(d_guide_in && d_cost_in && d_guide_inout && d_cost_inout, "null pointer");
    if (int e = check_levels(rows_inout, cols_inout, rows_in, cols_in)) return e;
    SSG_REQUIRE(storage == SSG_STORAGE_F32, "coarse levels are float32 (storage must be SSG_STORAGE_F32)");
    SSG_REQUIRE(candidate_count >= 1 && candidate_count <= SSG_MAX_CANDIDATES, "candidate_count out of range");
    SSG_REQUIRE(instances >= 1 && instances <= 65535, "instances out of range");
    if (int e = check_aligned(d_cost_in, 16, "d_cost_in")) return e;  // staged by 16-byte copies
    if (int e = check_cells(d_cost_inout, SSG_STORAGE_F32, "d_cost_inout")) return e;
    const int chunks = chunks_of(candidate_count);
    return launch_up<8, float, false, G4>(d_guide_in, static_cast<const float*>(d_cost_in), rows_in, cols_in,
                                      d_guide_inout, static_cast<float*>(d_cost_inout), rows_inout, cols_inout, chunks,
                                      chunks * 8, instances, weight_up, weight_down, var_inv_i, SelectOut{},
                                      as_stream(stream));
}

extern "C" int ssg_isb_filter_batch(uint8_t* const* d_guides, void* const* d_costs, int level_count, int rows,
                                    int cols, int candidate_count, int instances, int storage,
                                    const float* weight_up, const float* weight_down, float var_inv_i, void* stream)
{
    SSG_REQUIRE(d_guides && d_costs && weight_up && weight_down, "null pointer");
    SSG_REQUIRE(level_count >= 2 && level_count <= SSG_MAX_LEVELS, "level_count %d outside [2, %d]", level_count,
                SSG_MAX_LEVELS);
    SSG_REQUIRE(rows > 0 && cols > 0, "sizes must be positive");
    SSG_REQUIRE(instances >= 1 && instances <= 65535, "instances out of range");
    SSG_REQUIRE(candidate_count >= 1 && candidate_count <= SSG_MAX_CANDIDATES, "candidate_count out of range");
    for (int s = 0; s < level_count; ++s) {
        SSG_REQUIRE(d_guides[s] && d_costs[s], "level %d is NULL", s);
        if (s > 0)
            if (int e = check_cells(d_costs[s], SSG_STORAGE_F32, "a float32 level")) return e;
    }
    const int chunks = chunks_of(candidate_count);
    cudaStream_t st = as_stream(stream);
    // small levels as one fused tail (SSG_TUNE_ISB_TAIL: the largest first level, in pixels)
    const int first = tail_first(rows, cols, level_count, tuning(SSG_TUNE_ISB_TAIL));
    for (int s = 1; s < level_count && s <= first; ++s)
        if (int e = ssg_isb_downsample_batch(d_guides[s - 1], d_costs[s - 1], level_rows(rows, s - 1),
                                             level_rows(cols, s - 1), d_guides[s], d_costs[s], level_rows(rows, s),
                                             level_rows(cols, s), candidate_count, instances,
                                             s == 1 ? storage : SSG_STORAGE_F32, var_inv_i, stream))
            return e;
    if (first < level_count) {
        float* costs[SSG_MAX_LEVELS] = {};
        for (int s = 1; s < level_count; ++s) costs[s] = static_cast<float*>(d_costs[s]);
        if (int e = launch_tail<8>(d_guides, costs, level_count, first, rows, cols, chunks, instances, weight_up,
                                   weight_down, var_inv_i, st))
            return e;
    }
    for (int s = (first < level_count ? first : level_count - 1) - 1; s >= 1; --s)
        if (int e = ssg_isb_upsample_batch(d_guides[s + 1], d_costs[s + 1], level_rows(rows, s + 1),
                                           level_rows(cols, s + 1), d_guides[s], d_costs[s], level_rows(rows, s),
                                           level_rows(cols, s), candidate_count, instances, SSG_STORAGE_F32,
                                           weight_up[s], weight_down[s], var_inv_i, stream))
            return e;
    return SSG_OK;
}

extern "C" int ssg_isb_upsample_select_batch(const uint8_t* d_guide_in, const void* d_cost_in, int rows_in,
                                             int cols_in, uint8_t* d_guide_inout, const void* d_cost_fine,
                                             int rows_fine, int cols_fine, int candidate_count, int instances,
                                             int storage, float weight_up, float weight_down, float var_inv_i,
                                             const float* candidates, float* d_distance, int32_t* d_index,
                                             float* d_distance_copy, void* stream)
{
    SSG_REQUIRE(d_guide_in && d_cost_in && d_guide_inout && d_cost_fine && d_distance && candidates, "null pointer");
    if (int e = check_levels(rows_fine, cols_fine, rows_in, cols_in)) return e;
    SSG_REQUIRE(storage == SSG_STORAGE_F16 || storage == SSG_STORAGE_UNORM16 || storage == SSG_STORAGE_F32,
                "unknown fine-level storage %d", storage);
    SSG_REQUIRE(candidate_count >= 1 && candidate_count <= SSG_MAX_CANDIDATES, "candidate_count out of range");
    SSG_REQUIRE(instances >= 1 && instances <= 65535, "instances out of range");
    if (int e = check_aligned(d_cost_in, 16, "d_cost_in")) return e;  // staged by 16-byte copies
    if (int e = check_cells(d_cost_fine, storage, "d_cost_fine")) return e;
    const int chunks = chunks_of(candidate_count);
    SelectOut so = select_constants(candidates, candidate_count, d_distance, d_index);
    so.distance2 = d_distance_copy;
    const float* coarse = static_cast<const float*>(d_cost_in);
    void* fine = const_cast<void*>(d_cost_fine);  // read only in the selecting variant
    cudaStream_t st = as_stream(stream);
    if (storage == SSG_STORAGE_F16)
        return launch_up<8, __half, true, G4>(d_guide_in, coarse, rows_in, cols_in, d_guide_inout,
                                          static_cast<__half*>(fine), rows_fine, cols_fine, chunks, candidate_count,
                                          instances, weight_up, weight_down, var_inv_i, so, st);
    if (storage == SSG_STORAGE_UNORM16)
        return launch_up<8, uint16_t, true, G4>(d_guide_in, coarse, rows_in, cols_in, d_guide_inout,
                                            static_cast<uint16_t*>(fine), rows_fine, cols_fine, chunks,
                                            candidate_count, instances, weight_up, weight_down, var_inv_i, so, st);
    return launch_up<8, float, true, G4>(d_guide_in, coarse, rows_in, cols_in, d_guide_inout, static_cast<float*>(fine),
                                     rows_fine, cols_fine, chunks, candidate_count, instances, weight_up, weight_down,
                                     var_inv_i, so, st);
}

extern "C" int ssg_select_distance_batch(const void* d_cost, int candidate_count, int64_t pixels, int instances,
                                         int storage, const float* candidates, float* d_distance, int32_t* d_index,
                                         void* stream)
{
    SSG_REQUIRE(d_cost && d_distance && candidates, "null pointer");
    SSG_REQUIRE(pixels > 0 && instances >= 1 && instances <= 65535, "invalid sizes");
    SSG_REQUIRE(candidate_count >= 1 && candidate_count <= SSG_MAX_CANDIDATES, "candidate_count out of range");
    SSG_REQUIRE(storage == SSG_STORAGE_F16 || storage == SSG_STORAGE_UNORM16 || storage == SSG_STORAGE_F32,
                "unknown storage %d", storage);
    if (int e = check_cells(d_cost, storage, "d_cost")) return e;
    const SelectOut so = select_constants(candidates, candidate_count, d_distance, d_index);
    const dim3 grid(grid_1d(pixels, kBatchBlock), instances);
    const int chunks = chunks_of(candidate_count);
    cudaStream_t st = as_stream(stream);
    if (storage == SSG_STORAGE_F16)
        select_kernel<8, __half><<<grid, kBatchBlock, 0, st>>>(static_cast<const __half*>(d_cost), pixels, chunks,
                                                               candidate_count, so.d0, so.dl, so.q, d_distance, d_index);
    else if (storage == SSG_STORAGE_UNORM16)
        select_kernel<8, uint16_t><<<grid, kBatchBlock, 0, st>>>(static_cast<const uint16_t*>(d_cost), pixels, chunks,
                                                                 candidate_count, so.d0, so.dl, so.q, d_distance,
                                                                 d_index);
    else
        select_kernel<8, float><<<grid, kBatchBlock, 0, st>>>(static_cast<const float*>(d_cost), pixels, chunks,
                                                              candidate_count, so.d0, so.dl, so.q, d_distance, d_index);
    return launch_status("select_kernel");
}

namespace ssg {
uint32_t take_stitch_status(cudaError_t* err);  // ssg_stitch.cu
}

extern "C" int ssg_take_device_status(uint32_t* status)
{
    SSG_REQUIRE(status, "null pointer");
    uint32_t zero = 0;
    cudaError_t e = cudaMemcpyFromSymbol(status, ssg::g_tma_status, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(ssg::g_tma_status, &zero, sizeof(uint32_t));
    if (e == cudaSuccess) *status |= ssg::take_stitch_status(&e);
    if (e != cudaSuccess) return ssg::fail(SSG_ERR_CUDA, "device status: %s", cudaGetErrorString(e));
    return SSG_OK;
}
