// Tensor-memory-accelerator (TMA) tile loads with mbarrier completion, for kernels that stage
// tiles of a chunked cost level in shared memory (cp.async.bulk.tensor, sm_90 and later).
//
// Host: tensor maps are encoded with the driver's cuTensorMapEncodeTiled, looked up once through
// the runtime (no link against the driver library).  Device: one elected thread arms an mbarrier
// with the expected byte count and issues the copies; every thread waits on the barrier's phase
// with a bounded number of polls.  A wait that runs out records kTmaTimeout in the translation
// unit's status word (g_tma_status, sticky until ssg_take_device_status reads and clears it) and
// raises the launch's abort word (g_tma_abort, cleared by the host before every launch that
// waits on TMA tiles, so it only shortens the waits of the launch that failed).  The block then
// writes nothing more: it stops issuing copies, waits (again bounded) for the copies it has in
// flight so that none lands in shared memory after it exits, and returns.
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>

#include "ssg_common.cuh"

namespace ssg {

constexpr uint32_t kTmaTimeout = SSG_STATUS_TMA_TIMEOUT;
constexpr int kTmaMaxPolls = 1 << 20;   // each poll may suspend the thread for a short while
constexpr int kTmaShortPolls = 4096;    // the limit while a copy is withheld on purpose (tests)

static __device__ uint32_t g_tma_status;  // sticky: kTmaTimeout once any wait ran out
static __device__ uint32_t g_tma_abort;   // nonzero once a wait of the current launch ran out

// Encodes a map of a float32 tensor of `rank` dims (dims[0] innermost, strides in bytes for dims
// 1..rank-1) read in boxes of `box`; returns false when the driver refuses it.
bool encode_tensor_map(CUtensorMap* map, const void* base, int rank, const uint64_t* dims, const uint64_t* strides,
                       const uint32_t* box);

__device__ __forceinline__ uint32_t smem_address(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_address(bar)), "r"(count) : "memory");
}

// the barrier initialisation is visible to the async proxy (TMA) before any copy completes on it
__device__ __forceinline__ void mbar_init_fence()
{
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

// shared-memory writes of this thread are ordered before later async-proxy (TMA) writes
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_address(bar)), "r"(bytes)
                 : "memory");
}

// 4-D tile load: box at coordinates (c0 innermost .. c3) into dst (128-byte aligned), completing
// on bar
__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];\n" ::"r"(smem_address(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_address(bar))
        : "memory");
}

// Waits for the barrier phase of parity `parity`, at most `max_polls` polls; false when the polls
// ran out (recorded in g_tma_status and g_tma_abort).  `early_out`: also false at once when
// another wait of this launch has run out, so that a broken copy costs one bounded wait per
// resident block rather than one per tile.  Waits for copies already issued (the drain before a
// failed block exits) pass early_out = false.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int max_polls = kTmaMaxPolls,
                                          bool early_out = true)
{
    const uint32_t a = smem_address(bar);
    for (int i = 0; i < max_polls; ++i) {
        if (early_out && (i & 1023) == 0 && *reinterpret_cast<volatile uint32_t*>(&g_tma_abort) != 0) return false;
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    atomicOr(&g_tma_status, kTmaTimeout);
    atomicExch(&g_tma_abort, 1u);
    return false;
}

// Clears the abort word before a launch that waits on TMA tiles (a one-thread kernel enqueued on
// its stream, so a captured graph clears it on every replay).  Launches on other streams share the word: a clear
// can only lengthen another launch's failed waits, never hide a failure, which g_tma_status keeps.
cudaError_t clear_tma_abort(cudaStream_t st);

}  // namespace ssg
