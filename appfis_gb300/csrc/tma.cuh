// Tensor-memory-accelerator (TMA) plumbing: host-side tensor-map encoding and the device-side
// mbarrier / bulk-tensor-copy primitives (inline PTX, sm_90 and later; used here for sm_103a).
//
// A CTA stages tiles of several fields into shared memory with cp.async.bulk.tensor; each
// pipeline stage has one mbarrier that thread 0 arms with the stage's byte count before it
// issues the copies, and that every consumer waits on with the stage's phase parity.  Waits
// are bounded (about one second of wall clock); a wait that gives up is reported through the
// library's device status word, never by trapping.
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>

#include "gb_common.cuh"

namespace gb {

// Encodes a 3-D tiled tensor map over a padded field: x fastest, extents dx/dy/dz elements,
// row stride `pitch` elements, plane stride pitch*py elements, box bx x by x 1, zero fill
// outside the extents.  The base must be 16-byte aligned and pitch*esize a multiple of 16.
int tensor_map_3d(CUtensorMap* map, CUtensorMapDataType type, size_t esize, const void* base, uint64_t dx, uint64_t dy,
                  uint64_t dz, uint64_t pitch, uint64_t py, uint32_t bx, uint32_t by);

// Device status word of the current device (zeroed at creation).  Kernels set bits in it when
// a bounded wait gives up; appfis_gb_stream_sync and the _job entry points report and clear it.
int status_word(unsigned** out);
// Reads and clears the current device's status word after the work that may set it has
// finished; returns APPFIS_GB_ETIMEOUT (with `what` in the message) if a bit was set.
int check_status(const char* what);

enum StatusBits : unsigned { ST_TMA_TIMEOUT = 1u, ST_SMEM_ALIGN = 2u };

inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

namespace tma {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void bar_init(uint64_t* bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Makes initialised barriers visible to the other threads and to the async (TMA) proxy.
__device__ __forceinline__ void fence_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Arrives once on `bar` and adds `bytes` to the transaction count of its current phase.
__device__ __forceinline__ void arrive_expect(uint64_t* bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// Copies the box at element coordinates (x, y, z) of `map` into shared memory at dst (128-byte
// aligned); completion is signalled on `bar` as transaction bytes.  x * element size must be a
// multiple of 16 bytes.
__device__ __forceinline__ void load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

// Copies `bytes` (a multiple of 16) from global src to shared dst, both 16-byte aligned, as one
// bulk copy; completion is signalled on `bar` as transaction bytes.
__device__ __forceinline__ void load_1d(void* dst, const void* src, unsigned bytes, uint64_t* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
                 "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void prefetch_map(const CUtensorMap* map)
{
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// Tests the phase; a thread whose phase is not complete is suspended (up to ~0.5 ms, woken
// early when the phase completes), so waiting warps do not spin on the issue slots that the
// working warps need.
__device__ __forceinline__ bool try_wait(uint64_t* bar, unsigned parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\tselp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity), "r"(500000u)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Waits for the phase with `parity` of `bar` to complete; gives up after `limit_ns` of wall
// clock (default one second; at most 2^22 tests) and returns false.
constexpr uint64_t DRAIN_NS = 10000000ull;  // 10 ms: waits for copies in flight after a failure
__device__ __forceinline__ bool wait(uint64_t* bar, unsigned parity, uint64_t limit_ns = 1000000000ull)
{
    if (try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (unsigned n = 0; n < (1u << 22); n++) {
        if (try_wait(bar, parity)) return true;
        if (global_ns() - t0 > limit_ns) break;
    }
    return false;
}

}  // namespace tma
}  // namespace gb
