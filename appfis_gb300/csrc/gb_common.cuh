// Shared plumbing of the C-ABI library: status codes, the last-error message, argument checks,
// CUDA error capture and a grow-only per-device workspace.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <string>

#include "appfis_gb.h"

namespace gb {

// Records msg as this thread's last error and returns `code`.
int fail(int code, const char* fmt, ...);
// Returns OK, or records the CUDA error of `e` (with `what`) and returns APPFIS_GB_ECUDA.
int cuda_status(cudaError_t e, const char* what);
// Checks the launch that just happened on this thread.
inline int launched(const char* what) { return cuda_status(cudaGetLastError(), what); }

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Device workspace: one grow-only allocation per (device, slot), reused across calls.  Calls
// that use the same slot on the same device must not overlap on the GPU.
enum Slot { WS_REDUCE = 0, WS_JOB_A, WS_JOB_B, WS_JOB_C, WS_JOB_D, WS_JOB_E, WS_JOB_F, WS_LIFE_C, WS_LIFE_D, WS_LIFE_E, WS_LIFE_F, WS_FLOOD_Z, WS_FLOOD_SRC, WS_F64_PARTIALS, WS_FLOOD_MAPS, WS_SLOTS };
int workspace(int slot, size_t bytes, void** out);
// Pinned host staging buffer, grow-only, per slot (0..1).
int pinned(int slot, size_t bytes, void** out);

inline unsigned ceil_div(size_t a, size_t b) { return (unsigned)((a + b - 1) / b); }

// Splits n planes into the fewest chunks of at most `target` planes, all of (nearly) equal size,
// and returns the chunk size.
inline int balanced_chunk(int n, int target)
{
    const int chunks = (n + target - 1) / target;
    return (n + chunks - 1) / chunks;
}

// Chunk size for a grid with `per_chunk` CTAs per chunk of planes: among the balanced chunks of
// about lo..hi planes (steps of 8), the one whose grid fills `slots` resident CTAs best over its
// waves, counting the `halo` planes each chunk reads beyond its own as waste.
inline int wave_chunk(int n, int lo, int hi, long long per_chunk, long long slots, int halo)
{
    int best = balanced_chunk(n, lo);
    double score = -1.0;
    for (int t = lo; t <= hi; t += 8) {
        const int kz = balanced_chunk(n, t), chunks = (n + kz - 1) / kz;
        const long long ctas = per_chunk * chunks, waves = (ctas + slots - 1) / slots;
        const double sc = (double)ctas / (double)(waves * slots) * kz / (kz + halo);
        if (sc > score + 1e-9) {
            score = sc;
            best = kz;
        }
    }
    return best;
}

// Number of SMs of the current device (cached).
int sm_count();

// The non-blocking stream the _job entry points run on, one per device (created on first use).
int job_stream(cudaStream_t* out);

// Test plan of the bounded device-side waits (set by appfis_gb_test_stall_next): returns true,
// with the plan's limit, once for the next call of the given kind, and clears the plan.
enum TestStall { TEST_NONE = 0, TEST_FLOOD_BARRIER = 1, TEST_TMA_SHORTFALL = 2 };
bool take_test_stall(int kind, unsigned long long* limit);

#define GB_TRY(expr)                 \
    do {                             \
        int _st = (expr);            \
        if (_st != APPFIS_GB_OK)     \
            return _st;              \
    } while (0)

#define GB_CUDA(expr) GB_TRY(::gb::cuda_status((expr), #expr))

}  // namespace gb
