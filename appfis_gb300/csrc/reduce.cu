// Box reductions MAX / MIN / SUM over a padded field (the reference's Execute{1,2,3}DReduce).
//
// Reference: GPU path Appfis/Runtime_CUDA.hpp:554-740 launches one thread per element of the
// WHOLE padded array masked by the Config box, writes block partials into the grid's `next`
// buffer (so a SINGLE grid's input is overwritten), loops multi-pass kernels, then copies one
// scalar to the host and synchronises; CPU path Appfis/Runtime.hpp:597-913.  Seeds: MAX starts
// from numeric_limits<T>::min(), MIN from max(), SUM from 0 (kept here, including MAX's
// smallest-positive seed for floating types).
//
// Here: one launch.  Each block walks whole rows of the box (coalesced along x), reduces in
// registers + warp shuffles, writes one partial to a workspace array; the last block to finish
// (ticket counter) folds the partials in block order.  Fixed grid size and fixed combine order
// make the result deterministic; floating sums accumulate in double.  The input is never written.
#include <cfloat>
#include <climits>
#include <mutex>
#include <type_traits>

#include "gb_common.cuh"

namespace {

template <class T> struct Acc { typedef double type; };
template <> struct Acc<int32_t> { typedef long long type; };

template <class T> __device__ __forceinline__ T max_seed();
template <> __device__ __forceinline__ float max_seed<float>() { return FLT_MIN; }
template <> __device__ __forceinline__ double max_seed<double>() { return DBL_MIN; }
template <> __device__ __forceinline__ int32_t max_seed<int32_t>() { return INT_MIN; }
template <class T> __device__ __forceinline__ T min_seed();
template <> __device__ __forceinline__ float min_seed<float>() { return FLT_MAX; }
template <> __device__ __forceinline__ double min_seed<double>() { return DBL_MAX; }
template <> __device__ __forceinline__ int32_t min_seed<int32_t>() { return INT_MAX; }

template <class T, int OP>
__device__ __forceinline__ typename Acc<T>::type seed()
{
    typedef typename Acc<T>::type A;
    return OP == APPFIS_GB_MAX ? (A)max_seed<T>() : (OP == APPFIS_GB_MIN ? (A)min_seed<T>() : (A)0);
}

template <int OP, class A>
__device__ __forceinline__ A combine(A a, A b)
{
    return OP == APPFIS_GB_MAX ? (b > a ? b : a) : (OP == APPFIS_GB_MIN ? (b < a ? b : a) : a + b);
}

template <int OP, class A>
__device__ __forceinline__ A block_reduce(A v, A neutral, A* sh)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = combine<OP>(v, __shfl_down_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : neutral;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = combine<OP>(v, __shfl_down_sync(0xffffffffu, v, o));
    }
    return v;
}

template <class T, int OP>
__global__ void __launch_bounds__(256) reduce_box(const T* __restrict__ f, int px, int py, int x0, int x1, int y0, int y1,
                                                  int z0, int z1, typename Acc<T>::type* __restrict__ partials,
                                                  unsigned* __restrict__ ticket, void* __restrict__ result)
{
    typedef typename Acc<T>::type A;
    __shared__ A sh[32];
    __shared__ bool last;
    A v = seed<T, OP>();
    const int nyb = y1 - y0;
    const long long rows = (long long)nyb * (z1 - z0);
    for (long long r = blockIdx.x; r < rows; r += gridDim.x) {
        const int j = y0 + (int)(r % nyb), k = z0 + (int)(r / nyb);
        const T* row = f + ((size_t)k * py + j) * (size_t)px;
        for (int i = x0 + threadIdx.x; i < x1; i += blockDim.x) v = combine<OP>(v, (A)__ldg(row + i));
    }
    v = block_reduce<OP>(v, seed<T, OP>(), sh);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = v;
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    A w = seed<T, OP>();
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) w = combine<OP>(w, ((volatile A*)partials)[b]);
    __syncthreads();
    w = block_reduce<OP>(w, seed<T, OP>(), sh);
    if (threadIdx.x == 0) {
        if (std::is_floating_point<A>::value) *reinterpret_cast<double*>(result) = (double)w;
        else *reinterpret_cast<long long*>(result) = (long long)w;
        *ticket = 0;  // ready for the next call
    }
}

constexpr int RED_THREADS = 256;

template <class T>
int launch_reduce(const void* field, int px, int py, const int* b, int op, void* res, cudaStream_t st)
{
    typedef typename Acc<T>::type A;
    const long long rows = (long long)(b[3] - b[2]) * (b[5] - b[4]);
    const int grid = (int)std::max<long long>(1, std::min<long long>(rows, (long long)gb::sm_count() * 4));
    void* ws;
    GB_TRY(gb::workspace(gb::WS_REDUCE, 256 + sizeof(A) * (size_t)grid, &ws));
    unsigned* ticket = reinterpret_cast<unsigned*>(ws);
    A* partials = reinterpret_cast<A*>(reinterpret_cast<char*>(ws) + 256);
    GB_CUDA(cudaMemsetAsync(ticket, 0, sizeof(unsigned), st));
    const T* f = reinterpret_cast<const T*>(field);
    switch (op) {
    case APPFIS_GB_MAX:
        reduce_box<T, APPFIS_GB_MAX><<<grid, RED_THREADS, 0, st>>>(f, px, py, b[0], b[1], b[2], b[3], b[4], b[5], partials, ticket, res);
        break;
    case APPFIS_GB_MIN:
        reduce_box<T, APPFIS_GB_MIN><<<grid, RED_THREADS, 0, st>>>(f, px, py, b[0], b[1], b[2], b[3], b[4], b[5], partials, ticket, res);
        break;
    default:
        reduce_box<T, APPFIS_GB_SUM><<<grid, RED_THREADS, 0, st>>>(f, px, py, b[0], b[1], b[2], b[3], b[4], b[5], partials, ticket, res);
    }
    return gb::launched("reduce_box");
}

// ---------------------------------------------------------------- allocation-free variant
// Some callers cannot allocate device memory at the moment they need a reduction: a host
// framework whose caching allocator has reserved the device memory, a library embedded in a
// runtime that owns every allocation, or a latency-critical loop that cannot take the implicit
// synchronisation of a first cudaMalloc/cudaFree.  For them the same reduction kernel can take
// its scratch (one ticket counter and one partial per block) from a fixed array that is part of
// the library image instead of the grow-only workspace.  64 KiB holds the ticket and 8160
// partials; the kernel uses at most 4 blocks per SM (608 on a GB300), so every box fits on
// current GPUs.  Every device that loads the library keeps this array until the process exits
// (under lazy module loading the runtime commits it on the first use of the module on a device).
constexpr size_t NOALLOC_SCRATCH_BYTES = 64 * 1024;
constexpr size_t NOALLOC_MAX_PARTIALS = (NOALLOC_SCRATCH_BYTES - 256) / sizeof(double);
static __device__ __align__(256) unsigned char g_reduce_scratch[NOALLOC_SCRATCH_BYTES];

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_addr[NOALLOC_MAX_DEVICES] = {};

// Device address of the scratch array on the current device.  On the host the array's name
// only stands for the symbol, so its address is looked up once per device (first call on that
// device, with it current) and cached.
int noalloc_scratch(void** out)
{
    int dev = 0;
    GB_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return gb::fail(APPFIS_GB_EINVAL, "reduce_noalloc: device %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_reduce_scratch);
        if (e != cudaSuccess || !p) return gb::cuda_status(e != cudaSuccess ? e : cudaErrorInvalidSymbol, "cudaGetSymbolAddress(reduce scratch)");
        g_noalloc_addr[dev] = p;
    }
    *out = g_noalloc_addr[dev];
    return APPFIS_GB_OK;
}

template <class T>
int launch_reduce_noalloc(const void* field, int px, int py, const int* b, int op, void* res, cudaStream_t st)
{
    typedef typename Acc<T>::type A;
    const long long rows = (long long)(b[3] - b[2]) * (b[5] - b[4]);
    const int grid = (int)std::max<long long>(1, std::min<long long>(rows, (long long)gb::sm_count() * 4));
    if ((size_t)grid > NOALLOC_MAX_PARTIALS)
        return gb::fail(APPFIS_GB_EINVAL, "reduce_noalloc: %d partial sums needed, the fixed scratch holds %zu", grid,
                        NOALLOC_MAX_PARTIALS);
    void* ws = nullptr;
    GB_TRY(noalloc_scratch(&ws));
    unsigned* ticket = reinterpret_cast<unsigned*>(ws);
    A* partials = reinterpret_cast<A*>(reinterpret_cast<char*>(ws) + 256);
    GB_CUDA(cudaMemsetAsync(ticket, 0, sizeof(unsigned), st));  // the array keeps the last call's contents
    const T* f = reinterpret_cast<const T*>(field);
    switch (op) {
    case APPFIS_GB_MAX:
        reduce_box<T, APPFIS_GB_MAX><<<grid, RED_THREADS, 0, st>>>(f, px, py, b[0], b[1], b[2], b[3], b[4], b[5], partials, ticket, res);
        break;
    case APPFIS_GB_MIN:
        reduce_box<T, APPFIS_GB_MIN><<<grid, RED_THREADS, 0, st>>>(f, px, py, b[0], b[1], b[2], b[3], b[4], b[5], partials, ticket, res);
        break;
    default:
        reduce_box<T, APPFIS_GB_SUM><<<grid, RED_THREADS, 0, st>>>(f, px, py, b[0], b[1], b[2], b[3], b[4], b[5], partials, ticket, res);
    }
    return gb::launched("reduce_box (fixed scratch)");
}

}  // namespace

extern "C" {

int appfis_gb_reduce_noalloc(const void* field, int dtype, int px, int py, const int* box, int op, void* dev_result,
                             void* stream)
{
    if (!field || !box || !dev_result) return gb::fail(APPFIS_GB_EINVAL, "reduce_noalloc: null argument");
    if (op < APPFIS_GB_MAX || op > APPFIS_GB_SUM) return gb::fail(APPFIS_GB_EINVAL, "reduce_noalloc: unknown op %d", op);
    for (int a = 0; a < 3; a++)
        if (box[2 * a] < 0 || box[2 * a + 1] < box[2 * a]) return gb::fail(APPFIS_GB_EINVAL, "reduce_noalloc: bad box axis %d", a);
    if (box[1] > px || box[3] > py || px < 1 || py < 1) return gb::fail(APPFIS_GB_EINVAL, "reduce_noalloc: box outside the field");
    if (box[0] == box[1] || box[2] == box[3] || box[4] == box[5]) return gb::fail(APPFIS_GB_EINVAL, "reduce_noalloc: empty box");
    cudaStream_t st = gb::as_stream(stream);
    switch (dtype) {
    case APPFIS_GB_F32: return launch_reduce_noalloc<float>(field, px, py, box, op, dev_result, st);
    case APPFIS_GB_F64: return launch_reduce_noalloc<double>(field, px, py, box, op, dev_result, st);
    case APPFIS_GB_I32: return launch_reduce_noalloc<int32_t>(field, px, py, box, op, dev_result, st);
    default: return gb::fail(APPFIS_GB_EINVAL, "reduce_noalloc: unknown dtype %d", dtype);
    }
}

int appfis_gb_reduce(const void* field, int dtype, int px, int py, const int* box, int op, void* dev_result, void* stream)
{
    if (!field || !box || !dev_result) return gb::fail(APPFIS_GB_EINVAL, "reduce: null argument");
    if (op < APPFIS_GB_MAX || op > APPFIS_GB_SUM) return gb::fail(APPFIS_GB_EINVAL, "reduce: unknown op %d", op);
    for (int a = 0; a < 3; a++)
        if (box[2 * a] < 0 || box[2 * a + 1] < box[2 * a]) return gb::fail(APPFIS_GB_EINVAL, "reduce: bad box axis %d", a);
    if (box[1] > px || box[3] > py || px < 1 || py < 1) return gb::fail(APPFIS_GB_EINVAL, "reduce: box outside the field");
    if (box[0] == box[1] || box[2] == box[3] || box[4] == box[5])
        return gb::fail(APPFIS_GB_EINVAL, "reduce: empty box");
    cudaStream_t st = gb::as_stream(stream);
    switch (dtype) {
    case APPFIS_GB_F32: return launch_reduce<float>(field, px, py, box, op, dev_result, st);
    case APPFIS_GB_F64: return launch_reduce<double>(field, px, py, box, op, dev_result, st);
    case APPFIS_GB_I32: return launch_reduce<int32_t>(field, px, py, box, op, dev_result, st);
    default: return gb::fail(APPFIS_GB_EINVAL, "reduce: unknown dtype %d", dtype);
    }
}

int appfis_gb_reduce_host(const void* field, int dtype, int px, int py, const int* box, int op, double* result, void* stream)
{
    if (!result) return gb::fail(APPFIS_GB_EINVAL, "reduce_host: null result");
    void* d;
    GB_TRY(gb::workspace(gb::WS_JOB_F, 64, &d));
    cudaStream_t st = gb::as_stream(stream);
    GB_TRY(appfis_gb_reduce(field, dtype, px, py, box, op, d, st));
    union { double f; long long i; } u;
    GB_CUDA(cudaMemcpyAsync(&u, d, 8, cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    *result = dtype == APPFIS_GB_I32 ? (double)u.i : u.f;
    return APPFIS_GB_OK;
}

}  // extern "C"
