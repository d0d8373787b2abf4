// Runtime plumbing of the C ABI: last-error message, status helpers, grow-only workspace.
//
// The reference keeps one CUDA stream in a singleton (Appfis/Topology.hpp:104-151) and ignores
// CUDA return codes after initialisation; here every call returns a status and the message of
// the last failure is kept per host thread.
#include <mutex>
#include <vector>

#include "gb_common.cuh"
#include "tma.cuh"

namespace gb {

static thread_local std::string t_last_error;

namespace {
std::mutex g_test_mu;
int g_test_kind = TEST_NONE;
unsigned long long g_test_limit = 0;
}  // namespace

bool take_test_stall(int kind, unsigned long long* limit)
{
    std::lock_guard<std::mutex> lk(g_test_mu);
    if (g_test_kind != kind) return false;
    *limit = g_test_limit;
    g_test_kind = TEST_NONE;
    return true;
}

int fail(int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    t_last_error = buf;
    return code;
}

int cuda_status(cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return APPFIS_GB_OK;
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return fail(APPFIS_GB_ENOMEM, "%s: %s", what, cudaGetErrorString(e));
    }
    return fail(APPFIS_GB_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}

namespace {
struct Buf {
    void* p = nullptr;
    size_t n = 0;
};
std::mutex g_mu;
std::vector<std::vector<Buf>> g_dev;  // [device][slot]
Buf g_pinned[2];
std::vector<int> g_sms;
std::vector<unsigned*> g_status;  // [device]
std::vector<cudaStream_t> g_job_streams;  // [device]
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_encode_once;
}  // namespace

int workspace(int slot, size_t bytes, void** out)
{
    if (slot < 0 || slot >= WS_SLOTS) return fail(APPFIS_GB_EINVAL, "workspace slot %d", slot);
    int dev = 0;
    GB_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_mu);
    if ((int)g_dev.size() <= dev) g_dev.resize(dev + 1, std::vector<Buf>(WS_SLOTS));
    Buf& b = g_dev[dev][slot];
    if (b.n < bytes) {
        if (b.p) {
            cudaError_t e = cudaFree(b.p);
            b.p = nullptr;
            b.n = 0;
            GB_TRY(cuda_status(e, "cudaFree(workspace)"));
        }
        size_t want = bytes < 256 ? 256 : bytes;
        GB_TRY(cuda_status(cudaMalloc(&b.p, want), "cudaMalloc(workspace)"));
        b.n = want;
    }
    *out = b.p;
    return APPFIS_GB_OK;
}

int pinned(int slot, size_t bytes, void** out)
{
    if (slot < 0 || slot > 1) return fail(APPFIS_GB_EINVAL, "pinned slot %d", slot);
    std::lock_guard<std::mutex> lk(g_mu);
    Buf& b = g_pinned[slot];
    if (b.n < bytes) {
        if (b.p) {
            cudaFreeHost(b.p);
            b.p = nullptr;
            b.n = 0;
        }
        GB_TRY(cuda_status(cudaMallocHost(&b.p, bytes), "cudaMallocHost(staging)"));
        b.n = bytes;
    }
    *out = b.p;
    return APPFIS_GB_OK;
}

int sm_count()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 152;
    std::lock_guard<std::mutex> lk(g_mu);
    if ((int)g_sms.size() <= dev) g_sms.resize(dev + 1, 0);
    if (g_sms[dev] == 0) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
        g_sms[dev] = n;
    }
    return g_sms[dev];
}

int job_stream(cudaStream_t* out)
{
    int dev = 0;
    GB_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_mu);
    if ((int)g_job_streams.size() <= dev) g_job_streams.resize(dev + 1, nullptr);
    if (!g_job_streams[dev]) GB_CUDA(cudaStreamCreateWithFlags(&g_job_streams[dev], cudaStreamNonBlocking));
    *out = g_job_streams[dev];
    return APPFIS_GB_OK;
}

int status_word(unsigned** out)
{
    int dev = 0;
    GB_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_mu);
    if ((int)g_status.size() <= dev) g_status.resize(dev + 1, nullptr);
    if (!g_status[dev]) {
        unsigned* p = nullptr;
        GB_TRY(cuda_status(cudaMalloc(&p, 256), "cudaMalloc(status word)"));
        GB_TRY(cuda_status(cudaMemset(p, 0, 256), "cudaMemset(status word)"));
        g_status[dev] = p;
    }
    *out = g_status[dev];
    return APPFIS_GB_OK;
}

int check_status(const char* what)
{
    int dev = 0;
    GB_CUDA(cudaGetDevice(&dev));
    unsigned* p = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if ((int)g_status.size() > dev) p = g_status[dev];
    }
    if (!p) return APPFIS_GB_OK;
    unsigned v = 0;
    GB_CUDA(cudaMemcpy(&v, p, sizeof v, cudaMemcpyDeviceToHost));
    if (v == 0) return APPFIS_GB_OK;
    GB_CUDA(cudaMemset(p, 0, sizeof v));
    return fail(APPFIS_GB_ETIMEOUT, "%s: a device-side wait gave up (status 0x%x: %s)", what, v,
                (v & ST_SMEM_ALIGN) ? "shared-memory staging misaligned" : "bulk copy did not complete within 1 s");
}

int tensor_map_3d(CUtensorMap* map, CUtensorMapDataType type, size_t esize, const void* base, uint64_t dx, uint64_t dy,
                  uint64_t dz, uint64_t pitch, uint64_t py, uint32_t bx, uint32_t by)
{
    std::call_once(g_encode_once, [] {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
        cudaGetLastError();
    });
    if (!g_encode) return fail(APPFIS_GB_ECUDA, "cuTensorMapEncodeTiled is not available from the driver");
    if (!aligned16(base) || (pitch * esize) % 16 != 0)
        return fail(APPFIS_GB_EINVAL, "tensor map: base or row stride not 16-byte aligned");
    const cuuint64_t dims[3] = {dx, dy, dz};
    const cuuint64_t strides[2] = {pitch * esize, pitch * py * esize};
    const cuuint32_t box[3] = {bx, by, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = g_encode(map, type, 3, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(APPFIS_GB_ECUDA, "cuTensorMapEncodeTiled failed (CUresult %d)", (int)r);
    return APPFIS_GB_OK;
}

}  // namespace gb

extern "C" {

const char* appfis_gb_last_error(void) { return gb::t_last_error.c_str(); }

int appfis_gb_version(void) { return 10000; }

int appfis_gb_stream_sync(void* stream)
{
    GB_CUDA(cudaStreamSynchronize(gb::as_stream(stream)));
    return gb::check_status("appfis_gb_stream_sync");
}

int appfis_gb_test_stall_next(int kind, unsigned long long limit)
{
    if (kind != gb::TEST_NONE && kind != gb::TEST_FLOOD_BARRIER && kind != gb::TEST_TMA_SHORTFALL)
        return gb::fail(APPFIS_GB_EINVAL, "test_stall_next: kind %d", kind);
    if (kind == gb::TEST_FLOOD_BARRIER && (limit < 1 || limit > (1ull << 20)))
        return gb::fail(APPFIS_GB_EINVAL, "test_stall_next: barrier poll limit %llu (1 .. 2^20)", limit);
    if (kind == gb::TEST_TMA_SHORTFALL && (limit < 1000 || limit > 100000000ull))
        return gb::fail(APPFIS_GB_EINVAL, "test_stall_next: wait limit %llu ns (1 us .. 100 ms)", limit);
    std::lock_guard<std::mutex> lk(gb::g_test_mu);
    gb::g_test_kind = kind;
    gb::g_test_limit = limit;
    return APPFIS_GB_OK;
}

}  // extern "C"
