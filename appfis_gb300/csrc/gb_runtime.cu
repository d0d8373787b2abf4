// Runtime plumbing of the C ABI: last-error message, status helpers, grow-only workspace.
//
// The reference keeps one CUDA stream in a singleton (Appfis/Topology.hpp:104-151) and ignores
// CUDA return codes after initialisation; here every call returns a status and the message of
// the last failure is kept per host thread.
#include <mutex>
#include <vector>

#include "gb_common.cuh"

namespace gb {

static thread_local std::string t_last_error;

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

}  // namespace gb

extern "C" {

const char* appfis_gb_last_error(void) { return gb::t_last_error.c_str(); }

int appfis_gb_version(void) { return 10000; }

int appfis_gb_stream_sync(void* stream)
{
    return gb::cuda_status(cudaStreamSynchronize(gb::as_stream(stream)), "cudaStreamSynchronize");
}

}  // extern "C"
