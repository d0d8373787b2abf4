// 2-D heat (explicit 5-point Jacobi, FP32) on a DUAL grid with a Dirichlet ghost ring.
//
// Reference functor: HeatDiffusion/src/heat_appfis.hpp:166-174 (3-D FP64), restated in 2-D FP32:
//     next = c + cx*((l + r) - 2c) + cy*((u + d) - 2c)
// driven once per iteration by Execute2D -> Kernel2D (Appfis/Runtime_CUDA.hpp:345-369,1217-1230).
// The arithmetic below uses explicit round-to-nearest intrinsics in exactly that order (no FMA
// contraction), so every point is bit-identical to the reference's CPU path.
//
// The 1024^2 workload is 8.4 MB for both buffers, so it lives in L2; one launch per sweep would
// be launch-bound.  heat2d_blocked therefore runs S sweeps per launch on a tile held in shared
// memory (overlapped tiling: the tile plus an S-deep halo is loaded once, each sweep shrinks the
// valid region by one cell, the centre tile is written back).  Ghost-ring cells are loaded and
// held constant, so Dirichlet boundaries are exact for any S.
#include "gb_common.cuh"

namespace {

__device__ __forceinline__ float heat_point(float c, float l, float r, float u, float d, float cx, float cy)
{
    float two_c = __fmul_rn(2.0f, c);
    float x = __fmul_rn(cx, __fsub_rn(__fadd_rn(l, r), two_c));
    float y = __fmul_rn(cy, __fsub_rn(__fadd_rn(u, d), two_c));
    return __fadd_rn(__fadd_rn(c, x), y);
}

__global__ void __launch_bounds__(256) heat2d_sweep_k(const float* __restrict__ cur, float* __restrict__ nxt, int nx,
                                                       int ny, int pitch, float cx, float cy)
{
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = 1 + blockIdx.y * blockDim.y + threadIdx.y;
    if (i > nx || j > ny) return;
    const size_t c = (size_t)j * pitch + i;
    nxt[c] = heat_point(__ldg(cur + c), __ldg(cur + c - 1), __ldg(cur + c + 1), __ldg(cur + c - pitch), __ldg(cur + c + pitch),
                        cx, cy);
}

// Overlapped tiling: output tile TX x TY, halo S (runtime, <= SMAX), S sweeps per launch.
// Threads form a 32 x 8 grid that strides over the shared region (no index division).
template <int TX, int TY, int SMAX>
__global__ void __launch_bounds__(256) heat2d_blocked(const float* __restrict__ cur, float* __restrict__ nxt, int nx,
                                                       int ny, int pitch, int S, float cx, float cy)
{
    constexpr int RW = TX + 2 * SMAX, RH = TY + 2 * SMAX;  // shared region (max)
    extern __shared__ float sm[];
    float* A = sm;
    float* B = sm + RW * RH;
    const int rw = TX + 2 * S, rh = TY + 2 * S;  // region actually used
    const int ox = 1 + blockIdx.x * TX - S;      // padded coords of region (0,0)
    const int oy = 1 + blockIdx.y * TY - S;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;

    // load the region: all loads of a thread are issued before any is stored (one L2 round trip)
    constexpr int LR = (RH + 7) / 8, LC = (RW + 31) / 32;
    float v[LR][LC];
#pragma unroll
    for (int a = 0; a < LR; a++)
#pragma unroll
        for (int c = 0; c < LC; c++) {
            const int ry = ty + 8 * a, rx = tx + 32 * c, gy = oy + ry, gx = ox + rx;
            v[a][c] = (ry < rh && rx < rw && gx >= 0 && gx <= nx + 1 && gy >= 0 && gy <= ny + 1)
                          ? __ldg(cur + (size_t)gy * pitch + gx) : 0.0f;
        }
#pragma unroll
    for (int a = 0; a < LR; a++)
#pragma unroll
        for (int c = 0; c < LC; c++) {
            const int ry = ty + 8 * a, rx = tx + 32 * c;
            if (ry < rh && rx < rw) {
                A[ry * RW + rx] = v[a][c];
                B[ry * RW + rx] = v[a][c];  // ghost / outside cells keep their value in both buffers
            }
        }
    __syncthreads();

    // interior cells of the region (those updated by the sweep), in region coordinates
    const int ix0 = max(1 - ox, 0), ix1 = min(nx + 1 - ox, rw);  // gx in [1, nx]
    const int iy0 = max(1 - oy, 0), iy1 = min(ny + 1 - oy, rh);
    for (int s = 1; s <= S; s++) {
        // valid after this sweep: region cells [s, rw-s) x [s, rh-s)
        const int x0 = max(s, ix0), x1 = min(rw - s, ix1), y0 = max(s, iy0), y1 = min(rh - s, iy1);
        for (int ry = y0 + ty; ry < y1; ry += 8)
            for (int rx = x0 + tx; rx < x1; rx += 32) {
                const int q = ry * RW + rx;
                B[q] = heat_point(A[q], A[q - 1], A[q + 1], A[q - RW], A[q + RW], cx, cy);
            }
        __syncthreads();
        float* t = A;
        A = B;
        B = t;
    }

    for (int y = ty; y < TY; y += 8) {
        const int gy = 1 + blockIdx.y * TY + y;
        if (gy > ny) break;
        for (int x = tx; x < TX; x += 32) {
            const int gx = 1 + blockIdx.x * TX + x;
            if (gx <= nx) nxt[(size_t)gy * pitch + gx] = A[(y + S) * RW + (x + S)];
        }
    }
}

constexpr int HTX = 64, HTY = 32, HSMAX = 8;

int check_heat(const void* a, const void* b, int nx, int ny, int pitch)
{
    if (!a || !b || a == b) return gb::fail(APPFIS_GB_EINVAL, "heat2d: null or aliased buffers");
    if (nx < 1 || ny < 1 || pitch < nx + 2) return gb::fail(APPFIS_GB_EINVAL, "heat2d: bad size %d x %d pitch %d", nx, ny, pitch);
    return APPFIS_GB_OK;
}

}  // namespace

extern "C" {

int appfis_gb_heat2d_sweep(const float* cur, float* next, int nx, int ny, int pitch, float cx, float cy, void* stream)
{
    GB_TRY(check_heat(cur, next, nx, ny, pitch));
    dim3 blk(64, 4), grd(gb::ceil_div(nx, 64), gb::ceil_div(ny, 4));
    heat2d_sweep_k<<<grd, blk, 0, gb::as_stream(stream)>>>(cur, next, nx, ny, pitch, cx, cy);
    return gb::launched("heat2d_sweep");
}

int appfis_gb_heat2d(float* a, float* b, int nx, int ny, int pitch, int iters, float cx, float cy, int* cur_index,
                     void* stream)
{
    GB_TRY(check_heat(a, b, nx, ny, pitch));
    if (iters < 0) return gb::fail(APPFIS_GB_EINVAL, "heat2d: negative iteration count");
    cudaStream_t st = gb::as_stream(stream);
    constexpr size_t smem = sizeof(float) * 2 * (HTX + 2 * HSMAX) * (HTY + 2 * HSMAX);
    GB_CUDA(cudaFuncSetAttribute(heat2d_blocked<HTX, HTY, HSMAX>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grd(gb::ceil_div(nx, HTX), gb::ceil_div(ny, HTY));
    float* buf[2] = {a, b};
    int ci = 0;
    for (int done = 0; done < iters;) {
        const int S = std::min(HSMAX, iters - done);
        heat2d_blocked<HTX, HTY, HSMAX><<<grd, 256, smem, st>>>(buf[ci], buf[1 - ci], nx, ny, pitch, S, cx, cy);
        ci = 1 - ci;
        done += S;
    }
    GB_TRY(gb::launched("heat2d_blocked"));
    if (cur_index) *cur_index = ci;
    return APPFIS_GB_OK;
}

int appfis_gb_heat2d_job(float* field, int nx, int ny, int iters, float cx, float cy, double* stats)
{
    if (!field || nx < 1 || ny < 1 || iters < 0) return gb::fail(APPFIS_GB_EINVAL, "heat2d_job: bad arguments");
    cudaStream_t st;
    GB_TRY(gb::job_stream(&st));
    const int px = nx + 2, py = ny + 2;
    const size_t bytes = sizeof(float) * (size_t)px * py;
    void *a, *b, *res;
    GB_TRY(gb::workspace(gb::WS_JOB_A, bytes, &a));
    GB_TRY(gb::workspace(gb::WS_JOB_B, bytes, &b));
    GB_TRY(gb::workspace(gb::WS_JOB_F, 64, &res));
    GB_CUDA(cudaMemcpyAsync(a, field, bytes, cudaMemcpyHostToDevice, st));
    GB_CUDA(cudaMemcpyAsync(b, a, bytes, cudaMemcpyDeviceToDevice, st));  // ghost ring in both buffers
    int ci = 0;
    GB_TRY(appfis_gb_heat2d((float*)a, (float*)b, nx, ny, px, iters, cx, cy, &ci, st));
    float* latest = ci == 0 ? (float*)a : (float*)b;
    double s[3] = {0, 0, 0};
    if (stats) {
        const int box[6] = {1, nx + 1, 1, ny + 1, 0, 1};
        for (int op = 0; op < 3; op++) {
            GB_TRY(appfis_gb_reduce(latest, APPFIS_GB_F32, px, py, box, op, (char*)res + 8 * op, st));
        }
        GB_CUDA(cudaMemcpyAsync(s, res, sizeof s, cudaMemcpyDeviceToHost, st));
    }
    GB_CUDA(cudaMemcpyAsync(field, latest, bytes, cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    if (stats) for (int k = 0; k < 3; k++) stats[k] = s[k];
    return APPFIS_GB_OK;
}

}  // extern "C"
