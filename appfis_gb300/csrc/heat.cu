// 2-D heat (explicit 5-point Jacobi, FP32) on a DUAL grid with a Dirichlet ghost ring.
//
// Reference functor: HeatDiffusion/src/heat_appfis.hpp:166-174 (3-D FP64), restated in 2-D FP32:
//     next = c + cx*((l + r) - 2c) + cy*((u + d) - 2c)
// driven once per iteration by Execute2D -> Kernel2D (Appfis/Runtime_CUDA.hpp:345-369,1217-1230).
// The arithmetic below uses explicit round-to-nearest intrinsics in exactly that order (no FMA
// contraction), so every point is bit-identical to the reference's CPU path.
//
// The 1024^2 workload is 8.4 MB for both buffers, so it lives in L2; one launch per sweep would
// be launch-bound.  heat2d_regs therefore runs S sweeps per launch on a tile held on chip
// (overlapped tiling: the tile plus an S-deep halo is loaded once, each sweep shrinks the valid
// region by one cell, the centre tile is written back).  Ghost-ring cells are loaded and held
// constant, so Dirichlet boundaries are exact for any S.
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

// Overlapped tiling: output tile TX x TY, halo S <= SMAX, S sweeps per launch (S is a template
// argument: launch_heat_regs instantiates 1..SMAX and picks the launch's).  The
// (TX + 2 SMAX) x (TY + 2 SMAX) region is cut into 4 x 4 blocks, one per thread, held in
// registers for all S sweeps.  A sweep publishes each block's four edges (top and bottom rows,
// left and right columns, one 16-byte vector each) into shared memory, synchronises once, reads
// the facing edges of the four neighbour blocks and updates its 16 points: 8 shared-memory
// vector operations per 16 point-updates.  Ghost-ring cells and cells outside the field keep
// their values; every other cell of the region is updated each sweep (those outside the
// shrinking valid window only feed cells that are not written back).  The point update is
// heat_point, scalar: packed FP32-pair multiplies feeding pair adds are contracted to pair FMAs
// by the code generator, which would change the rounding.
constexpr int RBS = 4;  // block side

template <int BX, int BY>
struct HeatEdges {  // block edges, by sweep parity
    float4 t[2][BY][BX], b[2][BY][BX], l[2][BY][BX], r[2][BY][BX];
};

// One tile, S sweeps (unrolled: the sweep-to-sweep register copies become renaming).  MASK:
// the region reaches the ghost ring or beyond the field, so loads are guarded and only interior
// cells are updated; tiles whose whole region is interior take the unmasked form.
template <int TX, int TY, int SMAX, int S, bool MASK>
__device__ __forceinline__ void heat_tile(const float* __restrict__ cur, float* __restrict__ nxt, int nx, int ny, int pitch,
                                          float cx, float cy, HeatEdges<(TX + 2 * SMAX) / RBS, (TY + 2 * SMAX) / RBS>& e)
{
    constexpr int BX = (TX + 2 * SMAX) / RBS, BY = (TY + 2 * SMAX) / RBS;
    constexpr int rw = TX + 2 * S, rh = TY + 2 * S;  // region in use
    const int t = threadIdx.x, bx = t % BX, by = t / BX;
    const int ox = 1 + blockIdx.x * TX - S, oy = 1 + blockIdx.y * TY - S;  // padded coords of region (0,0)
    float v[RBS][RBS];
    unsigned upd = 0;  // MASK: bit 4r+c set for an interior cell of the region in use
#pragma unroll
    for (int r = 0; r < RBS; r++)
#pragma unroll
        for (int c = 0; c < RBS; c++) {
            const int rx = RBS * bx + c, ry = RBS * by + r, gx = ox + rx, gy = oy + ry;
            if (MASK) {
                const bool used = rx < rw && ry < rh;
                v[r][c] = (used && gx >= 0 && gx <= nx + 1 && gy >= 0 && gy <= ny + 1) ? __ldg(cur + (size_t)gy * pitch + gx) : 0.0f;
                if (used && gx >= 1 && gx <= nx && gy >= 1 && gy <= ny) upd |= 1u << (RBS * r + c);
            } else {
                v[r][c] = __ldg(cur + (size_t)gy * pitch + gx);
            }
        }
    const float4 z4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll
    for (int s = 1; s <= S; s++) {
        // one barrier per sweep: a buffer is rewritten two sweeps later, after every thread has
        // passed the next sweep's barrier and so finished reading it
        const int q = s & 1;
        e.t[q][by][bx] = make_float4(v[0][0], v[0][1], v[0][2], v[0][3]);
        e.b[q][by][bx] = make_float4(v[3][0], v[3][1], v[3][2], v[3][3]);
        e.l[q][by][bx] = make_float4(v[0][0], v[1][0], v[2][0], v[3][0]);
        e.r[q][by][bx] = make_float4(v[0][3], v[1][3], v[2][3], v[3][3]);
        __syncthreads();
        const float4 up = by > 0 ? e.b[q][by - 1][bx] : z4;
        const float4 dn = by < BY - 1 ? e.t[q][by + 1][bx] : z4;
        const float4 lf = bx > 0 ? e.r[q][by][bx - 1] : z4;
        const float4 rt = bx < BX - 1 ? e.l[q][by][bx + 1] : z4;
        const float upv[RBS] = {up.x, up.y, up.z, up.w}, dnv[RBS] = {dn.x, dn.y, dn.z, dn.w};
        const float lfv[RBS] = {lf.x, lf.y, lf.z, lf.w}, rtv[RBS] = {rt.x, rt.y, rt.z, rt.w};
        float nv[RBS][RBS];
#pragma unroll
        for (int r = 0; r < RBS; r++)
#pragma unroll
            for (int c = 0; c < RBS; c++) {
                const float l = c > 0 ? v[r][c - 1] : lfv[r], rr = c + 1 < RBS ? v[r][c + 1] : rtv[r];
                const float u = r > 0 ? v[r - 1][c] : upv[c], d = r + 1 < RBS ? v[r + 1][c] : dnv[c];
                const float h = heat_point(v[r][c], l, rr, u, d, cx, cy);
                nv[r][c] = !MASK || ((upd >> (RBS * r + c)) & 1u) ? h : v[r][c];
            }
#pragma unroll
        for (int r = 0; r < RBS; r++)
#pragma unroll
            for (int c = 0; c < RBS; c++) v[r][c] = nv[r][c];
    }
#pragma unroll
    for (int r = 0; r < RBS; r++)
#pragma unroll
        for (int c = 0; c < RBS; c++) {
            const int x = RBS * bx + c - S, y = RBS * by + r - S;  // output tile coordinates
            const int gx = 1 + blockIdx.x * TX + x, gy = 1 + blockIdx.y * TY + y;
            if (x >= 0 && x < TX && y >= 0 && y < TY && (!MASK || (gx <= nx && gy <= ny))) nxt[(size_t)gy * pitch + gx] = v[r][c];
        }
}

template <int TX, int TY, int SMAX, int S>
__global__ void __launch_bounds__(((TX + 2 * SMAX) / RBS) * ((TY + 2 * SMAX) / RBS))
    heat2d_regs(const float* __restrict__ cur, float* __restrict__ nxt, int nx, int ny, int pitch, float cx, float cy)
{
    constexpr int BX = (TX + 2 * SMAX) / RBS, BY = (TY + 2 * SMAX) / RBS;
    static_assert(BX * RBS == TX + 2 * SMAX && BY * RBS == TY + 2 * SMAX, "region in whole blocks");
    static_assert(S >= 1 && S <= SMAX, "sweeps per launch");
    __shared__ HeatEdges<BX, BY> e;
    // the whole region (TX + 2 SMAX wide, loaded in full) lies on interior cells
    const bool inner = S == SMAX && (int)blockIdx.x * TX >= S && (int)blockIdx.y * TY >= S &&
                       ((int)blockIdx.x + 1) * TX + S <= nx && ((int)blockIdx.y + 1) * TY + S <= ny;
    if (inner)
        heat_tile<TX, TY, SMAX, S, false>(cur, nxt, nx, ny, pitch, cx, cy, e);
    else
        heat_tile<TX, TY, SMAX, S, true>(cur, nxt, nx, ny, pitch, cx, cy, e);
}

template <int TX, int TY, int SMAX, int S = SMAX>
void launch_heat_regs(int s, dim3 grd, const float* cur, float* nxt, int nx, int ny, int pitch, float cx, float cy,
                      cudaStream_t st)
{
    if constexpr (S > 1) {
        if (s < S) return launch_heat_regs<TX, TY, SMAX, S - 1>(s, grd, cur, nxt, nx, ny, pitch, cx, cy, st);
    }
    constexpr int threads = ((TX + 2 * SMAX) / RBS) * ((TY + 2 * SMAX) / RBS);
    heat2d_regs<TX, TY, SMAX, S><<<grd, threads, 0, st>>>(cur, nxt, nx, ny, pitch, cx, cy);
}

// 48 x 32 output tiles: a 64 x 48 region, 16 x 12 blocks, 192 threads of at most 96 registers,
// 3 CTAs per SM.  The wider 64 x 32 tile (240 threads, 2 CTAs per SM) and every other shape
// tried (40-56 wide, 24-40 high) measured slower.
constexpr int HTX = 48, HTY = 32, HSMAX = 8;

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
    dim3 grd(gb::ceil_div(nx, HTX), gb::ceil_div(ny, HTY));
    float* buf[2] = {a, b};
    int ci = 0;
    for (int done = 0; done < iters;) {
        const int S = std::min(HSMAX, iters - done);
        launch_heat_regs<HTX, HTY, HSMAX>(S, grd, buf[ci], buf[1 - ci], nx, ny, pitch, cx, cy, st);
        ci = 1 - ci;
        done += S;
    }
    GB_TRY(gb::launched("heat2d_regs"));
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
