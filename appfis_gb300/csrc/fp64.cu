// FP64 sweeps: the heat, Himeno and radius-4 star functors instantiated with double.
//
// The reference's functors are templates on the element type, and two of its applications run
// in double (HeatDiffusion: Grid<double>, HeatDiffusion/src/heat_appfis.hpp:72; Triton:
// Triton/src/triton_appfis.hpp:108-122).  These kernels are those functors in double with every
// multiply and add rounded separately in the reference's order (explicit __d*_rn, no FMA
// contraction), so they reproduce the reference's CPU path built with double bit for bit.  They
// are also the precision reference of the engine: the FP32, FP16-storage, mixed-precision and
// time-blocked forms state their error against these results.
//
// One thread per point of a (32 x 8)-point block of one plane (z = blockIdx.z); neighbours come
// through the read-only cache.  FP64 arithmetic on a GB300 runs at a small fraction of the
// FP32 rate, so these sweeps are bounded by the FP64 pipe, not by HBM; they are not a fast path.
#include "gb_common.cuh"

namespace {

constexpr int BX = 32, BY = 8;

__global__ void __launch_bounds__(BX * BY) heat2d_f64(const double* __restrict__ cur, double* __restrict__ nxt, int nx, int ny,
                                                      int px, double cx, double cy)
{
    const int i = 1 + blockIdx.x * BX + threadIdx.x, j = 1 + blockIdx.y * BY + threadIdx.y;
    if (i > nx || j > ny) return;
    const size_t c = (size_t)j * px + i;
    const double v = __ldg(cur + c), two_c = __dmul_rn(2.0, v);
    const double x = __dmul_rn(cx, __dsub_rn(__dadd_rn(__ldg(cur + c - 1), __ldg(cur + c + 1)), two_c));
    const double y = __dmul_rn(cy, __dsub_rn(__dadd_rn(__ldg(cur + c - px), __ldg(cur + c + px)), two_c));
    nxt[c] = __dadd_rn(__dadd_rn(v, x), y);
}

struct CoefF64 {
    const double* f[12];  // a0 a1 a2 a3 b0 b1 b2 c0 c1 c2 bnd wrk1
};

// Himeno/src/himeno_appfis.hpp:178-198 in double; ss^2 summed per block (fixed order), the block
// partials folded in block order by fold_f64 into gosa[it].
__global__ void __launch_bounds__(BX * BY) himeno_f64(CoefF64 cf, const double* __restrict__ p, double* __restrict__ w2, int nx,
                                                      int ny, int nz, int px, int py, double omega, double* __restrict__ partials)
{
    const int i = 1 + blockIdx.x * BX + threadIdx.x, j = 1 + blockIdx.y * BY + threadIdx.y, k = 1 + blockIdx.z;
    double g = 0.0;
    if (i <= nx && j <= ny) {
        const size_t sx = 1, sy = (size_t)px, sz = (size_t)px * py, c = (size_t)k * sz + (size_t)j * sy + i;
        auto P = [&](int di, int dj, int dk) { return __ldg(p + c + di * (long long)sx + dj * (long long)sy + dk * (long long)sz); };
        auto C = [&](int n) { return __ldg(cf.f[n] + c); };
        double s0 = __dmul_rn(C(0), P(1, 0, 0));
        s0 = __dadd_rn(s0, __dmul_rn(C(1), P(0, 1, 0)));
        s0 = __dadd_rn(s0, __dmul_rn(C(2), P(0, 0, 1)));
        s0 = __dadd_rn(s0, __dmul_rn(C(4), __dadd_rn(__dsub_rn(__dsub_rn(P(1, 1, 0), P(1, -1, 0)), P(-1, 1, 0)), P(-1, -1, 0))));
        s0 = __dadd_rn(s0, __dmul_rn(C(5), __dadd_rn(__dsub_rn(__dsub_rn(P(0, 1, 1), P(0, -1, 1)), P(0, 1, -1)), P(0, -1, -1))));
        s0 = __dadd_rn(s0, __dmul_rn(C(6), __dadd_rn(__dsub_rn(__dsub_rn(P(1, 0, 1), P(-1, 0, 1)), P(1, 0, -1)), P(-1, 0, -1))));
        s0 = __dadd_rn(s0, __dmul_rn(C(7), P(-1, 0, 0)));
        s0 = __dadd_rn(s0, __dmul_rn(C(8), P(0, -1, 0)));
        s0 = __dadd_rn(s0, __dmul_rn(C(9), P(0, 0, -1)));
        s0 = __dadd_rn(s0, C(11));
        const double p0 = P(0, 0, 0);
        const double ss = __dmul_rn(__dsub_rn(__dmul_rn(s0, C(3)), p0), C(10));
        w2[c] = __dadd_rn(p0, __dmul_rn(omega, ss));
        g = __dmul_rn(ss, ss);
    }
    // block sum in a fixed order: warp shuffles, then the 8 warp sums in warp order
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) g = __dadd_rn(g, __shfl_down_sync(0xffffffffu, g, o));
    __shared__ double ws[BY];
    const int t = threadIdx.y * BX + threadIdx.x;
    if ((t & 31) == 0) ws[t >> 5] = g;
    __syncthreads();
    if (t == 0 && partials) {
        double s = 0.0;
        for (int n = 0; n < BY; n++) s = __dadd_rn(s, ws[n]);
        partials[((size_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x] = s;
    }
}

// One block folds n partials: each thread a contiguous run in order, then the runs in thread order.
__global__ void __launch_bounds__(1024) fold_f64(const double* __restrict__ part, size_t n, double* __restrict__ out)
{
    __shared__ double sh[1024];
    const size_t per = (n + 1023) / 1024, b = (size_t)threadIdx.x * per, e = b + per < n ? b + per : n;
    double s = 0.0;
    for (size_t q = b; q < e; q++) s = __dadd_rn(s, part[q]);
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = 512; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) sh[threadIdx.x] = __dadd_rn(sh[threadIdx.x], sh[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

struct StarWeightsF64 {
    double w[5];
};

// FDTD3d/src/fdtd3d_appfis.hpp:129-143 (mode 0) and the weighted form (mode 1) in double.
template <int MODE>
__global__ void __launch_bounds__(BX * BY) star_r4_f64(const double* __restrict__ cur, double* __restrict__ nxt, int nx, int ny,
                                                       int px, int py, double coeff, StarWeightsF64 wt)
{
    constexpr int R = 4;
    const int i = R + blockIdx.x * BX + threadIdx.x, j = R + blockIdx.y * BY + threadIdx.y, k = R + blockIdx.z;
    if (i >= nx + R || j >= ny + R) return;
    const long long sy = px, sz = (long long)px * py;
    const size_t c = (size_t)k * sz + (size_t)j * sy + i;
    double v = MODE == 0 ? __ldg(cur + c) : __dmul_rn(wt.w[0], __ldg(cur + c));
#pragma unroll
    for (int s = 1; s <= R; s++) {
        const double sx = __dadd_rn(__ldg(cur + c - s), __ldg(cur + c + s));
        const double syy = __dadd_rn(__ldg(cur + c - s * sy), __ldg(cur + c + s * sy));
        const double szz = __dadd_rn(__ldg(cur + c - s * sz), __ldg(cur + c + s * sz));
        const double ring = __dadd_rn(__dadd_rn(sx, syy), szz);
        v = MODE == 0 ? __dadd_rn(v, ring) : __dadd_rn(v, __dmul_rn(wt.w[s], ring));
    }
    if (MODE == 0) v = __dmul_rn(v, coeff);
    nxt[c] = v;
}

}  // namespace

extern "C" {

int appfis_gb_heat2d_f64(double* a, double* b, int nx, int ny, int pitch, int iters, double cx, double cy, int* cur_index,
                         void* stream)
{
    if (!a || !b || a == b) return gb::fail(APPFIS_GB_EINVAL, "heat2d_f64: null or aliased buffers");
    if (nx < 1 || ny < 1 || pitch < nx + 2 || iters < 0) return gb::fail(APPFIS_GB_EINVAL, "heat2d_f64: bad dims");
    cudaStream_t st = gb::as_stream(stream);
    double* buf[2] = {a, b};
    dim3 blk(BX, BY), grd(gb::ceil_div(nx, BX), gb::ceil_div(ny, BY));
    int ci = 0;
    for (int it = 0; it < iters; it++, ci = 1 - ci) heat2d_f64<<<grd, blk, 0, st>>>(buf[ci], buf[1 - ci], nx, ny, pitch, cx, cy);
    GB_TRY(gb::launched("heat2d_f64"));
    if (cur_index) *cur_index = ci;
    return APPFIS_GB_OK;
}

int appfis_gb_himeno_f64(const double* const* coef, double* p, double* wrk2, int nx, int ny, int nz, int pitch, int iters,
                         double omega, double* dev_gosa, int* cur_index, void* stream)
{
    if (!coef || !p || !wrk2 || p == wrk2) return gb::fail(APPFIS_GB_EINVAL, "himeno_f64: null or aliased buffers");
    if (nx < 1 || ny < 1 || nz < 1 || nz > 65535 || pitch < nx + 2 || iters < 0)
        return gb::fail(APPFIS_GB_EINVAL, "himeno_f64: bad dims");
    CoefF64 cf;
    for (int n = 0; n < 12; n++) {
        if (!coef[n]) return gb::fail(APPFIS_GB_EINVAL, "himeno_f64: null coefficient field %d", n);
        cf.f[n] = coef[n];
    }
    cudaStream_t st = gb::as_stream(stream);
    dim3 blk(BX, BY), grd(gb::ceil_div(nx, BX), gb::ceil_div(ny, BY), nz);
    const size_t nblk = (size_t)grd.x * grd.y * grd.z;
    void* ws = nullptr;
    if (dev_gosa) GB_TRY(gb::workspace(gb::WS_F64_PARTIALS, sizeof(double) * nblk, &ws));
    double* part = reinterpret_cast<double*>(ws);
    double* buf[2] = {p, wrk2};
    int ci = 0;
    for (int it = 0; it < iters; it++, ci = 1 - ci) {
        himeno_f64<<<grd, blk, 0, st>>>(cf, buf[ci], buf[1 - ci], nx, ny, nz, pitch, ny + 2, omega, part);
        if (dev_gosa) fold_f64<<<1, 1024, 0, st>>>(part, nblk, dev_gosa + it);
    }
    GB_TRY(gb::launched("himeno_f64"));
    if (cur_index) *cur_index = ci;
    return APPFIS_GB_OK;
}

int appfis_gb_star_r4_f64(double* a, double* b, int nx, int ny, int nz, int pitch, int iters, int mode, double coeff,
                          const double* weights, int* cur_index, void* stream)
{
    if (!a || !b || a == b) return gb::fail(APPFIS_GB_EINVAL, "star_r4_f64: null or aliased buffers");
    if (nx < 1 || ny < 1 || nz < 1 || nz > 65535 || pitch < nx + 8 || iters < 0)
        return gb::fail(APPFIS_GB_EINVAL, "star_r4_f64: bad dims");
    if (mode != 0 && mode != 1) return gb::fail(APPFIS_GB_EINVAL, "star_r4_f64: mode %d", mode);
    if (mode == 1 && !weights) return gb::fail(APPFIS_GB_EINVAL, "star_r4_f64: weighted mode needs 5 weights");
    StarWeightsF64 w = {{0, 0, 0, 0, 0}};
    if (weights)
        for (int n = 0; n < 5; n++) w.w[n] = weights[n];
    cudaStream_t st = gb::as_stream(stream);
    double* buf[2] = {a, b};
    dim3 blk(BX, BY), grd(gb::ceil_div(nx, BX), gb::ceil_div(ny, BY), nz);
    int ci = 0;
    for (int it = 0; it < iters; it++, ci = 1 - ci) {
        if (mode == 0) star_r4_f64<0><<<grd, blk, 0, st>>>(buf[ci], buf[1 - ci], nx, ny, pitch, ny + 8, coeff, w);
        else star_r4_f64<1><<<grd, blk, 0, st>>>(buf[ci], buf[1 - ci], nx, ny, pitch, ny + 8, coeff, w);
    }
    GB_TRY(gb::launched("star_r4_f64"));
    if (cur_index) *cur_index = ci;
    return APPFIS_GB_OK;
}

}  // extern "C"
