// Radius-4 3-D star stencil (FDTD3d): 2.5-D sweep with a register queue along z.
//
// Reference functor: FDTD3d/src/fdtd3d_appfis.hpp:129-143 (ghost width 4, :62):
//     val = c; for a in 1..4: val += (x-a + x+a) + (y-a + y+a) + (z-a + z+a); val *= coeff
// run once per time step by Execute3D -> Kernel3D with 8x8x4 blocks that read 25 points each.
//
// Here a CTA owns a 32 x (8*RY) tile of (x, y) columns and a chunk of z planes.  Each thread
// keeps the 9 z-values of its RY columns in registers (the queue shifts by one plane per
// step, so every input plane is read from memory once per CTA), writes its current plane
// into a shared tile, four edge groups fetch the 4-wide x/y halo of that plane, and the x/y
// neighbours come from shared memory.  Per point: one load, one store (8 B/LUP at FP32,
// 4 B/LUP at FP16 storage) plus the halo and z-chunk overlap.
//
// MODE 0: the reference form (uniform coefficient, same addition order as the reference, so
//         FP32 results are bit-identical to its CPU path).
// MODE 1: weighted form  val = w0*c + sum_a w_a*((x-a + x+a) + (y-a + y+a) + (z-a + z+a)),
//         which holds the 8th-order Laplacian update u <- u + nu*L8(u) with w0 = 1 + 3 nu c0,
//         w_a = nu c_a.
// Storage T = float or __half; arithmetic is FP32 in both.
#include <cuda_fp16.h>

#include "gb_common.cuh"

namespace {

constexpr int R = 4;
constexpr int TX = 32;

template <class T> __device__ __forceinline__ float ld(const T* p);
template <> __device__ __forceinline__ float ld<float>(const float* p) { return __ldg(p); }
template <> __device__ __forceinline__ float ld<__half>(const __half* p) { return __half2float(__ldg(p)); }
template <class T> __device__ __forceinline__ void st(T* p, float v);
template <> __device__ __forceinline__ void st<float>(float* p, float v) { *p = v; }
template <> __device__ __forceinline__ void st<__half>(__half* p, float v) { *p = __float2half_rn(v); }

struct StarW {
    float w[5];
};

template <class T, int MODE, int RY>
__global__ void __launch_bounds__(256) star_r4_sweep(const T* __restrict__ in, T* __restrict__ out, int nx, int ny, int nz,
                                                      int px, int py, int kz, float coeff, StarW wt)
{
    constexpr int TY = 8 * RY;
    constexpr int SW = TX + 2 * R;  // shared tile width
    __shared__ float tile[(TY + 2 * R) * SW];
    const int tx = threadIdx.x, ty = threadIdx.y, t = ty * TX + tx;
    const int x0 = R + blockIdx.x * TX, y0 = R + blockIdx.y * TY;
    const int k0 = R + blockIdx.z * kz, k1 = min(k0 + kz, nz + R);
    const int xe = nx + 2 * R, ye = ny + 2 * R;  // padded extents
    const size_t plane = (size_t)px * py;
    const int x = x0 + tx;

    float q[RY][2 * R + 1];
    // queue: z = k0-4 .. k0+3 in slots 0..7; slot 8 filled at the top of each step
#pragma unroll
    for (int r = 0; r < RY; r++) {
        const int y = y0 + ty + 8 * r;
        const bool in_pad = x < xe && y < ye;
#pragma unroll
        for (int m = 0; m < 2 * R; m++)
            q[r][m] = in_pad ? ld<T>(in + (size_t)(k0 - R + m) * plane + (size_t)y * px + x) : 0.0f;
    }
    // halo assignment (2 values per thread per plane)
    const int side = t >> 7, idx = t & 127;
    const int hx_lr = side ? x0 + TX + (idx & 3) : x0 - R + (idx & 3);  // left/right halo column
    const int hy_lr = y0 + (idx >> 2);                                   // rows y0 .. y0+31
    const int hx_tb = x0 + (idx & 31);
    const int hy_tb = side ? y0 + TY + (idx >> 5) : y0 - R + (idx >> 5);

    for (int k = k0; k < k1; k++) {
#pragma unroll
        for (int r = 0; r < RY; r++) {
            const int y = y0 + ty + 8 * r;
            const bool in_pad = x < xe && y < ye;
            q[r][2 * R] = in_pad ? ld<T>(in + (size_t)(k + R) * plane + (size_t)y * px + x) : 0.0f;
        }
        __syncthreads();  // previous plane's tile reads are done
#pragma unroll
        for (int r = 0; r < RY; r++) tile[(ty + 8 * r + R) * SW + tx + R] = q[r][R];
        const size_t pk = (size_t)k * plane;
        for (int h = hy_lr; h < y0 + TY; h += 32) {  // TY may exceed 32: cover every row
            float v = (hx_lr < xe && h < ye) ? ld<T>(in + pk + (size_t)h * px + hx_lr) : 0.0f;
            tile[(h - y0 + R) * SW + (hx_lr - x0 + R)] = v;
        }
        {
            float v = (hx_tb < xe && hy_tb < ye) ? ld<T>(in + pk + (size_t)hy_tb * px + hx_tb) : 0.0f;
            tile[(hy_tb - y0 + R) * SW + (hx_tb - x0 + R)] = v;
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < RY; r++) {
            const int yy = ty + 8 * r + R, xx = tx + R;
            const float* s = tile + yy * SW + xx;
            float v;
            if (MODE == 0) {
                v = q[r][R];
#pragma unroll
                for (int a = 1; a <= R; a++) {
                    const float sx = __fadd_rn(s[-a], s[a]);
                    const float sy = __fadd_rn(s[-a * SW], s[a * SW]);
                    const float sz = __fadd_rn(q[r][R - a], q[r][R + a]);
                    v = __fadd_rn(v, __fadd_rn(__fadd_rn(sx, sy), sz));
                }
                v = __fmul_rn(v, coeff);
            } else {
                v = wt.w[0] * q[r][R];
#pragma unroll
                for (int a = 1; a <= R; a++)
                    v += wt.w[a] * (((s[-a] + s[a]) + (s[-a * SW] + s[a * SW])) + (q[r][R - a] + q[r][R + a]));
            }
            const int y = y0 + ty + 8 * r;
            if (x < nx + R && y < ny + R) st<T>(out + (size_t)k * plane + (size_t)y * px + x, v);
        }
#pragma unroll
        for (int r = 0; r < RY; r++)
#pragma unroll
            for (int m = 0; m < 2 * R; m++) q[r][m] = q[r][m + 1];
    }
}

template <class T, int MODE, int RY>
void launch_star(const T* in, T* out, int nx, int ny, int nz, int px, int kz, float coeff, StarW w, cudaStream_t st)
{
    dim3 blk(TX, 8), grd(gb::ceil_div(nx, TX), gb::ceil_div(ny, 8 * RY), gb::ceil_div(nz, kz));
    star_r4_sweep<T, MODE, RY><<<grd, blk, 0, st>>>(in, out, nx, ny, nz, px, ny + 2 * R, kz, coeff, w);
}

template <class T>
int run_star(T* a, T* b, int nx, int ny, int nz, int pitch, int iters, int mode, float coeff, const float* w5, int ry,
             int kz, int* cur_index, cudaStream_t st)
{
    StarW w = {{0, 0, 0, 0, 0}};
    if (w5)
        for (int n = 0; n < 5; n++) w.w[n] = w5[n];
    T* buf[2] = {a, b};
    int ci = 0;
    for (int it = 0; it < iters; it++) {
        if (mode == 0) {
            if (ry == 2) launch_star<T, 0, 2>(buf[ci], buf[1 - ci], nx, ny, nz, pitch, kz, coeff, w, st);
            else launch_star<T, 0, 4>(buf[ci], buf[1 - ci], nx, ny, nz, pitch, kz, coeff, w, st);
        } else {
            if (ry == 2) launch_star<T, 1, 2>(buf[ci], buf[1 - ci], nx, ny, nz, pitch, kz, coeff, w, st);
            else launch_star<T, 1, 4>(buf[ci], buf[1 - ci], nx, ny, nz, pitch, kz, coeff, w, st);
        }
        ci = 1 - ci;
    }
    GB_TRY(gb::launched("star_r4_sweep"));
    if (cur_index) *cur_index = ci;
    return APPFIS_GB_OK;
}

}  // namespace

extern "C" {

int appfis_gb_star_r4(void* a, void* b, int dtype, int nx, int ny, int nz, int pitch, int iters, int mode, float coeff,
                      const float* weights, int tile_rows, int zchunk, int* cur_index, void* stream)
{
    if (!a || !b || a == b) return gb::fail(APPFIS_GB_EINVAL, "star_r4: null or aliased buffers");
    if (nx < 1 || ny < 1 || nz < 1 || pitch < nx + 2 * R) return gb::fail(APPFIS_GB_EINVAL, "star_r4: bad dims");
    if (mode != 0 && mode != 1) return gb::fail(APPFIS_GB_EINVAL, "star_r4: mode %d", mode);
    if (mode == 1 && !weights) return gb::fail(APPFIS_GB_EINVAL, "star_r4: weighted mode needs 5 weights");
    if (iters < 0) return gb::fail(APPFIS_GB_EINVAL, "star_r4: negative iteration count");
    const int ry = tile_rows <= 0 ? 4 : tile_rows;
    if (ry != 2 && ry != 4) return gb::fail(APPFIS_GB_EINVAL, "star_r4: tile_rows must be 2 or 4");
    const int kz = zchunk <= 0 ? 64 : zchunk;
    cudaStream_t st = gb::as_stream(stream);
    if (dtype == APPFIS_GB_F32)
        return run_star<float>((float*)a, (float*)b, nx, ny, nz, pitch, iters, mode, coeff, weights, ry, kz, cur_index, st);
    if (dtype == APPFIS_GB_F16)
        return run_star<__half>((__half*)a, (__half*)b, nx, ny, nz, pitch, iters, mode, coeff, weights, ry, kz, cur_index, st);
    return gb::fail(APPFIS_GB_EINVAL, "star_r4: dtype %d (F32 or F16)", dtype);
}

}  // extern "C"
