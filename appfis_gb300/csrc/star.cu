// Radius-4 3-D star stencil (FDTD3d): 2.5-D sweep with a register queue along z.
//
// Reference functor: FDTD3d/src/fdtd3d_appfis.hpp:129-143 (ghost width 4, :62):
//     val = c; for a in 1..4: val += (x-a + x+a) + (y-a + y+a) + (z-a + z+a); val *= coeff
// run once per time step by Execute3D -> Kernel3D with 8x8x4 blocks that read 25 points each.
//
// Every tile is a 2.5-D march: a CTA owns an (x, y) tile and a chunk of z planes, each thread
// keeps the 9 z-values of its columns in registers (the queue shifts by one plane per step, so
// every input plane is read from memory once per CTA) and the x/y neighbours come from a plane
// held in shared memory.  Per point: one load, one store (8 B/LUP at FP32, 4 B/LUP at FP16
// storage) plus the halo and z-chunk overlap.  Tiles (APPFIS_GB_STAR_*):
//   star_r4_tma    (TMA_X4 / TMA_X2) planes moved by the tensor memory accelerator into an
//                  mbarrier ring, 4 or 2 x points x 2 rows per thread, packed FP32-pair math;
//                  needs 16-byte rows (the default whenever they are);
//   star_r4_vec    (VEC) 4 x points per thread, register-staged plane loads;
//   star_r4_sweep  (SCALAR2 / SCALAR4) one x point, 2 or 4 rows per thread, any pitch.
//
// MODE 0: the reference form (uniform coefficient, same addition order as the reference, so
//         FP32 results are bit-identical to its CPU path).
// MODE 1: weighted form  val = w0*c + sum_a w_a*((x-a + x+a) + (y-a + y+a) + (z-a + z+a)),
//         which holds the 8th-order Laplacian update u <- u + nu*L8(u) with w0 = 1 + 3 nu c0,
//         w_a = nu c_a.
// Storage T = float or __half; arithmetic is FP32 in both.
#include <cuda_fp16.h>

#include <algorithm>
#include <cstdlib>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "gb_common.cuh"
#include "f32x2.cuh"
#include "tma.cuh"

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
    constexpr int NTY = 8;          // thread rows of the block (32 x 8 threads)
    constexpr int TY = NTY * RY;    // tile rows: each thread owns RY consecutive rows
    constexpr int SW = TX + 2 * R;  // shared plane width
    constexpr int SH = TY + 2 * R;
    constexpr int NHALO = 8 * TY + 8 * TX;          // x halo (2 sides x 4 x TY) + y halo (2 x 4 x TX)
    constexpr int HPT = (NHALO + 255) / 256;        // halo values per thread per plane
    __shared__ float tile[2][SH * SW];
    const int tx = threadIdx.x, ty = threadIdx.y, t = ty * TX + tx;
    const int x0 = R + blockIdx.x * TX, y0 = R + blockIdx.y * TY;
    const int k0 = R + blockIdx.z * kz, k1 = min(k0 + kz, nz + R);
    const int xe = nx + 2 * R, ye = ny + 2 * R;  // padded extents
    const size_t plane = (size_t)px * py;
    const int x = x0 + tx, yb = y0 + ty * RY;

    // halo items of this thread: padded (hx, hy) and shared offset, fixed for all planes
    int hoff[HPT];
    size_t hsrc[HPT];
    bool hok[HPT];
#pragma unroll
    for (int h = 0; h < HPT; h++) {
        const int item = t + 256 * h;
        int hx = 0, hy = 0;
        hok[h] = item < NHALO;
        if (item < 8 * TY) {
            const int side = item / (4 * TY), rem = item - side * 4 * TY;
            hx = side ? x0 + TX + (rem & 3) : x0 - R + (rem & 3);
            hy = y0 + (rem >> 2);
        } else {
            const int it2 = item - 8 * TY;
            const int side = it2 / (4 * TX), rem = it2 - side * 4 * TX;
            hx = x0 + (rem % TX);
            hy = side ? y0 + TY + rem / TX : y0 - R + rem / TX;
        }
        hoff[h] = (hy - y0 + R) * SW + (hx - x0 + R);
        hok[h] = hok[h] && hx < xe && hy < ye;
        hsrc[h] = (size_t)hy * px + hx;
    }

    float q[RY][2 * R + 1];  // z queue of each owned point: planes k-4 .. k+4
#pragma unroll
    for (int r = 0; r < RY; r++) {
        const int y = yb + r;
        const bool in_pad = x < xe && y < ye;
#pragma unroll
        for (int m = 0; m < 2 * R; m++)
            q[r][m] = in_pad ? ld<T>(in + (size_t)(k0 - R + m) * plane + (size_t)y * px + x) : 0.0f;
    }
    float hv[HPT];
#pragma unroll
    for (int h = 0; h < HPT; h++) hv[h] = hok[h] ? ld<T>(in + (size_t)k0 * plane + hsrc[h]) : 0.0f;
    // plane k0 into tile[0]
#pragma unroll
    for (int r = 0; r < RY; r++) tile[0][(ty * RY + r + R) * SW + tx + R] = q[r][R];
#pragma unroll
    for (int h = 0; h < HPT; h++)
        if (t + 256 * h < NHALO) tile[0][hoff[h]] = hv[h];
    __syncthreads();

    for (int k = k0; k < k1; k++) {
        const int b = (k - k0) & 1;
        // prefetch: plane k+4 for the queues, plane k+1 for the halo
#pragma unroll
        for (int r = 0; r < RY; r++) {
            const int y = yb + r;
            q[r][2 * R] = (x < xe && y < ye) ? ld<T>(in + (size_t)(k + R) * plane + (size_t)y * px + x) : 0.0f;
        }
        if (k + 1 < k1) {
#pragma unroll
            for (int h = 0; h < HPT; h++) hv[h] = hok[h] ? ld<T>(in + (size_t)(k + 1) * plane + hsrc[h]) : 0.0f;
        }
        const float* s = tile[b];
        float col[RY + 2 * R];  // the thread's column in this plane, rows yb-4 .. yb+RY+3
#pragma unroll
        for (int m = 0; m < RY + 2 * R; m++) col[m] = s[(ty * RY + m) * SW + tx + R];
#pragma unroll
        for (int r = 0; r < RY; r++) {
            const float* row = s + (ty * RY + r + R) * SW + tx + R;
            float v;
            if (MODE == 0) {
                v = q[r][R];
#pragma unroll
                for (int a = 1; a <= R; a++) {
                    const float sx = __fadd_rn(row[-a], row[a]);
                    const float sy = __fadd_rn(col[r + R - a], col[r + R + a]);
                    const float sz = __fadd_rn(q[r][R - a], q[r][R + a]);
                    v = __fadd_rn(v, __fadd_rn(__fadd_rn(sx, sy), sz));
                }
                v = __fmul_rn(v, coeff);
            } else {
                v = wt.w[0] * q[r][R];
#pragma unroll
                for (int a = 1; a <= R; a++)
                    v += wt.w[a] * (((row[-a] + row[a]) + (col[r + R - a] + col[r + R + a])) + (q[r][R - a] + q[r][R + a]));
            }
            const int y = yb + r;
            if (x < nx + R && y < ny + R) st<T>(out + (size_t)k * plane + (size_t)y * px + x, v);
        }
#pragma unroll
        for (int r = 0; r < RY; r++)
#pragma unroll
            for (int m = 0; m < 2 * R; m++) q[r][m] = q[r][m + 1];
        if (k + 1 < k1) {  // plane k+1 into the other buffer (its last readers passed the previous barrier)
            float* d = tile[1 - b];
#pragma unroll
            for (int r = 0; r < RY; r++) d[(ty * RY + r + R) * SW + tx + R] = q[r][R];
#pragma unroll
            for (int h = 0; h < HPT; h++)
                if (t + 256 * h < NHALO) d[hoff[h]] = hv[h];
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------- vectorised form
// Each thread owns 4 consecutive x points of one row (16 x 16 threads = a 64 x 16 tile), so a
// row of the shared plane is read as float4 (x-window x-4 .. x+7 = three 16-byte reads) and the
// y-window as one float4 per row.  The z queue holds 9 float4 planes; the plane loop is unrolled
// by 9 so the queue rotates by register renaming instead of moves.  Requires 16-byte aligned
// rows: pitch % 4 == 0 (FP32) / pitch % 8 == 0 (FP16, 8-byte half4 loads) and an aligned base.
constexpr int VX = 4, VTX = 64, VTY = 16;
constexpr int VSW = VTX + 2 * R, VSH = VTY + 2 * R;

template <class T> struct Vec4;
template <> struct Vec4<float> {
    static __device__ __forceinline__ float4 ld(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }
    static __device__ __forceinline__ void st(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
};
template <> struct Vec4<__half> {
    static __device__ __forceinline__ float4 ld(const __half* p)
    {
        const uint2 u = __ldg(reinterpret_cast<const uint2*>(p));
        const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&u.x));
        const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&u.y));
        return make_float4(a.x, a.y, b.x, b.y);
    }
    static __device__ __forceinline__ void st(__half* p, float4 v)
    {
        const __half2 a = __floats2half2_rn(v.x, v.y), b = __floats2half2_rn(v.z, v.w);
        uint2 u;
        u.x = *reinterpret_cast<const uint32_t*>(&a);
        u.y = *reinterpret_cast<const uint32_t*>(&b);
        *reinterpret_cast<uint2*>(p) = u;
    }
};

__device__ __forceinline__ float f4(const float4& v, int c) { return c == 0 ? v.x : (c == 1 ? v.y : (c == 2 ? v.z : v.w)); }

template <class T, int MODE>
__global__ void __launch_bounds__(256) star_r4_vec(const T* __restrict__ in, T* __restrict__ out, int nx, int ny, int nz, int px,
                                                    int py, int kz, float coeff, StarW wt)
{
    __shared__ __align__(16) float tile[2][VSH * VSW];
    const int tx = threadIdx.x, ty = threadIdx.y, t = ty * 16 + tx;
    const int x0 = R + blockIdx.x * VTX, y0 = R + blockIdx.y * VTY;
    const int k0 = R + blockIdx.z * kz, k1 = min(k0 + kz, nz + R);
    const int xe = nx + 2 * R, ye = ny + 2 * R;
    const size_t plane = (size_t)px * py;
    const int x = x0 + VX * tx, y = y0 + ty;
    const bool inpad = x < xe && y < ye;  // x % 4 == 0 and xe % 4 == 0 when pitch is aligned: all 4 in or out
    const size_t own = (size_t)y * px + x;
    // halo vectors of this thread: y halo = 8 rows x 16 vectors (items 0..127); x halo = 2 sides x 16
    // rows (items 128..159); 160 items over 256 threads
    const bool has_h = t < 160;
    int hoff = 0;
    size_t hsrc = 0;
    bool hok = false;
    if (has_h) {
        int hx, hy;
        if (t < 128) {
            const int row = t >> 4;  // 0..7: rows y0-4..y0-1, y0+VTY..y0+VTY+3
            hy = row < 4 ? y0 - R + row : y0 + VTY + (row - 4);
            hx = x0 + VX * (t & 15);
        } else {
            const int it = t - 128, side = it >> 4;
            hy = y0 + (it & 15);
            hx = side ? x0 + VTX : x0 - R;
        }
        hoff = (hy - y0 + R) * VSW + (hx - x0 + R);
        hok = hx < xe && hy < ye;
        hsrc = (size_t)hy * px + hx;
    }
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 q[9];
#pragma unroll
    for (int m = 0; m < 8; m++) q[m] = inpad ? Vec4<T>::ld(in + (size_t)(k0 - R + m) * plane + own) : z4;
    float4 hv = (has_h && hok) ? Vec4<T>::ld(in + (size_t)k0 * plane + hsrc) : z4;
    {
        float* d = tile[0];
        *reinterpret_cast<float4*>(d + (ty + R) * VSW + R + VX * tx) = q[R];
        if (has_h) *reinterpret_cast<float4*>(d + hoff) = hv;
    }
    __syncthreads();
    for (int kb = k0; kb < k1; kb += 9) {
#pragma unroll
        for (int P = 0; P < 9; P++) {
            const int k = kb + P;
            if (k < k1) {
                const int b = (k - k0) & 1;
                q[(P + 8) % 9] = inpad ? Vec4<T>::ld(in + (size_t)(k + R) * plane + own) : z4;
                const bool more = k + 1 < k1;
                if (more) hv = (has_h && hok) ? Vec4<T>::ld(in + (size_t)(k + 1) * plane + hsrc) : z4;
                const float* s = tile[b];
                const float* rowp = s + (ty + R) * VSW + R + VX * tx;  // this thread's 4 points
                const float4 xl = *reinterpret_cast<const float4*>(rowp - 4);
                const float4 xc = *reinterpret_cast<const float4*>(rowp);
                const float4 xr = *reinterpret_cast<const float4*>(rowp + 4);
                float4 ym[R], yp[R];
#pragma unroll
                for (int a = 1; a <= R; a++) {
                    ym[a - 1] = *reinterpret_cast<const float4*>(rowp - a * VSW);
                    yp[a - 1] = *reinterpret_cast<const float4*>(rowp + a * VSW);
                }
                const float xw[12] = {xl.x, xl.y, xl.z, xl.w, xc.x, xc.y, xc.z, xc.w, xr.x, xr.y, xr.z, xr.w};
                float res[4];
#pragma unroll
                for (int c = 0; c < 4; c++) {
                    const float cen = f4(q[(P + 4) % 9], c);
                    float v;
                    if (MODE == 0) {
                        v = cen;
#pragma unroll
                        for (int a = 1; a <= R; a++) {
                            const float sx = __fadd_rn(xw[4 + c - a], xw[4 + c + a]);
                            const float sy = __fadd_rn(f4(ym[a - 1], c), f4(yp[a - 1], c));
                            const float sz = __fadd_rn(f4(q[(P + 4 - a) % 9], c), f4(q[(P + 4 + a) % 9], c));
                            v = __fadd_rn(v, __fadd_rn(__fadd_rn(sx, sy), sz));
                        }
                        v = __fmul_rn(v, coeff);
                    } else {
                        v = wt.w[0] * cen;
#pragma unroll
                        for (int a = 1; a <= R; a++)
                            v += wt.w[a] * (((xw[4 + c - a] + xw[4 + c + a]) + (f4(ym[a - 1], c) + f4(yp[a - 1], c))) +
                                            (f4(q[(P + 4 - a) % 9], c) + f4(q[(P + 4 + a) % 9], c)));
                    }
                    res[c] = v;
                }
                if (x < nx + R && y < ny + R) {
                    if (x + VX <= nx + R) {
                        Vec4<T>::st(out + (size_t)k * plane + own, make_float4(res[0], res[1], res[2], res[3]));
                    } else {  // ragged last vector of a row: only the interior lanes
                        for (int c = 0; c < VX && x + c < nx + R; c++) st<T>(out + (size_t)k * plane + own + c, res[c]);
                    }
                }
                if (more) {
                    float* d = tile[1 - b];
                    *reinterpret_cast<float4*>(d + (ty + R) * VSW + R + VX * tx) = q[(P + 5) % 9];
                    if (has_h) *reinterpret_cast<float4*>(d + hoff) = hv;
                }
                __syncthreads();
            }
        }
    }
}

// ---------------------------------------------------------------- TMA-staged form
// A (16*VXT) x 16 (x, y) tile per CTA of 16 x 8 threads; each thread owns VXT consecutive x
// points (4 or 2) of RYT = 2 consecutive rows, and every plane is moved by the tensor memory
// accelerator: plane pl arrives as one (16*VXT + 8) x 24 box (the x/y halo included; the box x
// origin is the tile's first ghost column, a 16*VXT-point boundary of the padded row, so every
// copy starts 16-byte aligned) in slot (pl - k0 + 4) % TNS of a shared ring, signalled on that
// slot's mbarrier.  Thread 0 keeps TNS - 5 planes in flight beyond the newest one in use.  Each
// thread pushes its centre values of plane k+4 into its z queue (registers); the x/y windows of
// plane k come from the ring, except the thread's own rows, which are the queue's centre
// entries.  The arithmetic runs on x pairs with packed FP32-pair instructions, except the x sums
// at odd shifts: their operand pairs straddle register pairs, and two scalar adds cost less than
// assembling the pairs (the same round-to-nearest additions either way).  VXT = 4 reads
// 16-byte shared vectors (fewer shared-memory wavefronts); VXT = 2 halves the queue registers
// (twice the resident warps).  Global traffic: each plane read once per CTA (plus the 8-plane
// z-chunk overlap), each result written once.
constexpr int TNS = 8;   // ring slots: planes k..k+4 resident, 3 more in flight

// TRY rows per thread (2, or 4 for the tile that spreads each plane's fixed per-thread work --
// the mbarrier wait, the ring addresses, the barrier, the store predicates -- over 16 points);
// the tile has 8 thread rows, TTY = 8 * TRY rows.
template <class T, int VXT, int TRY = 2>
struct TmaStar {
    static constexpr int TTY = 8 * TRY;             // tile rows
    static constexpr int TX = 16 * VXT;             // tile x points
    static constexpr int SW = TX + 2 * R, SH = TTY + 2 * R;
    static constexpr int BOX = SW * SH * (int)sizeof(T);  // bytes per plane box
    static constexpr int SLOT = (BOX + 127) / 128 * 128;
    static constexpr int smem() { return TNS * SLOT + TNS * 8; }
};

// VXT consecutive values, loaded from shared memory (FP32 or FP16 storage) and stored to global
template <int VXT>
struct VecN {
    float v[VXT];
};
template <class T, int VXT> __device__ __forceinline__ VecN<VXT> ldsv(const T* p);
template <> __device__ __forceinline__ VecN<4> ldsv<float, 4>(const float* p)
{
    const float4 a = *reinterpret_cast<const float4*>(p);
    return {{a.x, a.y, a.z, a.w}};
}
template <> __device__ __forceinline__ VecN<2> ldsv<float, 2>(const float* p)
{
    const float2 a = *reinterpret_cast<const float2*>(p);
    return {{a.x, a.y}};
}
template <> __device__ __forceinline__ VecN<4> ldsv<__half, 4>(const __half* p)
{
    const uint2 u = *reinterpret_cast<const uint2*>(p);
    const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&u.x));
    const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&u.y));
    return {{a.x, a.y, b.x, b.y}};
}
template <> __device__ __forceinline__ VecN<2> ldsv<__half, 2>(const __half* p)
{
    const float2 a = __half22float2(*reinterpret_cast<const __half2*>(p));
    return {{a.x, a.y}};
}
template <class T, int VXT> __device__ __forceinline__ void stgv(T* p, const float* r);
template <> __device__ __forceinline__ void stgv<float, 4>(float* p, const float* r)
{
    *reinterpret_cast<float4*>(p) = make_float4(r[0], r[1], r[2], r[3]);
}
template <> __device__ __forceinline__ void stgv<float, 2>(float* p, const float* r)
{
    *reinterpret_cast<float2*>(p) = make_float2(r[0], r[1]);
}
template <> __device__ __forceinline__ void stgv<__half, 4>(__half* p, const float* r)
{
    Vec4<__half>::st(p, make_float4(r[0], r[1], r[2], r[3]));
}
template <> __device__ __forceinline__ void stgv<__half, 2>(__half* p, const float* r)
{
    *reinterpret_cast<__half2*>(p) = __floats2half2_rn(r[0], r[1]);
}

// Waits: `wait_ns` per mbarrier wait (1 s in production); `shortfall` (testing only, 0 in
// production) arms the first plane's barrier with that many bytes more than its copy delivers,
// so that its wait runs out.
template <class T, int MODE, int VXT, int TRY>
__global__ void __launch_bounds__(128, VXT == 4 ? (TRY == 2 ? 4 : 2) : 6) star_r4_tma(const __grid_constant__ CUtensorMap map, T* __restrict__ out,
                                                                     int nx, int ny, int nz, int px, int py, int kz, float coeff,
                                                                     StarW wt, unsigned* __restrict__ status,
                                                                     unsigned long long wait_ns, unsigned shortfall)
{
    namespace f2 = gb::f2;
    typedef TmaStar<T, VXT, TRY> Lay;
    constexpr int SW = Lay::SW, TTY = Lay::TTY;
    extern __shared__ __align__(128) unsigned char tsm[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(tsm + TNS * Lay::SLOT);
    const int tx = threadIdx.x, ty = threadIdx.y, t = ty * 16 + tx;
    const int bx0 = blockIdx.x * Lay::TX, by0 = blockIdx.y * TTY;  // box origin (padded coordinates)
    const int x = R + bx0 + VXT * tx, y = R + by0 + TRY * ty;       // this thread's first point
    const int k0 = R + blockIdx.z * kz, k1 = min(k0 + kz, nz + R);
    const int plast = k1 + R - 1;                                   // last plane the chunk reads
    const size_t plane = (size_t)px * py;
    if (gb::tma::smem_u32(tsm) & 127u) {
        if (t == 0) atomicOr(status, (unsigned)gb::ST_SMEM_ALIGN);
        return;
    }
    if (t == 0) {
        for (int n = 0; n < TNS; n++) gb::tma::bar_init(&bar[n], 1);
        gb::tma::fence_init();
        gb::tma::prefetch_map(&map);
    }
    __syncthreads();
    const int pbase = k0 - R;  // plane of slot 0, phase 0
    // plane offsets from pbase are never negative: unsigned arithmetic makes the ring index a mask
    auto slot = [&](int pl) { return reinterpret_cast<const T*>(tsm + ((unsigned)(pl - pbase) % TNS) * Lay::SLOT); };
    int last_issued = pbase - 1;  // thread 0 only
    auto issue = [&](int pl) {
        last_issued = pl;
        const unsigned n = (unsigned)(pl - pbase) % TNS;
        gb::tma::arrive_expect(&bar[n], Lay::BOX + (pl == pbase ? shortfall : 0u));
        gb::tma::load_3d(tsm + n * Lay::SLOT, &map, bx0, by0, pl, &bar[n]);
    };
    auto ready = [&](int pl, uint64_t limit) {
        return gb::tma::wait(&bar[(unsigned)(pl - pbase) % TNS], ((unsigned)(pl - pbase) / TNS) & 1u, limit);
    };
    if (t == 0)
        for (int pl = pbase; pl < pbase + TNS && pl <= plast; pl++) issue(pl);

    const int own = (TRY * ty + R) * SW + R + VXT * tx;  // this thread's first row, VXT points, in a slot
    bool bad = false;
    VecN<VXT> q[TRY][9];
#pragma unroll
    for (int m = 0; m < 8; m++) {  // planes k0-4 .. k0+3
        if (!bad && !ready(pbase + m, wait_ns)) bad = true;
#pragma unroll
        for (int r = 0; r < TRY; r++) q[r][m] = ldsv<T, VXT>(slot(pbase + m) + own + r * SW);
    }
    // planes k0-4 .. k0-1 only fed the queue: their slots take planes pbase+8 .. pbase+11
    bad = __syncthreads_or(bad);
    if (t == 0 && !bad)
        for (int pl = pbase + TNS; pl < pbase + TNS + R && pl <= plast; pl++) issue(pl);

    for (int kb = k0; kb < k1 && !bad; kb += 9) {
#pragma unroll
        for (int P = 0; P < 9; P++) {
            const int k = kb + P;
            if (k < k1 && !bad) {
                if (!ready(k + R, wait_ns)) bad = true;
#pragma unroll
                for (int r = 0; r < TRY; r++) q[r][(P + 8) % 9] = ldsv<T, VXT>(slot(k + R) + own + r * SW);
                const T* rowp = slot(k) + own;
                // y-window rows m = -4..-1 and TRY..TRY+3 relative to the first row
                VecN<VXT> wv[8];
#pragma unroll
                for (int a = 1; a <= R; a++) {
                    wv[a - 1] = ldsv<T, VXT>(rowp - a * SW);
                    wv[R + a - 1] = ldsv<T, VXT>(rowp + (TRY - 1 + a) * SW);
                }
#pragma unroll
                for (int r = 0; r < TRY; r++) {
                    // x window: x-4 .. x+VXT+3 (the centre VXT values are the queue's)
                    float xw[VXT + 2 * R];
#pragma unroll
                    for (int b = 0; b < R; b += VXT) {
                        const VecN<VXT> lo = ldsv<T, VXT>(rowp + r * SW - R + b), hi = ldsv<T, VXT>(rowp + r * SW + VXT + b);
#pragma unroll
                        for (int e = 0; e < VXT; e++) {
                            xw[b + e] = lo.v[e];
                            xw[R + VXT + b + e] = hi.v[e];
                        }
                    }
#pragma unroll
                    for (int e = 0; e < VXT; e++) xw[R + e] = q[r][(P + 4) % 9].v[e];
                    // rows relative to the first row: own rows come from the queue
                    const VecN<VXT>* ym[R];
                    const VecN<VXT>* yp[R];
#pragma unroll
                    for (int a = 1; a <= R; a++) {
                        const int mm = r - a, mp = r + a;
                        ym[a - 1] = mm >= 0 ? &q[mm < TRY ? mm : 0][(P + 4) % 9] : &wv[-mm - 1];
                        yp[a - 1] = mp < TRY ? &q[mp][(P + 4) % 9] : &wv[R + mp - TRY];
                    }
                    float res[VXT];
#pragma unroll
                    for (int c = 0; c < VXT; c += 2) {
                        const float2 cen = make_float2(xw[R + c], xw[R + c + 1]);
                        float2 v;
                        if (MODE == 0) {
                            v = cen;
#pragma unroll
                            for (int a = 1; a <= R; a++) {
                                const float2 sx = (a & 1) ? make_float2(__fadd_rn(xw[R + c - a], xw[R + c + a]),
                                                                        __fadd_rn(xw[R + c + 1 - a], xw[R + c + 1 + a]))
                                                          : f2::add(make_float2(xw[R + c - a], xw[R + c + 1 - a]),
                                                                    make_float2(xw[R + c + a], xw[R + c + 1 + a]));
                                const float2 sy = f2::add(make_float2(ym[a - 1]->v[c], ym[a - 1]->v[c + 1]),
                                                          make_float2(yp[a - 1]->v[c], yp[a - 1]->v[c + 1]));
                                const VecN<VXT>& zm = q[r][(P + 4 - a) % 9];
                                const VecN<VXT>& zp = q[r][(P + 4 + a) % 9];
                                const float2 sz = f2::add(make_float2(zm.v[c], zm.v[c + 1]), make_float2(zp.v[c], zp.v[c + 1]));
                                v = f2::add(v, f2::add(f2::add(sx, sy), sz));
                            }
                            v = f2::mul(v, f2::splat(coeff));
                        } else {
                            v = f2::mul(f2::splat(wt.w[0]), cen);
#pragma unroll
                            for (int a = 1; a <= R; a++) {
                                const float2 sx = (a & 1) ? make_float2(__fadd_rn(xw[R + c - a], xw[R + c + a]),
                                                                        __fadd_rn(xw[R + c + 1 - a], xw[R + c + 1 + a]))
                                                          : f2::add(make_float2(xw[R + c - a], xw[R + c + 1 - a]),
                                                                    make_float2(xw[R + c + a], xw[R + c + 1 + a]));
                                const float2 sy = f2::add(make_float2(ym[a - 1]->v[c], ym[a - 1]->v[c + 1]),
                                                          make_float2(yp[a - 1]->v[c], yp[a - 1]->v[c + 1]));
                                const VecN<VXT>& zm = q[r][(P + 4 - a) % 9];
                                const VecN<VXT>& zp = q[r][(P + 4 + a) % 9];
                                const float2 sz = f2::add(make_float2(zm.v[c], zm.v[c + 1]), make_float2(zp.v[c], zp.v[c + 1]));
                                v = f2::fma(f2::splat(wt.w[a]), f2::add(f2::add(sx, sy), sz), v);
                            }
                        }
                        res[c] = v.x;
                        res[c + 1] = v.y;
                    }
                    const int yr = y + r;
                    if (!bad && x < nx + R && yr < ny + R) {
                        T* o = out + (size_t)k * plane + (size_t)yr * px + x;
                        if (x + VXT <= nx + R) {
                            stgv<T, VXT>(o, res);
                        } else {  // ragged last vector of a row: only the interior lanes
                            for (int c = 0; c < VXT && x + c < nx + R; c++) st<T>(o + c, res[c]);
                        }
                    }
                }
                // plane k's slot is free once every thread is past this barrier: it takes plane k+TNS
                bad = __syncthreads_or(bad);
                if (t == 0 && !bad && k + TNS <= plast) issue(k + TNS);
            }
        }
    }
    if (bad && t == 0) {  // a wait gave up: report and let the copies still in flight land
        atomicOr(status, (unsigned)gb::ST_TMA_TIMEOUT);
        for (int pl = max(pbase, last_issued - TNS + 1); pl <= last_issued; pl++) ready(pl, gb::tma::DRAIN_NS);
    }
}

// ---------------------------------------------------------------- time-blocked form: two steps per launch
// A CTA owns a 64 x TY output tile and a chunk of z planes, and advances it by TWO time steps
// while each input plane crosses the chip once: the output of step 1 ("level 1") is never
// written to memory.  Level 1 is needed on the tile plus a 4-wide ring (its x/y neighbours for
// step 2), so the CTA's 18 x (TY + 8) threads cover that 72 x (TY + 8) region, each thread 4
// consecutive x points of one row:
//   * input planes (level 0) arrive by TMA as 88 x (TY + 16) boxes (the region plus 8 more on
//     each side in x, so that the box origin is 8-element aligned for FP16 too, and 4 in y) in
//     an 8-slot mbarrier ring;
//   * when input plane p lands, every thread pushes its 4 values into a 9-deep register queue
//     (level 0, planes p-8 .. p) and computes level 1 at plane p-4 from that queue (z) and the
//     box of plane p-4 (x, y); points of the ghost halo keep their input value;
//   * level-1 plane p-4 goes to a 6-slot shared-memory ring (FP32) and into a second 9-deep
//     register queue; the 16 x TY threads over the output tile then compute step 2 at plane
//     p-8 from that queue (z) and the ring's plane p-8 (x, y), and store it.
// One CTA barrier per plane: level-1 ring slots are rewritten six planes after their last read.
// Per output point and two steps: one read and one write of the field (plus the halo overlap
// of neighbouring tiles through L2 and 16 planes per z chunk), against two reads and two writes
// for two single-step launches; the step-1 work is done on (TY + 8) x 72 points per 64 x TY
// outputs.  The per-point arithmetic and its order are the single-step TMA tile's, so results
// are bit-identical to two single-step launches (FP32 storage; with FP16 storage the level-1
// values stay FP32 instead of being rounded to FP16 between the steps).
constexpr int TB_NS = 8;  // level-0 ring slots: planes p-4 .. p resident, 3 more in flight
constexpr int TB_L1 = 6;  // level-1 ring slots

template <class T, int TY>
struct TbStar {
    static constexpr int OX = 64;                       // output tile width
    static constexpr int RX = OX + 2 * R;               // level-1 region width (72)
    static constexpr int RH = TY + 2 * R;               // level-1 region height
    static constexpr int BXW = OX + 6 * R;              // level-0 box width (88)
    static constexpr int BH = TY + 4 * R;               // level-0 box height
    static constexpr int NT = (RX / 4) * RH;            // threads (18 x RH)
    static constexpr int BOX = BXW * BH * (int)sizeof(T);
    static constexpr int SLOT = (BOX + 127) / 128 * 128;
    static constexpr int L1P = RX * RH * 4;             // a level-1 plane (FP32)
    static constexpr int L1S = (L1P + 127) / 128 * 128;
    static constexpr int smem() { return TB_NS * SLOT + TB_L1 * L1S + TB_NS * 8; }
};

// Four points of one row: x window xw[0..11] (x-4 .. x+7, centre xw[4..7]), y neighbours
// ym[a-1] / yp[a-1] (rows -a / +a), z queue q (9 planes, the centre at index (P + 4) % 9).
template <int MODE>
__device__ __forceinline__ void star4(const float* xw, const VecN<4>* ym, const VecN<4>* yp, const VecN<4>* q, int P, float coeff,
                                      const StarW& wt, float* res)
{
    namespace f2 = gb::f2;
#pragma unroll
    for (int c = 0; c < 4; c += 2) {
        const float2 cen = make_float2(xw[R + c], xw[R + c + 1]);
        float2 v = MODE == 0 ? cen : f2::mul(f2::splat(wt.w[0]), cen);
#pragma unroll
        for (int a = 1; a <= R; a++) {
            const float2 sx = (a & 1) ? make_float2(__fadd_rn(xw[R + c - a], xw[R + c + a]), __fadd_rn(xw[R + c + 1 - a], xw[R + c + 1 + a]))
                                      : f2::add(make_float2(xw[R + c - a], xw[R + c + 1 - a]), make_float2(xw[R + c + a], xw[R + c + 1 + a]));
            const float2 sy = f2::add(make_float2(ym[a - 1].v[c], ym[a - 1].v[c + 1]), make_float2(yp[a - 1].v[c], yp[a - 1].v[c + 1]));
            const VecN<4>& zm = q[(P + 4 - a) % 9];
            const VecN<4>& zp = q[(P + 4 + a) % 9];
            const float2 sz = f2::add(make_float2(zm.v[c], zm.v[c + 1]), make_float2(zp.v[c], zp.v[c + 1]));
            if (MODE == 0) v = f2::add(v, f2::add(f2::add(sx, sy), sz));
            else v = f2::fma(f2::splat(wt.w[a]), f2::add(f2::add(sx, sy), sz), v);
        }
        if (MODE == 0) v = f2::mul(v, f2::splat(coeff));
        res[c] = v.x;
        res[c + 1] = v.y;
    }
}

template <class T, int MODE, int TY>
__global__ void __launch_bounds__(TbStar<T, TY>::NT, 1) star_r4_tb2(const __grid_constant__ CUtensorMap map, T* __restrict__ out, int nx,
                                                                    int ny, int nz, int px, int py, int kz, float coeff, StarW wt,
                                                                    unsigned* __restrict__ status, unsigned long long wait_ns)
{
    typedef TbStar<T, TY> Lay;
    extern __shared__ __align__(128) unsigned char tsm[];
    float* l1 = reinterpret_cast<float*>(tsm + TB_NS * Lay::SLOT);
    uint64_t* bar = reinterpret_cast<uint64_t*>(tsm + TB_NS * Lay::SLOT + TB_L1 * Lay::L1S);
    const int t = threadIdx.x, tx = t % (Lay::RX / 4), ty = t / (Lay::RX / 4);
    const int rx0 = blockIdx.x * Lay::OX, ry0 = blockIdx.y * TY;     // region origin (padded coordinates)
    const int bx0 = rx0 - 2 * R, by0 = ry0 - R;                       // box origin
    const int x = rx0 + 4 * tx, y = ry0 + ty;                         // this thread's first point, its row
    const int k0 = R + blockIdx.z * kz, k1 = min(k0 + kz, nz + R);
    const int pbase = k0 - 2 * R, plast = k1 + 2 * R - 1;             // input planes of the chunk
    const bool out_thread = tx >= 1 && tx <= Lay::OX / 4 && ty >= R && ty < R + TY;
    const size_t plane = (size_t)px * py;
    if (gb::tma::smem_u32(tsm) & 127u) {
        if (t == 0) atomicOr(status, (unsigned)gb::ST_SMEM_ALIGN);
        return;
    }
    if (t == 0) {
        for (int n = 0; n < TB_NS; n++) gb::tma::bar_init(&bar[n], 1);
        gb::tma::fence_init();
        gb::tma::prefetch_map(&map);
    }
    __syncthreads();
    auto slot = [&](int pl) { return reinterpret_cast<const T*>(tsm + ((unsigned)(pl - pbase) % TB_NS) * Lay::SLOT); };
    auto l1slot = [&](int q) { return l1 + (size_t)((unsigned)(q - pbase) % TB_L1) * (Lay::L1S / 4); };
    int last_issued = pbase - 1;
    auto issue = [&](int pl) {
        last_issued = pl;
        const unsigned n = (unsigned)(pl - pbase) % TB_NS;
        gb::tma::arrive_expect(&bar[n], Lay::BOX);
        gb::tma::load_3d(tsm + n * Lay::SLOT, &map, bx0, by0, pl, &bar[n]);
    };
    auto ready = [&](int pl, uint64_t limit) {
        return gb::tma::wait(&bar[(unsigned)(pl - pbase) % TB_NS], ((unsigned)(pl - pbase) / TB_NS) & 1u, limit);
    };
    if (t == 0)
        for (int pl = pbase; pl < pbase + TB_NS && pl <= plast; pl++) issue(pl);

    // interior masks of this thread's 4 points (x) and row (y); planes are checked per plane
    bool xin[4];
#pragma unroll
    for (int e = 0; e < 4; e++) xin[e] = x + e >= R && x + e < nx + R;
    const bool yin = y >= R && y < ny + R;
    const int bown = (ty + R) * Lay::BXW + 4 * tx + 2 * R;  // this thread's 4 points in a box
    const int lown = ty * Lay::RX + 4 * tx;                 // ... in a level-1 plane
    VecN<4> q0[9], q1[9];
#pragma unroll
    for (int m = 0; m < 9; m++)
#pragma unroll
        for (int e = 0; e < 4; e++) q0[m].v[e] = q1[m].v[e] = 0.0f;
    bool bad = false;
    const int iters = plast - pbase + 1;
    for (int ib = 0; ib < iters && !bad; ib += 9) {
#pragma unroll
        for (int P = 0; P < 9; P++) {
            const int it = ib + P;
            if (it < iters && !bad) {
                const int pl = pbase + it;
                if (!ready(pl, wait_ns)) bad = true;
                q0[(P + 8) % 9] = ldsv<T, 4>(slot(pl) + bown);  // level 0, plane pl (queue holds pl-8 .. pl)
                const int q1p = pl - R;                          // level-1 plane computed now
                if (!bad && it >= 2 * R) {
                    const T* b = slot(q1p) + bown;
                    float xw[12];
                    {
                        const VecN<4> lo = ldsv<T, 4>(b - R), hi = ldsv<T, 4>(b + 4);
#pragma unroll
                        for (int e = 0; e < 4; e++) {
                            xw[e] = lo.v[e];
                            xw[8 + e] = hi.v[e];
                            xw[4 + e] = q0[(P + 4) % 9].v[e];
                        }
                    }
                    VecN<4> ym[R], yp[R];
#pragma unroll
                    for (int a = 1; a <= R; a++) {
                        ym[a - 1] = ldsv<T, 4>(b - a * Lay::BXW);
                        yp[a - 1] = ldsv<T, 4>(b + a * Lay::BXW);
                    }
                    float res[4];
                    star4<MODE>(xw, ym, yp, q0, P, coeff, wt, res);
                    const bool zin = q1p >= R && q1p < nz + R;
                    VecN<4> lv;
#pragma unroll
                    for (int e = 0; e < 4; e++) lv.v[e] = (zin && yin && xin[e]) ? res[e] : q0[(P + 4) % 9].v[e];
                    *reinterpret_cast<float4*>(l1slot(q1p) + lown) = make_float4(lv.v[0], lv.v[1], lv.v[2], lv.v[3]);
                    q1[(P + 8) % 9] = lv;  // level 1, plane q1p (queue holds q1p-8 .. q1p)
                }
                // the level-1 plane is complete; the box of plane q1p is no longer needed
                bad = __syncthreads_or(bad);
                if (t == 0 && !bad && it >= R && pl + R <= plast) issue(pl + R);
                const int q2 = q1p - R;  // output plane
                if (!bad && it >= 4 * R && out_thread) {
                    const float* b = l1slot(q2) + lown;
                    float xw[12];
                    {
                        const float4 lo = *reinterpret_cast<const float4*>(b - R), hi = *reinterpret_cast<const float4*>(b + 4);
                        xw[0] = lo.x; xw[1] = lo.y; xw[2] = lo.z; xw[3] = lo.w;
                        xw[8] = hi.x; xw[9] = hi.y; xw[10] = hi.z; xw[11] = hi.w;
#pragma unroll
                        for (int e = 0; e < 4; e++) xw[4 + e] = q1[(P + 4) % 9].v[e];
                    }
                    VecN<4> ym[R], yp[R];
#pragma unroll
                    for (int a = 1; a <= R; a++) {
                        ym[a - 1] = ldsv<float, 4>(b - a * Lay::RX);
                        yp[a - 1] = ldsv<float, 4>(b + a * Lay::RX);
                    }
                    float res[4];
                    star4<MODE>(xw, ym, yp, q1, P, coeff, wt, res);
                    if (yin && x < nx + R) {
                        T* o = out + (size_t)q2 * plane + (size_t)y * px + x;
                        if (x + 4 <= nx + R) stgv<T, 4>(o, res);
                        else
                            for (int e = 0; e < 4 && x + e < nx + R; e++) st<T>(o + e, res[e]);
                    }
                }
            }
        }
    }
    if (bad && t == 0) {  // a wait gave up: report and let the copies still in flight land
        atomicOr(status, (unsigned)gb::ST_TMA_TIMEOUT);
        for (int pl = max(pbase, last_issued - TB_NS + 1); pl <= last_issued; pl++) ready(pl, gb::tma::DRAIN_NS);
    }
}

// Runs `pairs` double steps (a -> b in two steps per launch, ping-pong); the caller does any odd
// step with the single-step tile.
template <class T, int TY>
int run_star_tb2(T** buf, int nx, int ny, int nz, int pitch, int pairs, int mode, float coeff, StarW w, int kz, cudaStream_t st)
{
    typedef TbStar<T, TY> Lay;
    const CUtensorMapDataType dt = sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
    CUtensorMap maps[2];
    for (int n = 0; n < 2; n++)
        GB_TRY(gb::tensor_map_3d(&maps[n], dt, sizeof(T), buf[n], nx + 2 * R, ny + 2 * R, nz + 2 * R, pitch, ny + 2 * R, Lay::BXW,
                                 Lay::BH));
    unsigned* status;
    GB_TRY(gb::status_word(&status));
    constexpr int smem = Lay::smem();
    auto kern = mode == 0 ? star_r4_tb2<T, 0, TY> : star_r4_tb2<T, 1, TY>;
    GB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    int tkz = kz;
    if (tkz <= 0) {  // whole waves of the one resident CTA per SM, counting the 16 extra planes a chunk reads
        const long long per_chunk = (long long)gb::ceil_div(nx, Lay::OX) * gb::ceil_div(ny, TY);
        tkz = gb::wave_chunk(nz, 64, 256, per_chunk, gb::sm_count(), 4 * R);
    }
    dim3 blk(Lay::NT), grd(gb::ceil_div(nx, Lay::OX), gb::ceil_div(ny, TY), gb::ceil_div(nz, tkz));
    int ci = 0;
    for (int it = 0; it < pairs; it++) {
        kern<<<grd, blk, smem, st>>>(maps[ci], buf[1 - ci], nx, ny, nz, pitch, ny + 2 * R, tkz, coeff, w, status, 1000000000ull);
        ci = 1 - ci;
    }
    return gb::launched("star_r4_tb2");
}

template <class T, int MODE, int RY>
void launch_star(const T* in, T* out, int nx, int ny, int nz, int px, int kz, float coeff, StarW w, cudaStream_t st)
{
    dim3 blk(TX, 8), grd(gb::ceil_div(nx, TX), gb::ceil_div(ny, 8 * RY), gb::ceil_div(nz, kz));
    static_assert(RY >= 1, "rows per thread");
    star_r4_sweep<T, MODE, RY><<<grd, blk, 0, st>>>(in, out, nx, ny, nz, px, ny + 2 * R, kz, coeff, w);
}

template <class T, int VXT, int TRY = 2>
int run_star_tma(T** buf, int nx, int ny, int nz, int pitch, int iters, int mode, float coeff, StarW w, int kz, int* cur_index,
                 cudaStream_t st)
{
    typedef TmaStar<T, VXT, TRY> Lay;
    constexpr int TTY = Lay::TTY;
    const CUtensorMapDataType dt = sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
    CUtensorMap maps[2];
    for (int n = 0; n < 2; n++)
        GB_TRY(gb::tensor_map_3d(&maps[n], dt, sizeof(T), buf[n], nx + 2 * R, ny + 2 * R, nz + 2 * R, pitch, ny + 2 * R, Lay::SW,
                                 Lay::SH));
    unsigned* status;
    GB_TRY(gb::status_word(&status));
    constexpr int smem = Lay::smem();
    auto kern = mode == 0 ? star_r4_tma<T, 0, VXT, TRY> : star_r4_tma<T, 1, VXT, TRY>;
    GB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    // default z chunk: 32-64 planes per CTA, the length whose grid fills the resident CTAs in the
    // most nearly whole waves, counting the 8 halo planes each chunk re-reads (512^3: 47 planes,
    // 2816 CTAs in 4.6 waves of 608)
    int tkz = kz;
    if (tkz <= 0) {
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 16 * (TTY / TRY), smem) != cudaSuccess || per_sm < 1)
            per_sm = 1;
        tkz = gb::wave_chunk(nz, 32, 64, (long long)gb::ceil_div(nx, Lay::TX) * gb::ceil_div(ny, TTY),
                             (long long)per_sm * gb::sm_count(), 2 * R);
    }
    dim3 blk(16, TTY / TRY), grd(gb::ceil_div(nx, Lay::TX), gb::ceil_div(ny, TTY), gb::ceil_div(nz, tkz));
    unsigned long long wait_ns = 1000000000ull, test_ns = 0;
    unsigned shortfall = 0;
    if (iters > 0 && gb::take_test_stall(gb::TEST_TMA_SHORTFALL, &test_ns)) {  // a test runs the first launch's waits out
        wait_ns = test_ns;
        shortfall = 16;
    }
    int ci = 0;
    for (int it = 0; it < iters; it++) {
        kern<<<grd, blk, smem, st>>>(maps[ci], buf[1 - ci], nx, ny, nz, pitch, ny + 2 * R, tkz, coeff, w, status, wait_ns, shortfall);
        wait_ns = 1000000000ull;
        shortfall = 0;
        ci = 1 - ci;
    }
    GB_TRY(gb::launched("star_r4_tma"));
    if (cur_index) *cur_index = ci;
    return APPFIS_GB_OK;
}

// ---------------------------------------------------------------- autotuner
// The kernel (tile, time-blocking depth) and z chunk of a shape are chosen by timing: every
// candidate runs once from a into b (b's interior is overwritten, a and both halos are not:
// kernels write interior points only), then three more times between CUDA events on the
// caller's stream, and the fastest time per step wins.  Candidates: on 16-byte aligned rows the
// TMA-staged tiles with 4 or 2 x points per thread (depth 1) and the two-step tiles with 64 x 16
// or 64 x 8 outputs (depth 2), otherwise the vector and scalar tiles; z chunks of the tile's
// default and 32 .. 256 planes.  Depths 3 and 4 are not candidates: a depth-D tile keeps D
// register queues of 9 planes per point (36 D registers per thread of 4 points) over a region
// 8 (D - 1) points wider and taller than its output, so at D = 3 a 64 x 8 output tile needs
// 20 x 24 threads x about 160 registers (77 K > the 64 K register file of an SM), and smaller
// tiles redo more step-1 work than the bytes they save.  The result is kept per device and shape
// (and dtype, form, pitch) for the process; APPFIS_GB_STAR_AUTO uses it.  With the environment
// variable APPFIS_GB_TUNE_FILE set, results are also read from / appended to that text file.
struct TuneKey {
    int dev, dtype, mode, nx, ny, nz, pitch;
    bool operator<(const TuneKey& o) const
    {
        const int a[7] = {dev, dtype, mode, nx, ny, nz, pitch}, b[7] = {o.dev, o.dtype, o.mode, o.nx, o.ny, o.nz, o.pitch};
        return std::lexicographical_compare(a, a + 7, b, b + 7);
    }
};
struct TuneVal {
    int tile, kz;
    float ms_per_step;
};
std::mutex g_tune_mu;
std::map<TuneKey, TuneVal> g_tune;
bool g_tune_file_read = false;

const char* tune_file() { return std::getenv("APPFIS_GB_TUNE_FILE"); }

// GPU name (spaces removed) so that a tune file shared between machines keys by device model.
std::string device_tag(int dev)
{
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return "unknown";
    std::string n(prop.name);
    n.erase(std::remove(n.begin(), n.end(), ' '), n.end());
    return n;
}

void read_tune_file_locked()
{
    if (g_tune_file_read) return;
    g_tune_file_read = true;
    const char* path = tune_file();
    if (!path) return;
    FILE* f = std::fopen(path, "r");
    if (!f) return;
    int dev = 0;
    cudaGetDevice(&dev);
    const std::string tag = device_tag(dev);
    char name[128], kind[32];
    TuneKey k;
    TuneVal v;
    while (std::fscanf(f, "%31s %127s %d %d %d %d %d %d %d %d %f", kind, name, &k.dtype, &k.mode, &k.nx, &k.ny, &k.nz, &k.pitch, &v.tile,
                       &v.kz, &v.ms_per_step) == 11)
        if (std::string(kind) == "star_r4" && tag == name) {
            k.dev = dev;
            g_tune[k] = v;
        }
    std::fclose(f);
}

bool tuned(const TuneKey& k, TuneVal* v)
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    read_tune_file_locked();
    auto it = g_tune.find(k);
    if (it == g_tune.end()) return false;
    *v = it->second;
    return true;
}

void record_tune(const TuneKey& k, const TuneVal& v)
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[k] = v;
    const char* path = tune_file();
    if (!path) return;
    if (FILE* f = std::fopen(path, "a")) {
        std::fprintf(f, "star_r4 %s %d %d %d %d %d %d %d %d %.6f\n", device_tag(k.dev).c_str(), k.dtype, k.mode, k.nx, k.ny, k.nz, k.pitch,
                     v.tile, v.kz, v.ms_per_step);
        std::fclose(f);
    }
}

template <class T>
int run_star(T* a, T* b, int nx, int ny, int nz, int pitch, int iters, int mode, float coeff, const float* w5, int tile,
             int kz, int* cur_index, cudaStream_t st);

int steps_per_launch(int tile) { return (tile == APPFIS_GB_STAR_TB2 || tile == APPFIS_GB_STAR_TB2_8) ? 2 : 1; }

template <class T>
int tune_star(T* a, T* b, int dtype, int nx, int ny, int nz, int pitch, int mode, float coeff, const float* w5, TuneVal* best,
              cudaStream_t st)
{
    const bool rows16 = (pitch * sizeof(T)) % 16 == 0 && gb::aligned16(a) && gb::aligned16(b);
    const bool vec4 = pitch % 4 == 0 && ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b)) % (sizeof(T) * 4)) == 0;
    std::vector<int> tiles;
    if (rows16)
        tiles = {APPFIS_GB_STAR_TMA_X4, APPFIS_GB_STAR_TMA_X4R4, APPFIS_GB_STAR_TMA_X2, APPFIS_GB_STAR_TB2, APPFIS_GB_STAR_TB2_8};
    else if (vec4) tiles = {APPFIS_GB_STAR_VEC, APPFIS_GB_STAR_SCALAR4};
    else tiles = {APPFIS_GB_STAR_SCALAR4, APPFIS_GB_STAR_SCALAR2};
    std::vector<int> chunks = {0};
    for (int c : {32, 48, 64, 96, 128, 256})
        if (c < nz) chunks.push_back(c);
    cudaEvent_t e0, e1;
    GB_CUDA(cudaEventCreate(&e0));
    GB_CUDA(cudaEventCreate(&e1));
    best->ms_per_step = 1e30f;
    int rc = APPFIS_GB_OK;
    for (int tile : tiles) {
        for (int kz : chunks) {
            const int steps = steps_per_launch(tile);
            rc = run_star<T>(a, b, nx, ny, nz, pitch, steps, mode, coeff, w5, tile, kz, nullptr, st);  // warm-up
            if (rc != APPFIS_GB_OK) break;
            cudaEventRecord(e0, st);
            for (int r = 0; r < 3 && rc == APPFIS_GB_OK; r++) rc = run_star<T>(a, b, nx, ny, nz, pitch, steps, mode, coeff, w5, tile, kz, nullptr, st);
            cudaEventRecord(e1, st);
            if (rc != APPFIS_GB_OK) break;
            if (cudaEventSynchronize(e1) != cudaSuccess) {
                rc = gb::launched("star_r4 tuning");
                break;
            }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            ms /= 3.0f * steps;
            if (ms < best->ms_per_step) *best = TuneVal{tile, kz, ms};
        }
        if (rc != APPFIS_GB_OK) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    GB_TRY(rc);
    GB_TRY(gb::check_status("star_r4 tuning"));  // a bounded wait of a TMA tile that gave up
    int dev = 0;
    GB_CUDA(cudaGetDevice(&dev));
    record_tune(TuneKey{dev, dtype, mode, nx, ny, nz, pitch}, *best);
    return APPFIS_GB_OK;
}

template <class T>
int run_star(T* a, T* b, int nx, int ny, int nz, int pitch, int iters, int mode, float coeff, const float* w5, int tile,
             int kz, int* cur_index, cudaStream_t st)
{
    StarW w = {{0, 0, 0, 0, 0}};
    if (w5)
        for (int n = 0; n < 5; n++) w.w[n] = w5[n];
    T* buf[2] = {a, b};
    const bool rows16 = (pitch * sizeof(T)) % 16 == 0 && gb::aligned16(a) && gb::aligned16(b);
    const bool vec4 = pitch % 4 == 0 && ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b)) % (sizeof(T) * 4)) == 0;
    if (tile == APPFIS_GB_STAR_AUTO)  // TMA-staged when rows are 16-byte aligned, else vectors, else scalar
        tile = rows16 ? APPFIS_GB_STAR_TMA_X4 : (vec4 ? APPFIS_GB_STAR_VEC : APPFIS_GB_STAR_SCALAR4);
    if ((tile == APPFIS_GB_STAR_TMA_X4 || tile == APPFIS_GB_STAR_TMA_X2 || tile == APPFIS_GB_STAR_TB2 || tile == APPFIS_GB_STAR_TB2_8 ||
         tile == APPFIS_GB_STAR_TMA_X4R4) &&
        !rows16)
        return gb::fail(APPFIS_GB_EINVAL, "star_r4: the TMA-staged tiles need 16-byte aligned rows and fields");
    if (tile == APPFIS_GB_STAR_VEC && !vec4)
        return gb::fail(APPFIS_GB_EINVAL, "star_r4: the vector tile needs a pitch of a multiple of 4 and aligned fields");
    if (tile == APPFIS_GB_STAR_TB2 || tile == APPFIS_GB_STAR_TB2_8) {
        // pairs of steps in the time-blocked tile, an odd last step in the single-step tile
        const int pairs = iters / 2;
        if (pairs > 0) {
            if (tile == APPFIS_GB_STAR_TB2) GB_TRY((run_star_tb2<T, 16>(buf, nx, ny, nz, pitch, pairs, mode, coeff, w, kz, st)));
            else GB_TRY((run_star_tb2<T, 8>(buf, nx, ny, nz, pitch, pairs, mode, coeff, w, kz, st)));
        }
        int ci = pairs % 2;
        if (iters % 2) {
            T* b2[2] = {buf[ci], buf[1 - ci]};
            GB_TRY((run_star_tma<T, 4>(b2, nx, ny, nz, pitch, 1, mode, coeff, w, 0, nullptr, st)));
            ci = 1 - ci;
        }
        if (cur_index) *cur_index = ci;
        return APPFIS_GB_OK;
    }
    if (tile == APPFIS_GB_STAR_TMA_X4) return run_star_tma<T, 4>(buf, nx, ny, nz, pitch, iters, mode, coeff, w, kz, cur_index, st);
    if (tile == APPFIS_GB_STAR_TMA_X4R4)
        return run_star_tma<T, 4, 4>(buf, nx, ny, nz, pitch, iters, mode, coeff, w, kz, cur_index, st);
    if (tile == APPFIS_GB_STAR_TMA_X2) return run_star_tma<T, 2>(buf, nx, ny, nz, pitch, iters, mode, coeff, w, kz, cur_index, st);
    if (kz <= 0) kz = 32;
    int ci = 0;
    for (int it = 0; it < iters; it++) {
        if (tile == APPFIS_GB_STAR_VEC) {
            dim3 blk(16, 16), grd(gb::ceil_div(nx, VTX), gb::ceil_div(ny, VTY), gb::ceil_div(nz, kz));
            if (mode == 0) star_r4_vec<T, 0><<<grd, blk, 0, st>>>(buf[ci], buf[1 - ci], nx, ny, nz, pitch, ny + 2 * R, kz, coeff, w);
            else star_r4_vec<T, 1><<<grd, blk, 0, st>>>(buf[ci], buf[1 - ci], nx, ny, nz, pitch, ny + 2 * R, kz, coeff, w);
        } else if (mode == 0) {
            if (tile == APPFIS_GB_STAR_SCALAR2) launch_star<T, 0, 2>(buf[ci], buf[1 - ci], nx, ny, nz, pitch, kz, coeff, w, st);
            else launch_star<T, 0, 4>(buf[ci], buf[1 - ci], nx, ny, nz, pitch, kz, coeff, w, st);
        } else {
            if (tile == APPFIS_GB_STAR_SCALAR2) launch_star<T, 1, 2>(buf[ci], buf[1 - ci], nx, ny, nz, pitch, kz, coeff, w, st);
            else launch_star<T, 1, 4>(buf[ci], buf[1 - ci], nx, ny, nz, pitch, kz, coeff, w, st);
        }
        ci = 1 - ci;
    }
    GB_TRY(gb::launched("star_r4 sweep"));
    if (cur_index) *cur_index = ci;
    return APPFIS_GB_OK;
}

}  // namespace

extern "C" {

int appfis_gb_star_r4(void* a, void* b, int dtype, int nx, int ny, int nz, int pitch, int iters, int mode, float coeff,
                      const float* weights, int tile, int zchunk, int* cur_index, void* stream)
{
    if (!a || !b || a == b) return gb::fail(APPFIS_GB_EINVAL, "star_r4: null or aliased buffers");
    if (nx < 1 || ny < 1 || nz < 1 || pitch < nx + 2 * R) return gb::fail(APPFIS_GB_EINVAL, "star_r4: bad dims");
    if (mode != 0 && mode != 1) return gb::fail(APPFIS_GB_EINVAL, "star_r4: mode %d", mode);
    if (mode == 1 && !weights) return gb::fail(APPFIS_GB_EINVAL, "star_r4: weighted mode needs 5 weights");
    if (iters < 0) return gb::fail(APPFIS_GB_EINVAL, "star_r4: negative iteration count");
    if (tile != APPFIS_GB_STAR_AUTO && tile != APPFIS_GB_STAR_SCALAR2 && tile != APPFIS_GB_STAR_SCALAR4 &&
        tile != APPFIS_GB_STAR_TMA_X4 && tile != APPFIS_GB_STAR_TMA_X2 && tile != APPFIS_GB_STAR_VEC && tile != APPFIS_GB_STAR_TB2 &&
        tile != APPFIS_GB_STAR_TB2_8 && tile != APPFIS_GB_STAR_TMA_X4R4)
        return gb::fail(APPFIS_GB_EINVAL, "star_r4: unknown tile %d", tile);
    int kz = zchunk <= 0 ? 0 : zchunk;  // 0: the tile's default (TMA-staged: 32-64 planes chosen for whole waves; 32 otherwise)
    cudaStream_t st = gb::as_stream(stream);
    if (tile == APPFIS_GB_STAR_AUTO) {  // a tuned choice for this device and shape, if there is one
        int dev = 0;
        TuneVal v;
        if (cudaGetDevice(&dev) == cudaSuccess && tuned(TuneKey{dev, dtype, mode, nx, ny, nz, pitch}, &v)) {
            tile = v.tile;
            if (zchunk <= 0) kz = v.kz;
        }
    }
    if (dtype == APPFIS_GB_F32)
        return run_star<float>((float*)a, (float*)b, nx, ny, nz, pitch, iters, mode, coeff, weights, tile, kz, cur_index, st);
    if (dtype == APPFIS_GB_F16)
        return run_star<__half>((__half*)a, (__half*)b, nx, ny, nz, pitch, iters, mode, coeff, weights, tile, kz, cur_index, st);
    return gb::fail(APPFIS_GB_EINVAL, "star_r4: dtype %d (F32 or F16)", dtype);
}

int appfis_gb_star_r4_tune(void* a, void* b, int dtype, int nx, int ny, int nz, int pitch, int mode, float coeff,
                           const float* weights, int* tile_out, int* zchunk_out, float* ms_per_step_out, void* stream)
{
    if (!a || !b || a == b) return gb::fail(APPFIS_GB_EINVAL, "star_r4_tune: null or aliased buffers");
    if (nx < 1 || ny < 1 || nz < 1 || pitch < nx + 2 * R) return gb::fail(APPFIS_GB_EINVAL, "star_r4_tune: bad dims");
    if (mode != 0 && mode != 1) return gb::fail(APPFIS_GB_EINVAL, "star_r4_tune: mode %d", mode);
    if (mode == 1 && !weights) return gb::fail(APPFIS_GB_EINVAL, "star_r4_tune: weighted mode needs 5 weights");
    cudaStream_t st = gb::as_stream(stream);
    TuneVal best{0, 0, 0.f};
    if (dtype == APPFIS_GB_F32) GB_TRY(tune_star<float>((float*)a, (float*)b, dtype, nx, ny, nz, pitch, mode, coeff, weights, &best, st));
    else if (dtype == APPFIS_GB_F16)
        GB_TRY(tune_star<__half>((__half*)a, (__half*)b, dtype, nx, ny, nz, pitch, mode, coeff, weights, &best, st));
    else return gb::fail(APPFIS_GB_EINVAL, "star_r4_tune: dtype %d (F32 or F16)", dtype);
    if (tile_out) *tile_out = best.tile;
    if (zchunk_out) *zchunk_out = best.kz;
    if (ms_per_step_out) *ms_per_step_out = best.ms_per_step;
    return APPFIS_GB_OK;
}

}  // extern "C"
