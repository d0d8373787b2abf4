// Himeno 19-point Jacobi (FP32 plain form and FP16-storage defect-correction form), with the
// per-sweep gosa = sum(ss^2) reduced in double inside the sweep.
//
// Reference functor: Himeno/src/himeno_appfis.hpp:178-198, run by Execute3D once per iteration
// on a DUAL p grid and 12 SINGLE coefficient grids (:74-86, :108-114).  The reference computes
// no gosa; ss is exactly its :195 expression.
//
// Plain form: one launch per sweep, a 2.5-D z-march with the p planes in a shared ring and the
// 12 coefficient streams read once: himeno_tma (tiles moved by the tensor memory accelerator)
// when rows and fields are 16-byte aligned, else himeno_ring<0> (register-prefetched loads).
// The sum uses round-to-nearest intrinsics in the reference's order (no FMA contraction), so p
// is bit-identical to the reference CPU path.
//
// Defect-correction form (FP16 storage, FP32 arithmetic).  With p = P + e (P an FP32 master
// frozen between corrections) the Jacobi update p' = p + w*bnd*(a3*(N p + wrk1) - p) becomes
//     e' = e + w*bnd*(a3*N e - e) + D,    D = w*ss(P)   (the FP32 defect of the master),
// an exact rewrite (N = the 18 neighbour terms of s0 without wrk1).  Inner sweeps read e, D and
// the ten neighbour/boundary coefficient fields (a0 a1 a2 b0 b1 b2 c0 c1 c2 bnd) in FP16 and the
// diagonal scale a3 in FP32 (it multiplies the whole neighbour sum, so its rounding would bias
// every point coherently): 30 B per point per sweep instead of 56.  Every `period` sweeps a
// correction pass folds e into P, recomputes D from the FP32 coefficients and restarts e at 0,
// which bounds the FP16 error to the last period's correction.  The sweep's own ss is
// (e' - e)/w (FP32, before rounding e').  Inner sweeps: himeno_mixed2 (TMA-staged, two points
// per thread) when the FP16 rows are 16-byte aligned, else himeno_ring<1>.
#include <cuda_fp16.h>

#include <type_traits>

#include "gb_common.cuh"
#include "f32x2.cuh"
#include "tma.cuh"

namespace {

struct Coef12 {
    const float* c[12];  // a0 a1 a2 a3 b0 b1 b2 c0 c1 c2 bnd wrk1
};
struct H10 {
    const __half* c[10];  // a0 a1 a2 b0 b1 b2 c0 c1 c2 bnd in FP16
    const float* a3;      // FP32
};

__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }

// gosa without atomics: each block of a sweep writes the sums of its values to
// part[vals * block + v]; block 0 of the next launch on the stream, after its own work, folds the
// previous launch's sums into that launch's gosa values (the previous launch has finished by
// then), and himeno_gosa_fold folds those of the last launch before a correction pass or the end.
// Each value is folded in a fixed order (strided per thread, then a shuffle tree, then the warps
// in order), so gosa is deterministic.
struct GosaIO {
    double* part;        // this launch's block sums (null: no gosa)
    const double* prev;  // the previous launch's block sums (null: nothing to fold)
    double* prev_out;    // its gosa values
    unsigned prev_n;     // its block count
    int prev_vals;       // its sums per block (1, or 2 for a two-sweep pass)
};

__device__ __forceinline__ double block_sum(double v, double* sh)
{
    const int nthreads = blockDim.x * blockDim.y;
    const int t = threadIdx.y * blockDim.x + threadIdx.x;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();  // sh may still be read from an earlier call
    if ((t & 31) == 0) sh[t >> 5] = v;
    __syncthreads();
    double s = 0.0;
    if (t == 0)
        for (int q = 0; q < (nthreads >> 5); q++) s += sh[q];
    return s;  // thread 0
}

__device__ void gosa_fold(const GosaIO& g)
{
    __shared__ double sh[32];
    const int nthreads = blockDim.x * blockDim.y;
    const int t = threadIdx.y * blockDim.x + threadIdx.x;
    for (int w = 0; w < g.prev_vals; w++) {
        double v = 0.0;
        for (unsigned b = t; b < g.prev_n; b += nthreads) v += g.prev[(size_t)g.prev_vals * b + w];
        const double s = block_sum(v, sh);
        if (t == 0) g.prev_out[w] = s;
    }
}

// The end of a sweep kernel: this block's sums of its NV values, then (block 0) the fold of the
// previous launch.
template <int NV>
__device__ __forceinline__ void gosa_end(const double (&v)[NV], const GosaIO& g)
{
    __shared__ double sh[32];
    if (g.part) {
        const unsigned b = (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
#pragma unroll
        for (int w = 0; w < NV; w++) {
            const double s = block_sum(v[w], sh);
            if (threadIdx.x == 0 && threadIdx.y == 0) g.part[(size_t)NV * b + w] = s;
        }
    }
    if (g.prev && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0) gosa_fold(g);
}

__global__ void himeno_gosa_fold(GosaIO g) { gosa_fold(g); }

// Per-thread sum of squares in two floats (hi + lo, ~48 significant bits): the square is split
// exactly with an FMA and added with an exact two-sum, so a thread's few dozen terms stay within
// ~1e-13 relative of the exact sum with FP32 instructions only (this part's FP64 rate is a small
// fraction of its FP32 rate, and one FP64 multiply-add per point would cost more than the
// point's memory traffic).  The block and grid sums that follow are in double.
struct SqAcc {
    float hi = 0.0f, lo = 0.0f;
    __device__ __forceinline__ void add_sq(float x)
    {
        const float p = __fmul_rn(x, x);
        const float e = __fmaf_rn(x, x, -p);  // p + e == x*x exactly
        const float s = __fadd_rn(hi, p);
        const float bb = __fsub_rn(s, hi);
        const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));  // hi + p == s + err
        hi = s;
        lo = __fadd_rn(lo, __fadd_rn(err, e));
    }
    __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

// 19-point s0 in the reference's order, on any readable field F (F(di,dj,dk) -> float)
#define HIMENO_S0(F, A0, A1, A2, B0, B1, B2, C0, C1, C2, W1)                                               \
    fadd(fadd(fadd(fadd(fadd(fadd(fadd(fadd(fadd(fmul(A0, F(1, 0, 0)), fmul(A1, F(0, 1, 0))), fmul(A2, F(0, 0, 1))), \
                                           fmul(B0, fadd(fsub(fsub(F(1, 1, 0), F(1, -1, 0)), F(-1, 1, 0)), F(-1, -1, 0)))), \
                                      fmul(B1, fadd(fsub(fsub(F(0, 1, 1), F(0, -1, 1)), F(0, 1, -1)), F(0, -1, -1)))),      \
                                 fmul(B2, fadd(fsub(fsub(F(1, 0, 1), F(-1, 0, 1)), F(1, 0, -1)), F(-1, 0, -1)))),           \
                            fmul(C0, F(-1, 0, 0))),                                                                         \
                       fmul(C1, F(0, -1, 0))),                                                                              \
                  fmul(C2, F(0, 0, -1))),                                                                                   \
         W1)

// ---------------------------------------------------------------- defect-correction form
// FP16 copies of the ten neighbour / boundary coefficient fields (over the interior).
__global__ void himeno_half_coef(Coef12 cf, __half* __restrict__ w, size_t field, int nx, int ny, int nz, int px, int py)
{
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = 1 + blockIdx.y;
    const int k = 1 + blockIdx.z;
    if (i > nx) return;
    const size_t c = ((size_t)k * py + j) * px + i;
    const int map[10] = {0, 1, 2, 4, 5, 6, 7, 8, 9, 10};  // a0 a1 a2 b0 b1 b2 c0 c1 c2 bnd
#pragma unroll
    for (int n = 0; n < 10; n++) w[n * field + c] = __float2half_rn(cf.c[map[n]][c]);
}

// Correction pass: P' = P + e, D = omega*ss(P'), e_next = 0.  Reads P and e at neighbours.
template <int BX, int BY>
__global__ void __launch_bounds__(BX* BY) himeno_correct(Coef12 cf, const float* __restrict__ P, const __half* __restrict__ e,
                                                          float* __restrict__ Pn, __half* __restrict__ D,
                                                          __half* __restrict__ enext, int nx, int ny, int nz, int px,
                                                          int py, int kz, float omega, float inv_omega, int prime, GosaIO gz)
{
    const int i = 1 + blockIdx.x * BX + threadIdx.x;
    const int j = 1 + blockIdx.y * BY + threadIdx.y;
    const int k0 = 1 + blockIdx.z * kz, k1 = min(k0 + kz, nz + 1);
    const bool act = i <= nx && j <= ny;
    const ptrdiff_t plane = (ptrdiff_t)px * py;
    ptrdiff_t c = ((ptrdiff_t)k0 * py + j) * px + i;
    float g = 0.0f;
    for (int k = k0; act && k < k1; k++) {
#define QF(di, dj, dk)                                                                                      \
    (__ldg(P + c + (ptrdiff_t)(di) + (ptrdiff_t)(dj) * px + (ptrdiff_t)(dk) * (ptrdiff_t)plane) +          \
     __half2float(e[c + (ptrdiff_t)(di) + (ptrdiff_t)(dj) * px + (ptrdiff_t)(dk) * (ptrdiff_t)plane]))
        const float q0 = QF(0, 0, 0);
        const float s0 = HIMENO_S0(QF, __ldg(cf.c[0] + c), __ldg(cf.c[1] + c), __ldg(cf.c[2] + c), __ldg(cf.c[4] + c),
                                   __ldg(cf.c[5] + c), __ldg(cf.c[6] + c), __ldg(cf.c[7] + c), __ldg(cf.c[8] + c),
                                   __ldg(cf.c[9] + c), __ldg(cf.c[11] + c));
#undef QF
        const float ss = (s0 * __ldg(cf.c[3] + c) - q0) * __ldg(cf.c[10] + c);
        const __half dh = __float2half_rn(omega * ss);
        Pn[c] = q0;
        D[c] = dh;
        enext[c] = prime ? dh : __float2half_rn(0.0f);
        if (prime) {  // the next sweep from e = 0 gives e = D exactly, with ss = D / omega
            const float s1 = __half2float(dh) * inv_omega;
            g = __fmaf_rn(s1, s1, g);
        }
        c += plane;
    }
    gosa_end<1>({(double)g}, gz);
}

// ---------------------------------------------------------------- 2.5-D forms with a shared plane ring
// A CTA of RX x RY threads owns an (x, y) tile and marches a chunk of z.  p (or e) planes k-1,
// k, k+1 live in a 4-slot shared ring with a one-cell x/y halo: plane k+2 is loaded into
// registers one iteration ahead and written to its slot after the sweep of plane k, so one
// barrier per plane suffices and every p value comes from memory once per CTA.  The point's
// coefficients for plane k+1 are loaded while plane k is computed.  All neighbour reads are
// shared-memory reads, so the only global traffic is the compulsory streams.
constexpr int RX = 32, RY = 8;
constexpr int RW = RX + 2, RH = RY + 2, RSLOT = RW * RH;
constexpr int RHALO = RSLOT - RX * RY;  // 84 halo cells per plane

// (row, col) in the slot of halo item h (0 <= h < RHALO): top row, bottom row, left col, right col
__device__ __forceinline__ int halo_slot(int h)
{
    if (h < RW) return h;                                     // row 0
    h -= RW;
    if (h < RW) return (RH - 1) * RW + h;                     // row RH-1
    h -= RW;
    if (h < RY) return (h + 1) * RW;                          // col 0, rows 1..RY
    h -= RY;
    return (h + 1) * RW + RW - 1;                             // col RW-1
}

template <class L>
__device__ __forceinline__ float ring_load(const L* f, size_t idx, bool ok);
template <> __device__ __forceinline__ float ring_load<float>(const float* f, size_t idx, bool ok) { return ok ? __ldg(f + idx) : 0.0f; }
template <> __device__ __forceinline__ float ring_load<__half>(const __half* f, size_t idx, bool ok)
{
    return ok ? __half2float(__ldg(f + idx)) : 0.0f;
}

// Loads plane k of field f for this thread: its centre value and (threads < RHALO) one halo value.
template <class L>
__device__ __forceinline__ void ring_fetch(const L* f, int k, int i, int j, int hi, int hj, int nx, int ny, int px,
                                           size_t plane, int t, float& c, float& h)
{
    const size_t base = (size_t)k * plane;
    c = ring_load<L>(f, base + (size_t)j * px + i, i <= nx + 1 && j <= ny + 1);
    h = t < RHALO ? ring_load<L>(f, base + (size_t)hj * px + hi, hi <= nx + 1 && hj <= ny + 1) : 0.0f;
}

__device__ __forceinline__ void ring_store(float* slot, int t, int tx, int ty, int hs, float c, float h)
{
    slot[(ty + 1) * RW + tx + 1] = c;
    if (t < RHALO) slot[hs] = h;
}

template <int MODE>  // 0: plain FP32 sweep of p; 1: FP16 correction sweep of e
__global__ void __launch_bounds__(RX* RY) himeno_ring(Coef12 cf, H10 hf, const void* __restrict__ pin, void* __restrict__ pout,
                                                       const __half* __restrict__ D, int nx, int ny, int nz, int px, int py,
                                                       int kz, float omega, float inv_omega, GosaIO gz)
{
    __shared__ float ring[4][RSLOT];
    const int tx = threadIdx.x, ty = threadIdx.y, t = ty * RX + tx;
    const int i = 1 + blockIdx.x * RX + tx, j = 1 + blockIdx.y * RY + ty;
    const int k0 = 1 + blockIdx.z * kz, k1 = min(k0 + kz, nz + 1);
    const size_t plane = (size_t)px * py;
    const bool act = i <= nx && j <= ny;
    // this thread's halo cell (fixed for all planes)
    int hs = 0, hi = 0, hj = 0;
    if (t < RHALO) {
        hs = halo_slot(t);
        hi = blockIdx.x * RX + hs % RW;  // padded coords: slot (0,0) is (i0-1, j0-1)
        hj = blockIdx.y * RY + hs / RW;
    }
    typedef typename std::conditional<MODE == 0, float, __half>::type L;
    const L* f = reinterpret_cast<const L*>(pin);
    float c, h;
    // planes k0-1, k0, k0+1 into slots, k0+2 in registers
#pragma unroll
    for (int d = -1; d <= 1; d++) {
        ring_fetch<L>(f, k0 + d, i, j, hi, hj, nx, ny, px, plane, t, c, h);
        ring_store(ring[(k0 + d) & 3], t, tx, ty, hs, c, h);
    }
    float nc = 0.0f, nh = 0.0f;
    if (k0 + 2 <= nz + 1) ring_fetch<L>(f, k0 + 2, i, j, hi, hj, nx, ny, px, plane, t, nc, nh);
    // coefficients of plane k0
    const size_t c0 = ((size_t)k0 * py + j) * px + i;
    float co[12];
    if (act) {
        if (MODE == 0) {
#pragma unroll
            for (int n = 0; n < 12; n++) co[n] = __ldcs(cf.c[n] + c0);
        } else {
#pragma unroll
            for (int n = 0; n < 10; n++) co[n] = __half2float(__ldcs(hf.c[n] + c0));
            co[10] = __ldcs(hf.a3 + c0);
            co[11] = __half2float(__ldcs(D + c0));
        }
    }
    __syncthreads();
    SqAcc g;
    for (int k = k0; k < k1; k++) {
        const size_t cc = ((size_t)k * py + j) * px + i;
        // prefetch the next plane's coefficients
        float cn[12];
        const bool more = k + 1 < k1;
        if (act && more) {
            const size_t c1 = cc + plane;
            if (MODE == 0) {
#pragma unroll
                for (int n = 0; n < 12; n++) cn[n] = __ldcs(cf.c[n] + c1);
            } else {
#pragma unroll
                for (int n = 0; n < 10; n++) cn[n] = __half2float(__ldcs(hf.c[n] + c1));
                cn[10] = __ldcs(hf.a3 + c1);
                cn[11] = __half2float(__ldcs(D + c1));
            }
        }
        if (act) {
            const float* sm = ring[(k - 1) & 3];
            const float* s0 = ring[k & 3];
            const float* sp = ring[(k + 1) & 3];
            const int q = (ty + 1) * RW + tx + 1;
#define RF(di, dj, dk) (((dk) < 0 ? sm : ((dk) > 0 ? sp : s0))[q + (di) + (dj) * RW])
            if (MODE == 0) {
                const float s0v = HIMENO_S0(RF, co[0], co[1], co[2], co[4], co[5], co[6], co[7], co[8], co[9], co[11]);
                const float pc = RF(0, 0, 0);
                const float ss = fmul(fsub(fmul(s0v, co[3]), pc), co[10]);
                reinterpret_cast<float*>(pout)[cc] = fadd(pc, fmul(omega, ss));
                g.add_sq(ss);
            } else {
                // neighbour sum N e (no wrk1), then e' = e + w*bnd*(a3*N e - e) + D
                float ne = co[0] * RF(1, 0, 0) + co[1] * RF(0, 1, 0) + co[2] * RF(0, 0, 1);
                ne += co[3] * ((RF(1, 1, 0) - RF(1, -1, 0)) - (RF(-1, 1, 0) - RF(-1, -1, 0)));
                ne += co[4] * ((RF(0, 1, 1) - RF(0, -1, 1)) - (RF(0, 1, -1) - RF(0, -1, -1)));
                ne += co[5] * ((RF(1, 0, 1) - RF(-1, 0, 1)) - (RF(1, 0, -1) - RF(-1, 0, -1)));
                ne += co[6] * RF(-1, 0, 0) + co[7] * RF(0, -1, 0) + co[8] * RF(0, 0, -1);
                const float e0 = RF(0, 0, 0);
                const float v = e0 + omega * co[9] * (co[10] * ne - e0) + co[11];
                reinterpret_cast<__half*>(pout)[cc] = __float2half_rn(v);
                const float ss = (v - e0) * inv_omega;
                g.add_sq(ss);
            }
#undef RF
        }
        if (more) {
            // plane k+2 (fetched last iteration) into its slot; its last readers (plane k-1's sweep)
            // passed the previous barrier
            ring_store(ring[(k + 2) & 3], t, tx, ty, hs, nc, nh);
            if (k + 3 <= nz + 1) ring_fetch<L>(f, k + 3, i, j, hi, hj, nx, ny, px, plane, t, nc, nh);
#pragma unroll
            for (int n = 0; n < 12; n++) co[n] = cn[n];
        }
        __syncthreads();
    }
    gosa_end<1>({g.value()}, gz);
}

// ---------------------------------------------------------------- TMA-staged FP32 sweep
// Same tile, z-march and arithmetic as himeno_ring<0>, but every stream is moved by the tensor
// memory accelerator: for plane k, one pipeline stage holds the twelve coefficient tiles of
// plane k (32 x 8 each) and p's plane k+1 (40 x 10, the halo included, its x origin rounded down
// to a 16-byte boundary).  Thread 0 keeps S stages in flight; the other threads only read
// shared memory.  The CTA's x tile starts on a 32-point boundary of the padded row (thread tx
// owns padded x = 32*bx + tx, interior points only), so every tile copy starts 16-byte aligned;
// this needs a pitch of a multiple of 4 elements and 16-byte aligned fields.
struct TileMaps {
    CUtensorMap m[13];  // 0..11: the per-point fields, 12: the iterated field
};

struct TmaLayout {
    static constexpr int XO = 4;                          // ring box x origin = tile x - XO
    static constexpr int W = RX + 2 * XO;                 // ring box width (40)
    static constexpr int RB = W * (RY + 2) * 4;           // ring box bytes
    static constexpr int PB = (RB + 127) / 128 * 128;     // ring slot bytes
    static constexpr int CT = 12 * 1024;                  // the coefficient tiles of one plane
    __host__ __device__ static constexpr int tile_off(int n) { return n * 1024; }
    static constexpr int smem(int S) { return S * CT + (S + 2) * PB + S * 8; }
};

template <int S>
__global__ void __launch_bounds__(RX* RY) himeno_tma(const __grid_constant__ TileMaps maps, float* __restrict__ pout, int nx, int ny,
                                                      int nz, int pitch, int py, int kz, float omega,
                                                      GosaIO gz, unsigned* __restrict__ status)
{
    typedef TmaLayout Lay;
    typedef float L;
    constexpr int P = S + 2;  // ring slots: planes k-1 .. k+S
    extern __shared__ __align__(128) unsigned char tsm[];
    unsigned char* stages = tsm;
    unsigned char* slots = tsm + S * Lay::CT;
    uint64_t* bar = reinterpret_cast<uint64_t*>(tsm + S * Lay::CT + P * Lay::PB);

    const int tx = threadIdx.x, ty = threadIdx.y, t = ty * RX + tx;
    const int x0 = blockIdx.x * RX, y0 = 1 + blockIdx.y * RY;
    const int i = x0 + tx, j = y0 + ty;
    const int k0 = 1 + blockIdx.z * kz, k1 = min(k0 + kz, nz + 1);
    const bool act = i >= 1 && i <= nx && j <= ny;
    if (gb::tma::smem_u32(tsm) & 127u) {  // uniform: the copies need 128-byte aligned destinations
        if (t == 0) atomicOr(status, (unsigned)gb::ST_SMEM_ALIGN);
        gosa_end<1>({__longlong_as_double(0x7ff8000000000000ll)}, gz);
        return;
    }
    if (t == 0) {
#pragma unroll
        for (int s = 0; s < S; s++) gb::tma::bar_init(&bar[s], 1);
        gb::tma::fence_init();
        for (int n = 0; n < 13; n++) gb::tma::prefetch_map(&maps.m[n]);
    }
    __syncthreads();

    auto slot = [&](int pl) { return slots + ((pl - (k0 - 1)) % P) * Lay::PB; };
    // thread 0: stage of plane k = the per-point tiles of plane k and the iterated field's plane k+1
    // (the first stage also brings planes k0-1 and k0)
    auto issue = [&](int k) {
        const int s = (k - k0) % S;
        unsigned char* st = stages + s * Lay::CT;
        gb::tma::arrive_expect(&bar[s], Lay::CT + Lay::RB * (k == k0 ? 3 : 1));
        if (k == k0) {
            gb::tma::load_3d(slot(k0 - 1), &maps.m[12], x0 - Lay::XO, y0 - 1, k0 - 1, &bar[s]);
            gb::tma::load_3d(slot(k0), &maps.m[12], x0 - Lay::XO, y0 - 1, k0, &bar[s]);
        }
#pragma unroll
        for (int n = 0; n < 12; n++) gb::tma::load_3d(st + Lay::tile_off(n), &maps.m[n], x0, y0, k, &bar[s]);
        gb::tma::load_3d(slot(k + 1), &maps.m[12], x0 - Lay::XO, y0 - 1, k + 1, &bar[s]);
    };
    if (t == 0)
        for (int k = k0; k < min(k0 + S, k1); k++) issue(k);

    SqAcc g;
    bool bad = false;
    int k = k0;
    const int cq = ty * RX + tx;                        // this point in a per-point tile
    const int q = (ty + 1) * Lay::W + tx + Lay::XO;     // this point in a ring slot
    for (; k < k1; k++) {
        const int s = (k - k0) % S;
        if (!gb::tma::wait(&bar[s], (unsigned)((k - k0) / S) & 1u)) bad = true;
        if (act && !bad) {
            const unsigned char* st = stages + s * Lay::CT;
            const L* sm = reinterpret_cast<const L*>(slot(k - 1));
            const L* s0 = reinterpret_cast<const L*>(slot(k));
            const L* sp = reinterpret_cast<const L*>(slot(k + 1));
            const size_t cc = ((size_t)k * py + j) * pitch + i;
            float co[12];
#pragma unroll
            for (int n = 0; n < 12; n++) co[n] = reinterpret_cast<const float*>(st + Lay::tile_off(n))[cq];
#define RF(di, dj, dk) (((dk) < 0 ? sm : ((dk) > 0 ? sp : s0))[q + (di) + (dj) * Lay::W])
            const float s0v = HIMENO_S0(RF, co[0], co[1], co[2], co[4], co[5], co[6], co[7], co[8], co[9], co[11]);
            const float pc = RF(0, 0, 0);
            const float ss = fmul(fsub(fmul(s0v, co[3]), pc), co[10]);
            pout[cc] = fadd(pc, fmul(omega, ss));
            g.add_sq(ss);
#undef RF
        }
        // everyone is done with stage s and with the slot of plane k-1: refill them with plane k+S
        if (__syncthreads_or(bad)) break;
        if (t == 0 && k + S < k1) issue(k + S);
    }
    if (k < k1) {  // a wait gave up: report, let the copies still in flight land, poison gosa
        if (t == 0) {
            atomicOr(status, (unsigned)gb::ST_TMA_TIMEOUT);
            for (int kk = k; kk < min(k + S, k1); kk++)
                gb::tma::wait(&bar[(kk - k0) % S], (unsigned)((kk - k0) / S) & 1u, gb::tma::DRAIN_NS);
        }
    }
    gosa_end<1>({k < k1 ? __longlong_as_double(0x7ff8000000000000ll) : g.value()}, gz);
}

// ---------------------------------------------------------------- FP16 inner sweep, two points per thread
// The defect-correction sweep is instruction-bound in the one-point form (each FP16 neighbour
// is converted where it is read, and every point pays the loop, wait and barrier overhead), so
// this form gives each thread an x pair and does the arithmetic with packed FP32 pair
// instructions.  Tile 64 x 8 points (32 x 8 threads).  Per plane k a pipeline stage brings the
// eleven FP16/FP32 per-point tiles of plane k (a0 a1 a2 b0 b1 b2 c0 c1 c2 bnd as FP16, a3 as
// FP32, D as FP16) and the FP16 box of e plane k+2 (80 x 10, x origin = tile x - 8).  The threads
// convert that box once into an FP32 ring slot (planes k .. k+2 resident), and each thread keeps
// its pair's neighbour sets of planes k-1 and k in registers, so a plane costs a pair 9 FP32
// shared loads (paired where the pair's columns are contiguous).
constexpr int MY = 8, MXO = 8;  // tile rows; x halo of the e box
constexpr int MIX_S = 2;

// The tile of width TW and its byte sizes.
template <int TW>
struct MixTile {
    static constexpr int X = TW, W = TW + 2 * MXO;
    static constexpr int EB = W * (MY + 2) * 2, ES = (EB + 127) / 128 * 128;
    static constexpr int CT = 10 * X * MY * 2 + X * MY * 4 + X * MY * 2;
    static constexpr int STG = CT + ES, R32 = W * (MY + 2);
    static constexpr int RB = (3 * R32 * 4 + 127) / 128 * 128;  // the 3-slot ring, a 128-byte multiple
    static constexpr int smem(int S) { return S * STG + RB + 3 * ES + S * 8; }
};

template <int TW>
__device__ __forceinline__ void e_box_to_f32(const unsigned char* src, float* dst, int t)
{
    const __half2* h = reinterpret_cast<const __half2*>(src);
    float2* d = reinterpret_cast<float2*>(dst);
    for (int q = t; q < MixTile<TW>::R32 / 2; q += TW / 2 * MY) d[q] = __half22float2(h[q]);
}

// The values of one e plane that a pair's 19-point sum takes from it when the plane is the one
// above or below: the pair itself, the pairs at y +- 1 and the singles at x - 1 and x + 2.  As
// the z-march advances, the set read for plane k+1 serves again as plane k's centre row and then
// as plane k-1, so a step reads only plane k+1's set and plane k's four xy-diagonal singles.
struct PlaneSet {
    float2 c, yp, ym;
    float l, r;
};

__device__ __forceinline__ PlaneSet plane_set(const float* __restrict__ b, int q, int W)
{
    PlaneSet p;
    p.c = *reinterpret_cast<const float2*>(b + q);
    p.yp = *reinterpret_cast<const float2*>(b + q + W);
    p.ym = *reinterpret_cast<const float2*>(b + q - W);
    p.l = b[q - 1];
    p.r = b[q + 2];
    return p;
}

// The xy-diagonal singles of the centre plane: (x-1, y+1), (x+2, y+1), (x-1, y-1), (x+2, y-1).
__device__ __forceinline__ float4 plane_diag(const float* __restrict__ b, int q, int W)
{
    return make_float4(b[q + W - 1], b[q + W + 2], b[q - W - 1], b[q - W + 2]);
}

// One x pair of the FP16 defect-correction sweep from planes k-1 (m), k (z, with its diagonal
// singles d) and k+1 (p), with the pair's coefficients co = a0 a1 a2 b0 b1 b2 c0 c1 c2 bnd, a3
// and D: the new values v and ss = (v - e) / omega.  Terms with x neighbours take one value
// from the next pair over, so their operands straddle register pairs: those are formed lane by
// lane with scalar round-to-nearest operations (the same per-lane arithmetic as the packed ones).
__device__ __forceinline__ void mix_pair(const PlaneSet& m, const PlaneSet& z, float4 d, const PlaneSet& p, const float2 (&co)[10],
                                         float2 a3, float2 D, float2 wsplat, float2 isplat, float2& v, float2& ss)
{
    namespace f2 = gb::f2;
    const float2 e0 = z.c, yp = z.yp, ym = z.ym, zp = p.c, zm = m.c;
    const float e0l = z.l, e0r = z.r, ypl = d.x, ypr = d.y, yml = d.z, ymr = d.w;
    const float zpl = p.l, zpr = p.r, zml = m.l, zmr = m.r;
    // diagonal rows (dy, dz) = (+-1, +-1): centre pair only
    const float2 ypzp = p.yp, ymzp = p.ym, ypzm = m.yp, ymzm = m.ym;
    // F(+1, dy, dz) = (centre.y, right), F(-1, dy, dz) = (left, centre.x)
    const float2 xp = make_float2(e0.y, e0r), xm = make_float2(e0l, e0.x);
    const float2 xpyp = make_float2(yp.y, ypr), xmyp = make_float2(ypl, yp.x);
    const float2 xpym = make_float2(ym.y, ymr), xmym = make_float2(yml, ym.x);
    const float2 xpzp = make_float2(zp.y, zpr), xmzp = make_float2(zpl, zp.x);
    const float2 xpzm = make_float2(zm.y, zmr), xmzm = make_float2(zml, zm.x);
    float2 ne = make_float2(__fmul_rn(co[0].x, xp.x), __fmul_rn(co[0].y, xp.y));
    ne = f2::fma(co[1], yp, ne);
    ne = f2::fma(co[2], zp, ne);
    const float2 txy = make_float2(__fsub_rn(__fsub_rn(xpyp.x, xpym.x), __fsub_rn(xmyp.x, xmym.x)),
                                   __fsub_rn(__fsub_rn(xpyp.y, xpym.y), __fsub_rn(xmyp.y, xmym.y)));
    ne = f2::fma(co[3], txy, ne);
    ne = f2::fma(co[4], f2::sub(f2::sub(ypzp, ymzp), f2::sub(ypzm, ymzm)), ne);
    const float2 txz = make_float2(__fsub_rn(__fsub_rn(xpzp.x, xmzp.x), __fsub_rn(xpzm.x, xmzm.x)),
                                   __fsub_rn(__fsub_rn(xpzp.y, xmzp.y), __fsub_rn(xpzm.y, xmzm.y)));
    ne = f2::fma(co[5], txz, ne);
    ne = make_float2(__fmaf_rn(co[6].x, xm.x, ne.x), __fmaf_rn(co[6].y, xm.y, ne.y));
    ne = f2::fma(co[7], ym, ne);
    ne = f2::fma(co[8], zm, ne);
    v = f2::add(f2::fma(f2::mul(wsplat, co[9]), f2::sub(f2::mul(a3, ne), e0), e0), D);
    ss = f2::mul(f2::sub(v, e0), isplat);
}

// TW: tile width in x points (64 or 72: the launcher takes the one whose whole tiles cover the
// grid's columns with less overhang).
template <int S, int TW>
__global__ void __launch_bounds__(TW / 2 * MY) himeno_mixed2(const __grid_constant__ TileMaps maps, __half* __restrict__ eout,
                                                             int nx, int ny, int nz, int pitch, int py, int kz, float omega,
                                                             float inv_omega, GosaIO gz, unsigned* __restrict__ status)
{
    namespace f2 = gb::f2;
    typedef MixTile<TW> L;
    constexpr int MX = L::X, MW = L::W, MEB = L::EB, MES = L::ES, MCT = L::CT, MSTG = L::STG, MR32 = L::R32;
    extern __shared__ __align__(128) unsigned char tsm[];
    unsigned char* stages = tsm;
    float* ring = reinterpret_cast<float*>(tsm + S * MSTG);
    unsigned char* pro = tsm + S * MSTG + L::RB;  // copy destinations stay 128-byte aligned
    uint64_t* bar = reinterpret_cast<uint64_t*>(pro + 3 * MES);
    const int tx = threadIdx.x, ty = threadIdx.y, t = ty * (MX / 2) + tx;
    // the copies are issued by the last warp's first thread: the e box conversion leaves that
    // warp the fewest pairs, so the issue work does not delay the plane's slowest warp
    const int issuer = MX / 2 * MY - 32;
    const int x0 = blockIdx.x * MX, y0 = 1 + blockIdx.y * MY;
    const int xa = x0 + 2 * tx, j = y0 + ty;
    const int k0 = 1 + blockIdx.z * kz, k1 = min(k0 + kz, nz + 1);
    const bool acta = xa >= 1 && xa <= nx && j <= ny, actb = xa + 1 <= nx && j <= ny;
    if (gb::tma::smem_u32(tsm) & 127u) {
        if (t == 0) atomicOr(status, (unsigned)gb::ST_SMEM_ALIGN);
        gosa_end<1>({__longlong_as_double(0x7ff8000000000000ll)}, gz);
        return;
    }
    if (t == issuer) {
#pragma unroll
        for (int s = 0; s < S; s++) gb::tma::bar_init(&bar[s], 1);
        gb::tma::fence_init();
        for (int n = 0; n < 13; n++) gb::tma::prefetch_map(&maps.m[n]);
    }
    __syncthreads();
    // e planes k-1 .. k+1 in a 3-slot FP32 ring: a step reads plane k+1's set and plane k's
    // diagonals (plane k-1 is in the register queue), so plane k+2 can take plane k-1's slot
    auto slot = [&](int pl) { return ring + ((unsigned)(pl - (k0 - 1)) % 3u) * MR32; };
    auto issue = [&](int k) {
        const int s = (k - k0) % S;
        unsigned char* st = stages + s * MSTG;
        gb::tma::arrive_expect(&bar[s], MCT + MEB * (k == k0 ? 4 : 1));
        if (k == k0)
            for (int d = 0; d < 3; d++) gb::tma::load_3d(pro + d * MES, &maps.m[12], x0 - MXO, y0 - 1, k0 - 1 + d, &bar[s]);
#pragma unroll
        for (int n = 0; n < 10; n++) gb::tma::load_3d(st + n * MX * MY * 2, &maps.m[n], x0, y0, k, &bar[s]);
        gb::tma::load_3d(st + 10 * MX * MY * 2, &maps.m[10], x0, y0, k, &bar[s]);
        gb::tma::load_3d(st + 10 * MX * MY * 2 + MX * MY * 4, &maps.m[11], x0, y0, k, &bar[s]);
        gb::tma::load_3d(st + MCT, &maps.m[12], x0 - MXO, y0 - 1, k + 2, &bar[s]);
    };
    if (t == issuer)
        for (int k = k0; k < min(k0 + S, k1); k++) issue(k);

    float2 g = make_float2(0.0f, 0.0f);
    bool bad = false;
    int k = k0;
    const int cq = ty * MX + 2 * tx;          // this pair in a per-point tile (elements)
    const int q = (ty + 1) * MW + 2 * tx + MXO;  // this pair in a ring slot
    const float2 wsplat = f2::splat(omega), isplat = f2::splat(inv_omega);
    PlaneSet pm, pz;  // planes k-1 and k of this pair (register queue)
    for (; k < k1; k++) {
        const int s = (k - k0) % S;
        if (!gb::tma::wait(&bar[s], (unsigned)((k - k0) / S) & 1u)) bad = true;
        const unsigned char* st = stages + s * MSTG;
        if (k == k0) {  // uniform
            for (int d = 0; d < 3; d++) e_box_to_f32<TW>(pro + d * MES, slot(k0 - 1 + d), t);
            __syncthreads();
            pm = plane_set(slot(k0 - 1), q, MW);
            pz = plane_set(slot(k0), q, MW);
            __syncthreads();  // plane k0-1's slot is read before plane k0+2 takes it
        }
        e_box_to_f32<TW>(st + MCT, slot(k + 2), t);  // plane k+2 into the slot plane k-1 left
        {
            float2 co[10];
#pragma unroll
            for (int n = 0; n < 10; n++) co[n] = __half22float2(reinterpret_cast<const __half2*>(st + n * MX * MY * 2)[cq / 2]);
            const float2 a3 = reinterpret_cast<const float2*>(st + 10 * MX * MY * 2)[cq / 2];
            const float2 D = __half22float2(reinterpret_cast<const __half2*>(st + 10 * MX * MY * 2 + MX * MY * 4)[cq / 2]);
            const PlaneSet pp = plane_set(slot(k + 1), q, MW);
            float2 v, ss;
            mix_pair(pm, pz, plane_diag(slot(k), q, MW), pp, co, a3, D, wsplat, isplat, v, ss);
            pm = pz;
            pz = pp;
            const size_t cc = ((size_t)k * py + j) * pitch + xa;
            const __half2 hv = __float22half2_rn(v);
            if (!bad) {
                if (acta && actb) {
                    *reinterpret_cast<__half2*>(eout + cc) = hv;
                } else {
                    if (acta) eout[cc] = __low2half(hv);
                    if (actb) eout[cc + 1] = __high2half(hv);
                }
            }
            ss.x = acta ? ss.x : 0.0f;
            ss.y = actb ? ss.y : 0.0f;
            g = f2::fma(ss, ss, g);
        }
        // everyone is done with stage s, the slot of plane k-1 and the conversions of plane k+2
        if (__syncthreads_or(bad)) break;
        if (t == issuer && k + S < k1) issue(k + S);
    }
    if (k < k1 && t == 0) {  // a wait gave up: report and let the copies still in flight land
        atomicOr(status, (unsigned)gb::ST_TMA_TIMEOUT);
        for (int kk = k; kk < min(k + S, k1); kk++)
                gb::tma::wait(&bar[(kk - k0) % S], (unsigned)((kk - k0) / S) & 1u, gb::tma::DRAIN_NS);
    }
    gosa_end<1>({k < k1 ? __longlong_as_double(0x7ff8000000000000ll) : (double)g.x + (double)g.y}, gz);
}

// ---------------------------------------------------------------- FP16 inner sweeps, two per pass
// Two defect-correction sweeps per pass over a 56 x 8 output tile, so the ten FP16 coefficient
// tiles, a3 and D of a plane (the 30 bytes a single sweep reads per point, 26 of them these) are
// read once for both.  A stage brings them for plane q as 72 x 10 boxes (x from tile x - 8: the
// tile and a one-point ring, x-aligned for the copy) and the FP16 e box of plane q+1 (72 x 12).
// Sweep 1 computes e1 on the tile and its ring (30 x pairs from tile x - 2, 10 rows) from an FP32
// ring of e planes; e1 is rounded to FP16 and back, as a stored sweep would round it, and is 0
// outside the interior (the e fields' ghost cells are 0), so sweep 2, on the tile from an FP32
// ring of e1 planes, gives the same bits as two single sweeps.  Step i (plane q = k0 - 1 + i)
// runs sweep 1 of plane q, then sweep 2 of plane q - 1 with the previous step's stage: four
// stages keep two planes in flight.  Both sweeps use mix_pair, the single sweep's arithmetic.
constexpr int T2X = 56, T2Y = 8, T2W = 72;                     // output tile, box width
constexpr int T2P1X = (T2X + 4) / 2, T2P1 = T2P1X * (T2Y + 2);  // sweep-1 pairs (30 x 10)
constexpr int T2P2X = T2X / 2, T2P2 = T2P2X * T2Y;              // sweep-2 pairs (28 x 8)
constexpr int T2NT = 320;                                       // threads (>= T2P1)
constexpr int T2CBYTES = T2W * (T2Y + 2) * 2, T2ABYTES = T2W * (T2Y + 2) * 4, T2EBYTES = T2W * (T2Y + 4) * 2;
constexpr int T2CB = (T2CBYTES + 127) / 128 * 128;              // FP16 per-point box slot
constexpr int T2AB = (T2ABYTES + 127) / 128 * 128;              // a3 box slot
constexpr int T2EB = (T2EBYTES + 127) / 128 * 128;              // e box slot
constexpr int T2STG = 11 * T2CB + T2AB + T2EB;                  // 10 coefficients + D, a3, e of plane q+1
constexpr int T2R0 = T2W * (T2Y + 4), T2R1 = T2W * (T2Y + 2);   // floats per e / e1 ring slot
constexpr int T2R0B = (3 * T2R0 * 4 + 127) / 128 * 128;         // the two rings (3 slots each), 128-byte multiples
constexpr int T2R1B = (3 * T2R1 * 4 + 127) / 128 * 128;
constexpr int T2S = 4;
constexpr int t2_smem() { return T2S * T2STG + T2R0B + T2R1B + 2 * T2EB + T2S * 8; }
static_assert(T2STG % 128 == 0 && T2CB % 128 == 0 && T2AB % 128 == 0 && T2EB % 128 == 0, "copy destinations 128-byte aligned");
static_assert(T2P1 <= T2NT && T2P2 <= T2NT, "thread count");

__device__ __forceinline__ void e_box72_to_f32(const unsigned char* src, float* dst, int t)
{
    const __half2* h = reinterpret_cast<const __half2*>(src);
    float2* d = reinterpret_cast<float2*>(dst);
    for (int q = t; q < T2R0 / 2; q += T2NT) d[q] = __half22float2(h[q]);
}

__global__ void __launch_bounds__(T2NT, 2) himeno_mixed_tb2(const __grid_constant__ TileMaps maps, __half* __restrict__ eout, int nx,
                                                            int ny, int nz, int pitch, int py, int kz, float omega, float inv_omega,
                                                            GosaIO gz, unsigned* __restrict__ status)
{
    namespace f2 = gb::f2;
    extern __shared__ __align__(128) unsigned char tsm[];
    unsigned char* stages = tsm;
    float* ring0 = reinterpret_cast<float*>(tsm + T2S * T2STG);
    float* ring1 = reinterpret_cast<float*>(tsm + T2S * T2STG + T2R0B);
    unsigned char* pro = tsm + T2S * T2STG + T2R0B + T2R1B;
    uint64_t* bar = reinterpret_cast<uint64_t*>(pro + 2 * T2EB);
    const int t = threadIdx.x, issuer = T2NT - 32;  // the copies: the last warp (no sweep-2 pairs)
    const int x0 = blockIdx.x * T2X, y0 = 1 + blockIdx.y * T2Y;
    const int k0 = 1 + blockIdx.z * kz, k1 = min(k0 + kz, nz + 1);
    const int qlo = k0 - 1, nst = k1 - k0 + 2;  // sweep 1 runs on planes qlo .. k1
    const double nan = __longlong_as_double(0x7ff8000000000000ll);
    if (gb::tma::smem_u32(tsm) & 127u) {
        if (t == 0) atomicOr(status, (unsigned)gb::ST_SMEM_ALIGN);
        gosa_end<2>({nan, nan}, gz);
        return;
    }
    if (t == issuer) {
#pragma unroll
        for (int s = 0; s < T2S; s++) gb::tma::bar_init(&bar[s], 1);
        gb::tma::fence_init();
        for (int n = 0; n < 13; n++) gb::tma::prefetch_map(&maps.m[n]);
    }
    __syncthreads();
    auto r0slot = [&](int pl) { return ring0 + ((unsigned)(pl - qlo + 1) % 3u) * T2R0; };  // e planes from qlo - 1
    auto r1slot = [&](int pl) { return ring1 + ((unsigned)(pl - qlo) % 3u) * T2R1; };      // e1 planes from qlo
    int last_issued = -1;  // the issuing thread only
    auto issue = [&](int i) {
        const int s = i % T2S, q = qlo + i;
        unsigned char* st = stages + s * T2STG;
        last_issued = i;
        gb::tma::arrive_expect(&bar[s], 11 * T2CBYTES + T2ABYTES + T2EBYTES + (i == 0 ? 2 * T2EBYTES : 0));
        if (i == 0)
            for (int d = 0; d < 2; d++) gb::tma::load_3d(pro + d * T2EB, &maps.m[12], x0 - 8, y0 - 2, qlo - 1 + d, &bar[s]);
#pragma unroll
        for (int n = 0; n < 10; n++) gb::tma::load_3d(st + n * T2CB, &maps.m[n], x0 - 8, y0 - 1, q, &bar[s]);
        gb::tma::load_3d(st + 10 * T2CB, &maps.m[11], x0 - 8, y0 - 1, q, &bar[s]);         // D
        gb::tma::load_3d(st + 11 * T2CB, &maps.m[10], x0 - 8, y0 - 1, q, &bar[s]);         // a3
        gb::tma::load_3d(st + 11 * T2CB + T2AB, &maps.m[12], x0 - 8, y0 - 2, q + 1, &bar[s]);  // e of plane q+1
    };
    if (t == issuer)
        for (int i = 0; i < min(T2S, nst); i++) issue(i);

    // sweep-1 pair of this thread (tile and ring), sweep-2 pair (tile)
    const bool has1 = t < T2P1, has2 = t < T2P2;
    const int p1x = t % T2P1X, p1y = t / T2P1X;
    const int x1 = x0 - 2 + 2 * p1x, y1 = y0 - 1 + p1y;
    const int c1 = p1y * T2W + 6 + 2 * p1x;        // in a per-point box and in an e1 slot
    const int q1 = (p1y + 1) * T2W + 6 + 2 * p1x;  // in an e slot
    const bool in1a = x1 >= 1 && x1 <= nx && y1 >= 1 && y1 <= ny, in1b = x1 + 1 >= 1 && x1 + 1 <= nx && y1 >= 1 && y1 <= ny;
    const bool own1 = x1 >= x0 && x1 <= x0 + T2X - 2 && y1 >= y0 && y1 < y0 + T2Y;
    const int p2x = t % T2P2X, p2y = t / T2P2X;
    const int x2 = x0 + 2 * p2x, y2 = y0 + p2y;
    const int c2i = (p2y + 1) * T2W + 8 + 2 * p2x;  // in a per-point box and in an e1 slot
    const bool act2a = x2 >= 1 && x2 <= nx && y2 <= ny, act2b = x2 + 1 <= nx && y2 <= ny;
    const float2 wsplat = f2::splat(omega), isplat = f2::splat(inv_omega);
    auto load_pair = [&](const unsigned char* st, int c, float2 (&co)[10], float2& a3, float2& D) {
#pragma unroll
        for (int n = 0; n < 10; n++) co[n] = __half22float2(reinterpret_cast<const __half2*>(st + n * T2CB)[c / 2]);
        D = __half22float2(reinterpret_cast<const __half2*>(st + 10 * T2CB)[c / 2]);
        a3 = reinterpret_cast<const float2*>(st + 11 * T2CB)[c / 2];
    };
    float2 g1 = make_float2(0.0f, 0.0f), g2 = make_float2(0.0f, 0.0f);
    PlaneSet m1, z1, m2, z2;  // register queues: e planes q-1, q (sweep 1); e1 planes k-1, k (sweep 2)
    bool bad = false;
    int i = 0;
    for (; i < nst; i++) {
        const int s = i % T2S, q = qlo + i;
        if (!gb::tma::wait(&bar[s], (unsigned)(i / T2S) & 1u)) bad = true;
        const unsigned char* st = stages + s * T2STG;
        if (!bad) {
            if (i == 0)
                for (int d = 0; d < 2; d++) e_box72_to_f32(pro + d * T2EB, r0slot(qlo - 1 + d), t);
            e_box72_to_f32(st + 11 * T2CB + T2AB, r0slot(q + 1), t);
        }
        // e planes q-1 .. q+1 are in; everyone is done with step i-1 (its sweep 2 read stage i-2)
        if (__syncthreads_or(bad)) break;
        if (t == issuer && i >= 2 && i + 2 < nst) issue(i + 2);
        if (has1) {  // sweep 1, plane q
            float2 co[10], a3, D, v, ss;
            load_pair(st, c1, co, a3, D);
            if (i == 0) {
                m1 = plane_set(r0slot(q - 1), q1, T2W);
                z1 = plane_set(r0slot(q), q1, T2W);
            }
            const PlaneSet p1 = plane_set(r0slot(q + 1), q1, T2W);
            mix_pair(m1, z1, plane_diag(r0slot(q), q1, T2W), p1, co, a3, D, wsplat, isplat, v, ss);
            m1 = z1;
            z1 = p1;
            const bool zin = q >= 1 && q <= nz;
            const float2 vr = __half22float2(__float22half2_rn(v));  // as a stored sweep rounds it
            *reinterpret_cast<float2*>(r1slot(q) + c1) = make_float2(zin && in1a ? vr.x : 0.0f, zin && in1b ? vr.y : 0.0f);
            if (own1 && q >= k0 && q < k1) {
                ss.x = in1a ? ss.x : 0.0f;
                ss.y = in1b ? ss.y : 0.0f;
                g1 = f2::fma(ss, ss, g1);
            }
        }
        __syncthreads();  // e1 plane q is in
        if (i >= 2 && has2) {  // sweep 2, plane q - 1 (k0 .. k1-1), with stage i-1
            const int k = q - 1;
            float2 co[10], a3, D, v, ss;
            load_pair(stages + ((i - 1) % T2S) * T2STG, c2i, co, a3, D);
            if (i == 2) {
                m2 = plane_set(r1slot(k - 1), c2i, T2W);
                z2 = plane_set(r1slot(k), c2i, T2W);
            }
            const PlaneSet p2 = plane_set(r1slot(k + 1), c2i, T2W);
            mix_pair(m2, z2, plane_diag(r1slot(k), c2i, T2W), p2, co, a3, D, wsplat, isplat, v, ss);
            m2 = z2;
            z2 = p2;
            const size_t cc = ((size_t)k * py + y2) * pitch + x2;
            const __half2 hv = __float22half2_rn(v);
            if (act2a && act2b) {
                *reinterpret_cast<__half2*>(eout + cc) = hv;
            } else {
                if (act2a) eout[cc] = __low2half(hv);
                if (act2b) eout[cc + 1] = __high2half(hv);
            }
            ss.x = act2a ? ss.x : 0.0f;
            ss.y = act2b ? ss.y : 0.0f;
            g2 = f2::fma(ss, ss, g2);
        }
    }
    if (i < nst && t == issuer) {  // a wait gave up: report and let the copies still in flight land
        atomicOr(status, (unsigned)gb::ST_TMA_TIMEOUT);
        for (int j = i; j <= last_issued; j++) gb::tma::wait(&bar[j % T2S], (unsigned)(j / T2S) & 1u, gb::tma::DRAIN_NS);
    }
    const bool ok = i == nst;
    gosa_end<2>({ok ? (double)g1.x + (double)g1.y : nan, ok ? (double)g2.x + (double)g2.y : nan}, gz);
}

// ---------------------------------------------------------------- TMA-staged correction pass
// P' = P + e, D = omega*ss(P'), e_next = 0, on the same 32 x 8 tile and z-march as himeno_tma.
// A stage brings the twelve FP32 coefficient tiles of plane k and the P (FP32, 40 x 10) and e
// (FP16, 48 x 10) boxes of plane k+2; the threads add them once into an FP32 ring of Q = P + e
// (planes k-1 .. k+2), so the 19-point sum reads shared memory only.
struct CorrMaps {
    CUtensorMap m[14];  // 0..11 coefficients, 12 P, 13 e
};
constexpr int CPB = (TmaLayout::RB + 127) / 128 * 128;  // P box slot (40 x 10 FP32)
constexpr int CEB = 48 * (RY + 2) * 2;                   // e box bytes (48 x 10 FP16)
constexpr int CES = (CEB + 127) / 128 * 128;
constexpr int CSTG = TmaLayout::CT + CPB + CES;          // one stage
constexpr int CQ = TmaLayout::W * (RY + 2);              // floats per Q ring slot
constexpr int CORR_S = 2;
constexpr int corr_smem(int S) { return S * CSTG + 4 * CQ * 4 + 3 * (CPB + CES) + S * 8; }

// Q = P + e over one 40 x 10 box (e's box starts 4 columns further left)
__device__ __forceinline__ void q_box(const unsigned char* pbox, const unsigned char* ebox, float* q, int t)
{
    const float* P = reinterpret_cast<const float*>(pbox);
    const __half* E = reinterpret_cast<const __half*>(ebox);
    for (int idx = t; idx < CQ; idx += RX * RY) {
        const int r = idx / TmaLayout::W, c = idx - r * TmaLayout::W;
        q[idx] = P[idx] + __half2float(E[r * 48 + c + 4]);
    }
}

template <int S>
__global__ void __launch_bounds__(RX* RY) himeno_correct_tma(const __grid_constant__ CorrMaps maps, float* __restrict__ Pn,
                                                              __half* __restrict__ D, __half* __restrict__ enext, int nx, int ny,
                                                              int nz, int pitch, int py, int kz, float omega, float inv_omega,
                                                              int prime, GosaIO gz, unsigned* __restrict__ status)
{
    typedef TmaLayout Lay;
    extern __shared__ __align__(128) unsigned char tsm[];
    unsigned char* stages = tsm;
    float* ring = reinterpret_cast<float*>(tsm + S * CSTG);
    unsigned char* pro = tsm + S * CSTG + 4 * CQ * 4;
    uint64_t* bar = reinterpret_cast<uint64_t*>(pro + 3 * (CPB + CES));
    const int tx = threadIdx.x, ty = threadIdx.y, t = ty * RX + tx;
    const int x0 = blockIdx.x * RX, y0 = 1 + blockIdx.y * RY;
    const int i = x0 + tx, j = y0 + ty;
    const int k0 = 1 + blockIdx.z * kz, k1 = min(k0 + kz, nz + 1);
    const bool act = i >= 1 && i <= nx && j <= ny;
    if (gb::tma::smem_u32(tsm) & 127u) {
        if (t == 0) atomicOr(status, (unsigned)gb::ST_SMEM_ALIGN);
        gosa_end<1>({__longlong_as_double(0x7ff8000000000000ll)}, gz);
        return;
    }
    if (t == 0) {
#pragma unroll
        for (int s = 0; s < S; s++) gb::tma::bar_init(&bar[s], 1);
        gb::tma::fence_init();
        for (int n = 0; n < 14; n++) gb::tma::prefetch_map(&maps.m[n]);
    }
    __syncthreads();
    auto slot = [&](int pl) { return ring + ((pl - (k0 - 1)) & 3) * CQ; };
    auto issue = [&](int k) {
        const int s = (k - k0) % S;
        unsigned char* st = stages + s * CSTG;
        gb::tma::arrive_expect(&bar[s], Lay::CT + (Lay::RB + CEB) * (k == k0 ? 4 : 1));
        if (k == k0)
            for (int d = 0; d < 3; d++) {
                unsigned char* b = pro + d * (CPB + CES);
                gb::tma::load_3d(b, &maps.m[12], x0 - Lay::XO, y0 - 1, k0 - 1 + d, &bar[s]);
                gb::tma::load_3d(b + CPB, &maps.m[13], x0 - 8, y0 - 1, k0 - 1 + d, &bar[s]);
            }
#pragma unroll
        for (int n = 0; n < 12; n++) gb::tma::load_3d(st + Lay::tile_off(n), &maps.m[n], x0, y0, k, &bar[s]);
        gb::tma::load_3d(st + Lay::CT, &maps.m[12], x0 - Lay::XO, y0 - 1, k + 2, &bar[s]);
        gb::tma::load_3d(st + Lay::CT + CPB, &maps.m[13], x0 - 8, y0 - 1, k + 2, &bar[s]);
    };
    if (t == 0)
        for (int k = k0; k < min(k0 + S, k1); k++) issue(k);

    bool bad = false;
    int k = k0;
    float g = 0.0f;
    const int cq = ty * RX + tx;
    const int q = (ty + 1) * Lay::W + tx + Lay::XO;
    for (; k < k1; k++) {
        const int s = (k - k0) % S;
        if (!gb::tma::wait(&bar[s], (unsigned)((k - k0) / S) & 1u)) bad = true;
        const unsigned char* st = stages + s * CSTG;
        if (k == k0) {  // uniform
            for (int d = 0; d < 3; d++) q_box(pro + d * (CPB + CES), pro + d * (CPB + CES) + CPB, slot(k0 - 1 + d), t);
            __syncthreads();
        }
        q_box(st + Lay::CT, st + Lay::CT + CPB, slot(k + 2), t);  // plane k+2 into the slot plane k-2 left
        if (act && !bad) {
            const float* sm = slot(k - 1);
            const float* s0 = slot(k);
            const float* sp = slot(k + 1);
            float co[12];
#pragma unroll
            for (int n = 0; n < 12; n++) co[n] = reinterpret_cast<const float*>(st + Lay::tile_off(n))[cq];
#define RF(di, dj, dk) (((dk) < 0 ? sm : ((dk) > 0 ? sp : s0))[q + (di) + (dj) * Lay::W])
            const float s0v = HIMENO_S0(RF, co[0], co[1], co[2], co[4], co[5], co[6], co[7], co[8], co[9], co[11]);
            const float q0 = RF(0, 0, 0);
#undef RF
            const float ss = (s0v * co[3] - q0) * co[10];
            const size_t cc = ((size_t)k * py + j) * pitch + i;
            const __half dh = __float2half_rn(omega * ss);
            Pn[cc] = q0;
            D[cc] = dh;
            enext[cc] = prime ? dh : __float2half_rn(0.0f);
            if (prime) {  // the next sweep from e = 0 gives e = D exactly, with ss = D / omega
                const float s1 = __half2float(dh) * inv_omega;
                g = __fmaf_rn(s1, s1, g);
            }
        }
        // everyone is done with stage s, the slot of plane k-1 and the sums of plane k+2
        if (__syncthreads_or(bad)) break;
        if (t == 0 && k + S < k1) issue(k + S);
    }
    if (k < k1 && t == 0) {  // a wait gave up: report and let the copies still in flight land
        atomicOr(status, (unsigned)gb::ST_TMA_TIMEOUT);
        for (int kk = k; kk < min(k + S, k1); kk++)
            gb::tma::wait(&bar[(kk - k0) % S], (unsigned)((kk - k0) / S) & 1u, gb::tma::DRAIN_NS);
    }
    gosa_end<1>({k < k1 ? __longlong_as_double(0x7ff8000000000000ll) : (double)g}, gz);
}

// HKZ: z planes per CTA (nz is split into equal chunks of at most HKZ planes)
constexpr int HBX = 32, HBY = 4, HKZ = 32;
constexpr int TMA_S_PLAIN = 3;

// Tensor maps of the plain form: the 12 FP32 coefficient fields and the iterated p buffer.
int plain_maps(const float* const* coef, const float* pin, int nx, int ny, int nz, int pitch, TileMaps* m)
{
    const int py = ny + 2;
    for (int n = 0; n < 12; n++)
        GB_TRY(gb::tensor_map_3d(&m->m[n], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, coef[n], nx + 2, py, nz + 2, pitch, py, RX, RY));
    return gb::tensor_map_3d(&m->m[12], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, pin, nx + 2, py, nz + 2, pitch, py,
                             TmaLayout::W, RY + 2);
}

bool plain_tma_ok(const float* const* coef, const float* p, const float* wrk2, int pitch)
{
    if (pitch % 4 != 0 || !gb::aligned16(p) || !gb::aligned16(wrk2)) return false;
    for (int n = 0; n < 12; n++)
        if (!gb::aligned16(coef[n])) return false;
    return true;
}

int check_dims(int nx, int ny, int nz, int pitch)
{
    if (nx < 1 || ny < 1 || nz < 1 || pitch < nx + 2) return gb::fail(APPFIS_GB_EINVAL, "himeno: bad dims %d %d %d pitch %d", nx, ny, nz, pitch);
    if ((size_t)pitch * (ny + 2) * (nz + 2) > ((size_t)1 << 36)) return gb::fail(APPFIS_GB_EINVAL, "himeno: grid too large");
    return APPFIS_GB_OK;
}

// The gosa block sums of a sequence of sweep launches (two buffers, used in turn) and the fold
// still owed for the last launch.
struct GosaSeq {
    double* buf[2] = {nullptr, nullptr};
    int cur = 0;
    GosaIO pend = {};
    // the scratch for launches of at most `blocks` blocks of `vals` sums each (no-op without gosa)
    int init(bool on, size_t blocks, int vals)
    {
        if (!on) return APPFIS_GB_OK;
        void* ws;
        const size_t n = blocks * (size_t)vals;
        GB_TRY(gb::workspace(gb::WS_REDUCE, 2 * sizeof(double) * n, &ws));
        buf[0] = reinterpret_cast<double*>(ws);
        buf[1] = buf[0] + n;
        return APPFIS_GB_OK;
    }
    // the GosaIO of the next launch (grid grd, `vals` sums per block, gosa values at out; out
    // null: no gosa), which folds the previous launch's sums
    GosaIO next(dim3 grd, int vals, double* out)
    {
        GosaIO g = {nullptr, pend.prev, pend.prev_out, pend.prev_n, pend.prev_vals};
        pend = {};
        if (out && buf[0]) {
            g.part = buf[cur];
            pend.prev = buf[cur];
            pend.prev_out = out;
            pend.prev_n = grd.x * grd.y * grd.z;
            pend.prev_vals = vals;
            cur ^= 1;
        }
        return g;
    }
    // folds what is owed (before a launch that takes no GosaIO, and at the end)
    int flush(cudaStream_t st)
    {
        if (!pend.prev) return APPFIS_GB_OK;
        himeno_gosa_fold<<<1, 256, 0, st>>>(pend);
        pend = {};
        return gb::launched("himeno_gosa_fold");
    }
};

}  // namespace

extern "C" {

int appfis_gb_himeno(const float* const* coef, float* p, float* wrk2, int nx, int ny, int nz, int pitch, int iters,
                     float omega, double* dev_gosa, int* cur_index, void* stream)
{
    if (!coef || !p || !wrk2 || p == wrk2) return gb::fail(APPFIS_GB_EINVAL, "himeno: null or aliased buffers");
    for (int n = 0; n < 12; n++)
        if (!coef[n]) return gb::fail(APPFIS_GB_EINVAL, "himeno: coefficient %d is null", n);
    GB_TRY(check_dims(nx, ny, nz, pitch));
    if (iters < 0) return gb::fail(APPFIS_GB_EINVAL, "himeno: negative iteration count");
    cudaStream_t st = gb::as_stream(stream);
    Coef12 cf;
    for (int n = 0; n < 12; n++) cf.c[n] = coef[n];
    dim3 blk(RX, RY), grd(gb::ceil_div(nx, RX), gb::ceil_div(ny, RY), gb::ceil_div(nz, HKZ));
    GosaSeq gs;
    float* buf[2] = {p, wrk2};
    int ci = 0;
    if (plain_tma_ok(coef, p, wrk2, pitch)) {
        // TMA-staged form: tile x origins on 32-point boundaries of the padded row
        TileMaps maps[2];
        GB_TRY(plain_maps(coef, p, nx, ny, nz, pitch, &maps[0]));
        maps[1] = maps[0];
        GB_TRY(gb::tensor_map_3d(&maps[1].m[12], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, wrk2, nx + 2, ny + 2, nz + 2, pitch,
                                 ny + 2, TmaLayout::W, RY + 2));
        unsigned* status;
        GB_TRY(gb::status_word(&status));
        constexpr int smem = TmaLayout::smem(TMA_S_PLAIN);
        GB_CUDA(cudaFuncSetAttribute(himeno_tma<TMA_S_PLAIN>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        // z chunks of 16-48 planes whose grid fills the resident CTAs in whole waves (each chunk
        // re-reads 2 halo planes of p)
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, himeno_tma<TMA_S_PLAIN>, RX * RY, smem) != cudaSuccess ||
            per_sm < 1)
            per_sm = 1;
        const long long cols = (long long)(nx / RX + 1) * gb::ceil_div(ny, RY);
        const int kz = gb::wave_chunk(nz, 16, 48, cols, (long long)per_sm * gb::sm_count(), 2);
        dim3 tgrd(nx / RX + 1, gb::ceil_div(ny, RY), gb::ceil_div(nz, kz));
        GB_TRY(gs.init(dev_gosa, (size_t)tgrd.x * tgrd.y * tgrd.z, 1));
        for (int it = 0; it < iters; it++) {
            himeno_tma<TMA_S_PLAIN><<<tgrd, blk, smem, st>>>(maps[ci], buf[1 - ci], nx, ny, nz, pitch, ny + 2, kz, omega,
                                                            gs.next(tgrd, 1, dev_gosa ? dev_gosa + it : nullptr), status);
            ci = 1 - ci;
        }
        GB_TRY(gb::launched("himeno_tma<plain>"));
        GB_TRY(gs.flush(st));
        if (cur_index) *cur_index = ci;
        return APPFIS_GB_OK;
    }
    GB_TRY(gs.init(dev_gosa, (size_t)grd.x * grd.y * grd.z, 1));
    H10 none = {};
    for (int it = 0; it < iters; it++) {
        himeno_ring<0><<<grd, blk, 0, st>>>(cf, none, buf[ci], buf[1 - ci], nullptr, nx, ny, nz, pitch, ny + 2, HKZ, omega, 0.0f,
                                            gs.next(grd, 1, dev_gosa ? dev_gosa + it : nullptr));
        ci = 1 - ci;
    }
    GB_TRY(gb::launched("himeno_ring<plain>"));
    GB_TRY(gs.flush(st));
    if (cur_index) *cur_index = ci;
    return APPFIS_GB_OK;
}

int appfis_gb_himeno_mixed(const float* const* coef, float* p, float* p_work, void* half_work, int nx, int ny, int nz,
                           int pitch, int iters, int period, float omega, double* dev_gosa, int* cur_index, void* stream)
{
    return appfis_gb_himeno_mixed_ex(coef, p, p_work, half_work, nx, ny, nz, pitch, iters, period, omega, 0, dev_gosa, cur_index,
                                     stream);
}

int appfis_gb_himeno_mixed_ex(const float* const* coef, float* p, float* p_work, void* half_work, int nx, int ny, int nz,
                              int pitch, int iters, int period, float omega, int sweeps_per_pass, double* dev_gosa, int* cur_index,
                              void* stream)
{
    if (!coef || !p || !p_work || !half_work || p == p_work) return gb::fail(APPFIS_GB_EINVAL, "himeno_mixed: null or aliased buffers");
    if (sweeps_per_pass < 0 || sweeps_per_pass > 2)
        return gb::fail(APPFIS_GB_EINVAL, "himeno_mixed: sweeps_per_pass %d (0, 1 or 2)", sweeps_per_pass);
    for (int n = 0; n < 12; n++)
        if (!coef[n]) return gb::fail(APPFIS_GB_EINVAL, "himeno_mixed: coefficient %d is null", n);
    GB_TRY(check_dims(nx, ny, nz, pitch));
    if (iters < 0 || period < 1) return gb::fail(APPFIS_GB_EINVAL, "himeno_mixed: bad iters %d / period %d", iters, period);
    if (omega == 0.0f) return gb::fail(APPFIS_GB_EINVAL, "himeno_mixed: omega must be non-zero");
    cudaStream_t st = gb::as_stream(stream);
    const size_t field = (size_t)pitch * (ny + 2) * (nz + 2);
    __half* hw = reinterpret_cast<__half*>(half_work);
    __half* Hc = hw;                  // 10 FP16 coefficient fields
    __half* E[2] = {hw + 10 * field, hw + 11 * field};
    __half* Dd = hw + 12 * field;
    Coef12 cf;
    for (int n = 0; n < 12; n++) cf.c[n] = coef[n];
    H10 hf;
    for (int n = 0; n < 10; n++) hf.c[n] = Hc + n * field;
    hf.a3 = coef[3];
    GB_CUDA(cudaMemsetAsync(hw, 0, sizeof(__half) * 13 * field, st));
    GB_CUDA(cudaMemsetAsync(p_work, 0, sizeof(float) * field, st));
    himeno_half_coef<<<dim3(gb::ceil_div(nx, 128), ny, nz), 128, 0, st>>>(cf, Hc, field, nx, ny, nz, pitch, ny + 2);
    dim3 blk(HBX, HBY), grd(gb::ceil_div(nx, HBX), gb::ceil_div(ny, HBY), gb::ceil_div(nz, HKZ));
    dim3 rblk(RX, RY), rgrd(gb::ceil_div(nx, RX), gb::ceil_div(ny, RY), gb::ceil_div(nz, HKZ));
    // TMA-staged inner sweeps (two points per thread) when the FP16 rows are 16-byte aligned
    // (pitch a multiple of 8)
    const bool use_tma = pitch % 8 == 0 && gb::aligned16(hw) && gb::aligned16(coef[3]);
    // A tile costs the same per plane however few of its columns lie inside the grid, so the
    // inner sweep takes the tile width whose whole tiles overhang columns 0 .. nx+1 less: 257
    // interior columns take four 72-wide tiles (288 columns) rather than five 64-wide ones (320).
    const int tiles64 = gb::ceil_div(nx + 1, 64), tiles72 = gb::ceil_div(nx + 1, 72);
    const int tw = tiles72 * 72 < tiles64 * 64 ? 72 : 64;
    const int tiles_x = tw == 72 ? tiles72 : tiles64;
    const int tsmem = tw == 72 ? MixTile<72>::smem(MIX_S) : MixTile<64>::smem(MIX_S);
    const int tbox_e = tw == 72 ? MixTile<72>::W : MixTile<64>::W;
    auto tkern = tw == 72 ? himeno_mixed2<MIX_S, 72> : himeno_mixed2<MIX_S, 64>;
    int tkz = gb::balanced_chunk(nz, HKZ);
    if (use_tma) {  // z chunks that fill the resident CTAs in whole waves (only e re-reads a halo)
        GB_CUDA(cudaFuncSetAttribute(tkern, cudaFuncAttributeMaxDynamicSharedMemorySize, tsmem));
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tkern, tw / 2 * MY, tsmem) != cudaSuccess || per_sm < 1)
            per_sm = 1;
        tkz = gb::wave_chunk(nz, 32, 64, (long long)tiles_x * gb::ceil_div(ny, MY), (long long)per_sm * gb::sm_count(), 0);
    }
    dim3 tblk(tw / 2, MY), tgrd(tiles_x, gb::ceil_div(ny, MY), gb::ceil_div(nz, tkz));
    TileMaps tmaps[2];
    unsigned* status = nullptr;
    if (use_tma) {
        const int py = ny + 2;
        for (int n = 0; n < 10; n++)
            GB_TRY(gb::tensor_map_3d(&tmaps[0].m[n], CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, hf.c[n], nx + 2, py, nz + 2, pitch, py, tw, MY));
        GB_TRY(gb::tensor_map_3d(&tmaps[0].m[10], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, coef[3], nx + 2, py, nz + 2, pitch, py, tw, MY));
        GB_TRY(gb::tensor_map_3d(&tmaps[0].m[11], CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, Dd, nx + 2, py, nz + 2, pitch, py, tw, MY));
        tmaps[1] = tmaps[0];
        for (int b = 0; b < 2; b++)
            GB_TRY(gb::tensor_map_3d(&tmaps[b].m[12], CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, E[b], nx + 2, py, nz + 2, pitch, py, tbox_e,
                                     MY + 2));
        GB_TRY(gb::status_word(&status));
    }
    // two sweeps per pass on request (measured slower than one per launch on every shape tried:
    // the ring recompute and the second barrier per plane cost more than the bytes saved)
    if (sweeps_per_pass == 2 && !use_tma)
        return gb::fail(APPFIS_GB_EINVAL, "himeno_mixed: two sweeps per pass need 16-byte aligned rows (pitch %% 8 == 0)");
    const bool two = use_tma && sweeps_per_pass == 2;
    TileMaps t2maps[2];
    dim3 t2grd(1, 1, 1);
    int t2kz = 1;
    if (two) {
        const int py = ny + 2;
        for (int n = 0; n < 10; n++)
            GB_TRY(gb::tensor_map_3d(&t2maps[0].m[n], CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, hf.c[n], nx + 2, py, nz + 2, pitch, py, T2W,
                                     T2Y + 2));
        GB_TRY(gb::tensor_map_3d(&t2maps[0].m[10], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, coef[3], nx + 2, py, nz + 2, pitch, py, T2W,
                                 T2Y + 2));
        GB_TRY(gb::tensor_map_3d(&t2maps[0].m[11], CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, Dd, nx + 2, py, nz + 2, pitch, py, T2W, T2Y + 2));
        t2maps[1] = t2maps[0];
        for (int b = 0; b < 2; b++)
            GB_TRY(gb::tensor_map_3d(&t2maps[b].m[12], CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, E[b], nx + 2, py, nz + 2, pitch, py, T2W,
                                     T2Y + 4));
        constexpr int smem2 = t2_smem();
        GB_CUDA(cudaFuncSetAttribute(himeno_mixed_tb2, cudaFuncAttributeMaxDynamicSharedMemorySize, smem2));
        GB_CUDA(cudaFuncSetAttribute(himeno_mixed_tb2, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, himeno_mixed_tb2, T2NT, smem2) != cudaSuccess || per_sm < 1)
            per_sm = 1;
        const int t2x = gb::ceil_div(nx + 1, T2X), t2y = gb::ceil_div(ny, T2Y);
        t2kz = gb::wave_chunk(nz, 32, 64, (long long)t2x * t2y, (long long)per_sm * gb::sm_count(), 2);
        t2grd = dim3(t2x, t2y, gb::ceil_div(nz, t2kz));
    }
    float* P[2] = {p, p_work};
    // correction maps: [P buffer][e buffer]
    CorrMaps cmaps[2][2];
    constexpr int csmem = corr_smem(CORR_S);
    int ckz = tkz;  // the correction pass's own z chunk: whole waves of its resident CTAs
    if (use_tma) {
        GB_CUDA(cudaFuncSetAttribute(himeno_correct_tma<CORR_S>, cudaFuncAttributeMaxDynamicSharedMemorySize, csmem));
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, himeno_correct_tma<CORR_S>, RX * RY, csmem) != cudaSuccess ||
            per_sm < 1)
            per_sm = 1;
        ckz = gb::wave_chunk(nz, 16, 64, (long long)(nx / RX + 1) * gb::ceil_div(ny, RY), (long long)per_sm * gb::sm_count(), 2);
    }
    dim3 cgrd(nx / RX + 1, gb::ceil_div(ny, RY), gb::ceil_div(nz, ckz));
    GosaSeq gs;  // block sums of the sweeps and of the correction passes (which do a sweep each)
    {
        const unsigned nb1 = use_tma ? tgrd.x * tgrd.y * tgrd.z : rgrd.x * rgrd.y * rgrd.z;
        const unsigned nb2 = two ? 2 * t2grd.x * t2grd.y * t2grd.z : 0;
        const unsigned nb3 = use_tma ? cgrd.x * cgrd.y * cgrd.z : grd.x * grd.y * grd.z;
        GB_TRY(gs.init(dev_gosa, std::max(std::max(nb1, nb2), nb3), 1));
    }
    if (use_tma) {
        const int py = ny + 2;
        for (int n = 0; n < 12; n++)
            GB_TRY(gb::tensor_map_3d(&cmaps[0][0].m[n], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, coef[n], nx + 2, py, nz + 2, pitch, py, RX, RY));
        for (int a = 0; a < 2; a++)
            for (int b = 0; b < 2; b++) {
                if (a || b) cmaps[a][b] = cmaps[0][0];
                GB_TRY(gb::tensor_map_3d(&cmaps[a][b].m[12], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, P[a], nx + 2, py, nz + 2, pitch, py,
                                         TmaLayout::W, RY + 2));
                GB_TRY(gb::tensor_map_3d(&cmaps[a][b].m[13], CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, E[b], nx + 2, py, nz + 2, pitch, py, 48,
                                         RY + 2));
            }
    }
    int pc = 0, ec = 0;
    const float inv_omega = 1.0f / omega;
    // The correction pass: P' = P + e into the other P buffer and D; with `prime` it also does
    // the next period's first inner sweep, which from e = 0 yields e = D exactly (all neighbour
    // terms vanish), so it writes e = D and that sweep's gosa; otherwise e = 0.
    auto correct = [&](bool prime, double* g) {
        const GosaIO gz = gs.next(use_tma ? cgrd : grd, 1, prime ? g : nullptr);
        if (use_tma)
            himeno_correct_tma<CORR_S><<<cgrd, rblk, csmem, st>>>(cmaps[pc][ec], P[1 - pc], Dd, E[1 - ec], nx, ny, nz, pitch, ny + 2,
                                                                 ckz, omega, inv_omega, prime ? 1 : 0, gz, status);
        else
            himeno_correct<HBX, HBY><<<grd, blk, 0, st>>>(cf, P[pc], E[ec], P[1 - pc], Dd, E[1 - ec], nx, ny, nz, pitch, ny + 2,
                                                          HKZ, omega, inv_omega, prime ? 1 : 0, gz);
        pc = 1 - pc;
        ec = 1 - ec;
    };
    // periods of `period` sweeps, each opened by a correction pass that does its first sweep;
    // the last correction closes the run
    for (int it = 0;;) {
        const bool prime = it < iters;
        correct(prime, dev_gosa ? dev_gosa + it : nullptr);
        if (!prime) break;
        const int end = std::min(iters, it + period);
        it += 1;
        while (it < end) {
            if (two && end - it >= 2) {
                himeno_mixed_tb2<<<t2grd, T2NT, t2_smem(), st>>>(t2maps[ec], E[1 - ec], nx, ny, nz, pitch, ny + 2, t2kz, omega, inv_omega,
                                                               gs.next(t2grd, 2, dev_gosa ? dev_gosa + it : nullptr), status);
                it += 2;
            } else {
                if (use_tma)
                    tkern<<<tgrd, tblk, tsmem, st>>>(tmaps[ec], E[1 - ec], nx, ny, nz, pitch, ny + 2, tkz, omega, inv_omega,
                                                     gs.next(tgrd, 1, dev_gosa ? dev_gosa + it : nullptr), status);
                else
                    himeno_ring<1><<<rgrd, rblk, 0, st>>>(cf, hf, E[ec], E[1 - ec], Dd, nx, ny, nz, pitch, ny + 2, HKZ, omega,
                                                          inv_omega, gs.next(rgrd, 1, dev_gosa ? dev_gosa + it : nullptr));
                it += 1;
            }
            ec = 1 - ec;
        }
    }
    GB_TRY(gs.flush(st));
    GB_TRY(gb::launched("himeno_mixed"));
    if (cur_index) *cur_index = pc;
    return APPFIS_GB_OK;
}

int appfis_gb_himeno_job(const float* coef_host, float* p_host, int nx, int ny, int nz, int iters, float omega, int form,
                         int period, double* gosa_host)
{
    if (!coef_host || !p_host) return gb::fail(APPFIS_GB_EINVAL, "himeno_job: null input");
    if (form != 0 && form != 1) return gb::fail(APPFIS_GB_EINVAL, "himeno_job: form %d", form);
    GB_TRY(check_dims(nx, ny, nz, nx + 2));
    cudaStream_t st;
    GB_TRY(gb::job_stream(&st));
    // device rows padded to a multiple of 8 elements (16-byte FP32 and FP16 rows: the TMA-staged
    // kernels); host rows are dense
    const int dense = nx + 2, pitch = (dense + 7) / 8 * 8;
    const size_t rows = (size_t)(ny + 2) * (nz + 2), field = (size_t)pitch * rows;
    const size_t hrow = sizeof(float) * dense, drow = sizeof(float) * pitch;
    void *dc, *da, *db, *dh, *dg;
    GB_TRY(gb::workspace(gb::WS_JOB_A, sizeof(float) * 12 * field, &dc));
    GB_TRY(gb::workspace(gb::WS_JOB_B, sizeof(float) * field, &da));
    GB_TRY(gb::workspace(gb::WS_JOB_C, sizeof(float) * field, &db));
    GB_TRY(gb::workspace(gb::WS_JOB_E, sizeof(double) * (iters > 0 ? iters : 1), &dg));
    GB_CUDA(cudaMemcpy2DAsync(dc, drow, coef_host, hrow, hrow, 12 * rows, cudaMemcpyHostToDevice, st));
    GB_CUDA(cudaMemcpy2DAsync(da, drow, p_host, hrow, hrow, rows, cudaMemcpyHostToDevice, st));
    GB_CUDA(cudaMemcpyAsync(db, da, sizeof(float) * field, cudaMemcpyDeviceToDevice, st));  // ghost ring in both
    const float* cp[12];
    for (int n = 0; n < 12; n++) cp[n] = reinterpret_cast<const float*>(dc) + n * field;
    int ci = 0;
    if (form == 0) {
        GB_TRY(appfis_gb_himeno(cp, (float*)da, (float*)db, nx, ny, nz, pitch, iters, omega, gosa_host ? (double*)dg : nullptr,
                                &ci, st));
    } else {
        GB_TRY(gb::workspace(gb::WS_JOB_D, sizeof(__half) * 13 * field, &dh));
        GB_TRY(appfis_gb_himeno_mixed(cp, (float*)da, (float*)db, dh, nx, ny, nz, pitch, iters, period, omega,
                                      gosa_host ? (double*)dg : nullptr, &ci, st));
    }
    GB_CUDA(cudaMemcpy2DAsync(p_host, hrow, ci == 0 ? da : db, drow, hrow, rows, cudaMemcpyDeviceToHost, st));
    if (gosa_host && iters > 0) GB_CUDA(cudaMemcpyAsync(gosa_host, dg, sizeof(double) * iters, cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    return gb::check_status("himeno_job");
}

}  // extern "C"
