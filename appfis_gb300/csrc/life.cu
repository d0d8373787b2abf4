// GameOfLife on a periodic grid: byte-per-cell (SWAR, 16 cells per thread per row) and
// bit-packed (32 cells per word) sweeps, pack/unpack, population count, whole-run job.
//
// Reference semantics (GameOfLife/src/game_appfis.hpp:121-135): a live cell whose 8-neighbour
// count is < 2 or > 4 is cleared in `next`; a dead cell with count 3 is set in `next`; any
// other cell leaves `next` untouched, so `next` keeps the state of two generations back (the
// DUAL grid's buffers swap every generation, Appfis/Runtime.hpp:318-319).  In bit-slice form:
//     new = (cur & keep & old) | (~cur & (birth | old)),  keep = (cnt in 2..4), birth = (cnt == 3).
// The periodic halo refresh of the reference (pack, MPI self-exchange, unpack every
// generation, Appfis/Communication.hpp:612-678) becomes index wrap-around inside the sweep.
//
// Layout: interior cells only, x fastest, row pitch nx bytes (u8) or nx/32 words (bits).
// The byte-per-cell sweep (life_u8_bulk) stages its rows in shared memory with bulk copies; the
// one-generation bit-packed sweep (life_bits_sweep) marches down a strip of rows per warp,
// keeping the row above / at / below in registers and exchanging the words at lane boundaries
// with warp shuffles.  Runs of 16 or more bit-packed generations use life_bits_tb, which
// advances a tile held in shared memory by 16 generations per launch.
#include "gb_common.cuh"
#include "tma.cuh"

namespace {

constexpr uint32_t FULL = 0xffffffffu;
constexpr uint32_t LSB = 0x01010101u;  // bit 0 of each byte
constexpr int LIFE_ROWS = 32;           // rows per warp task (bit-packed sweep)

// ------------------------------------------------------------------------------ rule logic
// Per byte lane (u8 form): cnt in 0..8 in each byte, c/o in {0,1} per byte.
template <int RULE>
__device__ __forceinline__ uint32_t rule_bytes(uint32_t cnt, uint32_t c, uint32_t o)
{
    uint32_t b0 = cnt & LSB, b1 = (cnt >> 1) & LSB, b2 = (cnt >> 2) & LSB, b3 = (cnt >> 3) & LSB;
    if (RULE == APPFIS_GB_LIFE_REFERENCE) {
        uint32_t birth = b0 & b1 & ~(b2 | b3);
        uint32_t keep = ~b3 & ((~b2 & b1) | (b2 & ~b1 & ~b0));
        return ((c & keep & o) | (~c & (birth | o))) & LSB;
    } else {
        return (b1 & ~(b2 | b3) & (b0 | c)) & LSB;
    }
}


// ------------------------------------------------------------------------------ generic form
// One thread per cell, any nx, ny (used when nx is not a multiple of 16).
template <int RULE>
__global__ void life_u8_generic(const uint8_t* __restrict__ cur, uint8_t* __restrict__ out, int nx, int ny)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= nx || j >= ny) return;
    int im = i == 0 ? nx - 1 : i - 1, ip = i == nx - 1 ? 0 : i + 1;
    size_t rm = (size_t)(j == 0 ? ny - 1 : j - 1) * nx, r0 = (size_t)j * nx, rp = (size_t)(j == ny - 1 ? 0 : j + 1) * nx;
    uint32_t cnt = cur[rm + im] + cur[rm + i] + cur[rm + ip] + cur[r0 + im] + cur[r0 + ip] + cur[rp + im] + cur[rp + i] +
                   cur[rp + ip];
    uint32_t c = cur[r0 + i];
    uint32_t o = out[r0 + i];
    out[r0 + i] = (uint8_t)rule_bytes<RULE>(cnt, c, RULE == APPFIS_GB_LIFE_REFERENCE ? o : 0u);
}

// ------------------------------------------------------------------------------ u8 form, bulk-staged
struct RowU8 {         // 16 cells of one row, one per byte (SWAR)
    uint32_t w[4];     // the cells
    uint32_t s3[4];    // per byte: left + self + right
};

// A CTA owns a strip of UB_W cells (256 threads x 16) of UB_ROWS consecutive rows.  Each row it
// needs arrives in a shared-memory slot by bulk copies (the cur row with a 16-byte periodic halo
// on each side, and for output rows the t-1 row), UB_RING - 1 rows ahead of the row it computes,
// signalled on the slot's mbarrier: every copy is a contiguous run of up to 4 KB, and the rows in
// flight need no registers.  Each thread carries the row summaries of the rows above and at its
// output row and reads the row below from the slot (one 16-byte vector and the two neighbour
// words), so every row is summarised once.  Waits are bounded; a wait that gives up sets the
// device status word.
constexpr int UB_W = 4096;      // strip width in cells (bytes)
constexpr int UB_ROWS = 32;     // output rows per CTA
constexpr int UB_RING = 6;      // row slots
constexpr int UB_OLD = 16 + UB_W + 16;      // offset of the t-1 row in a slot
constexpr int UB_SLOT = UB_OLD + UB_W;      // 8224 bytes
constexpr int UB_SMEM = UB_RING * UB_SLOT + UB_RING * 8;

__device__ __forceinline__ RowU8 slot_row_u8(const unsigned char* s, int t)
{
    const unsigned char* p = s + 16 + 16 * t;
    const uint4 v = *reinterpret_cast<const uint4*>(p);
    const uint32_t lw = *reinterpret_cast<const uint32_t*>(p - 4);   // cell x-1 in the top byte
    const uint32_t rw = *reinterpret_cast<const uint32_t*>(p + 16);  // cell x+16 in the low byte
    RowU8 r;
    r.w[0] = v.x;
    r.w[1] = v.y;
    r.w[2] = v.z;
    r.w[3] = v.w;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const uint32_t prev = k == 0 ? lw : r.w[k - 1];
        const uint32_t next = k == 3 ? rw : r.w[k + 1];
        r.s3[k] = __funnelshift_l(prev, r.w[k], 8) + r.w[k] + __funnelshift_r(r.w[k], next, 8);
    }
    return r;
}

template <int RULE>
__global__ void __launch_bounds__(256) life_u8_bulk(const uint8_t* __restrict__ cur, uint8_t* __restrict__ out, int nx, int ny,
                                                     int strips, unsigned* __restrict__ status)
{
    extern __shared__ __align__(128) unsigned char ub[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(ub + UB_RING * UB_SLOT);
    const int t = threadIdx.x;
    const int strip = blockIdx.x % strips, band = blockIdx.x / strips;
    const int x0 = strip * UB_W, w = min(UB_W, nx - x0);
    const int j0 = band * UB_ROWS, j1 = min(j0 + UB_ROWS, ny);
    const int rbase = j0 - 1;  // row of slot 0, first use
    const bool active = 16 * t < w;
    if (gb::tma::smem_u32(ub) & 15u) {
        if (t == 0) atomicOr(status, (unsigned)gb::ST_SMEM_ALIGN);
        return;
    }
    if (t == 0) {
        for (int n = 0; n < UB_RING; n++) gb::tma::bar_init(&bar[n], 1);
        gb::tma::fence_init();
    }
    __syncthreads();
    int last_issued = rbase - 1;  // thread 0 only
    auto issue = [&](int r) {     // cur row r (periodic) with its halos; the t-1 row if r is an output row
        last_issued = r;
        const int n = (r - rbase) % UB_RING;
        unsigned char* d = ub + n * UB_SLOT;
        const int rr = r < 0 ? r + ny : (r >= ny ? r - ny : r);
        const uint8_t* row = cur + (size_t)rr * nx;
        const bool oldrow = RULE == APPFIS_GB_LIFE_REFERENCE && r >= j0 && r < j1;
        gb::tma::arrive_expect(&bar[n], 32 + w + (oldrow ? w : 0));
        gb::tma::load_1d(d, row + (x0 == 0 ? nx - 16 : x0 - 16), 16, &bar[n]);
        gb::tma::load_1d(d + 16, row + x0, w, &bar[n]);
        gb::tma::load_1d(d + 16 + w, row + (x0 + w == nx ? 0 : x0 + w), 16, &bar[n]);
        if (oldrow) gb::tma::load_1d(d + UB_OLD, out + (size_t)r * nx + x0, w, &bar[n]);
    };
    auto ready = [&](int r, uint64_t limit = 1000000000ull) {
        return gb::tma::wait(&bar[(r - rbase) % UB_RING], (unsigned)((r - rbase) / UB_RING) & 1u, limit);
    };
    auto slot = [&](int r) { return ub + ((r - rbase) % UB_RING) * UB_SLOT; };
    if (t == 0)
        for (int r = rbase; r < rbase + UB_RING && r <= j1; r++) issue(r);
    bool bad = !ready(rbase) || !ready(j0);
    RowU8 up = slot_row_u8(slot(rbase), t);
    RowU8 mid = slot_row_u8(slot(j0), t);
    bad = __syncthreads_or(bad);  // row j0-1 is read: its slot takes row j0-1+UB_RING
    if (t == 0 && !bad && rbase + UB_RING <= j1) issue(rbase + UB_RING);
    for (int j = j0; j < j1 && !bad; j++) {
        if (!ready(j + 1)) bad = true;
        const RowU8 dn = slot_row_u8(slot(j + 1), t);
        const uint4 o = RULE == APPFIS_GB_LIFE_REFERENCE ? *reinterpret_cast<const uint4*>(slot(j) + UB_OLD + 16 * t)
                                                         : make_uint4(0, 0, 0, 0);
        if (active && !bad) {
            const uint32_t ow[4] = {o.x, o.y, o.z, o.w};
            uint32_t nw[4];
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const uint32_t cnt = up.s3[k] + (mid.s3[k] - mid.w[k]) + dn.s3[k];
                nw[k] = rule_bytes<RULE>(cnt, mid.w[k], ow[k]);
            }
            *reinterpret_cast<uint4*>(out + (size_t)j * nx + x0 + 16 * t) = make_uint4(nw[0], nw[1], nw[2], nw[3]);
        }
        up = mid;
        mid = dn;
        // row j's slot (cur read at step j-1, t-1 read now) takes row j + UB_RING
        bad = __syncthreads_or(bad);
        if (t == 0 && !bad && j + UB_RING <= j1) issue(j + UB_RING);
    }
    if (bad && t == 0) {  // a wait gave up: report and let the copies still in flight land
        atomicOr(status, (unsigned)gb::ST_TMA_TIMEOUT);
        for (int r = max(rbase, last_issued - UB_RING + 1); r <= last_issued; r++) ready(r, gb::tma::DRAIN_NS);
    }
}

// ------------------------------------------------------------------------------ bit-packed form
struct RowBits {
    uint32_t w;       // 32 cells
    uint32_t a0, a1;  // left + self + right as 2-bit slices
};

// New word from the row sums of the rows above, at and below (each left + self + right, 0..3).
// S = up + mid + dn is the 3x3 sum including the cell, so the neighbour count is S - c:
//   reference rule (S234 with the stale carry): a live cell keeps o when S is 3, 4 or 5 and dies
//     otherwise; a dead cell is born when S is 3 and otherwise keeps o;
//   B3/S23: a live cell survives when S is 3 or 4; a dead cell is born when S is 3.
// Only S mod 8 is formed (S0..S2): S = 8 and 9 read as 0 and 1, which neither rule distinguishes
// from the true values (no birth, no survival either way).  Every step is one explicit 3-input
// logic instruction (lop3): 6 for the count (two full adders and the half adder folded into
// s2 = y ^ (x & c1)), 3 for the reference rule (the window S in 3..5, narrowed to S == 3 for a
// dead cell, then the keep/birth select with the stale value) and 2 for B3/S23.
// One 3-input logic instruction; LUT = f(0xF0, 0xCC, 0xAA) for the function f(a, b, c).
template <unsigned LUT>
__device__ __forceinline__ uint32_t lop3(uint32_t a, uint32_t b, uint32_t c)
{
    uint32_t d;
    asm("lop3.b32 %0, %1, %2, %3, %4;" : "=r"(d) : "r"(a), "r"(b), "r"(c), "n"(LUT));
    return d;
}
constexpr unsigned XOR3 = 0x96, MAJ3 = 0xE8;

template <int RULE>
__device__ __forceinline__ uint32_t life_combine(const RowBits& up, const RowBits& mid, const RowBits& dn, uint32_t o)
{
    const uint32_t s0 = lop3<XOR3>(up.a0, mid.a0, dn.a0);
    const uint32_t c1 = lop3<MAJ3>(up.a0, mid.a0, dn.a0);
    const uint32_t x = lop3<XOR3>(up.a1, mid.a1, dn.a1);
    const uint32_t y = lop3<MAJ3>(up.a1, mid.a1, dn.a1);
    const uint32_t s1 = x ^ c1;
    const uint32_t s2 = lop3<0x78>(y, x, c1);  // y ^ (x & c1)
    const uint32_t c = mid.w;
    if (RULE == APPFIS_GB_LIFE_REFERENCE) {
        const uint32_t in345 = lop3<0x38>(s2, s1, s0);  // S in 3..5: (~s2 & s1 & s0) | (s2 & ~s1)
        const uint32_t d = lop3<0xD0>(in345, c, s2);    // live: S in 3..5; dead: S == 3
        return lop3<0x8E>(c, o, d);                      // c ? o & d : o | d
    } else {
        const uint32_t in34 = lop3<0x18>(s2, s1, s0);   // S in 3..4
        return lop3<0xD0>(in34, c, s2);                  // live: S in 3..4; dead: S == 3
    }
}
struct RawBits {
    uint32_t w, lw, rw;
};

__device__ __forceinline__ RawBits load_raw_bits(const uint32_t* __restrict__ bits, int nw, int row, int xw, bool active,
                                                 int lane)
{
    const uint32_t* p = bits + (size_t)row * nw;
    RawBits r;
    r.w = active ? __ldg(p + xw) : 0u;
    r.lw = lane == 0 ? __ldg(p + (xw == 0 ? nw - 1 : xw - 1)) : 0u;
    r.rw = (active && (lane == 31 || xw + 1 >= nw)) ? __ldg(p + (xw + 1 >= nw ? 0 : xw + 1)) : 0u;
    return r;
}

__device__ __forceinline__ RowBits finish_row_bits(const RawBits& raw, int xw, int nw, int lane)
{
    uint32_t lw = __shfl_up_sync(FULL, raw.w, 1);
    uint32_t rw = __shfl_down_sync(FULL, raw.w, 1);
    if (lane == 0) lw = raw.lw;
    if (lane == 31 || xw + 1 >= nw) rw = raw.rw;
    const uint32_t w = raw.w;
    const uint32_t L = __funnelshift_l(lw, w, 1);  // bit b = cell x-1
    const uint32_t R = __funnelshift_r(w, rw, 1);  // bit b = cell x+1
    RowBits r;
    r.w = w;
    r.a0 = L ^ w ^ R;
    r.a1 = (L & w) | (R & (L ^ w));
    return r;
}

// Warp tasks: 32 words (1024 cells) per row over LIFE_ROWS rows, grid-stride, one row prefetched.
template <int RULE>
__global__ void __launch_bounds__(256) life_bits_sweep(const uint32_t* __restrict__ cur, uint32_t* __restrict__ out,
                                                        int nw, int ny, int strips, int tasks)
{
    const int lane = threadIdx.x & 31;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int task = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; task < tasks; task += nwarps) {
        const int strip = task % strips, seg = task / strips;
        const int xw = strip * 32 + lane;
        const bool active = xw < nw;
        const int j0 = seg * LIFE_ROWS, j1 = min(j0 + LIFE_ROWS, ny);
        RowBits up = finish_row_bits(load_raw_bits(cur, nw, j0 == 0 ? ny - 1 : j0 - 1, xw, active, lane), xw, nw, lane);
        RowBits mid = finish_row_bits(load_raw_bits(cur, nw, j0, xw, active, lane), xw, nw, lane);
        RawBits rdn = load_raw_bits(cur, nw, j0 == ny - 1 ? 0 : j0 + 1, xw, active, lane);
        uint32_t o = (RULE == APPFIS_GB_LIFE_REFERENCE && active) ? out[(size_t)j0 * nw + xw] : 0u;
        for (int j = j0; j < j1; j++) {
            RawBits rnext = {0u, 0u, 0u};
            uint32_t onext = 0u;
            if (j + 1 < j1) {
                const int r2 = j + 2 >= ny ? j + 2 - ny : j + 2;
                rnext = load_raw_bits(cur, nw, r2, xw, active, lane);
                if (RULE == APPFIS_GB_LIFE_REFERENCE && active) onext = out[(size_t)(j + 1) * nw + xw];
            }
            const RowBits dn = finish_row_bits(rdn, xw, nw, lane);
            if (active) out[(size_t)j * nw + xw] = life_combine<RULE>(up, mid, dn, o);
            up = mid;
            mid = dn;
            rdn = rnext;
            o = onext;
        }
    }
}

// ------------------------------------------------------------------------------ bit-packed, time-blocked
// TB_STEPS generations per launch on a tile held in shared memory.  A CTA owns output words
// [30*tx, 30*tx + 30) x rows [R*ty, R*ty + R) and loads a 32-word x (R + 2*TB_STEPS)-row region
// around it (periodic wrap at load time, so the region is a consistent periodic window even on
// the grid's last tiles).  Lane 0 / 31 hold the halo words: their outer bits go stale by one
// cell per generation, which never reaches the output words for up to 31 generations; rows go
// stale from the region's top/bottom by one row per generation, which never reaches the R
// output rows for up to TB_STEPS generations.  Both states (t and t-1) are kept: each
// generation writes the new state in place over the t-1 plane (new(x) reads only old(x) and
// the current plane), then the planes swap.  The launch reads two planes and writes two planes
// (the next launch needs both), so global traffic per generation drops by ~TB_STEPS/1.5.
constexpr int TB_ROWS = 256;  // output rows per tile (72 KB of dynamic shared memory, 3 CTAs per SM)
constexpr int TB_STEPS = 16;  // generations per launch (max)
constexpr int TB_WARPS = 8;
constexpr int TB_RR = TB_ROWS + 2 * TB_STEPS;

// Row summary of one word for the bit-sliced neighbour count.  Lanes 0 / 31 get their own word
// back from the shuffles, so their outer bit is wrong; those lanes are the stale halo, whose
// wrong bits travel one cell per generation and never reach an output word.
__device__ __forceinline__ RowBits tile_row(uint32_t w)
{
    const uint32_t lw = __shfl_up_sync(FULL, w, 1);
    const uint32_t rw = __shfl_down_sync(FULL, w, 1);
    const uint32_t L = __funnelshift_l(lw, w, 1), R = __funnelshift_r(w, rw, 1);
    RowBits r;
    r.w = w;
    r.a0 = lop3<XOR3>(L, w, R);
    r.a1 = lop3<MAJ3>(L, w, R);
    return r;
}

template <int RULE>
__global__ void __launch_bounds__(TB_WARPS * 32) life_bits_tb(const uint32_t* __restrict__ curG, const uint32_t* __restrict__ oldG,
                                                               uint32_t* __restrict__ outCur, uint32_t* __restrict__ outOld,
                                                               int nw, int ny, int tiles_x, int tiles, int steps)
{
    extern __shared__ uint32_t tbsm[];  // two (TB_RR x 32)-word planes
    uint32_t(*sA)[32] = reinterpret_cast<uint32_t(*)[32]>(tbsm);
    uint32_t(*sB)[32] = reinterpret_cast<uint32_t(*)[32]>(tbsm + TB_RR * 32);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const int tx = tile % tiles_x, ty = tile / tiles_x;
        int wx = (tx * 30 - 1 + lane) % nw;
        if (wx < 0) wx += nw;
        const int row0 = ty * TB_ROWS - TB_STEPS;
        for (int r = warp; r < TB_RR; r += TB_WARPS) {
            int gy = (row0 + r) % ny;
            if (gy < 0) gy += ny;
            const size_t g = (size_t)gy * nw + wx;
            sA[r][lane] = __ldg(curG + g);
            sB[r][lane] = RULE == APPFIS_GB_LIFE_REFERENCE ? __ldg(oldG + g) : 0u;
        }
        __syncthreads();
        uint32_t(*cur)[32] = sA;
        uint32_t(*old)[32] = sB;
        for (int t = 1; t <= steps; t++) {
            // rows valid after generation t: [t, TB_RR - t), split evenly over the warps; each warp
            // marches its chunk carrying the row summaries (one new row summary per output row)
            const int lo = t, n = TB_RR - 2 * t, chunk = (n + TB_WARPS - 1) / TB_WARPS;
            const int r0 = lo + warp * chunk, r1 = min(lo + n, r0 + chunk);
            if (r0 < r1) {
                RowBits up = tile_row(cur[r0 - 1][lane]);
                RowBits mid = tile_row(cur[r0][lane]);
#pragma unroll 8  // 8 rows per trip: the up/mid/dn rotation becomes register renaming
                for (int r = r0; r < r1; r++) {
                    const RowBits dn = tile_row(cur[r + 1][lane]);
                    const uint32_t o = RULE == APPFIS_GB_LIFE_REFERENCE ? old[r][lane] : 0u;
                    old[r][lane] = life_combine<RULE>(up, mid, dn, o);
                    up = mid;
                    mid = dn;
                }
            }
            __syncthreads();
            uint32_t(*tmp)[32] = cur;
            cur = old;
            old = tmp;
        }
        const int wout = tx * 30 - 1 + lane;
        if (lane >= 1 && lane <= 30 && wout < nw) {
            for (int r = TB_STEPS + warp; r < TB_STEPS + TB_ROWS; r += TB_WARPS) {
                const int gy = ty * TB_ROWS + (r - TB_STEPS);
                if (gy < ny) {
                    const size_t g = (size_t)gy * nw + wout;
                    outCur[g] = cur[r][lane];
                    outOld[g] = old[r][lane];
                }
            }
        }
        __syncthreads();
    }
}

__global__ void life_pack(const uint8_t* __restrict__ cells, uint32_t* __restrict__ bits, size_t nwords)
{
    size_t w = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nwords) return;
    const uint4* p = reinterpret_cast<const uint4*>(cells + w * 32);
    uint4 a = __ldg(p), b = __ldg(p + 1);
    uint32_t v[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w}, out = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        uint32_t x = v[k] & LSB;                 // bit 0 of bytes 0..3 -> bits 0, 8, 16, 24
        x = (x | (x >> 7)) & 0x00030003u;        // bytes 0,1 -> bits 0,1 ; bytes 2,3 -> bits 16,17
        x = (x | (x >> 14)) & 0x0000000fu;       // -> bits 0..3
        out |= x << (4 * k);
    }
    bits[w] = out;
}

__global__ void life_unpack(const uint32_t* __restrict__ bits, uint8_t* __restrict__ cells, size_t nwords)
{
    size_t w = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nwords) return;
    uint32_t b = __ldg(bits + w), v[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
        uint32_t x = (b >> (4 * k)) & 0xfu;
        x = (x | (x << 14)) & 0x00030003u;
        x = (x | (x << 7)) & LSB;
        v[k] = x;
    }
    uint4* p = reinterpret_cast<uint4*>(cells + w * 32);
    p[0] = make_uint4(v[0], v[1], v[2], v[3]);
    p[1] = make_uint4(v[4], v[5], v[6], v[7]);
}

// The reference's layout: int cells 0/1 on a (nx + 2g) x (ny + 2g) grid with a periodic ghost
// ring of width g (GameOfLife/src/game_appfis.hpp:58-62).  From it: the u8 interior; into it:
// every padded cell from the interior cell it wraps to (the ghost ring as the periodic exchange
// leaves it, corners included).
__global__ void life_from_i32(const int32_t* __restrict__ f, int px, int g, uint8_t* __restrict__ cells, int nx, int ny)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nx) return;
    for (int j = blockIdx.y; j < ny; j += gridDim.y) cells[(size_t)j * nx + i] = __ldg(f + (size_t)(j + g) * px + i + g) != 0;
}

__global__ void life_to_i32(const uint8_t* __restrict__ cells, int nx, int ny, int32_t* __restrict__ f, int px, int g)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nx + 2 * g) return;
    int si = (i - g) % nx;
    if (si < 0) si += nx;
    for (int j = blockIdx.y; j < ny + 2 * g; j += gridDim.y) {
        int sj = (j - g) % ny;
        if (sj < 0) sj += ny;
        f[(size_t)j * px + i] = __ldg(cells + (size_t)sj * nx + si);
    }
}

// Population: popcount over 32-bit words (u8 cells are 0/1, so popc of 4 bytes = live bytes).
__global__ void popcount_words(const uint32_t* __restrict__ words, size_t n, unsigned long long* __restrict__ out)
{
    unsigned long long s = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        s += __popc(__ldg(words + i));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(FULL, s, o);
    __shared__ unsigned long long part[32];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(FULL, s, o);
        if (threadIdx.x == 0) atomicAdd(out, s);
    }
}

// tail of a byte array whose length is not a multiple of 4
__global__ void popcount_tail(const uint8_t* __restrict__ p, int n, unsigned long long* __restrict__ out)
{
    unsigned long long s = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s += p[i];
    if (s) atomicAdd(out, s);
}

// Blocks of 256 threads: as many as are resident at once, but no more than the warp tasks need.
template <class K>
unsigned resident_grid(K kernel, int tasks)
{
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 256, 0) != cudaSuccess || per_sm < 1) per_sm = 4;
    const size_t need = gb::ceil_div((size_t)tasks * 32, 256);
    return (unsigned)std::max<size_t>(1, std::min<size_t>(need, (size_t)per_sm * gb::sm_count()));
}

template <int RULE>
int run_u8(uint8_t* buf[2], int nx, int ny, int gens, int* cur_index, cudaStream_t st)
{
    int ci = 0;
    if (nx % 16 == 0) {
        unsigned* status;
        GB_TRY(gb::status_word(&status));
        GB_CUDA(cudaFuncSetAttribute(life_u8_bulk<RULE>, cudaFuncAttributeMaxDynamicSharedMemorySize, UB_SMEM));
        const int strips = (nx + UB_W - 1) / UB_W;
        const unsigned grid = (unsigned)strips * gb::ceil_div(ny, UB_ROWS);
        for (int g = 0; g < gens; g++) {
            life_u8_bulk<RULE><<<grid, 256, UB_SMEM, st>>>(buf[ci], buf[1 - ci], nx, ny, strips, status);
            ci = 1 - ci;
        }
    } else {
        dim3 blk(32, 8), grd(gb::ceil_div(nx, 32), gb::ceil_div(ny, 8));
        for (int g = 0; g < gens; g++) {
            life_u8_generic<RULE><<<grd, blk, 0, st>>>(buf[ci], buf[1 - ci], nx, ny);
            ci = 1 - ci;
        }
    }
    GB_TRY(gb::launched("life_u8 sweep"));
    if (cur_index) *cur_index = ci;
    return APPFIS_GB_OK;
}

// Time-blocked launches for whole blocks of TB_STEPS generations, single-generation sweeps for
// the remainder.  A launch reads a (cur, old) pair and writes another pair (its tiles read
// neighbours' halo rows, so it cannot write in place).  An even number of launches ping-pongs
// between (a, b) and a workspace pair; an odd number of three or more first goes round three
// pairs once ((a, b) -> W1 -> W2 -> (a, b)) and then ping-pongs, so the newest state ends in
// (a, b) without a copy; a single launch copies its pair back.  cur_index tells which of a, b
// holds the newest state.
template <int RULE>
int run_bits(uint32_t* buf[2], int nx, int ny, int gens, int* cur_index, cudaStream_t st)
{
    const int nw = nx / 32;
    int ci = 0;
    const size_t plane = (size_t)nw * ny;
    if (gens >= TB_STEPS) {
        const int launches = gens / TB_STEPS;
        void *wc, *wd, *we = nullptr, *wf = nullptr;
        GB_TRY(gb::workspace(gb::WS_LIFE_C, sizeof(uint32_t) * plane, &wc));
        GB_TRY(gb::workspace(gb::WS_LIFE_D, sizeof(uint32_t) * plane, &wd));
        if (launches % 2 == 1 && launches >= 3) {
            GB_TRY(gb::workspace(gb::WS_LIFE_E, sizeof(uint32_t) * plane, &we));
            GB_TRY(gb::workspace(gb::WS_LIFE_F, sizeof(uint32_t) * plane, &wf));
        }
        uint32_t* P[3][2] = {{buf[0], buf[1]}, {(uint32_t*)wc, (uint32_t*)wd}, {(uint32_t*)we, (uint32_t*)wf}};  // [pair][cur/old]
        const int tiles_x = (nw + 29) / 30, tiles = tiles_x * ((ny + TB_ROWS - 1) / TB_ROWS);
        int per_sm = 0;
        const int tsm = 2 * TB_RR * 32 * 4;
        GB_CUDA(cudaFuncSetAttribute(life_bits_tb<RULE>, cudaFuncAttributeMaxDynamicSharedMemorySize, tsm));
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, life_bits_tb<RULE>, TB_WARPS * 32, tsm) != cudaSuccess ||
            per_sm < 1)
            per_sm = 4;
        const int grid = std::max(1, std::min(tiles, per_sm * gb::sm_count()));
        int pair = 0;
        for (int n = 0; n < launches; n++) {
            const int next = (we && n < 3) ? (n + 1) % 3 : 1 - pair;  // the three-pair round first, then ping-pong
            life_bits_tb<RULE><<<grid, TB_WARPS * 32, tsm, st>>>(P[pair][0], P[pair][1], P[next][0], P[next][1], nw, ny, tiles_x,
                                                               tiles, TB_STEPS);
            pair = next;
        }
        GB_TRY(gb::launched("life_bits_tb"));
        if (pair != 0) {  // one launch: bring the (cur, old) pair back into (a, b)
            GB_CUDA(cudaMemcpyAsync(buf[0], P[pair][0], sizeof(uint32_t) * plane, cudaMemcpyDeviceToDevice, st));
            GB_CUDA(cudaMemcpyAsync(buf[1], P[pair][1], sizeof(uint32_t) * plane, cudaMemcpyDeviceToDevice, st));
        }
        gens -= launches * TB_STEPS;
    }
    if (gens > 0) {
        const int strips = (nw + 31) / 32;
        const int tasks = strips * ((ny + LIFE_ROWS - 1) / LIFE_ROWS);
        const unsigned grid = resident_grid(life_bits_sweep<RULE>, tasks);
        for (int g = 0; g < gens; g++) {
            life_bits_sweep<RULE><<<grid, 256, 0, st>>>(buf[ci], buf[1 - ci], nw, ny, strips, tasks);
            ci = 1 - ci;
        }
        GB_TRY(gb::launched("life_bits sweep"));
    }
    if (cur_index) *cur_index = ci;
    return APPFIS_GB_OK;
}

int check_life(const void* a, const void* b, int nx, int ny, int gens, int rule)
{
    if (!a || !b) return gb::fail(APPFIS_GB_EINVAL, "life: null buffer");
    if (a == b) return gb::fail(APPFIS_GB_EINVAL, "life: the two buffers must differ");
    if (nx < 1 || ny < 1) return gb::fail(APPFIS_GB_EINVAL, "life: bad size %d x %d", nx, ny);
    if ((size_t)nx * (size_t)ny > ((size_t)1 << 40)) return gb::fail(APPFIS_GB_EINVAL, "life: grid too large");
    if (gens < 0) return gb::fail(APPFIS_GB_EINVAL, "life: negative generation count");
    if (rule != APPFIS_GB_LIFE_REFERENCE && rule != APPFIS_GB_LIFE_B3S23)
        return gb::fail(APPFIS_GB_EINVAL, "life: unknown rule %d", rule);
    return APPFIS_GB_OK;
}

int population_u8(const uint8_t* cells, int64_t n, int64_t* dev_count, cudaStream_t st)
{
    GB_CUDA(cudaMemsetAsync(dev_count, 0, sizeof(int64_t), st));
    size_t nw = (size_t)n / 4;
    if (nw) {
        unsigned grid = (unsigned)std::min<size_t>(gb::ceil_div(nw, 256), (size_t)gb::sm_count() * 8);
        popcount_words<<<grid, 256, 0, st>>>(reinterpret_cast<const uint32_t*>(cells), nw,
                                             reinterpret_cast<unsigned long long*>(dev_count));
    }
    if (n % 4)
        popcount_tail<<<1, 32, 0, st>>>(cells + nw * 4, (int)(n % 4), reinterpret_cast<unsigned long long*>(dev_count));
    return gb::launched("life population");
}

}  // namespace

extern "C" {

int appfis_gb_life_u8(uint8_t* a, uint8_t* b, int nx, int ny, int gens, int rule, int* cur_index, void* stream)
{
    GB_TRY(check_life(a, b, nx, ny, gens, rule));
    if (nx % 16 == 0 && ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b)) & 15))
        return gb::fail(APPFIS_GB_EINVAL, "life_u8: buffers must be 16-byte aligned");
    uint8_t* buf[2] = {a, b};
    cudaStream_t st = gb::as_stream(stream);
    return rule == APPFIS_GB_LIFE_REFERENCE ? run_u8<APPFIS_GB_LIFE_REFERENCE>(buf, nx, ny, gens, cur_index, st)
                                            : run_u8<APPFIS_GB_LIFE_B3S23>(buf, nx, ny, gens, cur_index, st);
}

int appfis_gb_life_bits(uint32_t* a, uint32_t* b, int nx, int ny, int gens, int rule, int* cur_index, void* stream)
{
    GB_TRY(check_life(a, b, nx, ny, gens, rule));
    if (nx % 32) return gb::fail(APPFIS_GB_EINVAL, "life_bits: nx (%d) must be a multiple of 32", nx);
    uint32_t* buf[2] = {a, b};
    cudaStream_t st = gb::as_stream(stream);
    return rule == APPFIS_GB_LIFE_REFERENCE ? run_bits<APPFIS_GB_LIFE_REFERENCE>(buf, nx, ny, gens, cur_index, st)
                                            : run_bits<APPFIS_GB_LIFE_B3S23>(buf, nx, ny, gens, cur_index, st);
}

int appfis_gb_life_pack(const uint8_t* cells, uint32_t* bits, int nx, int ny, void* stream)
{
    if (!cells || !bits || nx < 1 || ny < 1 || nx % 32) return gb::fail(APPFIS_GB_EINVAL, "life_pack: bad arguments");
    if (reinterpret_cast<uintptr_t>(cells) & 15) return gb::fail(APPFIS_GB_EINVAL, "life_pack: cells must be 16-byte aligned");
    size_t nw = (size_t)nx * ny / 32;
    life_pack<<<gb::ceil_div(nw, 256), 256, 0, gb::as_stream(stream)>>>(cells, bits, nw);
    return gb::launched("life_pack");
}

int appfis_gb_life_unpack(const uint32_t* bits, uint8_t* cells, int nx, int ny, void* stream)
{
    if (!cells || !bits || nx < 1 || ny < 1 || nx % 32) return gb::fail(APPFIS_GB_EINVAL, "life_unpack: bad arguments");
    if (reinterpret_cast<uintptr_t>(cells) & 15) return gb::fail(APPFIS_GB_EINVAL, "life_unpack: cells must be 16-byte aligned");
    size_t nw = (size_t)nx * ny / 32;
    life_unpack<<<gb::ceil_div(nw, 256), 256, 0, gb::as_stream(stream)>>>(bits, cells, nw);
    return gb::launched("life_unpack");
}

int appfis_gb_life_from_i32(const int32_t* padded, int px, int ghost, uint8_t* cells, int nx, int ny, void* stream)
{
    if (!padded || !cells || nx < 1 || ny < 1 || ghost < 0 || ghost > nx || ghost > ny || px < nx + 2 * ghost)
        return gb::fail(APPFIS_GB_EINVAL, "life_from_i32: bad arguments");
    dim3 grd(gb::ceil_div(nx, 256), std::min(ny, 65535));
    life_from_i32<<<grd, 256, 0, gb::as_stream(stream)>>>(padded, px, ghost, cells, nx, ny);
    return gb::launched("life_from_i32");
}

int appfis_gb_life_to_i32(const uint8_t* cells, int nx, int ny, int32_t* padded, int px, int ghost, void* stream)
{
    if (!padded || !cells || nx < 1 || ny < 1 || ghost < 0 || ghost > nx || ghost > ny || px < nx + 2 * ghost)
        return gb::fail(APPFIS_GB_EINVAL, "life_to_i32: bad arguments");
    dim3 grd(gb::ceil_div(nx + 2 * ghost, 256), std::min(ny + 2 * ghost, 65535));
    life_to_i32<<<grd, 256, 0, gb::as_stream(stream)>>>(cells, nx, ny, padded, px, ghost);
    return gb::launched("life_to_i32");
}

int appfis_gb_life_population_u8(const uint8_t* cells, int64_t n, int64_t* dev_count, void* stream)
{
    if (!cells || !dev_count || n < 0) return gb::fail(APPFIS_GB_EINVAL, "life_population_u8: bad arguments");
    if (reinterpret_cast<uintptr_t>(cells) & 3) return gb::fail(APPFIS_GB_EINVAL, "life_population_u8: cells must be 4-byte aligned");
    return population_u8(cells, n, dev_count, gb::as_stream(stream));
}

int appfis_gb_life_population_bits(const uint32_t* bits, int64_t nwords, int64_t* dev_count, void* stream)
{
    if (!bits || !dev_count || nwords < 0) return gb::fail(APPFIS_GB_EINVAL, "life_population_bits: bad arguments");
    cudaStream_t st = gb::as_stream(stream);
    GB_CUDA(cudaMemsetAsync(dev_count, 0, sizeof(int64_t), st));
    if (nwords) {
        unsigned grid = (unsigned)std::min<size_t>(gb::ceil_div((size_t)nwords, 256), (size_t)gb::sm_count() * 8);
        popcount_words<<<grid, 256, 0, st>>>(bits, (size_t)nwords, reinterpret_cast<unsigned long long*>(dev_count));
    }
    return gb::launched("life_population_bits");
}

int appfis_gb_life_job(const uint8_t* cells_in, uint8_t* cells_out, int nx, int ny, int gens, int rule, int form,
                       int64_t* population)
{
    if (!cells_in) return gb::fail(APPFIS_GB_EINVAL, "life_job: null input");
    if (form != APPFIS_GB_FORM_U8 && form != APPFIS_GB_FORM_BITS) return gb::fail(APPFIS_GB_EINVAL, "life_job: form %d", form);
    GB_TRY(check_life(cells_in, cells_in + 1, nx, ny, gens, rule));
    if (form == APPFIS_GB_FORM_BITS && nx % 32) return gb::fail(APPFIS_GB_EINVAL, "life_job: bit form needs nx %% 32 == 0");
    cudaStream_t st;
    GB_TRY(gb::job_stream(&st));
    const size_t n = (size_t)nx * ny;
    const size_t nbytes = (n + 15) & ~(size_t)15;
    void *ua, *ub, *cnt;
    GB_TRY(gb::workspace(gb::WS_JOB_A, nbytes, &ua));
    GB_TRY(gb::workspace(gb::WS_JOB_F, 64, &cnt));
    GB_CUDA(cudaMemcpyAsync(ua, cells_in, n, cudaMemcpyHostToDevice, st));
    uint8_t* latest = nullptr;
    if (form == APPFIS_GB_FORM_U8) {
        GB_TRY(gb::workspace(gb::WS_JOB_B, nbytes, &ub));
        GB_CUDA(cudaMemsetAsync(ub, 0, n, st));
        int ci = 0;
        GB_TRY(appfis_gb_life_u8((uint8_t*)ua, (uint8_t*)ub, nx, ny, gens, rule, &ci, st));
        latest = ci == 0 ? (uint8_t*)ua : (uint8_t*)ub;
        GB_TRY(appfis_gb_life_population_u8(latest, (int64_t)n, (int64_t*)cnt, st));
    } else {
        void *wa, *wb;
        const size_t wbytes = n / 8;
        GB_TRY(gb::workspace(gb::WS_JOB_C, wbytes, &wa));
        GB_TRY(gb::workspace(gb::WS_JOB_D, wbytes, &wb));
        GB_TRY(appfis_gb_life_pack((const uint8_t*)ua, (uint32_t*)wa, nx, ny, st));
        GB_CUDA(cudaMemsetAsync(wb, 0, wbytes, st));
        int ci = 0;
        GB_TRY(appfis_gb_life_bits((uint32_t*)wa, (uint32_t*)wb, nx, ny, gens, rule, &ci, st));
        uint32_t* lw = ci == 0 ? (uint32_t*)wa : (uint32_t*)wb;
        GB_TRY(appfis_gb_life_population_bits(lw, (int64_t)(n / 32), (int64_t*)cnt, st));
        if (cells_out) GB_TRY(appfis_gb_life_unpack(lw, (uint8_t*)ua, nx, ny, st));
        latest = (uint8_t*)ua;
    }
    if (cells_out) GB_CUDA(cudaMemcpyAsync(cells_out, latest, n, cudaMemcpyDeviceToHost, st));
    int64_t pop = 0;
    GB_CUDA(cudaMemcpyAsync(&pop, cnt, sizeof pop, cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    if (population) *population = pop;
    return gb::check_status("life_job");  // a bounded wait of the u8 sweep that gave up
}

}  // extern "C"
