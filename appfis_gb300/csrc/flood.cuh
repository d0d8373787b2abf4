// Batched, persistent flood-model time stepping (kernels + host runner), instantiated for float
// (flood_f32.cu) and double (flood_f64.cu, built without FMA contraction).  See flood_core.cuh
// for the per-face / per-cell arithmetic and the reference it follows.
//
// One cooperative launch advances a batch of independent domains of uneven sizes to t_end.
// Work items are strips (SCOLS interior columns x ROWS rows) of all domains; in each phase a warp
// takes its first strip by index and the rest one at a time from a counter (a strip's cost
// follows the water, so a fixed stride leaves some warps with far more wet strips than others).
// Each step is phase A (wet/dry fix of the previous step + CFL dt, min per domain) and phase B
// (fluxes + update into the other state buffer), separated by grid barriers whose spin waits
// are bounded (on timeout the kernel records an error and returns).  Per-domain scalars
// (dt bits, simulated time, print index, step count) are double-buffered by step parity so no
// block ever reads a value another block is writing in the same phase; one thread commits them.
#pragma once

#include "flood_core.cuh"
#include "tma.cuh"

namespace flood {

template <class T>
struct Dom {
    T* h[2];
    T* qx[2];
    T* qy[2];
    const T* dem;
    const T* n2;
    int nx, ny, px, strips_x;
    long long strip0;  // first global strip of this domain
};

// Point sources of one domain (device copies of the caller's tables).
struct SrcDev {
    int n, nt;            // sources, hydrograph rows
    const int* cells;     // n cells: the reference's padded sub-grid index row * (nx + 2) + col
    const double* times;  // nt times (s)
    const double* flows;  // nt * n flows (m^3/s), row t = the n sources at times[t]
};

struct Ctl {
    int src_lo[MAXD];     // hydrograph row of each domain's sources (kept across steps)
    unsigned long long dtbits[3][MAXD];  // two-phase kernel: by step parity; fused kernel: by step mod 3
    double simtime[2][MAXD];
    int pid[2][MAXD];
    int steps[2][MAXD];
    unsigned bar_count;
    unsigned bar_gen;
    int error;
    unsigned ticket[2];  // phase A strip hand-out, by step parity
    unsigned ticketb[2];  // phase B strip hand-out, by step parity
};

struct Params {
    double dx, cn, hextra, t_end, print_interval, time_step;
    float fdx, fcn, fhextra;  // dx, cn, hextra rounded to float once on the host (float kernel)
    int max_steps, ndom;
    long long total_strips;
    double* dtlog;  // [ndom][max_steps] or null
    unsigned char* zc;  // [2][total_strips] dry-step counters (null: every strip every step)
    unsigned long long spin_limit;  // polls before a grid-barrier wait gives up
    int stall_cta;                  // testing: this CTA skips its arrival at the first barrier (-1: none)
    const SrcDev* srcs;             // [ndom] point sources, or null (no source phase)
    const CUtensorMap* maps;        // staged fused pass: [ndom][8] row maps (h0 h1 qx0 qx1 qy0 qy1 dem n2)
    unsigned long long wait_ns;     // staged: limit of one wait for a stage of rows
    unsigned tx_extra;              // testing: bytes added to each warp's first stage (it cannot complete)
};

constexpr unsigned long long SPIN_LIMIT = 1ull << 25;
constexpr int STEP_CAP = 1000000;  // steps per domain when the caller sets no limit

// Grid-wide barrier of the cooperative launch.  Every wait is bounded (`limit` polls, each with
// a short sleep); a wait that gives up records error 1 and every CTA leaves its loop.  `skip`
// (testing only) makes this CTA wait without arriving, so that the barrier cannot complete.
__device__ __forceinline__ bool grid_barrier(Ctl* ctl, unsigned long long limit, bool skip = false)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* vgen = &ctl->bar_gen;
        const unsigned g = *vgen;
        __threadfence();
        if (!skip && atomicAdd(&ctl->bar_count, 1u) == gridDim.x - 1) {
            ctl->bar_count = 0;
            __threadfence();
            atomicAdd(&ctl->bar_gen, 1u);
        } else {
            unsigned long long n = 0;
            while (*vgen == g) {
                if (++n > limit) {
                    atomicExch(&ctl->error, 1);
                    break;
                }
                if (*(volatile int*)&ctl->error) break;
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return *(volatile int*)&ctl->error == 0;
}

template <class T>
__device__ __forceinline__ int find_domain(const Dom<T>* d, int nd, long long s)
{
    int lo = 0, hi = nd - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (d[mid].strip0 <= s) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// A parameter in the kernel's type: the float kernel takes the host-rounded copy (the same value
// as converting on the device, without a double-to-float conversion on the FP64 pipe per strip).
template <class T>
__device__ __forceinline__ T typed(double d, float f)
{
    if constexpr (sizeof(T) == 4)
        return f;
    else
        return d;
}

// The dt of domain d's step from its CFL minimum in dtbits[slot] and the step's scalars [cur].
__device__ __forceinline__ double step_dt_at(const Ctl* ctl, int slot, int cur, int d, const Params& p, double big)
{
    double dt = __longlong_as_double((long long)ctl->dtbits[slot][d]);
    if (dt >= big - 1.0) dt = p.time_step;
    const double st = ctl->simtime[cur][d];
    const double next_print = p.print_interval * (ctl->pid[cur][d] + 1);
    if (st + dt > next_print) dt = next_print - st;
    return dt;
}

__device__ __forceinline__ double step_dt(const Ctl* ctl, int cur, int d, const Params& p, double big)
{
    return step_dt_at(ctl, cur, cur, d, p, big);
}

__device__ __forceinline__ bool is_active(const Ctl* ctl, int cur, int d, const Params& p)
{
    return ctl->simtime[cur][d] < p.t_end && ctl->steps[cur][d] < p.max_steps;
}

// ---------------------------------------------------------------- phase A: fix + dt
// The domain descriptor arrives by value (registers): read through the shared-memory copy, every
// field would be reloaded after each global store, which the compiler cannot prove disjoint.
// Rows are processed in groups of FA_ROWS with their h, qx, qy loads issued together, so a
// warp has several rows of loads in flight instead of one.
constexpr int FA_ROWS = 4;

// SC, LO: the strip geometry (SC columns per strip on lanes LO .. LO+SC-1; the two-phase kernel's
// 30 on lanes 1..30, the fused kernel's 28 on lanes 2..29); the CFL minimum goes to dtbits[slot].
template <class T, int SC = SCOLS, int LO = 1>
__device__ void phase_a(const Dom<T> D, Ctl* ctl, int slot, int d, long long local, int b, bool fix, bool want_dt,
                        const Params& p)
{
    const int lane = threadIdx.x & 31;
    const int loc = (int)local, sy = loc / D.strips_x, sx = loc - sy * D.strips_x;  // 32-bit: a domain has < 2^31 strips
    const int i = sx * SC + lane - LO + 1;  // lanes LO..LO+SC-1: the strip's interior columns
    const int j0 = 1 + sy * ROWS, j1 = min(j0 + ROWS, D.ny + 1);
    const T* __restrict__ h = D.h[b];
    T* __restrict__ qx = D.qx[b];
    T* __restrict__ qy = D.qy[b];
    const T* __restrict__ dem = D.dem;
    const int px = D.px;
    const T hextra = typed<T>(p.hextra, p.fhextra), E = K<T>::dry(), G = K<T>::g();
    const T dx = typed<T>(p.dx, p.fdx), cn = typed<T>(p.cn, p.fcn);
    T mn = K<T>::big();  // min in T (exact), widened once per warp: no per-cell FP64 work in float
    if (lane >= LO && lane < LO + SC && i <= D.nx) {
        for (int jb = j0; jb < j1; jb += FA_ROWS) {
            T hv[FA_ROWS], qxv[FA_ROWS], qyv[FA_ROWS];
#pragma unroll
            for (int r = 0; r < FA_ROWS; r++) {
                const size_t c = (size_t)(jb + r) * px + i;
                const bool in = jb + r < j1;
                hv[r] = in ? h[c] : T(0);
                qxv[r] = in ? qx[c] : T(0);
                qyv[r] = in ? qy[c] : T(0);
            }
#pragma unroll
            for (int r = 0; r < FA_ROWS; r++) {
                const size_t c = (size_t)(jb + r) * px + i;
                const T hij = hv[r];
                if (!(hij > hextra)) continue;  // dry: no fix, no dt (rows past j1 hold 0)
                T qxr = qxv[r], qyr = qyv[r];
                if (fix) {  // triton_appfis.hpp:1095-1112
                    const T lvl = hij + dem[c];
                    if (((lvl < dem[c + 1]) && (h[c + 1] < E)) || ((lvl < dem[c - 1]) && (h[c - 1] < E))) {
                        qxr = T(0);
                        qx[c] = qxr;
                    }
                    if (((lvl < dem[c - px]) && (h[c - px] < E)) || ((lvl < dem[c + px]) && (h[c + px] < E))) {
                        qyr = T(0);
                        qy[c] = qyr;
                    }
                }
                if (want_dt) {  // triton_appfis.hpp:567-586
                    const T dtx = dx / (fabs(qxr / hij) + sqrt(G * hij));
                    const T dty = dx / (fabs(qyr / hij) + sqrt(G * hij));
                    const T v = dtx < dty ? cn * dtx : cn * dty;
                    mn = v < mn ? v : mn;
                }
            }
        }
    }
    if (want_dt) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const T other = __shfl_down_sync(0xffffffffu, mn, o);
            mn = other < mn ? other : mn;
        }
        if (lane == 0 && mn < K<T>::big())
            atomicMin(&ctl->dtbits[slot][d], (unsigned long long)__double_as_longlong((double)mn));
    }
}

// ---------------------------------------------------------------- phase B: fluxes + update
// A cell's raw state (h, qx, qy, z); zero outside the padded row.
template <class T>
struct Raw {
    T h, qx, qy, z;
};

template <class T>
__device__ __forceinline__ Raw<T> load_raw(const T* __restrict__ h, const T* __restrict__ qx, const T* __restrict__ qy,
                                           const T* __restrict__ dem, int px, int nx, int i, int j)
{
    if (i > nx + 1) return Raw<T>{T(0), T(0), T(0), T(0)};
    const size_t c = (size_t)j * px + i;
    return Raw<T>{h[c], qx[c], qy[c], dem[c]};
}

template <class T>
__device__ __forceinline__ Cell<T> cell_of(const Raw<T>& r)
{
    return make_cell<T>(r.h, r.qx, r.qy, r.z);
}

// Each warp marches its strip's rows.  Lane l holds column 30*sx + l of the row: lanes 1..30 are
// the strip's interior cells, lanes 0 and 31 the neighbour columns, so one coalesced row load
// brings every cell the strip's faces need.  Lanes 0..30 compute the X face between their cell
// and the next lane's (lane 0's is the strip's left face), lanes 1..30 the Y faces and updates.
// The loads of row j+2 are issued while row j is computed.
template <class T>
__device__ bool phase_b(const Dom<T> D, long long local, int b, T dt, const Params& p)
{
    const int lane = threadIdx.x & 31;
    const int loc = (int)local, sy = loc / D.strips_x, sx = loc - sy * D.strips_x;  // 32-bit: a domain has < 2^31 strips
    const int i = sx * SCOLS + lane;
    const int j0 = 1 + sy * ROWS, j1 = min(j0 + ROWS, D.ny + 1);
    const bool own = lane >= 1 && lane <= SCOLS && i <= D.nx;  // cells this lane updates
    const bool xface = lane <= SCOLS && i <= D.nx;             // face i|i+1 is needed
    const T dx = typed<T>(p.dx, p.fdx), hextra = typed<T>(p.hextra, p.fhextra);
    const T one = T(1), zero = T(0);
    const T* __restrict__ h = D.h[b];
    const T* __restrict__ qx = D.qx[b];
    const T* __restrict__ qy = D.qy[b];
    const T* __restrict__ dem = D.dem;
    const T* __restrict__ n2 = D.n2;
    T* __restrict__ ho_ = D.h[1 - b];
    T* __restrict__ qxo_ = D.qx[1 - b];
    T* __restrict__ qyo_ = D.qy[1 - b];
    const int px = D.px, nx = D.nx, ny = D.ny;
    const Raw<T> zr = {zero, zero, zero, zero};
    bool dry = true;  // every cell this lane updated ends with h = qx = qy = 0

    Cell<T> cj = cell_of(load_raw(h, qx, qy, dem, px, nx, i, j0));
    Raw<T> rn = load_raw(h, qx, qy, dem, px, nx, i, j0 + 1);  // rows j0+1 <= ny+1 always exist
    T ycar[3] = {zero, zero, zero};  // rhs0 Y part of row j (from face j|j-1)
    bool ywet = false;
    if (own) {
        const Cell<T> cm = cell_of(load_raw(h, qx, qy, dem, px, nx, i, j0 - 1));
        T r2[3];
        ywet = face<T>(cj, cm, zero, one, dx, dt, hextra, ycar, r2);
    }
    for (int j = j0; j < j1; j++) {
        const Raw<T> rnn = j + 2 <= ny + 1 ? load_raw(h, qx, qy, dem, px, nx, i, j + 2) : zr;  // prefetch
        const size_t c = (size_t)j * px + i;
        const T n2v = own ? n2[c] : zero;
        const Cell<T> cn_ = cell_of(rn);
        // X face i|i+1 of row j: rhs0 of cell i, rhs1 of cell i+1 (the next lane)
        const Cell<T> right = shfl_cell(cj, 1, true);
        T xr1[3] = {zero, zero, zero}, xr2[3] = {zero, zero, zero};
        bool xwet = false;
        if (xface) xwet = face<T>(cj, right, one, zero, dx, dt, hextra, xr1, xr2);
        T lr[3];
        lr[0] = __shfl_up_sync(0xffffffffu, xr2[0], 1);
        lr[1] = __shfl_up_sync(0xffffffffu, xr2[1], 1);
        lr[2] = __shfl_up_sync(0xffffffffu, xr2[2], 1);
        const bool lwet = __shfl_up_sync(0xffffffffu, (int)xwet, 1) != 0;
        // Y face j+1|j: id1 = row j+1, id2 = row j
        T yn1[3] = {zero, zero, zero}, yr2[3] = {zero, zero, zero};
        bool ynwet = false;
        if (own) ynwet = face<T>(cn_, cj, zero, one, dx, dt, hextra, yn1, yr2);
        if (own) {
            T r0[3], r1[3];
#pragma unroll
            for (int k = 0; k < 3; k++) {
                r0[k] = xwet ? xr1[k] : zero;
                if (ywet) r0[k] = r0[k] + ycar[k];
                r1[k] = lwet ? lr[k] : zero;
                if (ynwet) r1[k] = r1[k] + yr2[k];
            }
            T hn, qxn, qyn;
            update<T>(cj.h, cj.qx, cj.qy, n2v, r0, r1, dt, hextra, hn, qxn, qyn);
            ho_[c] = hn;
            qxo_[c] = qxn;
            qyo_[c] = qyn;
            dry = dry && hn == zero && qxn == zero && qyn == zero;
        }
#pragma unroll
        for (int k = 0; k < 3; k++) ycar[k] = yn1[k];
        ywet = ynwet;
        cj = cn_;
        rn = rnn;
    }
    return __all_sync(0xffffffffu, dry);
}

// Dry-strip bookkeeping (Params::zc): zc[parity][s] counts the consecutive steps whose output of
// strip s was entirely dry (capped at 2).  Strip s may be left out of a step when it has been
// dry for two steps (both state buffers hold zeros there) and its four neighbour strips of the
// same domain are dry in the step's input.
template <class T>
__device__ __forceinline__ bool strip_idle(const Dom<T>& D, const unsigned char* zin, long long s)
{
    if (zin[s] < 2) return false;
    const long long local = s - D.strip0;
    const int loc = (int)local, sy = loc / D.strips_x, sx = loc - sy * D.strips_x;  // 32-bit: a domain has < 2^31 strips
    const int sy_n = (D.ny + ROWS - 1) / ROWS;
    if (sx > 0 && zin[s - 1] == 0) return false;
    if (sx + 1 < D.strips_x && zin[s + 1] == 0) return false;
    if (sy > 0 && zin[s - D.strips_x] == 0) return false;
    if (sy + 1 < sy_n && zin[s + D.strips_x] == 0) return false;
    return true;
}

// Per-domain control of a phase (state buffer, fix / dt / step flags, the step's dt), evaluated
// once per CTA per phase by one thread per domain into shared memory: the strip loops then do
// no FP64 work (this part's FP64 rate is a small fraction of its FP32 rate).
template <class T>
struct DomCtl {
    T dt[MAXD];
    unsigned char flags[MAXD];  // bit 0: state buffer b, bit 1: fix, bit 2: wants dt / runs phase B
};

// Strips of one phase: warp w first takes strip w, then strips nwarps + k for the tickets k it
// draws from *ctr (zeroed after the phase's grid barrier, for its next use two steps later).
// The next ticket is requested before the current strip is processed, so its latency hides
// behind the work.  Warps without a first strip draw none (a batch smaller than the grid costs
// no atomics).
template <class F>
__device__ __forceinline__ void for_strips(unsigned* ctr, long long first, long long nwarps, long long total, int lane, F&& body)
{
    long long s = first;
    unsigned tk = 0;
    if (s < total && lane == 0) tk = atomicAdd(ctr, 1u);
    while (s < total) {
        body(s);
        s = nwarps + (long long)__shfl_sync(0xffffffffu, tk, 0);
        if (s < total && lane == 0) tk = atomicAdd(ctr, 1u);
    }
}

// Point sources of domain d after step n's update (Triton/src/triton_appfis.hpp:352-373 picks
// the hydrograph rows around the step's start time on the host; :1115-1141 adds
// flow * dt / dx^2 to h at each source cell), in the reference's operation order, one thread
// per domain so that sources sharing a cell add in order.  A source cell's strip is marked wet
// for the dry-strip bookkeeping.
template <class T>
__device__ void apply_sources(const Dom<T>& D, const SrcDev& S, Ctl* ctl, int cur, int d, const Params& p, double big)
{
    if (S.n <= 0 || !is_active(ctl, cur, d, p)) return;
    const double dt = step_dt(ctl, cur, d, p, big);
    if (!(dt > 1e-9 * p.time_step)) return;
    const double simtime = ctl->simtime[cur][d];
    int lo = ctl->src_lo[d], hi = S.nt - 1;
    bool found = false;
    for (int r = lo; r < hi; r++)
        if (S.times[r + 1] > simtime) {
            lo = r;
            hi = r + 1;
            found = true;
            break;
        }
    if (!found) lo = hi;
    ctl->src_lo[d] = lo;
    T* h = D.h[(ctl->steps[cur][d] + 1) & 1];  // the state step n wrote
    unsigned char* zwet = p.zc ? p.zc + (size_t)(1 - cur) * p.total_strips : nullptr;
    for (int s = 0; s < S.n; s++) {
        const double fl = S.flows[(size_t)lo * S.n + s];
        double flow = fl;
        if (lo != hi) {
            const double fh = S.flows[(size_t)hi * S.n + s];
            flow = fl + (((fh - fl) * (simtime - S.times[lo])) / (S.times[hi] - S.times[lo]));
        }
        const double hs = (flow * dt) / (p.dx * p.dx);
        const int j = S.cells[s] / (D.nx + 2), i = S.cells[s] - j * (D.nx + 2);
        T* c = h + (size_t)j * D.px + i;
        *c = (T)((double)*c + hs);
        if (zwet) zwet[D.strip0 + (long long)((j - 1) / ROWS) * D.strips_x + (i - 1) / SCOLS] = 0;
    }
}

// CTAs per SM the FP32 kernel's register allocation targets (FP64: 1).
#ifndef FLOOD_F32_MIN_BLOCKS
#define FLOOD_F32_MIN_BLOCKS 3
#endif

// SKIP: dry strips are left out (Params::zc set); a separate instantiation, so the full sweep
// carries none of the bookkeeping.
template <class T, bool SKIP>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? FLOOD_F32_MIN_BLOCKS : 1) flood_persistent(const Dom<T>* __restrict__ gdoms, Ctl* ctl,
                                                                                Params p)
{
    __shared__ Dom<T> doms[MAXD];
    __shared__ DomCtl<T> dc;
    for (int k = threadIdx.x; k < p.ndom; k += blockDim.x) doms[k] = gdoms[k];
    __syncthreads();
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    const int lane = threadIdx.x & 31;
    const double big = (double)K<T>::big();

    for (int n = 0;; n++) {
        const int cur = n & 1;
        // phase A
        if (threadIdx.x < p.ndom) {
            const int d = threadIdx.x;
            const bool fix = ctl->steps[cur][d] != ctl->steps[1 - cur][d];
            const bool want = is_active(ctl, cur, d, p);
            dc.flags[d] = (unsigned char)((ctl->steps[cur][d] & 1) | (fix ? 2 : 0) | (want ? 4 : 0));
        }
        __syncthreads();
        for_strips(&ctl->ticket[cur], warp, nwarps, p.total_strips, lane, [&](long long s) {
            const int d = find_domain(doms, p.ndom, s);
            const int f = dc.flags[d];
            if (SKIP && p.zc[(size_t)cur * p.total_strips + s] >= 1) return;  // dry input: no fix, no dt
            if (f & 6) phase_a<T>(doms[d], ctl, cur, d, s - doms[d].strip0, f & 1, (f & 2) != 0, (f & 4) != 0, p);
        });
        if (!grid_barrier(ctl, p.spin_limit, n == 0 && (int)blockIdx.x == p.stall_cta)) return;
        if (blockIdx.x == 0 && threadIdx.x == 0) ctl->ticket[cur] = 0;  // next used two steps later, past a barrier
        int active = 0;
        if (threadIdx.x < p.ndom) {
            const int d = threadIdx.x;
            active = is_active(ctl, cur, d, p) ? 1 : 0;
            const double dt = active ? step_dt(ctl, cur, d, p, big) : 0.0;
            const bool run = active && dt > 1e-9 * p.time_step;
            dc.dt[d] = (T)dt;
            dc.flags[d] = (unsigned char)((ctl->steps[cur][d] & 1) | (run ? 4 : 0));
        }
        if (!__syncthreads_or(active)) {
            if (blockIdx.x == 0 && threadIdx.x == 0)  // leave the final scalars in both halves
                for (int d = 0; d < p.ndom; d++) {
                    ctl->simtime[1 - cur][d] = ctl->simtime[cur][d];
                    ctl->pid[1 - cur][d] = ctl->pid[cur][d];
                    ctl->steps[1 - cur][d] = ctl->steps[cur][d];
                }
            return;
        }
        // phase B
        for_strips(&ctl->ticketb[cur], warp, nwarps, p.total_strips, lane, [&](long long s) {
            const int d = find_domain(doms, p.ndom, s);
            const int f = dc.flags[d];
            if (SKIP) {
                const unsigned char* zin = p.zc + (size_t)cur * p.total_strips;
                unsigned char* zout = p.zc + (size_t)(1 - cur) * p.total_strips;
                const unsigned char z = zin[s];
                if (!(f & 4) || strip_idle(doms[d], zin, s)) {  // unchanged state
                    if (lane == 0) zout[s] = z;
                    return;
                }
                const bool dry = phase_b<T>(doms[d], s - doms[d].strip0, f & 1, dc.dt[d], p);
                if (lane == 0) zout[s] = dry ? (unsigned char)(z < 2 ? z + 1 : 2) : 0;
            } else if (f & 4) {
                phase_b<T>(doms[d], s - doms[d].strip0, f & 1, dc.dt[d], p);
            }
        });
        if (blockIdx.x == 0 && threadIdx.x == 0) {  // commit the per-domain scalars of step n
            for (int d = 0; d < p.ndom; d++) {
                if (is_active(ctl, cur, d, p)) {
                    const double dt = step_dt(ctl, cur, d, p, big);
                    // a collapsed (below 1e-9 of the step scale) or NaN time step stops the run
                    if (!(dt > 1e-9 * p.time_step)) atomicExch(&ctl->error, 2);
                    const double st = ctl->simtime[cur][d] + dt;
                    int pid = ctl->pid[cur][d];
                    if (st >= p.print_interval * (pid + 1)) pid++;
                    if (p.dtlog) p.dtlog[(size_t)d * p.max_steps + ctl->steps[cur][d]] = dt;
                    ctl->simtime[1 - cur][d] = st;
                    ctl->pid[1 - cur][d] = pid;
                    ctl->steps[1 - cur][d] = ctl->steps[cur][d] + 1;
                } else {
                    ctl->simtime[1 - cur][d] = ctl->simtime[cur][d];
                    ctl->pid[1 - cur][d] = ctl->pid[cur][d];
                    ctl->steps[1 - cur][d] = ctl->steps[cur][d];
                }
                ctl->dtbits[1 - cur][d] = (unsigned long long)__double_as_longlong(big);
            }
        }
        if (!grid_barrier(ctl, p.spin_limit)) return;
        if (blockIdx.x == 0 && threadIdx.x == 0) ctl->ticketb[cur] = 0;  // next used two steps later, past a barrier
        if (p.srcs) {  // the point sources of step n, seen by the next step's wet/dry fix and dt
            if (blockIdx.x == 0 && threadIdx.x < p.ndom)
                apply_sources<T>(doms[threadIdx.x], p.srcs[threadIdx.x], ctl, cur, threadIdx.x, p, big);
            if (!grid_barrier(ctl, p.spin_limit)) return;
        }
    }
}

// ---------------------------------------------------------------- fused step (full sweep)
// One pass per step: each warp updates its strip and the one-cell ring around it (the ring cells
// are updated again, with the same arithmetic, by the strips that own them), so the wet/dry fix
// of its own cells, which reads the updated depth and the bed of their four neighbours, and the
// CFL dt of the next step follow in the same pass; the two-phase kernel's separate read of the
// state for fix and dt (16 of its 48 bytes per cell-step) and one grid barrier per step go away.
// Strips are FCOLS columns: lane l holds column FCOLS*sx + l - 1, lanes 1..30 update their cell,
// lanes 2..29 own it (write it, fix it, take its dt).  The strip's rows and the row above and
// below it are updated; row r-1 is fixed once row r is.  The fields are bit-identical to the
// two-phase kernel's: the same face, update, fix and dt functions of the same values.
constexpr int FCOLS = 28;

// Staged rows (FP32, rows 16-byte aligned): each warp streams its strip's rows of the five
// input arrays (h, qx, qy of the step's state, dem, n2) into its own ring of FS_NS shared-memory
// stages by TMA, FS_TR rows per stage and array as a 36-column box whose origin, the strip's
// first column rounded down to a multiple of 4, is 16-byte aligned.  A stage's slot is refilled
// with the stage FS_NS further on as soon as its last row is read, so FS_NS - 1 stages are in
// flight while the warp computes, and no row is held in registers ahead of its use.  Cells
// outside the padded domain arrive as the boxes' zero fill.
constexpr int FS_TR = 4, FS_NS = 2, FS_BW = 36;
constexpr int FS_ABYTES = (FS_BW * FS_TR * 4 + 127) / 128 * 128;  // one array's box, 128-byte aligned
constexpr int FS_STAGE = 5 * FS_ABYTES;
constexpr int FS_WARPS = 8;  // warps per CTA (256 threads)
constexpr int FS_SMEM = FS_WARPS * FS_NS * FS_STAGE + FS_WARPS * FS_NS * 8;
constexpr unsigned FS_TX = 5u * FS_BW * FS_TR * 4u;  // bytes one stage's five boxes deliver

struct RowRing {
    unsigned char* buf;  // this warp's FS_NS stages
    uint64_t* bar;       // their barriers
    unsigned g;          // stages consumed by this warp so far: slot g % FS_NS, phase (g / FS_NS) & 1
    bool dead;           // a wait gave up: the warp does no further work (the run reports the error)
};

// D is the CTA's shared-memory copy of the domain descriptor, taken by reference: its eight
// array pointers are then read from shared memory where they are used instead of occupying 16
// registers for the whole strip (90.5 against 87.4 G cell-steps/s on the 32-domain batch).
// STAGED: rows come from the warp's TMA ring (`ring`, domain d's maps in p.maps); otherwise
// from global memory, the row after next loaded while a row is computed.  QUIET: rows whose
// neighbourhood is exactly dry take the short path below (the full sweep; with dry strips left
// out the strips that remain are seldom dry and the votes would only cost).
template <class T, bool STAGED = false, bool QUIET = true>
__device__ bool phase_bf(const Dom<T>& D, long long local, int b, T dt, const Params& p, unsigned long long* dt_next,
                         RowRing* ring = nullptr, int d = 0, Ctl* ctl = nullptr)
{
    const int lane = threadIdx.x & 31;
    const int loc = (int)local, sy = loc / D.strips_x, sx = loc - sy * D.strips_x;  // 32-bit: a domain has < 2^31 strips
    const int i = sx * FCOLS + lane - 1;
    const int j0 = 1 + sy * ROWS, j1 = min(j0 + ROWS, D.ny + 1);  // owned rows j0 .. j1-1
    const int nx = D.nx, ny = D.ny, px = D.px;
    const bool col = i >= 0 && i <= nx + 1;                            // a column of the padded domain
    const bool upd = lane >= 1 && lane <= 30 && i >= 1 && i <= nx;     // updates its cell
    const bool own = lane >= 2 && lane <= 29 && i <= nx;               // owns it
    const bool xface = lane <= 30 && i >= 0 && i <= nx;                // face i|i+1
    const T dx = typed<T>(p.dx, p.fdx), hextra = typed<T>(p.hextra, p.fhextra), cn = typed<T>(p.cn, p.fcn);
    const T one = T(1), zero = T(0), E = K<T>::dry(), G = K<T>::g();
    const T* __restrict__ h = D.h[b];
    const T* __restrict__ qx = D.qx[b];
    const T* __restrict__ qy = D.qy[b];
    const T* __restrict__ dem = D.dem;
    const T* __restrict__ n2 = D.n2;
    T* __restrict__ ho_ = D.h[1 - b];
    T* __restrict__ qxo_ = D.qx[1 - b];
    T* __restrict__ qyo_ = D.qy[1 - b];
    const Raw<T> zr = {zero, zero, zero, zero};
    auto raw = [&](int r) -> Raw<T> {  // state of row r (zero outside the padded domain)
        if (!col || r < 0 || r > ny + 1) return zr;
        const size_t c = (size_t)r * px + i;
        return Raw<T>{h[c], qx[c], qy[c], dem[c]};
    };
    const int ra = j0 - 1, rb = j1;  // rows updated (those outside 1..ny keep their state)
    // staged rows: strip rows ra-1 .. rb+1 (x = 0 .. nrow-1) in stages of FS_TR, read in order
    const int x0 = max(sx * FCOLS - 4, 0), off = i - x0;  // box origin column; this lane's column in the box
    const int y0 = ra - 1, nrow = rb - ra + 3, nst = (nrow + FS_TR - 1) / FS_TR;
    bool bad = false;  // staged: a wait gave up (warp-uniform)
    int issued = -1;   // staged: last stage issued
    auto issue = [&](int q) {  // warp-collective: stage q of the strip into its slot
        const unsigned G = ring->g + q, s = G % FS_NS;
        if (lane == 0) gb::tma::arrive_expect(&ring->bar[s], FS_TX + (G == 0 ? p.tx_extra : 0u));
        __syncwarp();
        if (lane < 5) {  // one array per lane: h, qx, qy of buffer b, dem, n2
            const CUtensorMap* mp = p.maps + (size_t)d * 8 + (lane < 3 ? 2 * lane + b : lane + 3);
            gb::tma::load_3d(ring->buf + s * FS_STAGE + lane * FS_ABYTES, mp, x0, y0 + q * FS_TR, 0, &ring->bar[s]);
        }
        issued = q;
    };
    // staged row x of the strip (state, and n2 into n2o); called once per row, in row order
    auto fetch = [&](int x, T& n2o) -> Raw<T> {
        const int q = x / FS_TR, rr = x - q * FS_TR;
        const unsigned G = ring->g + q, s = G % FS_NS;
        if (rr == 0 && !bad) bad = __any_sync(0xffffffffu, !gb::tma::wait(&ring->bar[s], (G / FS_NS) & 1u, p.wait_ns));
        const T* a = reinterpret_cast<const T*>(ring->buf + s * FS_STAGE) + rr * FS_BW + off;
        const int r = y0 + x;
        Raw<T> v = zr;
        if (col && r >= 0 && r <= ny + 1) v = Raw<T>{a[0], a[FS_ABYTES / 4], a[2 * FS_ABYTES / 4], a[3 * FS_ABYTES / 4]};
        n2o = upd && r >= 1 && r <= ny ? a[4 * FS_ABYTES / 4] : zero;
        if (rr == FS_TR - 1) {  // the stage is read: its slot takes stage q + FS_NS
            __syncwarp();
            if (!bad && q + FS_NS < nst) issue(q + FS_NS);
        }
        return v;
    };
    Cell<T> cj;
    Raw<T> rn;
    T n2c = zero;  // staged: n2 of row r
    Cell<T> cm;
    if constexpr (STAGED) {
        if (ring->dead) return false;
        __syncwarp();  // every lane is done with the previous strip's stages before their slots refill
        for (int q = 0; q < FS_NS && q < nst; q++) issue(q);
        T unused;
        cm = cell_of(fetch(0, unused));
        cj = cell_of(fetch(1, n2c));
    } else {
        cj = cell_of(raw(ra));
        rn = raw(ra + 1);
    }
    T ycar[3] = {zero, zero, zero};  // rhs0 Y part of row r (from face r|r-1)
    bool ywet = false;
    if (upd && ra >= 1) {
        if constexpr (!STAGED) cm = cell_of(raw(ra - 1));
        T r2[3];
        ywet = face<T>(cj, cm, zero, one, dx, dt, hextra, ycar, r2);
    }
    T h2 = zero, z2 = zero;                         // row r-2: updated depth, bed
    T h1 = zero, qx1 = zero, qy1 = zero, z1 = zero;  // row r-1: updated state, bed
    T mn = K<T>::big();
    bool dry = true;  // every cell this lane owns ends with h = qx = qy = 0
    // Quiet rows: when the depth of every cell of rows r-1 .. r+1 across the warp is exactly 0
    // (no Y face r|r-1 was wet, and rows r and r+1 are zero), no face of row r has water on
    // either side, so every face returns without a contribution and the update with zero
    // right-hand sides leaves the depth (+0 or -0) and sets both momenta to +0 (hextra > 0):
    // the same bits without the face arithmetic.
    const bool qok = QUIET && hextra > zero;
    bool dcur = QUIET && __all_sync(0xffffffffu, zero_bits(cj.h));
    for (int r = ra; r <= rb; r++) {
        const bool rin = r >= 1 && r <= ny;
        Raw<T> rnn;
        T n2v, n2n = zero;
        if constexpr (STAGED) {
            rn = fetch(r + 1 - y0, n2n);
            n2v = n2c;
        } else {
            rnn = r + 2 <= rb + 1 ? raw(r + 2) : zr;  // prefetch
            n2v = upd && rin ? n2[(size_t)r * px + i] : zero;
        }
        const Cell<T> cn_ = cell_of(rn);
        const bool dnext = QUIET && __all_sync(0xffffffffu, zero_bits(cn_.h));
        const bool quiet = qok && dcur && dnext && !__any_sync(0xffffffffu, ywet);
        dcur = dnext;
        T yn1[3] = {zero, zero, zero};
        bool ynwet = false;
        T hn = cj.h, qxn = cj.qx, qyn = cj.qy;
        if (quiet) {
            if (upd && rin) {
                qxn = zero;
                qyn = zero;
            }
        } else {
            // X face i|i+1 of row r: rhs0 of cell i, rhs1 of cell i+1 (the next lane)
            const Cell<T> right = shfl_cell(cj, 1, true);
            T xr1[3] = {zero, zero, zero}, xr2[3] = {zero, zero, zero};
            bool xwet = false;
            if (xface && rin) xwet = face<T>(cj, right, one, zero, dx, dt, hextra, xr1, xr2);
            T lr[3];
            lr[0] = __shfl_up_sync(0xffffffffu, xr2[0], 1);
            lr[1] = __shfl_up_sync(0xffffffffu, xr2[1], 1);
            lr[2] = __shfl_up_sync(0xffffffffu, xr2[2], 1);
            const bool lwet = __shfl_up_sync(0xffffffffu, (int)xwet, 1) != 0;
            // Y face r+1|r: id1 = row r+1, id2 = row r (row r's rhs1 and row r+1's rhs0)
            T yr2[3] = {zero, zero, zero};
            if (upd && r >= 0 && r <= ny) ynwet = face<T>(cn_, cj, zero, one, dx, dt, hextra, yn1, yr2);
            if (upd && rin) {
                T r0[3], r1[3];
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    r0[k] = xwet ? xr1[k] : zero;
                    if (ywet) r0[k] = r0[k] + ycar[k];
                    r1[k] = lwet ? lr[k] : zero;
                    if (ynwet) r1[k] = r1[k] + yr2[k];
                }
                update<T>(cj.h, cj.qx, cj.qy, n2v, r0, r1, dt, hextra, hn, qxn, qyn);
            }
        }
        // row r-1, one of the strip's own rows: wet/dry fix (triton_appfis.hpp:1095-1112) on the
        // updated state, then its CFL dt (:567-586), then the write; the neighbours' depth and
        // bed are fetched only when some owned cell is wet enough to need them
        if (r - 1 >= j0 && r - 1 < j1) {
            T hL = zero, hR = zero, zL = zero, zR = zero;
            if (!QUIET || __any_sync(0xffffffffu, own && h1 > hextra)) {
                hL = __shfl_up_sync(0xffffffffu, h1, 1);
                hR = __shfl_down_sync(0xffffffffu, h1, 1);
                zL = __shfl_up_sync(0xffffffffu, z1, 1);
                zR = __shfl_down_sync(0xffffffffu, z1, 1);
            }
            if (own) {
                T qxr = qx1, qyr = qy1;
                if (h1 > hextra) {
                    const T lvl = h1 + z1;
                    if (((lvl < zR) && (hR < E)) || ((lvl < zL) && (hL < E))) qxr = zero;
                    if (((lvl < z2) && (h2 < E)) || ((lvl < cj.z) && (hn < E))) qyr = zero;
                    const T dtx = dx / (fabs(qxr / h1) + sqrt(G * h1));
                    const T dty = dx / (fabs(qyr / h1) + sqrt(G * h1));
                    const T v = dtx < dty ? cn * dtx : cn * dty;
                    mn = v < mn ? v : mn;
                }
                const size_t c1 = (size_t)(r - 1) * px + i;
                ho_[c1] = h1;
                qxo_[c1] = qxr;
                qyo_[c1] = qyr;
                dry = dry && h1 == zero && qxr == zero && qyr == zero;
            }
        }
#pragma unroll
        for (int k = 0; k < 3; k++) ycar[k] = yn1[k];
        ywet = ynwet;
        h2 = h1;
        z2 = z1;
        h1 = hn;
        qx1 = qxn;
        qy1 = qyn;
        z1 = cj.z;
        cj = cn_;
        if constexpr (STAGED) {
            n2c = n2n;
        } else {
            rn = rnn;
        }
    }
    if constexpr (STAGED) {
        if (bad) {  // report, and let the copies still in flight land before the warp moves on
            if (lane == 0) {
                atomicExch(&ctl->error, 1);
                for (int q = max(0, issued - FS_NS + 1); q <= issued; q++) {
                    const unsigned G = ring->g + q;
                    gb::tma::wait(&ring->bar[G % FS_NS], (G / FS_NS) & 1u, gb::tma::DRAIN_NS);
                }
            }
            __syncwarp();
            ring->dead = true;
            return false;
        }
        ring->g += nst;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const T other = __shfl_down_sync(0xffffffffu, mn, o);
        mn = other < mn ? other : mn;
    }
    if (lane == 0 && mn < K<T>::big()) atomicMin(dt_next, (unsigned long long)__double_as_longlong((double)mn));
    return __all_sync(0xffffffffu, dry);
}

// The fused persistent kernel (full sweep, no point sources): a dt-only pass over the initial
// state, then one pass and one grid barrier per step.  The per-domain CFL minimum of step n is
// accumulated in dtbits[n % 3] during step n-1, read at the start of step n, and the slot of
// step n+2 is reset by block 0 during step n (nobody reads or writes it then).
// STAGED: the step's rows arrive through each warp's TMA ring (FS_SMEM bytes of dynamic shared
// memory; FP32 domains whose rows are 16-byte aligned).
template <class T, bool SKIP, bool STAGED = false>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? FLOOD_F32_MIN_BLOCKS : 1) flood_fused(const Dom<T>* __restrict__ gdoms, Ctl* ctl,
                                                                                          Params p)
{
    __shared__ Dom<T> doms[MAXD];
    __shared__ DomCtl<T> dc;
    extern __shared__ __align__(128) unsigned char fsm[];
    RowRing ring = {nullptr, nullptr, 0u, false};
    if constexpr (STAGED) {
        const int w = threadIdx.x >> 5;
        ring.buf = fsm + w * (FS_NS * FS_STAGE);
        ring.bar = reinterpret_cast<uint64_t*>(fsm + FS_WARPS * FS_NS * FS_STAGE) + w * FS_NS;
        if (gb::tma::smem_u32(fsm) & 127u) {  // the boxes need 128-byte aligned slots: do no work
            ring.dead = true;
            if (threadIdx.x == 0) atomicExch(&ctl->error, 3);
        } else if ((threadIdx.x & 31) == 0) {
            for (int k = 0; k < FS_NS; k++) gb::tma::bar_init(&ring.bar[k], 1);
            gb::tma::fence_init();
        }
    }
    for (int k = threadIdx.x; k < p.ndom; k += blockDim.x) doms[k] = gdoms[k];
    __syncthreads();
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    const int lane = threadIdx.x & 31;
    const double big = (double)K<T>::big();
    // dt of step 0 from the initial state (no fix before the first step)
    if (threadIdx.x < p.ndom) dc.flags[threadIdx.x] = is_active(ctl, 0, threadIdx.x, p) ? 4 : 0;
    __syncthreads();
    for_strips(&ctl->ticket[0], warp, nwarps, p.total_strips, lane, [&](long long s) {
        const int d = find_domain(doms, p.ndom, s);
        if (dc.flags[d] & 4) phase_a<T, FCOLS, 2>(doms[d], ctl, 0, d, s - doms[d].strip0, ctl->steps[0][d] & 1, false, true, p);
    });
    if (!grid_barrier(ctl, p.spin_limit, (int)blockIdx.x == p.stall_cta)) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->ticket[0] = 0;
    for (int n = 0;; n++) {
        const int cur = n & 1, ds = n % 3;
        int active = 0;
        if (threadIdx.x < p.ndom) {
            const int d = threadIdx.x;
            active = is_active(ctl, cur, d, p) ? 1 : 0;
            const double dt = active ? step_dt_at(ctl, ds, cur, d, p, big) : 0.0;
            const bool run = active && dt > 1e-9 * p.time_step;
            dc.dt[d] = (T)dt;
            dc.flags[d] = (unsigned char)((ctl->steps[cur][d] & 1) | (run ? 4 : 0));
        }
        if (!__syncthreads_or(active)) {
            if (blockIdx.x == 0 && threadIdx.x == 0)  // leave the final scalars in both halves
                for (int d = 0; d < p.ndom; d++) {
                    ctl->simtime[1 - cur][d] = ctl->simtime[cur][d];
                    ctl->pid[1 - cur][d] = ctl->pid[cur][d];
                    ctl->steps[1 - cur][d] = ctl->steps[cur][d];
                }
            return;
        }
        const int dn = (n + 1) % 3;
        for_strips(&ctl->ticketb[cur], warp, nwarps, p.total_strips, lane, [&](long long s) {
            const int d = find_domain(doms, p.ndom, s);
            const int f = dc.flags[d];
            if (SKIP) {  // the two-phase kernel's dry-strip rule (strip_idle), on this kernel's strips
                const unsigned char* zin = p.zc + (size_t)cur * p.total_strips;
                unsigned char* zout = p.zc + (size_t)(1 - cur) * p.total_strips;
                const unsigned char z = zin[s];
                if (!(f & 4) || strip_idle(doms[d], zin, s)) {  // unchanged state, no fix, no dt
                    if (lane == 0) zout[s] = z;
                    return;
                }
                const bool dry = phase_bf<T, STAGED, false>(doms[d], s - doms[d].strip0, f & 1, dc.dt[d], p,
                                                            &ctl->dtbits[dn][d], &ring, d, ctl);
                if (lane == 0) zout[s] = dry ? (unsigned char)(z < 2 ? z + 1 : 2) : 0;
            } else if (f & 4) {
                phase_bf<T, STAGED>(doms[d], s - doms[d].strip0, f & 1, dc.dt[d], p, &ctl->dtbits[dn][d], &ring, d, ctl);
            }
        });
        if (blockIdx.x == 0 && threadIdx.x == 0) {  // commit the per-domain scalars of step n
            for (int d = 0; d < p.ndom; d++) {
                if (is_active(ctl, cur, d, p)) {
                    const double dt = step_dt_at(ctl, ds, cur, d, p, big);
                    if (!(dt > 1e-9 * p.time_step)) atomicExch(&ctl->error, 2);
                    const double st = ctl->simtime[cur][d] + dt;
                    int pid = ctl->pid[cur][d];
                    if (st >= p.print_interval * (pid + 1)) pid++;
                    if (p.dtlog) p.dtlog[(size_t)d * p.max_steps + ctl->steps[cur][d]] = dt;
                    ctl->simtime[1 - cur][d] = st;
                    ctl->pid[1 - cur][d] = pid;
                    ctl->steps[1 - cur][d] = ctl->steps[cur][d] + 1;
                } else {
                    ctl->simtime[1 - cur][d] = ctl->simtime[cur][d];
                    ctl->pid[1 - cur][d] = ctl->pid[cur][d];
                    ctl->steps[1 - cur][d] = ctl->steps[cur][d];
                }
                ctl->dtbits[(n + 2) % 3][d] = (unsigned long long)__double_as_longlong(big);
            }
        }
        if (!grid_barrier(ctl, p.spin_limit)) return;
        if (blockIdx.x == 0 && threadIdx.x == 0) ctl->ticketb[cur] = 0;  // next used two steps later, past a barrier
    }
}

static __global__ void flood_init_ctl(Ctl* ctl, int ndom, double big, double t0)
{
    const int d = threadIdx.x + blockIdx.x * blockDim.x;
    if (d == 0) {
        ctl->bar_count = 0;
        ctl->bar_gen = 0;
        ctl->error = 0;
        ctl->ticket[0] = ctl->ticket[1] = 0;
        ctl->ticketb[0] = ctl->ticketb[1] = 0;
    }
    if (d < ndom) {
        ctl->src_lo[d] = 0;
        ctl->dtbits[2][d] = (unsigned long long)__double_as_longlong(big);
        for (int k = 0; k < 2; k++) {
            ctl->dtbits[k][d] = (unsigned long long)__double_as_longlong(big);
            ctl->simtime[k][d] = t0;
            ctl->pid[k][d] = 0;
            ctl->steps[k][d] = 0;
        }
    }
}

// Deterministic FP64 sum of h over each domain's interior (mass / cell area), one block per domain.
template <class T>
__global__ void flood_mass(const Dom<T>* __restrict__ doms, const Ctl* __restrict__ ctl, int use_steps, double* out)
{
    const Dom<T> D = doms[blockIdx.x];
    const int b = use_steps ? (ctl->steps[0][blockIdx.x] & 1) : 0;
    double s = 0.0;
    for (int j = 1; j <= D.ny; j++)
        for (int i = 1 + threadIdx.x; i <= D.nx; i += blockDim.x) s += (double)D.h[b][(size_t)j * D.px + i];
    __shared__ double sh[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
        out[blockIdx.x] = t;
    }
}

}  // namespace flood
