// Batched, persistent flood-model time stepping (kernels + host runner), instantiated for float
// (flood_f32.cu) and double (flood_f64.cu, built without FMA contraction).  See flood_core.cuh
// for the per-face / per-cell arithmetic and the reference it follows.
//
// One cooperative launch advances a batch of independent domains of uneven sizes to t_end.
// Work items are strips (32 columns x ROWS rows) of all domains, visited grid-stride by warps.
// Each step is phase A (wet/dry fix of the previous step + CFL dt, min per domain) and phase B
// (fluxes + update into the other state buffer), separated by grid barriers whose spin waits
// are bounded (on timeout the kernel records an error and returns).  Per-domain scalars
// (dt bits, simulated time, print index, step count) are double-buffered by step parity so no
// block ever reads a value another block is writing in the same phase; one thread commits them.
#pragma once

#include "flood_core.cuh"

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

struct Ctl {
    unsigned long long dtbits[2][MAXD];
    double simtime[2][MAXD];
    int pid[2][MAXD];
    int steps[2][MAXD];
    unsigned bar_count;
    unsigned bar_gen;
    int error;
};

struct Params {
    double dx, cn, hextra, t_end, print_interval, time_step;
    int max_steps, ndom;
    long long total_strips;
    double* dtlog;  // [ndom][max_steps] or null
};

constexpr unsigned long long SPIN_LIMIT = 1ull << 25;
constexpr int STEP_CAP = 1000000;  // steps per domain when the caller sets no limit

__device__ __forceinline__ bool grid_barrier(Ctl* ctl)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* vgen = &ctl->bar_gen;
        const unsigned g = *vgen;
        __threadfence();
        if (atomicAdd(&ctl->bar_count, 1u) == gridDim.x - 1) {
            ctl->bar_count = 0;
            __threadfence();
            atomicAdd(&ctl->bar_gen, 1u);
        } else {
            unsigned long long n = 0;
            while (*vgen == g) {
                if (++n > SPIN_LIMIT) {
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

__device__ __forceinline__ double step_dt(const Ctl* ctl, int cur, int d, const Params& p, double big)
{
    double dt = __longlong_as_double((long long)ctl->dtbits[cur][d]);
    if (dt >= big - 1.0) dt = p.time_step;
    const double st = ctl->simtime[cur][d];
    const double next_print = p.print_interval * (ctl->pid[cur][d] + 1);
    if (st + dt > next_print) dt = next_print - st;
    return dt;
}

__device__ __forceinline__ bool is_active(const Ctl* ctl, int cur, int d, const Params& p)
{
    return ctl->simtime[cur][d] < p.t_end && ctl->steps[cur][d] < p.max_steps;
}

// ---------------------------------------------------------------- phase A: fix + dt
template <class T>
__device__ void phase_a(const Dom<T>& D, Ctl* ctl, int cur, int d, long long local, bool fix, bool want_dt, const Params& p)
{
    const int lane = threadIdx.x & 31;
    const int sx = (int)(local % D.strips_x), sy = (int)(local / D.strips_x);
    const int i = 1 + sx * 32 + lane;
    const int j0 = 1 + sy * ROWS, j1 = min(j0 + ROWS, D.ny + 1);
    const int b = ctl->steps[cur][d] & 1;
    const T* h = D.h[b];
    T* qx = D.qx[b];
    T* qy = D.qy[b];
    const T hextra = (T)p.hextra, E = K<T>::dry(), G = K<T>::g();
    const T dx = (T)p.dx, cn = (T)p.cn;
    double mn = (double)K<T>::big();
    if (i <= D.nx) {
        for (int j = j0; j < j1; j++) {
            const size_t c = (size_t)j * D.px + i;
            const T hij = h[c];
            T qxv = qx[c], qyv = qy[c];
            if (fix && hij > hextra) {  // triton_appfis.hpp:1095-1112
                const T zij = D.dem[c];
                const T lvl = hij + zij;
                if (((lvl < D.dem[c + 1]) && (h[c + 1] < E)) || ((lvl < D.dem[c - 1]) && (h[c - 1] < E))) {
                    qxv = T(0);
                    qx[c] = qxv;
                }
                if (((lvl < D.dem[c - D.px]) && (h[c - D.px] < E)) || ((lvl < D.dem[c + D.px]) && (h[c + D.px] < E))) {
                    qyv = T(0);
                    qy[c] = qyv;
                }
            }
            if (want_dt && hij > hextra) {  // triton_appfis.hpp:567-586
                const T dtx = dx / (fabs(qxv / hij) + sqrt(G * hij));
                const T dty = dx / (fabs(qyv / hij) + sqrt(G * hij));
                const T v = dtx < dty ? cn * dtx : cn * dty;
                mn = fmin(mn, (double)v);
            }
        }
    }
    if (want_dt) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mn = fmin(mn, __shfl_down_sync(0xffffffffu, mn, o));
        if (lane == 0 && mn < (double)K<T>::big())
            atomicMin(&ctl->dtbits[cur][d], (unsigned long long)__double_as_longlong(mn));
    }
}

// ---------------------------------------------------------------- phase B: fluxes + update
template <class T>
__device__ __forceinline__ Cell<T> load_cell(const Dom<T>& D, int b, int i, int j)
{
    if (i > D.nx + 1) return make_cell<T>(T(0), T(0), T(0), T(0));
    const size_t c = (size_t)j * D.px + i;
    return make_cell<T>(D.h[b][c], D.qx[b][c], D.qy[b][c], D.dem[c]);
}

template <class T>
__device__ void phase_b(const Dom<T>& D, Ctl* ctl, int cur, int d, long long local, const Params& p)
{
    const int lane = threadIdx.x & 31;
    const int sx = (int)(local % D.strips_x), sy = (int)(local / D.strips_x);
    const int i = 1 + sx * 32 + lane;
    const int j0 = 1 + sy * ROWS, j1 = min(j0 + ROWS, D.ny + 1);
    const bool act = i <= D.nx;
    const int b = ctl->steps[cur][d] & 1;
    const T dt = (T)step_dt(ctl, cur, d, p, (double)K<T>::big());
    const T dx = (T)p.dx, hextra = (T)p.hextra;
    const T one = T(1), zero = T(0);

    Cell<T> cj = load_cell(D, b, i, j0);
    T ycar[3] = {zero, zero, zero};  // rhs0 Y part of row j (from face j|j-1)
    bool ywet = false;
    if (act) {
        const Cell<T> cm = load_cell(D, b, i, j0 - 1);
        T r2[3];
        ywet = face<T>(cj, cm, zero, one, dx, dt, hextra, ycar, r2);
    }
    for (int j = j0; j < j1; j++) {
        const Cell<T> cn_ = load_cell(D, b, i, j + 1);
        // X face i|i+1 of row j
        Cell<T> right = shfl_cell(cj, 1, true);
        if (lane == 31 && act) right = load_cell(D, b, i + 1, j);
        T xr1[3] = {zero, zero, zero}, xr2[3] = {zero, zero, zero};
        bool xwet = false;
        if (act) xwet = face<T>(cj, right, one, zero, dx, dt, hextra, xr1, xr2);
        // rhs1 X part of cell i comes from face i-1|i (left lane, or computed by lane 0)
        T lr[3];
        bool lwet;
        lr[0] = __shfl_up_sync(0xffffffffu, xr2[0], 1);
        lr[1] = __shfl_up_sync(0xffffffffu, xr2[1], 1);
        lr[2] = __shfl_up_sync(0xffffffffu, xr2[2], 1);
        lwet = __shfl_up_sync(0xffffffffu, (int)xwet, 1) != 0;
        if (lane == 0 && act) {
            const Cell<T> left = load_cell(D, b, i - 1, j);
            T t1[3];
            lwet = face<T>(left, cj, one, zero, dx, dt, hextra, t1, lr);
        }
        // Y face j+1|j: id1 = row j+1, id2 = row j
        T yn1[3] = {zero, zero, zero}, yr2[3] = {zero, zero, zero};
        bool ynwet = false;
        if (act) ynwet = face<T>(cn_, cj, zero, one, dx, dt, hextra, yn1, yr2);
        if (act) {
            T r0[3], r1[3];
#pragma unroll
            for (int k = 0; k < 3; k++) {
                r0[k] = xwet ? xr1[k] : zero;
                if (ywet) r0[k] = r0[k] + ycar[k];
                r1[k] = lwet ? lr[k] : zero;
                if (ynwet) r1[k] = r1[k] + yr2[k];
            }
            const size_t c = (size_t)j * D.px + i;
            T ho, qxo, qyo;
            update<T>(cj.h, cj.qx, cj.qy, D.n2[c], r0, r1, dt, hextra, ho, qxo, qyo);
            D.h[1 - b][c] = ho;
            D.qx[1 - b][c] = qxo;
            D.qy[1 - b][c] = qyo;
        }
#pragma unroll
        for (int k = 0; k < 3; k++) ycar[k] = yn1[k];
        ywet = ynwet;
        cj = cn_;
    }
}

template <class T>
__global__ void __launch_bounds__(256) flood_persistent(const Dom<T>* __restrict__ gdoms, Ctl* ctl, Params p)
{
    __shared__ Dom<T> doms[MAXD];
    __shared__ int s_any;
    for (int k = threadIdx.x; k < p.ndom; k += blockDim.x) doms[k] = gdoms[k];
    __syncthreads();
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    const double big = (double)K<T>::big();

    for (int n = 0;; n++) {
        const int cur = n & 1;
        // phase A
        for (long long s = warp; s < p.total_strips; s += nwarps) {
            const int d = find_domain(doms, p.ndom, s);
            const bool fix = ctl->steps[cur][d] != ctl->steps[1 - cur][d];
            const bool want = is_active(ctl, cur, d, p);
            if (fix || want) phase_a<T>(doms[d], ctl, cur, d, s - doms[d].strip0, fix, want, p);
        }
        if (!grid_barrier(ctl)) return;
        if (threadIdx.x == 0) {
            int any = 0;
            for (int d = 0; d < p.ndom; d++) any |= is_active(ctl, cur, d, p) ? 1 : 0;
            s_any = any;
        }
        __syncthreads();
        if (!s_any) {
            if (blockIdx.x == 0 && threadIdx.x == 0)  // leave the final scalars in both halves
                for (int d = 0; d < p.ndom; d++) {
                    ctl->simtime[1 - cur][d] = ctl->simtime[cur][d];
                    ctl->pid[1 - cur][d] = ctl->pid[cur][d];
                    ctl->steps[1 - cur][d] = ctl->steps[cur][d];
                }
            return;
        }
        // phase B
        for (long long s = warp; s < p.total_strips; s += nwarps) {
            const int d = find_domain(doms, p.ndom, s);
            if (is_active(ctl, cur, d, p) && step_dt(ctl, cur, d, p, big) > 1e-9 * p.time_step)
                phase_b<T>(doms[d], ctl, cur, d, s - doms[d].strip0, p);
        }
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
        if (!grid_barrier(ctl)) return;
    }
}

static __global__ void flood_init_ctl(Ctl* ctl, int ndom, double big, double t0)
{
    const int d = threadIdx.x + blockIdx.x * blockDim.x;
    if (d == 0) {
        ctl->bar_count = 0;
        ctl->bar_gen = 0;
        ctl->error = 0;
    }
    if (d < ndom) {
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
