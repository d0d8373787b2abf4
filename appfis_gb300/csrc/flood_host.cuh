// Host side of the batched flood run: domain table, control block, cooperative launch, and the
// host-buffer job (upload + padding, run, mass, download).  Included once per precision.
#pragma once

#include <cstring>
#include <type_traits>
#include <vector>

#include "flood.cuh"

namespace flood {

// Domain setup from FP64 interiors (the reference reads FP64 DEM / depth files):
// dem ghost ring = 1e6 (dem.SetBoundary(1e6), triton_appfis.hpp:195); n2 = manning^2 everywhere
// (FillData + Square + SetBoundaryCopy, :142-150, :198); h, q ghosts = 0 in both buffers.
template <class T>
__global__ void flood_setup(Dom<T> D, const double* __restrict__ dem, const double* __restrict__ h,
                            const double* __restrict__ qx, const double* __restrict__ qy, double manning)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;  // padded column
    const int j = blockIdx.y;                             // padded row
    if (i >= D.nx + 2) return;
    const size_t c = (size_t)j * D.px + i;
    const bool in = i >= 1 && i <= D.nx && j >= 1 && j <= D.ny;
    const size_t o = in ? (size_t)(j - 1) * D.nx + (i - 1) : 0;
    T* dm = const_cast<T*>(D.dem);
    T* nn = const_cast<T*>(D.n2);
    dm[c] = in ? (T)dem[o] : T(1e6);
    nn[c] = (T)manning * (T)manning;
    const T hv = in ? (T)h[o] : T(0);
    const T qxv = in && qx ? (T)qx[o] : T(0);
    const T qyv = in && qy ? (T)qy[o] : T(0);
    for (int b = 0; b < 2; b++) {
        D.h[b][c] = hv;
        D.qx[b][c] = qxv;
        D.qy[b][c] = qyv;
    }
}

template <class T>
__global__ void flood_extract(Dom<T> D, int b, double* __restrict__ h, double* __restrict__ qx, double* __restrict__ qy)
{
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = 1 + blockIdx.y;
    if (i > D.nx) return;
    const size_t c = (size_t)j * D.px + i, o = (size_t)(j - 1) * D.nx + (i - 1);
    h[o] = (double)D.h[b][c];
    qx[o] = (double)D.qx[b][c];
    qy[o] = (double)D.qy[b][c];
}

static __global__ void flood_results(const Ctl* __restrict__ ctl, int ndom, int* steps, double* simtime, int* status)
{
    const int d = threadIdx.x;
    if (d < ndom) {
        if (steps) steps[d] = ctl->steps[0][d];
        if (simtime) simtime[d] = ctl->simtime[0][d];
    }
    if (d == 0 && status)
        *status = ctl->error == 0   ? APPFIS_GB_OK
                  : ctl->error == 2 ? APPFIS_GB_ENUMERIC
                  : ctl->error == 3 ? APPFIS_GB_ECUDA  // staging buffers misaligned: no step was taken
                                    : APPFIS_GB_ETIMEOUT;
}

// scols: interior columns per strip (SCOLS for the two-phase kernel, FCOLS for the fused one).
template <class T>
int make_table(const appfis_gb_flood_domain* doms, int ndom, std::vector<Dom<T>>& tab, long long& total, int scols = SCOLS)
{
    total = 0;
    tab.resize(ndom);
    for (int d = 0; d < ndom; d++) {
        const appfis_gb_flood_domain& s = doms[d];
        if (s.nx < 1 || s.ny < 1 || s.pitch < s.nx + 2) return gb::fail(APPFIS_GB_EINVAL, "flood: domain %d has bad dims", d);
        for (int b = 0; b < 2; b++)
            if (!s.h[b] || !s.qx[b] || !s.qy[b]) return gb::fail(APPFIS_GB_EINVAL, "flood: domain %d state buffer %d is null", d, b);
        if (!s.dem || !s.n2) return gb::fail(APPFIS_GB_EINVAL, "flood: domain %d dem/n2 is null", d);
        Dom<T>& D = tab[d];
        for (int b = 0; b < 2; b++) {
            D.h[b] = (T*)s.h[b];
            D.qx[b] = (T*)s.qx[b];
            D.qy[b] = (T*)s.qy[b];
        }
        D.dem = (const T*)s.dem;
        D.n2 = (const T*)s.n2;
        D.nx = s.nx;
        D.ny = s.ny;
        D.px = s.pitch;
        D.strips_x = (s.nx + scols - 1) / scols;
        D.strip0 = total;
        total += (long long)D.strips_x * ((s.ny + ROWS - 1) / ROWS);
    }
    return APPFIS_GB_OK;
}

// Initialises one domain's device buffers from FP64 device interiors (nx*ny each).
template <class T>
int setup(const appfis_gb_flood_domain* dom, const double* dem, const double* h, const double* qx, const double* qy,
          double manning, cudaStream_t st)
{
    if (!dom || !dem || !h) return gb::fail(APPFIS_GB_EINVAL, "flood_setup: null argument");
    std::vector<Dom<T>> one;
    long long tot;
    GB_TRY(make_table<T>(dom, 1, one, tot));
    flood_setup<T><<<dim3(gb::ceil_div(dom->nx + 2, 128), dom->ny + 2), 128, 0, st>>>(one[0], dem, h, qx, qy, manning);
    return gb::launched("flood_setup");
}

// Copies the point-source tables of the batch (host arrays) into one device buffer; *out =
// nullptr when no domain has a source.
inline int upload_sources(const appfis_gb_flood_domain* doms, const appfis_gb_flood_sources* srcs, int ndom,
                          const SrcDev** out, cudaStream_t st)
{
    *out = nullptr;
    if (!srcs) return APPFIS_GB_OK;
    size_t cells = 0, rows = 0, vals = 0;
    for (int d = 0; d < ndom; d++) {
        const appfis_gb_flood_sources& S = srcs[d];
        if (S.n < 0 || (S.n > 0 && (S.nt < 1 || !S.cells || !S.times || !S.flows)))
            return gb::fail(APPFIS_GB_EINVAL, "flood: domain %d has a bad source table", d);
        const int px = doms[d].nx + 2;
        for (int k = 0; k < S.n; k++) {
            const int j = S.cells[k] / px, i = S.cells[k] - j * px;
            if (S.cells[k] < 0 || i < 1 || i > doms[d].nx || j < 1 || j > doms[d].ny)
                return gb::fail(APPFIS_GB_EINVAL, "flood: domain %d source %d is not an interior cell", d, k);
        }
        for (int r = 0; r + 1 < S.nt && S.n > 0; r++)
            if (!(S.times[r + 1] > S.times[r])) return gb::fail(APPFIS_GB_EINVAL, "flood: domain %d hydrograph times must increase", d);
        if (S.n > 0) {
            cells += S.n;
            rows += S.nt;
            vals += (size_t)S.nt * S.n;
        }
    }
    if (cells == 0) return APPFIS_GB_OK;
    const size_t head = (sizeof(SrcDev) * MAXD + 255) / 256 * 256;
    const size_t ibytes = (sizeof(int) * cells + 255) / 256 * 256;
    std::vector<char> host(head + ibytes + sizeof(double) * (rows + vals));
    void* dev;
    GB_TRY(gb::workspace(gb::WS_FLOOD_SRC, host.size(), &dev));
    SrcDev* tab = reinterpret_cast<SrcDev*>(host.data());
    int* ci = reinterpret_cast<int*>(host.data() + head);
    double* dv = reinterpret_cast<double*>(host.data() + head + ibytes);
    char* base = reinterpret_cast<char*>(dev);
    size_t oc = 0, od = 0;
    for (int d = 0; d < MAXD; d++) tab[d] = SrcDev{0, 0, nullptr, nullptr, nullptr};
    for (int d = 0; d < ndom; d++) {
        const appfis_gb_flood_sources& S = srcs[d];
        if (S.n <= 0) continue;
        tab[d].n = S.n;
        tab[d].nt = S.nt;
        tab[d].cells = reinterpret_cast<const int*>(base + head) + oc;
        std::memcpy(ci + oc, S.cells, sizeof(int) * S.n);
        oc += S.n;
        tab[d].times = reinterpret_cast<const double*>(base + head + ibytes) + od;
        std::memcpy(dv + od, S.times, sizeof(double) * S.nt);
        od += S.nt;
        tab[d].flows = reinterpret_cast<const double*>(base + head + ibytes) + od;
        std::memcpy(dv + od, S.flows, sizeof(double) * S.nt * S.n);
        od += (size_t)S.nt * S.n;
    }
    GB_CUDA(cudaMemcpyAsync(dev, host.data(), host.size(), cudaMemcpyHostToDevice, st));
    GB_CUDA(cudaStreamSynchronize(st));  // the host table is a local
    *out = reinterpret_cast<const SrcDev*>(dev);
    return APPFIS_GB_OK;
}

// Uploads the table, initialises the control block and launches the persistent kernel.
template <class T>
int run(const appfis_gb_flood_domain* doms, int ndom, const appfis_gb_flood_params* prm, double* dev_dtlog, int* dev_steps,
        double* dev_simtime, int* dev_status, cudaStream_t st, const appfis_gb_flood_sources* srcs = nullptr)
{
    if (!doms || !prm || ndom < 1 || ndom > MAXD) return gb::fail(APPFIS_GB_EINVAL, "flood: 1..%d domains required", MAXD);
    if (!(prm->dx > 0) || !(prm->courant > 0) || !(prm->print_interval > 0) || prm->max_steps < 0)
        return gb::fail(APPFIS_GB_EINVAL, "flood: bad parameters");
    // the fused pass for the full sweep without point sources
    if ((prm->flags & APPFIS_GB_FLOOD_TWO_PHASE) && (prm->flags & APPFIS_GB_FLOOD_FUSED))
        return gb::fail(APPFIS_GB_EINVAL, "flood: TWO_PHASE and FUSED are exclusive");
    bool any_src = false;
    for (int d = 0; srcs && d < ndom; d++) any_src = any_src || srcs[d].n > 0;
    // the fused pass by default in FP32; in FP64 (one CTA per SM at ~200 registers) the two-phase
    // form is faster (full sweep 21.2 against 22.9 s on the 32-domain batch)
    const bool fused = !any_src && !(prm->flags & APPFIS_GB_FLOOD_TWO_PHASE) &&
                       ((prm->flags & APPFIS_GB_FLOOD_FUSED) || std::is_same<T, float>::value);
    std::vector<Dom<T>> tab;
    long long total = 0;
    GB_TRY(make_table<T>(doms, ndom, tab, total, fused ? FCOLS : SCOLS));
    void *wt, *hs;
    GB_TRY(gb::workspace(gb::WS_REDUCE, sizeof(Ctl) + sizeof(Dom<T>) * MAXD + 256, &wt));
    Ctl* ctl = reinterpret_cast<Ctl*>(wt);
    Dom<T>* dtab = reinterpret_cast<Dom<T>*>(reinterpret_cast<char*>(wt) + ((sizeof(Ctl) + 255) / 256) * 256);
    GB_TRY(gb::pinned(1, sizeof(Dom<T>) * ndom, &hs));
    GB_CUDA(cudaStreamSynchronize(st));  // the pinned staging buffer may still feed an earlier copy
    std::memcpy(hs, tab.data(), sizeof(Dom<T>) * ndom);
    GB_CUDA(cudaMemcpyAsync(dtab, hs, sizeof(Dom<T>) * ndom, cudaMemcpyHostToDevice, st));
    const double big = std::is_same<T, float>::value ? 3.402823466e38 : 1.7976931348623157e308;
    flood_init_ctl<<<1, MAXD, 0, st>>>(ctl, ndom, big, prm->t_start);
    GB_TRY(gb::launched("flood_init_ctl"));

    Params p;
    p.dx = prm->dx;
    p.cn = prm->courant;
    p.hextra = prm->hextra;
    p.fdx = (float)prm->dx;
    p.fcn = (float)prm->courant;
    p.fhextra = (float)prm->hextra;
    p.t_end = prm->t_end;
    p.print_interval = prm->print_interval;
    p.time_step = prm->time_step;
    p.max_steps = prm->max_steps > 0 ? prm->max_steps : STEP_CAP;
    p.ndom = ndom;
    p.total_strips = total;
    p.dtlog = prm->max_steps > 0 ? dev_dtlog : nullptr;
    p.zc = nullptr;
    p.spin_limit = SPIN_LIMIT;
    p.stall_cta = -1;
    p.maps = nullptr;
    p.wait_ns = 1000000000ull;
    p.tx_extra = 0;
    GB_TRY(upload_sources(doms, srcs, ndom, &p.srcs, st));
    // the fused FP32 full sweep stages its rows by TMA when every domain's arrays and rows are
    // 16-byte aligned: 112.5 against 97.4 G cell-steps/s on the 32-domain batch.  With dry strips
    // left out it loads them directly (324 against 319: a warp's strips are then scattered, and
    // each one starts its ring from empty); so does UNSTAGED, or any other layout (same fields).
    bool staged = fused && std::is_same<T, float>::value && !(prm->flags & APPFIS_GB_FLOOD_UNSTAGED) &&
                  !(prm->flags & APPFIS_GB_FLOOD_SKIP_DRY);
    for (int d = 0; staged && d < ndom; d++) {
        const Dom<T>& D = tab[d];
        const void* a[8] = {D.h[0], D.h[1], D.qx[0], D.qx[1], D.qy[0], D.qy[1], D.dem, D.n2};
        for (int k = 0; k < 8; k++) staged = staged && gb::aligned16(a[k]);
        staged = staged && (D.px * sizeof(T)) % 16 == 0;
    }
    if (staged) {
        std::vector<CUtensorMap> maps(8 * (size_t)ndom);
        for (int d = 0; d < ndom; d++) {
            const Dom<T>& D = tab[d];
            const void* a[8] = {D.h[0], D.h[1], D.qx[0], D.qx[1], D.qy[0], D.qy[1], D.dem, D.n2};
            for (int k = 0; k < 8; k++)
                GB_TRY(gb::tensor_map_3d(&maps[8 * d + k], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, sizeof(T), a[k], D.nx + 2, D.ny + 2, 1,
                                         D.px, D.ny + 2, FS_BW, FS_TR));
        }
        void* dm;
        GB_TRY(gb::workspace(gb::WS_FLOOD_MAPS, sizeof(CUtensorMap) * maps.size(), &dm));
        GB_CUDA(cudaMemcpyAsync(dm, maps.data(), sizeof(CUtensorMap) * maps.size(), cudaMemcpyHostToDevice, st));
        GB_CUDA(cudaStreamSynchronize(st));  // the host copy is a local
        p.maps = reinterpret_cast<const CUtensorMap*>(dm);
        unsigned long long test_ns = 0;
        if (gb::take_test_stall(gb::TEST_TMA_SHORTFALL, &test_ns)) {  // a test runs the first stage's waits out
            p.wait_ns = test_ns;
            p.tx_extra = 16;
        }
    }
    unsigned long long test_limit = 0;
    if (gb::take_test_stall(gb::TEST_FLOOD_BARRIER, &test_limit)) {  // a test runs a barrier wait out
        p.spin_limit = test_limit;
        p.stall_cta = 0;
    }
    if (prm->flags & APPFIS_GB_FLOOD_SKIP_DRY) {
        void* z;
        GB_TRY(gb::workspace(gb::WS_FLOOD_Z, 2 * (size_t)total, &z));
        GB_CUDA(cudaMemsetAsync(z, 0, 2 * (size_t)total, st));
        p.zc = reinterpret_cast<unsigned char*>(z);
    }

    int dev = 0, per_sm = 0;
    GB_CUDA(cudaGetDevice(&dev));
    auto kern = staged  ? flood_fused<T, false, true>
                : fused ? (p.zc ? flood_fused<T, true> : flood_fused<T, false>)
                        : (p.zc ? flood_persistent<T, true> : flood_persistent<T, false>);
    const int smem = staged ? FS_SMEM : 0;
    if (staged) GB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, smem));
    if (per_sm < 1) return gb::fail(APPFIS_GB_ECUDA, "flood: kernel cannot be resident");
    long long want = (total * 32 + 255) / 256;  // one warp per strip at most
    int grid = (int)std::min<long long>(want, (long long)per_sm * gb::sm_count());
    if (grid < 1) grid = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const Dom<T>* cdt = dtab;
    GB_CUDA(cudaLaunchKernelEx(&cfg, kern, cdt, ctl, p));
    flood_results<<<1, MAXD, 0, st>>>(ctl, ndom, dev_steps, dev_simtime, dev_status);
    return gb::launched("flood_results");
}

template <class T>
int mass(const appfis_gb_flood_domain* doms, int ndom, const int* host_steps, double* dev_mass, cudaStream_t st)
{
    std::vector<Dom<T>> tab;
    long long total = 0;
    GB_TRY(make_table<T>(doms, ndom, tab, total));
    for (int d = 0; d < ndom; d++) {
        const int b = host_steps ? (host_steps[d] & 1) : 0;
        // one block per domain on a one-domain table: pass the chosen buffer as buffer 0
        Dom<T> D = tab[d];
        D.h[0] = D.h[b];
        void* hs;
        GB_TRY(gb::workspace(gb::WS_JOB_E, sizeof(Dom<T>) * MAXD, &hs));
        GB_CUDA(cudaMemcpyAsync(reinterpret_cast<Dom<T>*>(hs) + d, &D, sizeof(D), cudaMemcpyHostToDevice, st));
        GB_CUDA(cudaStreamSynchronize(st));
        flood_mass<T><<<1, 256, 0, st>>>(reinterpret_cast<Dom<T>*>(hs) + d, nullptr, 0, dev_mass + d);
    }
    return gb::launched("flood_mass");
}

// Host-buffer job: interiors in FP64 (like the reference's input files), computed in T.
template <class T>
int job(int ndom, const int* nx, const int* ny, const double* const* dem, double* const* h, double* const* qx,
        double* const* qy, double manning, const appfis_gb_flood_params* prm, int* steps_out, double* mass_out,
        double* dtlog_host)
{
    if (ndom < 1 || ndom > MAXD || !nx || !ny || !dem || !h || !prm) return gb::fail(APPFIS_GB_EINVAL, "flood_job: bad arguments");
    cudaStream_t st;
    GB_TRY(gb::job_stream(&st));
    std::vector<appfis_gb_flood_domain> doms(ndom);
    std::vector<size_t> off(ndom);
    size_t fields_elems = 0, max_int = 0;
    for (int d = 0; d < ndom; d++) {
        if (nx[d] < 1 || ny[d] < 1 || !dem[d] || !h[d]) return gb::fail(APPFIS_GB_EINVAL, "flood_job: domain %d", d);
        const int pitch = ((nx[d] + 2 + 31) / 32) * 32;
        off[d] = fields_elems;
        fields_elems += (size_t)pitch * (ny[d] + 2) * 8;
        max_int = std::max(max_int, (size_t)nx[d] * ny[d]);
        doms[d].nx = nx[d];
        doms[d].ny = ny[d];
        doms[d].pitch = pitch;
    }
    void *pool, *stage, *small;
    GB_TRY(gb::workspace(gb::WS_JOB_A, sizeof(T) * fields_elems, &pool));
    GB_TRY(gb::workspace(gb::WS_JOB_B, sizeof(double) * 4 * max_int, &stage));
    GB_TRY(gb::workspace(gb::WS_JOB_C, 4096 + sizeof(double) * (size_t)ndom * (prm->max_steps > 0 ? prm->max_steps : 1), &small));
    T* base = reinterpret_cast<T*>(pool);
    for (int d = 0; d < ndom; d++) {
        const size_t f = (size_t)doms[d].pitch * (ny[d] + 2);
        T* p = base + off[d];
        doms[d].h[0] = p;
        doms[d].h[1] = p + f;
        doms[d].qx[0] = p + 2 * f;
        doms[d].qx[1] = p + 3 * f;
        doms[d].qy[0] = p + 4 * f;
        doms[d].qy[1] = p + 5 * f;
        doms[d].dem = p + 6 * f;
        doms[d].n2 = p + 7 * f;
        std::vector<Dom<T>> one;
        long long tot;
        GB_TRY(make_table<T>(&doms[d], 1, one, tot));
        const size_t n = (size_t)nx[d] * ny[d];
        double* sd = reinterpret_cast<double*>(stage);
        GB_CUDA(cudaMemcpyAsync(sd, dem[d], sizeof(double) * n, cudaMemcpyHostToDevice, st));
        GB_CUDA(cudaMemcpyAsync(sd + n, h[d], sizeof(double) * n, cudaMemcpyHostToDevice, st));
        const bool hq = qx && qy && qx[d] && qy[d];
        if (hq) {
            GB_CUDA(cudaMemcpyAsync(sd + 2 * n, qx[d], sizeof(double) * n, cudaMemcpyHostToDevice, st));
            GB_CUDA(cudaMemcpyAsync(sd + 3 * n, qy[d], sizeof(double) * n, cudaMemcpyHostToDevice, st));
        }
        flood_setup<T><<<dim3(gb::ceil_div(nx[d] + 2, 128), ny[d] + 2), 128, 0, st>>>(
            one[0], sd, sd + n, hq ? sd + 2 * n : nullptr, hq ? sd + 3 * n : nullptr, manning);
        GB_TRY(gb::launched("flood_setup"));
    }
    int* dsteps = reinterpret_cast<int*>(small);
    int* dstatus = dsteps + MAXD;
    double* dmass = reinterpret_cast<double*>(reinterpret_cast<char*>(small) + 1024);
    double* dlog = reinterpret_cast<double*>(reinterpret_cast<char*>(small) + 4096);
    if (mass_out) GB_TRY(mass<T>(doms.data(), ndom, nullptr, dmass, st));
    std::vector<double> m0(ndom, 0.0);
    if (mass_out) {
        GB_CUDA(cudaMemcpyAsync(m0.data(), dmass, sizeof(double) * ndom, cudaMemcpyDeviceToHost, st));
        GB_CUDA(cudaStreamSynchronize(st));
    }
    GB_TRY(run<T>(doms.data(), ndom, prm, dlog, dsteps, nullptr, dstatus, st));
    std::vector<int> steps(ndom + 1);
    GB_CUDA(cudaMemcpyAsync(steps.data(), dsteps, sizeof(int) * ndom, cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaMemcpyAsync(&steps[ndom], dstatus, sizeof(int), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    if (steps[ndom] != APPFIS_GB_OK)
        return gb::fail(steps[ndom], steps[ndom] == APPFIS_GB_ENUMERIC ? "flood: the time step collapsed (zero or NaN)"
                                     : steps[ndom] == APPFIS_GB_ECUDA  ? "flood: row staging buffers misaligned"
                                                                       : "flood: a device-side wait timed out");
    if (mass_out) {
        GB_TRY(mass<T>(doms.data(), ndom, steps.data(), dmass, st));
        std::vector<double> m1(ndom);
        GB_CUDA(cudaMemcpyAsync(m1.data(), dmass, sizeof(double) * ndom, cudaMemcpyDeviceToHost, st));
        GB_CUDA(cudaStreamSynchronize(st));
        for (int d = 0; d < ndom; d++) {
            mass_out[2 * d] = m0[d];
            mass_out[2 * d + 1] = m1[d];
        }
    }
    for (int d = 0; d < ndom; d++) {
        std::vector<Dom<T>> one;
        long long tot;
        GB_TRY(make_table<T>(&doms[d], 1, one, tot));
        const size_t n = (size_t)nx[d] * ny[d];
        double* sd = reinterpret_cast<double*>(stage);
        flood_extract<T><<<dim3(gb::ceil_div(nx[d], 128), ny[d]), 128, 0, st>>>(one[0], steps[d] & 1, sd, sd + n, sd + 2 * n);
        GB_TRY(gb::launched("flood_extract"));
        GB_CUDA(cudaMemcpyAsync(h[d], sd, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
        if (qx && qx[d]) GB_CUDA(cudaMemcpyAsync(qx[d], sd + n, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
        if (qy && qy[d]) GB_CUDA(cudaMemcpyAsync(qy[d], sd + 2 * n, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
        GB_CUDA(cudaStreamSynchronize(st));  // the staging buffer is reused by the next domain
    }
    if (steps_out)
        for (int d = 0; d < ndom; d++) steps_out[d] = steps[d];
    if (dtlog_host && prm->max_steps > 0) {
        GB_CUDA(cudaMemcpyAsync(dtlog_host, dlog, sizeof(double) * (size_t)ndom * prm->max_steps, cudaMemcpyDeviceToHost, st));
        GB_CUDA(cudaStreamSynchronize(st));
    }
    return APPFIS_GB_OK;
}

}  // namespace flood
