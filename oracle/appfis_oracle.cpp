// CPU restatement of the reference's hot-path algorithms — THE ORACLE (test infrastructure only).
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this library, and
// only as the checker or as the timed CPU restatement; the product library never does.
//
// Every function restates one reference routine (msharif42/APPFIS, file:line cited per
// function) in plain C++ on padded, x-fastest arrays with the reference's index order
// (i + dimX*j + dimX*dimY*k, Appfis/Array.hpp:578-589) and the reference's floating-point
// operation order, so that on x86-64 and aarch64 builds with -ffp-contract=off its results
// are bit-identical to the reference's own APPFIS_CPU path run through the single-rank MPI
// stand-in (oracle/_ref).  That identity is checked by tests/test_oracle.py.
//
// Build: g++ -O2 -fopenmp -ffp-contract=off -shared -fPIC (see oracle/build_oracle.py).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

namespace {

inline size_t at2(int i, int j, int px) { return (size_t)j * px + i; }
inline size_t at3(int i, int j, int k, int px, int py) { return ((size_t)k * py + j) * px + i; }

// ---------------------------------------------------------------------------------------------
// Reductions: Appfis/Runtime.hpp:597-913 (Execute{1,2,3}DReduceCPU).  MAX is seeded with
// std::numeric_limits<T>::min() (the smallest POSITIVE value for float/double, :608/:696/:805),
// MIN with max(), SUM with 0; accumulation in T in k, j, i order (one OpenMP thread).
// ---------------------------------------------------------------------------------------------
template <class T>
T reduce_box(const T* a, int px, int py, const int* box, int op)
{
    T acc = op == 0 ? std::numeric_limits<T>::min() : (op == 1 ? std::numeric_limits<T>::max() : T(0));
    for (int k = box[4]; k < box[5]; k++)
        for (int j = box[2]; j < box[3]; j++)
            for (int i = box[0]; i < box[1]; i++)
            {
                T v = a[at3(i, j, k, px, py)];
                if (op == 0) { if (v > acc) acc = v; }
                else if (op == 1) { if (v < acc) acc = v; }
                else acc += v;
            }
    return acc;
}

// ---------------------------------------------------------------------------------------------
// Heat, 2-D restatement of HeatDiffusion/src/heat_appfis.hpp:166-174 (z term dropped):
//   next = c + cx*((l + r) - 2c) + cy*((u + d) - 2c)
// over the interior of a padded (nx+2)x(ny+2) field; the ghost ring holds the Dirichlet values
// in both buffers (Grid::SetBoundary, Appfis/Grid.hpp:529-678) and is never written.
// ---------------------------------------------------------------------------------------------
template <class T>
void heat2d(int nx, int ny, int iters, T cx, T cy, T* a, T* b, int threads)
{
    const int px = nx + 2;
    T* cur = a;
    T* nxt = b;
    for (int it = 0; it < iters; it++)
    {
#pragma omp parallel for num_threads(threads) schedule(static)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++)
            {
                T c = cur[at2(i, j, px)];
                T v = c + cx * (cur[at2(i - 1, j, px)] + cur[at2(i + 1, j, px)] - 2 * c)
                        + cy * (cur[at2(i, j - 1, px)] + cur[at2(i, j + 1, px)] - 2 * c);
                nxt[at2(i, j, px)] = v;
            }
        std::swap(cur, nxt);
    }
    if (cur != a) std::memcpy(a, cur, sizeof(T) * (size_t)px * (ny + 2));
}

// ---------------------------------------------------------------------------------------------
// Himeno 19-point Jacobi: Himeno/src/himeno_appfis.hpp:178-198, same summation order.
// coef = 12 padded fields a0 a1 a2 a3 b0 b1 b2 c0 c1 c2 bnd wrk1.  p, wrk: padded, zero
// ghost ring (the reference's Scatter fills only the interior).  gosa[it] = sum(ss^2) of
// sweep it, accumulated in double (ss exactly as :195).
// ---------------------------------------------------------------------------------------------
template <class T>
void himeno(int nx, int ny, int nz, int iters, T omega, const T* coef, T* p, T* wrk, double* gosa, int threads)
{
    const int px = nx + 2, py = ny + 2;
    const size_t padded = (size_t)px * py * (nz + 2);
    const T *a0 = coef, *a1 = coef + padded, *a2 = coef + 2 * padded, *a3 = coef + 3 * padded;
    const T *b0 = coef + 4 * padded, *b1 = coef + 5 * padded, *b2 = coef + 6 * padded;
    const T *c0 = coef + 7 * padded, *c1 = coef + 8 * padded, *c2 = coef + 9 * padded;
    const T *bnd = coef + 10 * padded, *w1 = coef + 11 * padded;
    T* cur = p;
    T* nxt = wrk;
    std::vector<double> gk(nz + 2);
    for (int it = 0; it < iters; it++)
    {
#pragma omp parallel for num_threads(threads) schedule(static)
        for (int k = 1; k <= nz; k++)
        {
            double g = 0.0;  // per-plane partial, summed in plane order below (thread-count independent)
            for (int j = 1; j <= ny; j++)
                for (int i = 1; i <= nx; i++)
                {
#define P(di, dj, dk) cur[at3(i + (di), j + (dj), k + (dk), px, py)]
                    size_t c = at3(i, j, k, px, py);
                    T s0 = a0[c] * P(1, 0, 0) + a1[c] * P(0, 1, 0) + a2[c] * P(0, 0, 1)
                         + b0[c] * (P(1, 1, 0) - P(1, -1, 0) - P(-1, 1, 0) + P(-1, -1, 0))
                         + b1[c] * (P(0, 1, 1) - P(0, -1, 1) - P(0, 1, -1) + P(0, -1, -1))
                         + b2[c] * (P(1, 0, 1) - P(-1, 0, 1) - P(1, 0, -1) + P(-1, 0, -1))
                         + c0[c] * P(-1, 0, 0) + c1[c] * P(0, -1, 0) + c2[c] * P(0, 0, -1) + w1[c];
                    T ss = (s0 * a3[c] - P(0, 0, 0)) * bnd[c];
                    nxt[c] = P(0, 0, 0) + omega * ss;
                    g += (double)ss * (double)ss;
#undef P
                }
            gk[k] = g;
        }
        double g = 0.0;
        for (int k = 1; k <= nz; k++) g += gk[k];
        if (gosa) gosa[it] = g;
        std::swap(cur, nxt);
    }
    if (cur != p) std::memcpy(p, cur, sizeof(T) * padded);
}

// ---------------------------------------------------------------------------------------------
// Radius-4 star.  Reference form, FDTD3d/src/fdtd3d_appfis.hpp:129-143:
//   val = c; for a in 1..4: val += (x-a + x+a) + (y-a + y+a) + (z-a + z+a); val *= coeff.
// Weighted form (the 8th-order Laplacian update u <- u + nu*L8(u) folded into weights):
//   val = wc*c + sum_a w[a] * ((x-a + x+a) + (y-a + y+a) + (z-a + z+a)).
// Padded fields with a zero ghost halo of width 4.
// ---------------------------------------------------------------------------------------------
template <class T>
void star_r4(int nx, int ny, int nz, int iters, int weighted, T coeff, const T* w, T* a, T* b, int threads)
{
    const int R = 4, px = nx + 2 * R, py = ny + 2 * R;
    const size_t padded = (size_t)px * py * (nz + 2 * R);
    T* cur = a;
    T* nxt = b;
    for (int it = 0; it < iters; it++)
    {
#pragma omp parallel for num_threads(threads) schedule(static)
        for (int k = R; k < nz + R; k++)
            for (int j = R; j < ny + R; j++)
                for (int i = R; i < nx + R; i++)
                {
                    size_t c = at3(i, j, k, px, py);
                    T v;
                    if (!weighted)
                    {
                        v = cur[c];
                        for (int s = 1; s <= R; s++)
                            v += (cur[c - s] + cur[c + s]) + (cur[c - (size_t)s * px] + cur[c + (size_t)s * px])
                               + (cur[c - (size_t)s * px * py] + cur[c + (size_t)s * px * py]);
                        v *= coeff;
                    }
                    else
                    {
                        v = w[0] * cur[c];
                        for (int s = 1; s <= R; s++)
                            v += w[s] * ((cur[c - s] + cur[c + s]) + (cur[c - (size_t)s * px] + cur[c + (size_t)s * px])
                                       + (cur[c - (size_t)s * px * py] + cur[c + (size_t)s * px * py]));
                    }
                    nxt[c] = v;
                }
        std::swap(cur, nxt);
    }
    if (cur != a) std::memcpy(a, cur, sizeof(T) * padded);
}

// ---------------------------------------------------------------------------------------------
// Triton shallow-water step, Triton/src/triton_appfis.hpp.  The X- and Y-direction flux functors
// (:608-824, :827-1043) are one Roe-type face solver with the normal (1,0) resp. (0,1) and the
// "right" cell at i+1 resp. j-1; it is written once here (roe_face) and called for both.
// ---------------------------------------------------------------------------------------------
template <class T>
struct Phys {
    static constexpr T g = T(9.81);          // G      (:53)
    static constexpr T sqrtg = T(3.132091953);  // SQRTG  (:54)
    static constexpr T eps = T(1e-12);       // EPS12  (:55)
    // "this cell is dry" threshold on depths: EPS12 in double; in float a depth that should be
    // exactly 0 keeps a rounding residual of ~1e-8 m, so the float form uses 1e-6 m.
    static constexpr T dry = sizeof(T) == sizeof(double) ? T(1e-12) : T(1e-6);
};

// One face; returns false when both cells are dry (the reference then writes nothing).
template <class T>
bool roe_face(T h1, T h2, T qx1, T qy1, T qx2, T qy2, T z1, T z2, T sqh1, T sqh2, T nx, T ny, T dx, T dt,
              T hextra, T d1[3], T d2[3])
{
    const T G = Phys<T>::g, SG = Phys<T>::sqrtg, E = Phys<T>::eps, ED = Phys<T>::dry;
    if (!(h1 > T(0) || h2 > T(0))) return false;
    T u1 = 0, v1 = 0, u2 = 0, v2 = 0;
    if (h1 >= hextra) { u1 = qx1 / h1; v1 = qy1 / h1; }
    if (h2 >= hextra) { u2 = qx2 / h2; v2 = qy2 / h2; }

    T h12 = T(0.5) * (h1 + h2);
    T dh = h2 - h1;
    T c12 = std::sqrt(G * h12);
    T u12 = (u1 * sqh1 + u2 * sqh2) / (sqh1 + sqh2);
    T v12 = (v1 * sqh1 + v2 * sqh2) / (sqh1 + sqh2);
    T un = u12 * nx + v12 * ny;

    T lam[3] = {un - c12, un, un + c12};  // eigenvalues            (:658-660)
    T lamE[3] = {0, 0, 0};                // entropy-fix parts      (:663-682)
    T e1 = u1 * nx + v1 * ny - SG * sqh1;
    T e2 = u2 * nx + v2 * ny - SG * sqh2;
    if (e1 < T(0) && e2 > T(0))
    {
        lamE[0] = lam[0] - e1 * (e2 - lam[0]) / (e2 - e1);
        lam[0] = e1 * (e2 - lam[0]) / (e2 - e1);
    }
    e1 = u1 * nx + v1 * ny + SG * sqh1;
    e2 = u2 * nx + v2 * ny + SG * sqh2;
    if (e1 < T(0) && e2 > T(0))
    {
        lamE[2] = lam[2] - e2 * (lam[2] - e1) / (e2 - e1);
        lam[2] = e2 * (lam[2] - e1) / (e2 - e1);
    }

    T ev[3][3] = {{T(1), u12 - c12 * nx, v12 - c12 * ny},   // eigenvectors (:684-692)
                  {T(0), -c12 * ny, c12 * nx},
                  {T(1), u12 + c12 * nx, v12 + c12 * ny}};
    T al[3];                                                 // wave strengths (:694-696)
    al[0] = T(0.5) * (dh - (((qx2 - qx1) * nx + (qy2 - qy1) * ny) - un * dh) / c12);
    al[1] = (((qy2 - qy1) - v12 * dh) * nx - ((qx2 - qx1) - u12 * dh) * ny) / c12;
    al[2] = T(0.5) * (dh + (((qx2 - qx1) * nx + (qy2 - qy1) * ny) - un * dh) / c12);

    // upwinded bed-slope source (:698-721)
    T dz = z2 - z1, l1 = z1 + h1, l2 = z2 + h2, dzp = dz, hp;
    if (dz >= T(0)) { hp = h1; if (l1 < z2) dzp = h1; }
    else { hp = h2; if (l2 < z1) dzp = -h2; }
    T be[3];
    be[0] = T(0.5) * G * (hp - T(0.5) * std::fabs(dzp)) * dzp / c12;

    // wet-wet correction (:724-730)
    hp = h1 + al[0];
    if (lam[0] * lam[2] < T(0) && hp > T(0) && h1 > T(0) && h2 > T(0))
    {
        be[0] = std::fmax(be[0], al[0] * lam[0] - h1 * dx * T(0.5) / dt);
        be[0] = std::fmin(be[0], -al[2] * lam[2] + h2 * dx * T(0.5) / dt);
    }
    be[1] = 0;
    be[2] = -be[0];

    for (int i = 0; i < 3; i++) d1[i] = d2[i] = 0;
    l1 = hp - be[0] / lam[0];
    l2 = hp + be[2] / lam[2];
    if (l2 < -ED && h2 < ED)
        d1[0] += (lam[0] * al[0] - be[0]) + (lam[2] * al[2] - be[2]);
    else if (l1 < -ED && h1 < ED)
        d2[0] += (lam[0] * al[0] - be[0]) + (lam[2] * al[2] - be[2]);
    else
        for (int i = 0; i < 3; i++)
        {
            T w = lam[i] * al[i] - be[i];
            T* d = lam[i] > T(0) ? d2 : d1;
            d[0] += w * ev[i][0];
            d[1] += w * ev[i][1];
            d[2] += w * ev[i][2];
        }
    for (int i = 0; i < 3; i++)
    {
        T w = lamE[i] * al[i];
        T* d = lamE[i] > T(0) ? d2 : d1;
        d[0] += w * ev[i][0];
        d[1] += w * ev[i][1];
        d[2] += w * ev[i][2];
    }
    for (int i = 0; i < 3; i++)
    {
        if (std::fabs(d1[i]) < E) d1[i] = 0;
        if (std::fabs(d2[i]) < E) d2[i] = 0;
    }
    return true;
}

template <class T>
struct TritonState {
    int nx, ny, px;
    std::vector<T> dem, n2, h, qx, qy, sq, r[6], dtv;
    T* R(int f) { return r[f].data(); }
};

enum { RH0, RH1, RQX0, RQX1, RQY0, RQY1 };

// One step of the reference time loop (:320-385) without sources; returns the dt used.
template <class T>
double triton_step(TritonState<T>& s, T dx, T cn, T hextra, double time_step, double print_interval, int& print_id,
                   double& simtime, int threads)
{
    const int nx = s.nx, ny = s.ny, px = s.px;
    const T G = Phys<T>::g, E = Phys<T>::eps;
    T* h = s.h.data();
    T* qx = s.qx.data();
    T* qy = s.qy.data();
    const T* dem = s.dem.data();

    // 1. CFL dt per interior cell (:567-586) and its MIN (Execute2DReduce, :325)
    T gdt = std::numeric_limits<T>::max();
    for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++)
        {
            size_t c = at2(i, j, px);
            T out = std::numeric_limits<T>::max();
            T hij = h[c];
            if (hij > hextra)
            {
                T dtx = dx / (std::fabs(qx[c] / hij) + std::sqrt(G * hij));
                T dty = dx / (std::fabs(qy[c] / hij) + std::sqrt(G * hij));
                out = dtx < dty ? cn * dtx : cn * dty;
            }
            if (out < gdt) gdt = out;
        }
    double dt = (double)gdt;
    if (dt >= (double)std::numeric_limits<T>::max() - 1.0) dt = time_step;          // :326-329
    if (simtime + dt > print_interval * (print_id + 1)) dt = print_interval * (print_id + 1) - simtime;  // :331-334
    const T tdt = (T)dt;

    // 2. sqrt(h) and RHS reset over the whole padded field (:589-605)
    const size_t padded = (size_t)px * (ny + 2);
    for (size_t c = 0; c < padded; c++)
    {
        s.sq[c] = h[c] > T(0) ? std::sqrt(h[c]) : T(0);
        for (int f = 0; f < 6; f++) s.r[f][c] = 0;
    }
    // 3. X faces i|i+1, i in [0, nx], j in [1, ny] (Config(dem,0,1,1,1)); RHS set
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int j = 1; j <= ny; j++)
        for (int i = 0; i <= nx; i++)
        {
            size_t a = at2(i, j, px), b = a + 1;
            T d1[3], d2[3];
            if (roe_face<T>(h[a], h[b], qx[a], qy[a], qx[b], qy[b], dem[a], dem[b], s.sq[a], s.sq[b], T(1), T(0), dx, tdt,
                            hextra, d1, d2))
            {
                s.r[RH0][a] = tdt * d1[0] / dx;
                s.r[RQX0][a] = tdt * d1[1] / dx;
                s.r[RQY0][a] = tdt * d1[2] / dx;
                s.r[RH1][b] = tdt * d2[0] / dx;
                s.r[RQX1][b] = tdt * d2[1] / dx;
                s.r[RQY1][b] = tdt * d2[2] / dx;
            }
        }
    // 4. Y faces j|j-1, i in [1, nx], j in [1, ny+1] (Config(dem,1,1,1,0)); RHS accumulated
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int i = 1; i <= nx; i++)
        for (int j = 1; j <= ny + 1; j++)
        {
            size_t a = at2(i, j, px), b = at2(i, j - 1, px);
            T d1[3], d2[3];
            if (roe_face<T>(h[a], h[b], qx[a], qy[a], qx[b], qy[b], dem[a], dem[b], s.sq[a], s.sq[b], T(0), T(1), dx, tdt,
                            hextra, d1, d2))
            {
                s.r[RH0][a] = s.r[RH0][a] + tdt * d1[0] / dx;
                s.r[RQX0][a] = s.r[RQX0][a] + tdt * d1[1] / dx;
                s.r[RQY0][a] = s.r[RQY0][a] + tdt * d1[2] / dx;
                s.r[RH1][b] = s.r[RH1][b] + tdt * d2[0] / dx;
                s.r[RQX1][b] = s.r[RQX1][b] + tdt * d2[1] / dx;
                s.r[RQY1][b] = s.r[RQY1][b] + tdt * d2[2] / dx;
            }
        }
    // 5. update + semi-implicit Manning friction (:1046-1092)
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++)
        {
            size_t c = at2(i, j, px);
            T hn = h[c];
            T hij = hn - s.r[RH0][c] - s.r[RH1][c];
            if (hij < T(0)) hij = 0;
            T qxij, qyij;
            if (hij < hextra) { qxij = 0; qyij = 0; }
            else
            {
                T mx = qx[c] - s.r[RQX0][c] - s.r[RQX1][c];
                T my = qy[c] - s.r[RQY0][c] - s.r[RQY1][c];
                T modM = std::sqrt(mx * mx + my * my);
                T nn = s.n2[c];
                if (nn > E && hn >= hextra && modM > E)
                {
                    T tt = tdt * G * nn * modM / (hn * hn * std::cbrt(hn));
                    if (sizeof(T) == sizeof(double)) {  // the reference's form
                        qxij = T(-0.5) * (mx - mx * std::sqrt(T(1) + T(4) * tt)) / tt;
                        qyij = T(-0.5) * (my - my * std::sqrt(T(1) + T(4) * tt)) / tt;
                    } else {  // FP32: the same quantity without the cancellation of 1 - sqrt(1 + 4 tt)
                        const T den = T(1) + std::sqrt(T(1) + T(4) * tt);
                        qxij = T(2) * mx / den;
                        qyij = T(2) * my / den;
                    }
                }
                else { qxij = mx; qyij = my; }
            }
            h[c] = hij;
            qx[c] = qxij;
            qy[c] = qyij;
        }
    // 6. wet/dry momentum fix on the updated depth (:1095-1112)
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++)
        {
            size_t c = at2(i, j, px);
            T hij = h[c], zij = dem[c];
            const T ED = Phys<T>::dry;
            if (hij > hextra)
            {
                if (((hij + zij < dem[c + 1]) && (h[c + 1] < ED)) || ((hij + zij < dem[c - 1]) && (h[c - 1] < ED))) qx[c] = 0;
                if (((hij + zij < dem[c - px]) && (h[c - px] < ED)) || ((hij + zij < dem[c + px]) && (h[c + px] < ED))) qy[c] = 0;
            }
        }
    simtime += dt;
    if (simtime >= print_interval * (print_id + 1)) print_id++;
    return dt;
}

template <class T>
int triton_run(int nx, int ny, double dx, double cn, double hextra, double mann, double t_end, double print_interval,
               double time_step, int max_steps, const double* dem, double* h, double* qx, double* qy, double* dts,
               double* simtime_out, int threads)
{
    TritonState<T> s;
    s.nx = nx;
    s.ny = ny;
    s.px = nx + 2;
    const size_t padded = (size_t)s.px * (ny + 2);
    s.dem.assign(padded, T(1e6));  // dem.SetBoundary(1e6) (:195)
    s.n2.assign(padded, (T)mann * (T)mann);  // nin Fill + Square + SetBoundaryCopy (:142-150, :198)
    s.h.assign(padded, T(0));
    s.qx.assign(padded, T(0));
    s.qy.assign(padded, T(0));
    s.sq.assign(padded, T(0));
    for (int f = 0; f < 6; f++) s.r[f].assign(padded, T(0));
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++)
        {
            size_t c = at2(i + 1, j + 1, s.px), o = (size_t)j * nx + i;
            s.dem[c] = (T)dem[o];
            s.h[c] = (T)h[o];
            s.qx[c] = (T)qx[o];
            s.qy[c] = (T)qy[o];
        }
    double simtime = 0.0;
    int print_id = 0, steps = 0;
    while (simtime < t_end && (max_steps <= 0 || steps < max_steps))
    {
        double dt = triton_step<T>(s, (T)dx, (T)cn, (T)hextra, time_step, print_interval, print_id, simtime, threads);
        if (dts) dts[steps] = dt;
        steps++;
    }
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++)
        {
            size_t c = at2(i + 1, j + 1, s.px), o = (size_t)j * nx + i;
            h[o] = (double)s.h[c];
            qx[o] = (double)s.qx[c];
            qy[o] = (double)s.qy[c];
        }
    if (simtime_out) *simtime_out = simtime;
    return steps;
}

}  // namespace

extern "C" {

// GameOfLife: GameOfLife/src/game_appfis.hpp:121-135 (S234 with the stale carry: `next` is
// written only when the state changes, so it keeps the state of two generations back) on a
// periodic grid (ghosts refreshed by the self-exchange, Appfis/Communication.hpp:612-678).
// cur: state at t on entry (interior nx*ny, 0/1); old: state at t-1 (zeros at t=0, since
// Array::AllocateMemory zero-fills, Appfis/Array.hpp:339-342).  On return cur holds the state
// after `gens` sweeps and old the one before it.
void oracle_gol(int nx, int ny, int gens, uint8_t* cur, uint8_t* old, int threads)
{
    uint8_t* c = cur;
    uint8_t* o = old;
    for (int g = 0; g < gens; g++)
    {
#pragma omp parallel for num_threads(threads) schedule(static)
        for (int j = 0; j < ny; j++)
        {
            int jm = j == 0 ? ny - 1 : j - 1, jp = j == ny - 1 ? 0 : j + 1;
            for (int i = 0; i < nx; i++)
            {
                int im = i == 0 ? nx - 1 : i - 1, ip = i == nx - 1 ? 0 : i + 1;
                int cnt = c[at2(im, jm, nx)] + c[at2(i, jm, nx)] + c[at2(ip, jm, nx)] + c[at2(im, j, nx)] + c[at2(ip, j, nx)]
                        + c[at2(im, jp, nx)] + c[at2(i, jp, nx)] + c[at2(ip, jp, nx)];
                if (c[at2(i, j, nx)] == 1) { if (cnt < 2 || cnt > 4) o[at2(i, j, nx)] = 0; }
                else { if (cnt == 3) o[at2(i, j, nx)] = 1; }
            }
        }
        std::swap(c, o);
    }
    if (c != cur)  // odd number of sweeps: the latest state sits in `old`
    {
        std::vector<uint8_t> t(cur, cur + (size_t)nx * ny);
        std::memcpy(cur, old, (size_t)nx * ny);
        std::memcpy(old, t.data(), (size_t)nx * ny);
    }
}

// Classic Conway B3/S23 on the same periodic grid (the rule the workload description names);
// NOT the reference's rule — provided so the B3/S23 kernel variant has its own checker.
void oracle_gol_b3s23(int nx, int ny, int gens, uint8_t* cur, int threads)
{
    std::vector<uint8_t> nxt((size_t)nx * ny);
    for (int g = 0; g < gens; g++)
    {
#pragma omp parallel for num_threads(threads) schedule(static)
        for (int j = 0; j < ny; j++)
        {
            int jm = j == 0 ? ny - 1 : j - 1, jp = j == ny - 1 ? 0 : j + 1;
            for (int i = 0; i < nx; i++)
            {
                int im = i == 0 ? nx - 1 : i - 1, ip = i == nx - 1 ? 0 : i + 1;
                int cnt = cur[at2(im, jm, nx)] + cur[at2(i, jm, nx)] + cur[at2(ip, jm, nx)] + cur[at2(im, j, nx)]
                        + cur[at2(ip, j, nx)] + cur[at2(im, jp, nx)] + cur[at2(i, jp, nx)] + cur[at2(ip, jp, nx)];
                nxt[at2(i, j, nx)] = (uint8_t)(cnt == 3 || (cnt == 2 && cur[at2(i, j, nx)]));
            }
        }
        std::memcpy(cur, nxt.data(), nxt.size());
    }
}

int64_t oracle_population(const uint8_t* cells, int64_t n)
{
    int64_t s = 0;
    for (int64_t i = 0; i < n; i++) s += cells[i];
    return s;
}

void oracle_heat2d_f32(int nx, int ny, int iters, float cx, float cy, float* a, float* b, int threads)
{
    heat2d<float>(nx, ny, iters, cx, cy, a, b, threads);
}
void oracle_heat2d_f64(int nx, int ny, int iters, double cx, double cy, double* a, double* b, int threads)
{
    heat2d<double>(nx, ny, iters, cx, cy, a, b, threads);
}

// box = {x0, x1, y0, y1, z0, z1} half-open, on a padded field of px*py*pz; op 0=MAX 1=MIN 2=SUM
double oracle_reduce_f32(const float* a, int px, int py, const int* box, int op) { return reduce_box<float>(a, px, py, box, op); }
double oracle_reduce_f64(const double* a, int px, int py, const int* box, int op) { return reduce_box<double>(a, px, py, box, op); }
int64_t oracle_reduce_i32(const int32_t* a, int px, int py, const int* box, int op) { return reduce_box<int32_t>(a, px, py, box, op); }

void oracle_himeno_f32(int nx, int ny, int nz, int iters, float omega, const float* coef, float* p, float* wrk, double* gosa, int threads)
{
    himeno<float>(nx, ny, nz, iters, omega, coef, p, wrk, gosa, threads);
}
void oracle_himeno_f64(int nx, int ny, int nz, int iters, double omega, const double* coef, double* p, double* wrk, double* gosa, int threads)
{
    himeno<double>(nx, ny, nz, iters, omega, coef, p, wrk, gosa, threads);
}

void oracle_star_r4_f32(int nx, int ny, int nz, int iters, int weighted, float coeff, const float* w, float* a, float* b, int threads)
{
    star_r4<float>(nx, ny, nz, iters, weighted, coeff, w, a, b, threads);
}
void oracle_star_r4_f64(int nx, int ny, int nz, int iters, int weighted, double coeff, const double* w, double* a, double* b, int threads)
{
    star_r4<double>(nx, ny, nz, iters, weighted, coeff, w, a, b, threads);
}

// Triton time loop without sources; dem/h/qx/qy are nx*ny interiors (FP64 in, FP64 out),
// `prec` 64 = computed in double (the reference), 32 = computed in float.
int oracle_triton(int prec, int nx, int ny, double dx, double cn, double hextra, double mann, double t_end,
                  double print_interval, double time_step, int max_steps, const double* dem, double* h, double* qx,
                  double* qy, double* dts, double* simtime, int threads)
{
    if (prec == 32)
        return triton_run<float>(nx, ny, dx, cn, hextra, mann, t_end, print_interval, time_step, max_steps, dem, h, qx, qy,
                                 dts, simtime, threads);
    return triton_run<double>(nx, ny, dx, cn, hextra, mann, t_end, print_interval, time_step, max_steps, dem, h, qx, qy, dts,
                              simtime, threads);
}

}  // extern "C"
