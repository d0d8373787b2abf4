// Triton flood model (2-D shallow water, Roe-type augmented solver) — device code shared by the
// FP32 (fast) and FP64 (reference-precision) instantiations.
//
// Reference: Triton/src/triton_appfis.hpp.  One time step of the reference (:320-385) is
//   dt      = cn * min over wet cells of dx / (|q/h| + sqrt(g h))        (:567-586, MIN reduce :325)
//   clamp   to the next print time                                      (:326-334)
//   sqrt(h), zero the six RHS arrays                                    (:589-605)
//   X faces i|i+1 (normal (1,0)), RHS set; Y faces j|j-1 (normal (0,1)), RHS accumulated
//                                                                        (:608-824, :827-1043)
//   h, q -= RHS with semi-implicit Manning friction                     (:1046-1092)
//   wet/dry momentum fix on the updated depth                           (:1095-1112)
// seven kernel launches over five to sixteen arrays, plus a host round trip for dt.
//
// Here a step is two phases over strips of 32 columns x FLOOD_ROWS rows (one warp each):
//   phase A: wet/dry fix of the previous step (in place on q), then the CFL dt of every wet
//            cell, min-reduced per domain in double (atomicMin on the ordered bits);
//   phase B: every face flux computed once (a lane's X face i|i+1 feeds its own rhs0 and, by
//            shuffle, the next lane's rhs1; the Y face j+1|j of a column feeds rhs1 now and
//            rhs0 of the next row in registers), the update + friction, written to the other
//            state buffer.
// The RHS arrays, sqrt(h) array and dt array of the reference never exist in memory.
// The RHS of a cell is accumulated in the reference's order (X part, then + Y part, dry faces
// contributing nothing), so the FP64 instantiation built without FMA contraction follows the
// reference's rounding sequence.  The FP32 instantiation makes two precision adaptations, both
// the same mathematics: a dry-cell depth threshold of 1e-6 m instead of 1e-12 (K<float>::dry)
// and the friction update 2m / (1 + sqrt(1 + 4tt)) in place of -(m - m sqrt(1 + 4tt)) / (2tt),
// which cancels catastrophically in float for small tt.
#pragma once

#include <math.h>

#include "gb_common.cuh"

namespace flood {

constexpr int ROWS = 32;        // rows per strip
constexpr int SCOLS = 30;       // interior columns per strip (a warp's lanes 1..30; lanes 0 and 31 hold the halo)
constexpr int MAXD = 64;        // domains per batch

template <class T> struct K;
template <> struct K<double> {
    static __device__ __forceinline__ double g() { return 9.81; }
    static __device__ __forceinline__ double sqrtg() { return 3.132091953; }
    static __device__ __forceinline__ double eps() { return 1e-12; }
    static __device__ __forceinline__ double big() { return 1.7976931348623157e308; }
    static __device__ __forceinline__ double dry() { return 1e-12; }
};
template <> struct K<float> {
    static __device__ __forceinline__ float g() { return 9.81f; }
    static __device__ __forceinline__ float sqrtg() { return 3.132091953f; }
    static __device__ __forceinline__ float eps() { return 1e-12f; }
    static __device__ __forceinline__ float big() { return 3.402823466e38f; }
    // A depth that is exactly 0 in double keeps a rounding residual of ~1e-8 m in float, so the
    // float form's "dry" test (EPS12 on depths in the reference) uses 1e-6 m.
    static __device__ __forceinline__ float dry() { return 1e-6f; }
};

// Exactly +0 or -0, tested on the bits (a float denormal, which the arithmetic flushes to zero,
// does not count).
template <class T>
__device__ __forceinline__ bool zero_bits(T v)
{
    if constexpr (sizeof(T) == 4)
        return (__float_as_uint(v) << 1) == 0u;
    else
        return ((unsigned long long)__double_as_longlong(v) << 1) == 0ull;
}

// A cell's state as the flux needs it.
template <class T>
struct Cell {
    T h, qx, qy, z, sq;
};

template <class T>
__device__ __forceinline__ Cell<T> make_cell(T h, T qx, T qy, T z)
{
    Cell<T> c;
    c.h = h;
    c.qx = qx;
    c.qy = qy;
    c.z = z;
    c.sq = h > T(0) ? sqrt(h) : T(0);
    return c;
}

template <class T>
__device__ __forceinline__ Cell<T> shfl_cell(const Cell<T>& c, int delta, bool down)
{
    Cell<T> o;
    if (down) {
        o.h = __shfl_down_sync(0xffffffffu, c.h, delta);
        o.qx = __shfl_down_sync(0xffffffffu, c.qx, delta);
        o.qy = __shfl_down_sync(0xffffffffu, c.qy, delta);
        o.z = __shfl_down_sync(0xffffffffu, c.z, delta);
        o.sq = __shfl_down_sync(0xffffffffu, c.sq, delta);
    } else {
        o.h = __shfl_up_sync(0xffffffffu, c.h, delta);
        o.qx = __shfl_up_sync(0xffffffffu, c.qx, delta);
        o.qy = __shfl_up_sync(0xffffffffu, c.qy, delta);
        o.z = __shfl_up_sync(0xffffffffu, c.z, delta);
        o.sq = __shfl_up_sync(0xffffffffu, c.sq, delta);
    }
    return o;
}

// The Roe-type face solver of triton_appfis.hpp:608-824 (X) and :827-1043 (Y): cell 1 = id1,
// cell 2 = id2, normal (nx, ny).  Writes the scaled contributions dt*d/dx to r1 (for id1's rhs0)
// and r2 (for id2's rhs1); returns false when both cells are dry (no contribution).
template <class T>
__device__ __forceinline__ bool face(const Cell<T>& a, const Cell<T>& b, T nx, T ny, T dx, T dt, T hextra, T r1[3],
                                     T r2[3])
{
    const T G = K<T>::g(), SG = K<T>::sqrtg(), E = K<T>::eps(), ED = K<T>::dry();
    const T h1 = a.h, h2 = b.h;
    if (!(h1 > T(0) || h2 > T(0))) return false;
    T u1 = T(0), v1 = T(0), u2 = T(0), v2 = T(0);
    if (h1 >= hextra) {
        u1 = a.qx / h1;
        v1 = a.qy / h1;
    }
    if (h2 >= hextra) {
        u2 = b.qx / h2;
        v2 = b.qy / h2;
    }
    const T sqh1 = a.sq, sqh2 = b.sq;
    const T h12 = T(0.5) * (h1 + h2);
    const T dh = h2 - h1;
    const T c12 = sqrt(G * h12);
    const T u12 = (u1 * sqh1 + u2 * sqh2) / (sqh1 + sqh2);
    const T v12 = (v1 * sqh1 + v2 * sqh2) / (sqh1 + sqh2);
    const T un = u12 * nx + v12 * ny;

    T l0 = un - c12, l1 = un, l2 = un + c12;  // eigenvalues
    T le0 = T(0), le2 = T(0);                 // entropy-fix parts (the middle one is always 0)
    T e1 = u1 * nx + v1 * ny - SG * sqh1;
    T e2 = u2 * nx + v2 * ny - SG * sqh2;
    if (e1 < T(0) && e2 > T(0)) {
        le0 = l0 - e1 * (e2 - l0) / (e2 - e1);
        l0 = e1 * (e2 - l0) / (e2 - e1);
    }
    e1 = u1 * nx + v1 * ny + SG * sqh1;
    e2 = u2 * nx + v2 * ny + SG * sqh2;
    if (e1 < T(0) && e2 > T(0)) {
        le2 = l2 - e2 * (l2 - e1) / (e2 - e1);
        l2 = e2 * (l2 - e1) / (e2 - e1);
    }
    // eigenvectors (rows)
    const T ev01 = u12 - c12 * nx, ev02 = v12 - c12 * ny;
    const T ev11 = -c12 * ny, ev12 = c12 * nx;
    const T ev21 = u12 + c12 * nx, ev22 = v12 + c12 * ny;
    const T dqx = b.qx - a.qx, dqy = b.qy - a.qy;
    const T al0 = T(0.5) * (dh - ((dqx * nx + dqy * ny) - un * dh) / c12);
    const T al1 = ((dqy - v12 * dh) * nx - (dqx - u12 * dh) * ny) / c12;
    const T al2 = T(0.5) * (dh + ((dqx * nx + dqy * ny) - un * dh) / c12);

    // upwinded bed-slope source
    const T z1 = a.z, z2 = b.z;
    const T dz = z2 - z1;
    T dzp = dz, hp;
    if (dz >= T(0)) {
        hp = h1;
        if (z1 + h1 < z2) dzp = h1;
    } else {
        hp = h2;
        if (z2 + h2 < z1) dzp = -h2;
    }
    T be0 = T(0.5) * G * (hp - T(0.5) * fabs(dzp)) * dzp / c12;
    hp = h1 + al0;
    if (l0 * l2 < T(0) && hp > T(0) && h1 > T(0) && h2 > T(0)) {  // subcritical wet-wet correction
        be0 = fmax(be0, al0 * l0 - h1 * dx * T(0.5) / dt);
        be0 = fmin(be0, -al2 * l2 + h2 * dx * T(0.5) / dt);
    }
    const T be2 = -be0;

    T d1[3] = {T(0), T(0), T(0)}, d2[3] = {T(0), T(0), T(0)};
    const T lft = hp - be0 / l0;   // left intermediate state
    const T rgt = hp + be2 / l2;   // right intermediate state
    if (rgt < -ED && h2 < ED) {
        d1[0] += (l0 * al0 - be0) + (l2 * al2 - be2);
    } else if (lft < -ED && h1 < ED) {
        d2[0] += (l0 * al0 - be0) + (l2 * al2 - be2);
    } else {
        const T w0 = l0 * al0 - be0, w1 = l1 * al1 - T(0), w2 = l2 * al2 - be2;
        if (l0 > T(0)) { d2[0] += w0 * T(1); d2[1] += w0 * ev01; d2[2] += w0 * ev02; }
        else { d1[0] += w0 * T(1); d1[1] += w0 * ev01; d1[2] += w0 * ev02; }
        if (l1 > T(0)) { d2[0] += w1 * T(0); d2[1] += w1 * ev11; d2[2] += w1 * ev12; }
        else { d1[0] += w1 * T(0); d1[1] += w1 * ev11; d1[2] += w1 * ev12; }
        if (l2 > T(0)) { d2[0] += w2 * T(1); d2[1] += w2 * ev21; d2[2] += w2 * ev22; }
        else { d1[0] += w2 * T(1); d1[1] += w2 * ev21; d1[2] += w2 * ev22; }
    }
    {  // entropy parts (the middle wave has none: 0 * alpha goes to d1)
        const T w0 = le0 * al0, w1 = T(0) * al1, w2 = le2 * al2;
        if (le0 > T(0)) { d2[0] += w0 * T(1); d2[1] += w0 * ev01; d2[2] += w0 * ev02; }
        else { d1[0] += w0 * T(1); d1[1] += w0 * ev01; d1[2] += w0 * ev02; }
        d1[0] += w1 * T(0); d1[1] += w1 * ev11; d1[2] += w1 * ev12;
        if (le2 > T(0)) { d2[0] += w2 * T(1); d2[1] += w2 * ev21; d2[2] += w2 * ev22; }
        else { d1[0] += w2 * T(1); d1[1] += w2 * ev21; d1[2] += w2 * ev22; }
    }
#pragma unroll
    for (int k = 0; k < 3; k++) {
        if (fabs(d1[k]) < E) d1[k] = T(0);
        if (fabs(d2[k]) < E) d2[k] = T(0);
        r1[k] = dt * d1[k] / dx;
        r2[k] = dt * d2[k] / dx;
    }
    return true;
}

// Update + semi-implicit Manning friction of one interior cell (:1046-1092).
template <class T>
__device__ __forceinline__ void update(T hn, T qx, T qy, T nn, const T r0[3], const T r1[3], T dt, T hextra, T& ho,
                                       T& qxo, T& qyo)
{
    const T G = K<T>::g(), E = K<T>::eps();
    T hij = hn - r0[0] - r1[0];
    if (hij < T(0)) hij = T(0);
    if (hij < hextra) {
        qxo = T(0);
        qyo = T(0);
    } else {
        const T mx = qx - r0[1] - r1[1];
        const T my = qy - r0[2] - r1[2];
        const T modM = sqrt(mx * mx + my * my);
        if (nn > E && hn >= hextra && modM > E) {
            const T tt = dt * G * nn * modM / (hn * hn * cbrt(hn));
            if (sizeof(T) == sizeof(double)) {  // the reference's form
                qxo = T(-0.5) * (mx - mx * sqrt(T(1) + T(4) * tt)) / tt;
                qyo = T(-0.5) * (my - my * sqrt(T(1) + T(4) * tt)) / tt;
            } else {  // float: the same quantity without the cancellation of 1 - sqrt(1 + 4 tt)
                const T den = T(1) + sqrt(T(1) + T(4) * tt);
                qxo = T(2) * mx / den;
                qyo = T(2) * my / den;
            }
        } else {
            qxo = mx;
            qyo = my;
        }
    }
    ho = hij;
}

}  // namespace flood
