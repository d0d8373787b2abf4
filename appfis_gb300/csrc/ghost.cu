// Periodic ghost-cell refresh of a padded field on the device.
//
// Reference: for one rank with periodic boundaries the halo exchange packs each face, sends it
// to itself through MPI and unpacks it into the opposite ghost layers, axis by axis
// (Appfis/Communication.hpp:612-678, pack/unpack Appfis/Runtime.hpp:916-1173; on GPU builds via
// pinned host buffers every iteration, Appfis/Runtime_CUDA.hpp:743-1198).  Axis a's low ghost
// layer g takes interior layer dim-2G+g and its high ghost layer dim-G+g takes layer G+g, over
// the full extent of the other axes, X first, then Y, then Z, so edges and corners come out as
// in the reference.  Here each axis is one kernel over the ghost slabs, in place.
#include "gb_common.cuh"

namespace {

template <class E>
__global__ void periodic_axis(E* __restrict__ f, int dx, int dy, int dz, int axis, int G)
{
    // slab: 2G layers along `axis` times the full extent of the two other axes
    const int dims[3] = {dx, dy, dz};
    const int a1 = axis == 0 ? 1 : 0, a2 = axis == 2 ? 1 : 2;
    const long long n1 = dims[a1], n2 = dims[a2];
    const long long total = (long long)2 * G * n1 * n2;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x) {
        const int u = (int)(t % n1);
        const long long r = t / n1;
        const int v = (int)(r % n2);
        const int layer = (int)(r / n2);  // 0..2G-1
        const int D = dims[axis];
        int dst, src;
        if (layer < G) {
            dst = layer;
            src = D - 2 * G + layer;
        } else {
            dst = D - G + (layer - G);
            src = G + (layer - G);
        }
        int cd[3], cs[3];
        cd[axis] = dst;
        cs[axis] = src;
        cd[a1] = cs[a1] = u;
        cd[a2] = cs[a2] = v;
        f[((size_t)cd[2] * dy + cd[1]) * dx + cd[0]] = f[((size_t)cs[2] * dy + cs[1]) * dx + cs[0]];
    }
}

template <class E>
int fill(void* field, int ndim, const int* pd, int G, cudaStream_t st)
{
    const int dx = pd[0], dy = ndim > 1 ? pd[1] : 1, dz = ndim > 2 ? pd[2] : 1;
    for (int axis = 0; axis < ndim; axis++) {
        const int dims[3] = {dx, dy, dz};
        const long long other = (long long)dims[axis == 0 ? 1 : 0] * dims[axis == 2 ? 1 : 2];
        const long long total = 2LL * G * other;
        const unsigned grid = (unsigned)std::max<long long>(1, std::min<long long>((total + 255) / 256, 4LL * gb::sm_count()));
        periodic_axis<E><<<grid, 256, 0, st>>>(reinterpret_cast<E*>(field), dx, dy, dz, axis, G);
    }
    return gb::launched("periodic_axis");
}

}  // namespace

extern "C" {

int appfis_gb_ghost_periodic(void* field, int elem_size, int ndim, const int* padded_dims, int ghost, void* stream)
{
    if (!field || !padded_dims || ndim < 1 || ndim > 3 || ghost < 0) return gb::fail(APPFIS_GB_EINVAL, "ghost_periodic: bad arguments");
    if (ghost == 0) return APPFIS_GB_OK;
    for (int a = 0; a < ndim; a++)
        if (padded_dims[a] < 3 * ghost) return gb::fail(APPFIS_GB_EINVAL, "ghost_periodic: axis %d too small for %d ghost layers", a, ghost);
    cudaStream_t st = gb::as_stream(stream);
    switch (elem_size) {
    case 1: return fill<uint8_t>(field, ndim, padded_dims, ghost, st);
    case 2: return fill<uint16_t>(field, ndim, padded_dims, ghost, st);
    case 4: return fill<uint32_t>(field, ndim, padded_dims, ghost, st);
    case 8: return fill<unsigned long long>(field, ndim, padded_dims, ghost, st);
    default: return gb::fail(APPFIS_GB_EINVAL, "ghost_periodic: element size %d", elem_size);
    }
}

}  // extern "C"
