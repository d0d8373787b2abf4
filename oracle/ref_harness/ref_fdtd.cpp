// Oracle harness: the reference's FDTD3d functor (FDTD3d/src/fdtd3d_appfis.hpp:129-143,
// radius-4 star, one uniform coefficient) run through the reference's own APPFIS_CPU runtime
// with a zero ghost halo of width 4 (fdtd3d_appfis.hpp:62).
//
// usage: ref_fdtd NX NY NZ ITERS THREADS COEFF in.f32 out.f32
//   in.f32  : NX*NY*NZ interior;  out.f32 : padded (NX+8)(NY+8)(NZ+8) field after ITERS sweeps
// stdout : {"seconds": <sweep loop wall time>}
#include "harness_io.hpp"
#include "FDTD3d/src/fdtd3d_appfis.hpp"

int main(int argc, char** argv)
{
    int nx = harness::arg_int(argc, argv, 1), ny = harness::arg_int(argc, argv, 2), nz = harness::arg_int(argc, argv, 3);
    int iters = harness::arg_int(argc, argv, 4), threads = harness::arg_int(argc, argv, 5);
    float coeff = (float)harness::arg_f(argc, argv, 6);
    const int radius = 4;
    std::vector<char> in = harness::read_file(argv[7], (size_t)nx * ny * nz * sizeof(float));
    const float* src = reinterpret_cast<const float*>(in.data());

    APPFIS::Attribute attribute;
    attribute.threads = threads;
    attribute.ghostLayer = radius;
    attribute.periodic = false;
    APPFIS::Initialize(argc, argv, APPFIS::DIM_3D, APPFIS::DIM_3D, attribute);

    APPFIS::Grid<float> g(APPFIS::DIM_3D, nx, ny, nz, APPFIS::DUAL);
    g.AllocateFullGrid();
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) g.GetFullGrid()->Set(i, j, k, src[((size_t)k * ny + j) * nx + i]);
    APPFIS::Scatter(g.GetFullGrid(), g.GetSubGrid());
    APPFIS::Config<float> config(g);
    config.GridsToUpdate(g);
    APPFIS::InitializeExecution(g);

    harness::Clock clock;
    for (int it = 0; it < iters; it++) APPFIS::Execute3D(config, coeff, radius, g.GetSubGrid(), g.GetSubGridNext());
    double secs = clock.seconds();

    APPFIS::FinalizeExecution(g);
    APPFIS::Array<float>* sub = g.GetSubGrid();
    harness::write_file(argv[8], sub->GetData(), (size_t)sub->GetSize() * sizeof(float));
    std::printf("{\"seconds\": %.9f}\n", secs);
    APPFIS::Finalize();
    return 0;
}
