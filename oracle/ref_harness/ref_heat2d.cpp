// Oracle harness: 2-D FP32 heat sweep in the reference's functor form, run through the
// reference's own APPFIS_CPU runtime (Grid, SetBoundary, Config, Execute2D, Execute2DReduce).
//
// The reference app is 3-D FP64 (HeatDiffusion/src/heat_appfis.hpp:166-174); the 2-D FP32
// workload restates that functor with the z term dropped:  c + cx(l+r-2c) + cy(u+d-2c).
//
// usage: ref_heat2d NX NY ITERS THREADS R TOP in.f32 out.f32
//   in.f32 : NX*NY interior values (x fastest)
//   TOP    : Dirichlet value of the UP face (the j=0 ghost row); all other faces 0
//   out.f32: (NX+2)*(NY+2) padded field after ITERS sweeps (ghost ring included)
// stdout : {"max": .., "min": .., "sum": .., "seconds": ..}
#include "harness_io.hpp"
#include "Appfis/Appfis.hpp"

namespace APPFIS
{
    PARALLEL void STENCIL(const int i, const int j, float cx, float cy, APPFIS::Array<float>* cur, APPFIS::Array<float>* next)
    {
        float val = cur->Get(i, j)
            + cx * (cur->Get(i - 1, j) + cur->Get(i + 1, j) - 2 * cur->Get(i, j))
            + cy * (cur->Get(i, j - 1) + cur->Get(i, j + 1) - 2 * cur->Get(i, j));
        next->Set(i, j, val);
    }
}

int main(int argc, char** argv)
{
    int nx = harness::arg_int(argc, argv, 1);
    int ny = harness::arg_int(argc, argv, 2);
    int iters = harness::arg_int(argc, argv, 3);
    int threads = harness::arg_int(argc, argv, 4);
    float r = (float)harness::arg_f(argc, argv, 5);
    float top = (float)harness::arg_f(argc, argv, 6);
    std::vector<char> in = harness::read_file(argv[7], (size_t)nx * ny * sizeof(float));
    const float* src = reinterpret_cast<const float*>(in.data());

    APPFIS::Attribute attribute;
    attribute.threads = threads;
    attribute.ghostLayer = 1;
    attribute.periodic = false;
    APPFIS::Initialize(argc, argv, APPFIS::DIM_2D, APPFIS::DIM_2D, attribute);

    APPFIS::Grid<float> g(APPFIS::DIM_2D, nx, ny, APPFIS::DUAL);
    g.AllocateFullGrid();
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) g.GetFullGrid()->Set(i, j, src[(size_t)j * nx + i]);
    APPFIS::Scatter(g.GetFullGrid(), g.GetSubGrid());
    g.SetBoundary(0.0f);
    g.SetBoundary(APPFIS::UP, top);
    APPFIS::Config<float> config(g);
    config.GridsToUpdate(g);
    APPFIS::InitializeExecution(g);

    harness::Clock clock;
    for (int it = 0; it < iters; it++) APPFIS::Execute2D(config, r, r, g.GetSubGrid(), g.GetSubGridNext());
    double secs = clock.seconds();

    float mx = 0, mn = 0, sm = 0;
    APPFIS::Execute2DReduce(config, mx, APPFIS::MAX, g);
    APPFIS::Execute2DReduce(config, mn, APPFIS::MIN, g);
    APPFIS::Execute2DReduce(config, sm, APPFIS::SUM, g);
    APPFIS::FinalizeExecution(g);

    APPFIS::Array<float>* sub = g.GetSubGrid();
    harness::write_file(argv[8], sub->GetData(), (size_t)sub->GetSize() * sizeof(float));
    std::printf("{\"max\": %.9g, \"min\": %.9g, \"sum\": %.9g, \"seconds\": %.9f}\n", mx, mn, sm, secs);
    APPFIS::Finalize();
    return 0;
}
