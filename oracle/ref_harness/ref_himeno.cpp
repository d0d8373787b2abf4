// Oracle harness: the reference's Himeno functor (Himeno/src/himeno_appfis.hpp:178-198) run
// through the reference's own APPFIS_CPU runtime, plus the per-sweep gosa = sum(ss^2) that the
// reference does not compute (ss exactly as himeno_appfis.hpp:195, accumulated in FP64 over the
// current p before each sweep).
//
// usage: ref_himeno NX NY NZ ITERS THREADS OMEGA coef.f32 p.f32 out.f32 gosa.f64
//   coef.f32 : 12 padded fields (a0 a1 a2 a3 b0 b1 b2 c0 c1 c2 bnd wrk1), each (NX+2)(NY+2)(NZ+2)
//   p.f32    : NX*NY*NZ interior of p (ghost ring stays 0, as after the reference's Scatter)
//   out.f32  : padded p after ITERS sweeps;  gosa.f64 : ITERS values
// stdout : {"sum": <Execute3DReduce SUM of p>, "seconds": <sweep loop wall time>}
#include "harness_io.hpp"
#include "Himeno/src/himeno_appfis.hpp"

int main(int argc, char** argv)
{
    int nx = harness::arg_int(argc, argv, 1), ny = harness::arg_int(argc, argv, 2), nz = harness::arg_int(argc, argv, 3);
    int iters = harness::arg_int(argc, argv, 4), threads = harness::arg_int(argc, argv, 5);
    float omega = (float)harness::arg_f(argc, argv, 6);
    size_t padded = (size_t)(nx + 2) * (ny + 2) * (nz + 2);
    std::vector<char> coef = harness::read_file(argv[7], 12 * padded * sizeof(float));
    std::vector<char> pin = harness::read_file(argv[8], (size_t)nx * ny * nz * sizeof(float));
    const float* cf = reinterpret_cast<const float*>(coef.data());
    const float* ps = reinterpret_cast<const float*>(pin.data());

    APPFIS::Attribute attribute;
    attribute.threads = threads;
    attribute.ghostLayer = 1;
    attribute.periodic = false;
    APPFIS::Initialize(argc, argv, APPFIS::DIM_3D, APPFIS::DIM_3D, attribute);

    APPFIS::Grid<float> gp(APPFIS::DIM_3D, nx, ny, nz, APPFIS::DUAL);
    std::vector<APPFIS::Grid<float>*> gc;
    for (int c = 0; c < 12; c++) gc.push_back(new APPFIS::Grid<float>(APPFIS::DIM_3D, nx, ny, nz, APPFIS::SINGLE));

    gp.AllocateFullGrid();
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) gp.GetFullGrid()->Set(i, j, k, ps[((size_t)k * ny + j) * nx + i]);
    APPFIS::Scatter(gp.GetFullGrid(), gp.GetSubGrid());
    for (int c = 0; c < 12; c++) gc[c]->GetSubGrid()->SetData(const_cast<float*>(cf + c * padded));

    APPFIS::Config<float> config(gp);
    config.GridsToUpdate(gp);
    APPFIS::InitializeExecution(gp, *gc[0], *gc[1], *gc[2], *gc[3], *gc[4], *gc[5], *gc[6], *gc[7], *gc[8], *gc[9], *gc[10], *gc[11]);

    std::vector<double> gosa(iters, 0.0);
    double secs = 0.0;
    for (int it = 0; it < iters; it++)
    {
        APPFIS::Array<float>* a[12];
        for (int c = 0; c < 12; c++) a[c] = gc[c]->GetSubGrid();
        APPFIS::Array<float>* p = gp.GetSubGrid();
        double g = 0.0;
        for (int k = 1; k <= nz; k++)
            for (int j = 1; j <= ny; j++)
                for (int i = 1; i <= nx; i++)
                {
                    float s0 = a[0]->Get(i, j, k) * p->Get(i + 1, j, k)
                        + a[1]->Get(i, j, k) * p->Get(i, j + 1, k)
                        + a[2]->Get(i, j, k) * p->Get(i, j, k + 1)
                        + a[4]->Get(i, j, k) * (p->Get(i + 1, j + 1, k) - p->Get(i + 1, j - 1, k) - p->Get(i - 1, j + 1, k) + p->Get(i - 1, j - 1, k))
                        + a[5]->Get(i, j, k) * (p->Get(i, j + 1, k + 1) - p->Get(i, j - 1, k + 1) - p->Get(i, j + 1, k - 1) + p->Get(i, j - 1, k - 1))
                        + a[6]->Get(i, j, k) * (p->Get(i + 1, j, k + 1) - p->Get(i - 1, j, k + 1) - p->Get(i + 1, j, k - 1) + p->Get(i - 1, j, k - 1))
                        + a[7]->Get(i, j, k) * p->Get(i - 1, j, k)
                        + a[8]->Get(i, j, k) * p->Get(i, j - 1, k)
                        + a[9]->Get(i, j, k) * p->Get(i, j, k - 1)
                        + a[11]->Get(i, j, k);
                    float ss = (s0 * a[3]->Get(i, j, k) - p->Get(i, j, k)) * a[10]->Get(i, j, k);
                    g += (double)ss * (double)ss;
                }
        gosa[it] = g;
        harness::Clock clock;
        APPFIS::Execute3D(config, omega, a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8], a[9], a[10], a[11],
                          gp.GetSubGrid(), gp.GetSubGridNext());
        secs += clock.seconds();
    }

    float sum = 0;
    APPFIS::Execute3DReduce(config, sum, APPFIS::SUM, gp);
    APPFIS::FinalizeExecution(gp);
    APPFIS::Array<float>* sub = gp.GetSubGrid();
    harness::write_file(argv[9], sub->GetData(), (size_t)sub->GetSize() * sizeof(float));
    harness::write_file(argv[10], gosa.data(), gosa.size() * sizeof(double));
    std::printf("{\"sum\": %.9g, \"seconds\": %.9f}\n", sum, secs);
    APPFIS::Finalize();
    return 0;
}
