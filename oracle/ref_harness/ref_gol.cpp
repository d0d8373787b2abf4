// Oracle harness: the reference's GameOfLife functor (GameOfLife/src/game_appfis.hpp:121-135)
// run through the reference's own APPFIS_CPU runtime on a seeded interior.
//
// usage: ref_gol NX NY GENERATIONS THREADS in.u8 out.u8
//   in.u8  : NX*NY cells (0/1, x fastest), the interior of the periodic grid
//   out.u8 : the interior after GENERATIONS sweeps
// stdout : {"live": <Execute2DReduce SUM>, "seconds": <sweep loop wall time>}
#include "harness_io.hpp"
#include "GameOfLife/src/game_appfis.hpp"

int main(int argc, char** argv)
{
    int nx = harness::arg_int(argc, argv, 1);
    int ny = harness::arg_int(argc, argv, 2);
    int gens = harness::arg_int(argc, argv, 3);
    int threads = harness::arg_int(argc, argv, 4);
    std::vector<char> in = harness::read_file(argv[5], (size_t)nx * ny);

    APPFIS::Attribute attribute;
    attribute.threads = threads;
    attribute.overlap = false;
    attribute.ghostLayer = 1;
    attribute.periodic = true;  // game_appfis.hpp:58
    APPFIS::Initialize(argc, argv, APPFIS::DIM_2D, APPFIS::DIM_2D, attribute);

    APPFIS::Grid<int> g(APPFIS::DIM_2D, nx, ny, APPFIS::DUAL);
    g.AllocateFullGrid();
    APPFIS::Array<int>* full = g.GetFullGrid();
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) full->Set(i, j, (int)(unsigned char)in[(size_t)j * nx + i]);

    APPFIS::Scatter(g.GetFullGrid(), g.GetSubGrid());
    APPFIS::Config<int> config(g);
    config.GridsToUpdate(g);
    APPFIS::InitializeExecution(g);

    harness::Clock clock;
    for (int it = 0; it < gens; it++) APPFIS::Execute2D(config, g.GetSubGrid(), g.GetSubGridNext());
    double secs = clock.seconds();

    int live = 0;
    APPFIS::Execute2DReduce(config, live, APPFIS::SUM, g);
    APPFIS::FinalizeExecution(g);
    APPFIS::Gather(g.GetFullGrid(), g.GetSubGrid());

    std::vector<unsigned char> out((size_t)nx * ny);
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) out[(size_t)j * nx + i] = (unsigned char)full->Get(i, j);
    harness::write_file(argv[6], out.data(), out.size());
    std::printf("{\"live\": %d, \"seconds\": %.9f}\n", live, secs);
    APPFIS::Finalize();
    return 0;
}
