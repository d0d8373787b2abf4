// Oracle harness: the reference's Triton flood-model functors (Triton/src/triton_appfis.hpp:567-1112:
// CFL dt, sqrt(h) + RHS reset, X- and Y-direction Roe-type fluxes, update + Manning friction,
// wet/dry momentum fix) run through the reference's own APPFIS_CPU runtime, in the order of the
// reference time loop (triton_appfis.hpp:316-386) without point sources and without case files:
// the DEM, initial depth and constants come from the command line / raw FP64 files instead of
// the .cfg reader.
//
// usage: ref_triton NX NY THREADS DX COURANT HEXTRA MANNING T_END PRINT_INTERVAL TIME_STEP MAX_STEPS
//                   dem.f64 h.f64 out.f64 dt.f64
//   dem.f64, h.f64 : NX*NY interiors;  out.f64 : h, qx, qy interiors (3*NX*NY) at the end
//   dt.f64         : the dt of every step taken;  MAX_STEPS <= 0 means "until T_END"
// stdout : {"steps": .., "simtime": .., "seconds": ..}
#include "harness_io.hpp"
#include "Triton/src/triton_appfis.hpp"

int main(int argc, char** argv)
{
    int nx = harness::arg_int(argc, argv, 1), ny = harness::arg_int(argc, argv, 2), threads = harness::arg_int(argc, argv, 3);
    double cell = harness::arg_f(argc, argv, 4), courant = harness::arg_f(argc, argv, 5), hextra = harness::arg_f(argc, argv, 6);
    double mann = harness::arg_f(argc, argv, 7), t_end = harness::arg_f(argc, argv, 8), print_interval = harness::arg_f(argc, argv, 9);
    double time_step = harness::arg_f(argc, argv, 10);
    int max_steps = harness::arg_int(argc, argv, 11);
    size_t n = (size_t)nx * ny;
    std::vector<char> demb = harness::read_file(argv[12], n * sizeof(double));
    std::vector<char> hb = harness::read_file(argv[13], n * sizeof(double));
    const double* dems = reinterpret_cast<const double*>(demb.data());
    const double* hs = reinterpret_cast<const double*>(hb.data());

    APPFIS::Attribute attribute;
    attribute.threads = threads;
    attribute.ghostLayer = 1;
    attribute.periodic = false;
    APPFIS::Initialize(argc, argv, APPFIS::DIM_2D, APPFIS::DIM_2D, attribute);

    typedef APPFIS::Grid<double> GD;
    GD dem(APPFIS::DIM_2D, nx, ny, APPFIS::SINGLE), nin(APPFIS::DIM_2D, nx, ny, APPFIS::SINGLE);
    GD hin(APPFIS::DIM_2D, nx, ny, APPFIS::SINGLE), uin(APPFIS::DIM_2D, nx, ny, APPFIS::SINGLE), vin(APPFIS::DIM_2D, nx, ny, APPFIS::SINGLE);
    GD sqrth(APPFIS::DIM_2D, nx, ny, APPFIS::SINGLE);
    GD rhsh0(APPFIS::DIM_2D, nx, ny, APPFIS::SINGLE), rhsh1(APPFIS::DIM_2D, nx, ny, APPFIS::SINGLE);
    GD rhsqx0(APPFIS::DIM_2D, nx, ny, APPFIS::SINGLE), rhsqx1(APPFIS::DIM_2D, nx, ny, APPFIS::SINGLE);
    GD rhsqy0(APPFIS::DIM_2D, nx, ny, APPFIS::SINGLE), rhsqy1(APPFIS::DIM_2D, nx, ny, APPFIS::SINGLE);
    GD dtv(APPFIS::DIM_2D, nx, ny, APPFIS::DUAL);

    dem.AllocateFullGrid(); nin.AllocateFullGrid(); hin.AllocateFullGrid(); uin.AllocateFullGrid(); vin.AllocateFullGrid();
    for (size_t c = 0; c < n; c++) { dem.GetFullGrid()->GetData()[c] = dems[c]; hin.GetFullGrid()->GetData()[c] = hs[c]; }
    nin.GetFullGrid()->FillData(mann);
    nin.GetFullGrid()->Square();

    APPFIS::Scatter(dem.GetFullGrid(), dem.GetSubGrid());
    dem.SetBoundary(1e6);
    APPFIS::Scatter(nin.GetFullGrid(), nin.GetSubGrid());
    nin.SetBoundaryCopy();
    APPFIS::Scatter(hin.GetFullGrid(), hin.GetSubGrid());

    APPFIS::Config<double> config(dem);
    APPFIS::Config<double> configF(dem, 0, 0, 0, 0);
    APPFIS::Config<double> configX(dem, 0, 1, 1, 1);
    APPFIS::Config<double> configY(dem, 1, 1, 1, 0);
    APPFIS::Config<double> configQ(dem);
    configQ.GridsToUpdate(uin, vin);

    APPFIS::InitializeExecution(dem, nin, hin, uin, vin, sqrth, rhsh0, rhsh1, rhsqx0, rhsqx1, rhsqy0, rhsqy1, dtv);

    double simtime = 0.0, global_dt = time_step;
    int it_count = 0, print_id = 0;
    std::vector<double> dts;
    harness::Clock clock;
    while (simtime < t_end && (max_steps <= 0 || it_count < max_steps))
    {
        it_count++;
        APPFIS::Execute2D(config, cell, courant, hextra, uin.GetSubGrid(), vin.GetSubGrid(), hin.GetSubGrid(), dtv.GetSubGrid());
        APPFIS::Execute2DReduce(config, global_dt, APPFIS::MIN, dtv);
        if (global_dt >= DBL_MAX - 1.0) global_dt = time_step;
        if (simtime + global_dt > print_interval * (print_id + 1)) global_dt = print_interval * (print_id + 1) - simtime;

        APPFIS::Execute2D(configF, hin.GetSubGrid(), sqrth.GetSubGrid(), rhsh0.GetSubGrid(), rhsh1.GetSubGrid(),
                          rhsqx0.GetSubGrid(), rhsqx1.GetSubGrid(), rhsqy0.GetSubGrid(), rhsqy1.GetSubGrid());
        APPFIS::Execute2D(configX, cell, global_dt, hextra, hin.GetSubGrid(), uin.GetSubGrid(), vin.GetSubGrid(), dem.GetSubGrid(),
                          sqrth.GetSubGrid(), rhsh0.GetSubGrid(), rhsh1.GetSubGrid(), rhsqx0.GetSubGrid(), rhsqx1.GetSubGrid(),
                          rhsqy0.GetSubGrid(), rhsqy1.GetSubGrid());
        APPFIS::Execute2D(configY, cell, global_dt, hextra, 0, hin.GetSubGrid(), uin.GetSubGrid(), vin.GetSubGrid(), dem.GetSubGrid(),
                          sqrth.GetSubGrid(), rhsh0.GetSubGrid(), rhsh1.GetSubGrid(), rhsqx0.GetSubGrid(), rhsqx1.GetSubGrid(),
                          rhsqy0.GetSubGrid(), rhsqy1.GetSubGrid());
        APPFIS::Execute2D(config, global_dt, hextra, hin.GetSubGrid(), uin.GetSubGrid(), vin.GetSubGrid(), dem.GetSubGrid(), nin.GetSubGrid(),
                          rhsh0.GetSubGrid(), rhsh1.GetSubGrid(), rhsqx0.GetSubGrid(), rhsqx1.GetSubGrid(), rhsqy0.GetSubGrid(), rhsqy1.GetSubGrid());
        APPFIS::HaloExchange(&hin);
        APPFIS::Execute2D(configQ, global_dt, hextra, hin.GetSubGrid(), uin.GetSubGrid(), vin.GetSubGrid(), dem.GetSubGrid());
        simtime += global_dt;
        dts.push_back(global_dt);
        if (simtime >= print_interval * (print_id + 1)) print_id++;
    }
    double secs = clock.seconds();

    APPFIS::FinalizeExecution(hin, uin, vin);
    std::vector<double> out(3 * n);
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++)
        {
            size_t c = (size_t)j * nx + i;
            out[c] = hin.GetSubGrid()->Get(i + 1, j + 1);
            out[n + c] = uin.GetSubGrid()->Get(i + 1, j + 1);
            out[2 * n + c] = vin.GetSubGrid()->Get(i + 1, j + 1);
        }
    harness::write_file(argv[14], out.data(), out.size() * sizeof(double));
    harness::write_file(argv[15], dts.data(), dts.size() * sizeof(double));
    std::printf("{\"steps\": %d, \"simtime\": %.17g, \"seconds\": %.9f}\n", it_count, simtime, secs);
    APPFIS::Finalize();
    return 0;
}
