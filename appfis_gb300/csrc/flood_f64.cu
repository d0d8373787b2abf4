// FP64 instantiation of the batched flood model, compiled with -fmad=false so that every
// multiply and add rounds separately, as in the reference's CPU build; with correctly rounded
// division and square root this follows the reference's FP64 rounding sequence (cbrt may
// differ in the last bit).
#include "flood_host.cuh"

namespace flood {

int run_f64(const appfis_gb_flood_domain* doms, int ndom, const appfis_gb_flood_params* prm, double* dtlog, int* steps,
            double* simtime, int* status, cudaStream_t st, const appfis_gb_flood_sources* srcs)
{
    return run<double>(doms, ndom, prm, dtlog, steps, simtime, status, st, srcs);
}

int setup_f64(const appfis_gb_flood_domain* dom, const double* dem, const double* h, const double* qx, const double* qy,
              double manning, cudaStream_t st)
{
    return setup<double>(dom, dem, h, qx, qy, manning, st);
}

int job_f64(int ndom, const int* nx, const int* ny, const double* const* dem, double* const* h, double* const* qx,
            double* const* qy, double manning, const appfis_gb_flood_params* prm, int* steps_out, double* mass_out,
            double* dtlog_host)
{
    return job<double>(ndom, nx, ny, dem, h, qx, qy, manning, prm, steps_out, mass_out, dtlog_host);
}

}  // namespace flood
