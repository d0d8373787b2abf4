// FP32 instantiation of the batched flood model (the fast form: FP32 state and arithmetic,
// FP64 dt reduction, simulated time and mass sums) and the C-ABI entry points for both types.
#include "flood_host.cuh"

namespace flood {
// defined in flood_f64.cu (built without FMA contraction)
int run_f64(const appfis_gb_flood_domain* doms, int ndom, const appfis_gb_flood_params* prm, double* dtlog, int* steps,
            double* simtime, int* status, cudaStream_t st, const appfis_gb_flood_sources* srcs);
int setup_f64(const appfis_gb_flood_domain* dom, const double* dem, const double* h, const double* qx, const double* qy,
              double manning, cudaStream_t st);
int job_f64(int ndom, const int* nx, const int* ny, const double* const* dem, double* const* h, double* const* qx,
            double* const* qy, double manning, const appfis_gb_flood_params* prm, int* steps_out, double* mass_out,
            double* dtlog_host);
}  // namespace flood

extern "C" {

int appfis_gb_flood_run(const appfis_gb_flood_domain* doms, int ndom, int dtype, const appfis_gb_flood_params* prm,
                        double* dev_dtlog, int* dev_steps, double* dev_simtime, int* dev_status, void* stream)
{
    cudaStream_t st = gb::as_stream(stream);
    if (dtype == APPFIS_GB_F32) return flood::run<float>(doms, ndom, prm, dev_dtlog, dev_steps, dev_simtime, dev_status, st);
    if (dtype == APPFIS_GB_F64) return flood::run_f64(doms, ndom, prm, dev_dtlog, dev_steps, dev_simtime, dev_status, st, nullptr);
    return gb::fail(APPFIS_GB_EINVAL, "flood_run: dtype %d (F32 or F64)", dtype);
}

int appfis_gb_flood_run_sources(const appfis_gb_flood_domain* doms, const appfis_gb_flood_sources* srcs, int ndom, int dtype,
                                const appfis_gb_flood_params* prm, double* dev_dtlog, int* dev_steps, double* dev_simtime,
                                int* dev_status, void* stream)
{
    if (!srcs) return gb::fail(APPFIS_GB_EINVAL, "flood_run_sources: null source tables");
    cudaStream_t st = gb::as_stream(stream);
    if (dtype == APPFIS_GB_F32)
        return flood::run<float>(doms, ndom, prm, dev_dtlog, dev_steps, dev_simtime, dev_status, st, srcs);
    if (dtype == APPFIS_GB_F64) return flood::run_f64(doms, ndom, prm, dev_dtlog, dev_steps, dev_simtime, dev_status, st, srcs);
    return gb::fail(APPFIS_GB_EINVAL, "flood_run_sources: dtype %d (F32 or F64)", dtype);
}

int appfis_gb_flood_setup(const appfis_gb_flood_domain* dom, int dtype, const double* dem, const double* h, const double* qx,
                          const double* qy, double manning, void* stream)
{
    cudaStream_t st = gb::as_stream(stream);
    if (dtype == APPFIS_GB_F32) return flood::setup<float>(dom, dem, h, qx, qy, manning, st);
    if (dtype == APPFIS_GB_F64) return flood::setup_f64(dom, dem, h, qx, qy, manning, st);
    return gb::fail(APPFIS_GB_EINVAL, "flood_setup: dtype %d (F32 or F64)", dtype);
}

int appfis_gb_flood_job(int ndom, const int* nx, const int* ny, const double* const* dem, double* const* h,
                        double* const* qx, double* const* qy, double manning, const appfis_gb_flood_params* prm, int dtype,
                        int* steps_out, double* mass_out, double* dtlog_host)
{
    if (dtype == APPFIS_GB_F32)
        return flood::job<float>(ndom, nx, ny, dem, h, qx, qy, manning, prm, steps_out, mass_out, dtlog_host);
    if (dtype == APPFIS_GB_F64)
        return flood::job_f64(ndom, nx, ny, dem, h, qx, qy, manning, prm, steps_out, mass_out, dtlog_host);
    return gb::fail(APPFIS_GB_EINVAL, "flood_job: dtype %d (F32 or F64)", dtype);
}

}  // extern "C"
