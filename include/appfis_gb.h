/*
 * appfis_gb.h — C ABI of the GB300-native APPFIS stencil engine (libappfis_gb.so).
 *
 * The reference (msharif42/APPFIS) exposes its hot path as header-only C++ templates: the user
 * writes APPFIS::Stencil overloads and calls Execute{1,2,3}D / Execute*DReduce / HaloExchange
 * per iteration (Appfis/Runtime.hpp:23-57).  This library is what those calls land on for the
 * five workloads: hand-written sm_103a kernels behind plain C entry points, so that the
 * drop-in C++ headers (appfis_gb300/Appfis/) and any FFI (ctypes, cgo, JNI) can bind them.
 *
 * Conventions
 *  - Every function returns a status (APPFIS_GB_OK = 0); appfis_gb_last_error() gives the
 *    calling thread's message of the last failure.  No exception crosses the ABI.
 *  - Device pointers are caller-owned, x-fastest, padded exactly like the reference's
 *    sub-grids (interior + 2*ghost per axis, Appfis/Common.hpp:197-226) unless stated.
 *    `pitch` is the row stride in elements (>= the padded x extent).
 *  - `stream` is a cudaStream_t (NULL = the legacy default stream).  Device entry points are
 *    asynchronous on that stream; results that land in host memory (suffix _job, *_host)
 *    synchronise it.
 *  - Two-buffer iterations (the reference's DUAL grids, Appfis/Grid.hpp:367-397) take both
 *    buffers and report in *cur_index which one holds the newest state (0 = a, 1 = b), which
 *    is what Grid::Swap tracks in the reference (Appfis/Grid.hpp:854-857).
 *  - Entry points with the suffix _job take HOST buffers and run a whole workload end to end
 *    (upload, iterate, download) on an internal stream with reused device workspace; calls
 *    from several host threads to the same _job function must be serialised by the caller.
 */
#ifndef APPFIS_GB_H
#define APPFIS_GB_H

#include <stdint.h>

#if defined(__GNUC__)
#define APPFIS_GB_API __attribute__((visibility("default")))
#else
#define APPFIS_GB_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define APPFIS_GB_OK 0
#define APPFIS_GB_EINVAL 1       /* bad argument: null pointer, size, pitch, unsupported combination */
#define APPFIS_GB_ECUDA 2        /* a CUDA runtime call or kernel launch failed */
#define APPFIS_GB_ENOMEM 3       /* device or pinned host allocation failed */
#define APPFIS_GB_ETIMEOUT 4     /* a bounded device-side wait gave up (no hang; context still usable) */
#define APPFIS_GB_ENUMERIC 5     /* the computation stopped itself: a time step collapsed to zero or NaN */

/* element types (reference Scatter/AllReduce support int, float, double: Communication.hpp:66-83) */
#define APPFIS_GB_F32 0
#define APPFIS_GB_F64 1
#define APPFIS_GB_I32 2
#define APPFIS_GB_F16 3          /* storage only (IEEE half); arithmetic stays FP32 */

/* reduction operators, same order as the reference enum REDUCTION { MAX, MIN, SUM } (Appfis/Env.hpp:32) */
#define APPFIS_GB_MAX 0
#define APPFIS_GB_MIN 1
#define APPFIS_GB_SUM 2

/* ----------------------------------------------------------------------------- runtime */
APPFIS_GB_API const char* appfis_gb_last_error(void);
APPFIS_GB_API int appfis_gb_version(void);
/* Blocks until all work on `stream` is done (replaces the reference's cudaStreamSynchronize
 * calls on its one stream, Appfis/Topology.hpp:151).  Then reads and clears the device status
 * word that kernels with bounded device-side waits set when a wait gives up (the results of
 * that launch are then invalid): returns APPFIS_GB_ETIMEOUT if it was set. */
APPFIS_GB_API int appfis_gb_stream_sync(void* stream);

/* Testing the bounded device-side waits (no counterpart in the reference, which has none): makes
 * the NEXT call of one kind run a wait out on purpose, so that a test can check that the call
 * ends with APPFIS_GB_ETIMEOUT and that the device stays usable.  Nothing faults or hangs: every
 * wait involved has a limit.  The plan applies to one call and is then cleared.
 *  kind 1: the next appfis_gb_flood_run / _job: CTA 0 does not arrive at the first grid
 *          barrier, and every barrier wait gives up after `limit` polls (1 .. 2^20; each poll
 *          sleeps ~64 ns): the run stops, its status is APPFIS_GB_ETIMEOUT.
 *  kind 2: the next TMA-staged radius-4 star launch (appfis_gb_star_r4): every CTA arms its
 *          first plane's mbarrier for 16 bytes more than the copy delivers, and waits at most
 *          `limit` ns (1e3 .. 1e8) per wait: the launch gives up, lets its copies land, and the
 *          next appfis_gb_stream_sync returns APPFIS_GB_ETIMEOUT.  The same plan applies to the
 *          next flood run that stages its rows by TMA (FP32 fused full sweep): every warp arms its
 *          first stage of rows for 16 bytes more, waits at most `limit` ns, lets its copies land
 *          and stops; the run's status is APPFIS_GB_ETIMEOUT.
 *  kind 0: clears a pending plan. */
APPFIS_GB_API int appfis_gb_test_stall_next(int kind, unsigned long long limit);

/* ----------------------------------------------------------------------------- reductions */
/* Execute{1,2,3}DReduce over a box (Appfis/Runtime.hpp:225-255 dispatch; GPU path
 * Appfis/Runtime_CUDA.hpp:554-740; CPU path Runtime.hpp:597-913; AllReduce Communication.hpp:752-789).
 * field: padded device field of type `dtype` with x pitch `px` and y extent `py` (rows per plane);
 * box = {x0, x1, y0, y1, z0, z1}, half-open (a Config's [start, end) per axis; use {0,1} for absent axes).
 * The result is written to the 8-byte device location dev_result: a double for F32/F64, an
 * int64 for I32.  MAX is seeded with std::numeric_limits<T>::min() like the reference (for
 * floating types that is the smallest positive normal, so an all-negative box returns it),
 * MIN with max(), SUM with 0.  Floating SUMs accumulate in double; every result is deterministic
 * (fixed-order tree: per-block partials, then the last block folds them in block order). */
APPFIS_GB_API int appfis_gb_reduce(const void* field, int dtype, int px, int py, const int* box, int op, void* dev_result,
                     void* stream);
/* Same reduction, same result, for callers that must not allocate device memory: a host
 * framework whose caching allocator has already reserved the device memory (a cudaMalloc there
 * fails, or fragments the framework's pool), a library embedded in another runtime that owns
 * every allocation, or a latency-critical loop where the implicit device synchronisation of a
 * first cudaMalloc/cudaFree would stall the pipeline.  No counterpart in the reference (its
 * reductions allocate nothing beyond the grid's own buffers).
 * The scratch (a ticket and one partial sum per block) lives in a fixed 64 KiB device array
 * inside the library, held by every device that loads it until the process exits; a box whose
 * reduction needs more than 8160 partial sums is rejected with APPFIS_GB_EINVAL (this kernel
 * uses at most 4 per SM).  The entry point calls no cudaMalloc, cudaFree or allocating library
 * routine.  Set-up: the first call on a device, with that device current, looks up the array's
 * device address (cudaGetSymbolAddress) and caches it; make that first call before any stream
 * capture.  Under CUDA's default lazy module loading the runtime commits the array's 64 KiB and
 * loads each (dtype, op) kernel instance on first use, so warm up every dtype/op pair you will
 * use before the device memory is handed to another allocator (or set CUDA_MODULE_LOADING=EAGER,
 * which loads everything when the library's module is first used).  Every call clears the
 * ticket with an asynchronous memset on `stream`.  All calls share the array, so calls that
 * overlap on the GPU (other streams, other host threads) race: order them. */
APPFIS_GB_API int appfis_gb_reduce_noalloc(const void* field, int dtype, int px, int py, const int* box, int op,
                                           void* dev_result, void* stream);
/* Same, returning the value on the host (synchronises `stream`). */
APPFIS_GB_API int appfis_gb_reduce_host(const void* field, int dtype, int px, int py, const int* box, int op, double* result,
                          void* stream);

/* ----------------------------------------------------------------------------- halo */
/* Periodic ghost refresh of a dense padded field (row pitch = padded_dims[0]) in place: the
 * single-rank form of Exchange for periodic grids (Appfis/Communication.hpp:612-678 with the
 * pack/unpack of Appfis/Runtime.hpp:916-1173), axis by axis over full faces so corners match.
 * elem_size 1, 2, 4 or 8 bytes; each padded axis must be >= 3*ghost. */
APPFIS_GB_API int appfis_gb_ghost_periodic(void* field, int elem_size, int ndim, const int* padded_dims, int ghost,
                                           void* stream);

/* ----------------------------------------------------------------------------- GameOfLife */
/* Replaces Execute2D(config, cur, next) with the GameOfLife functor + the periodic halo
 * exchange per generation (GameOfLife/src/game_appfis.hpp:79-82,121-135;
 * Appfis/Runtime_CUDA.hpp:345-369; Appfis/Communication.hpp:612-678).
 * Cells are u8 0/1 on the nx*ny INTERIOR only (row pitch nx): the periodic ghost ring of the
 * reference is not stored, the kernels wrap indices instead.
 * rule APPFIS_GB_LIFE_REFERENCE: the reference rule — a live cell dies when its count is < 2 or
 *   > 4, a dead cell is born when the count is 3, and otherwise the output buffer is left as it
 *   was (it then holds the state of two generations back).  Both buffers are read.
 * rule APPFIS_GB_LIFE_B3S23: Conway's B3/S23, a different function (not the reference's).
 * a = state at t, b = state at t-1 (zeros for the first call, as the reference zero-fills).
 * With nx a multiple of 16 both buffers must be 16-byte aligned (rows are bulk-copied). */
#define APPFIS_GB_LIFE_REFERENCE 0
#define APPFIS_GB_LIFE_B3S23 1
APPFIS_GB_API int appfis_gb_life_u8(uint8_t* a, uint8_t* b, int nx, int ny, int gens, int rule, int* cur_index, void* stream);
/* Bit-packed form: 32 cells per uint32 word, bit k of word w of row j = cell (32w + k, j);
 * nx must be a multiple of 32.  States are identical to appfis_gb_life_u8. */
APPFIS_GB_API int appfis_gb_life_pack(const uint8_t* cells, uint32_t* bits, int nx, int ny, void* stream);
APPFIS_GB_API int appfis_gb_life_unpack(const uint32_t* bits, uint8_t* cells, int nx, int ny, void* stream);
APPFIS_GB_API int appfis_gb_life_bits(uint32_t* a, uint32_t* b, int nx, int ny, int gens, int rule, int* cur_index, void* stream);
/* The reference's own layout (GameOfLife/src/game_appfis.hpp:58-62: int cells on a grid padded by
 * a periodic ghost ring of width `ghost`, row pitch px >= nx + 2*ghost, (ny + 2*ghost) rows) to the
 * u8 interior above, and back: to_i32 writes every padded cell from the interior cell it wraps to,
 * i.e. the interior plus the ghost ring as the reference's periodic exchange leaves it
 * (Appfis/Communication.hpp:612-678).  The drop-in's GameOfLife fast path uses these at the edges
 * of a run of generations. */
APPFIS_GB_API int appfis_gb_life_from_i32(const int32_t* padded, int px, int ghost, uint8_t* cells, int nx, int ny,
                                          void* stream);
APPFIS_GB_API int appfis_gb_life_to_i32(const uint8_t* cells, int nx, int ny, int32_t* padded, int px, int ghost,
                                        void* stream);
/* Population (Execute2DReduce SUM of the cells, game_appfis.hpp:84) into an int64 device location. */
APPFIS_GB_API int appfis_gb_life_population_u8(const uint8_t* cells, int64_t n, int64_t* dev_count, void* stream);
APPFIS_GB_API int appfis_gb_life_population_bits(const uint32_t* bits, int64_t nwords, int64_t* dev_count, void* stream);
/* Whole run from host buffers: cells_in (nx*ny u8) -> cells_out (nx*ny u8, may alias cells_in)
 * after `gens` generations; *population = live cells at the end.  form 0 = u8 kernels,
 * 1 = bit-packed kernels (nx % 32 == 0).  A NULL cells_out skips the field download. */
#define APPFIS_GB_FORM_U8 0
#define APPFIS_GB_FORM_BITS 1
APPFIS_GB_API int appfis_gb_life_job(const uint8_t* cells_in, uint8_t* cells_out, int nx, int ny, int gens, int rule, int form,
                       int64_t* population);

/* ----------------------------------------------------------------------------- Heat (2-D) */
/* Replaces the per-iteration Execute2D(config, cx, cy, cur, next) of the heat functor
 * (HeatDiffusion/src/heat_appfis.hpp:87-90,166-174, restated in 2-D FP32) on a DUAL grid with a
 * Dirichlet ghost ring (Grid::SetBoundary, Appfis/Grid.hpp:529-678) held in both buffers.
 * a, b: padded (nx+2) x (ny+2) fields with row pitch `pitch`; the update is
 *   next = c + cx*((l + r) - 2c) + cy*((u + d) - 2c)
 * evaluated with the same rounding sequence as the reference CPU path (no FMA contraction), so
 * results are bit-identical to it.  `iters` sweeps run as time-blocked launches (several sweeps
 * per launch in shared memory) with the identical per-point arithmetic. */
APPFIS_GB_API int appfis_gb_heat2d(float* a, float* b, int nx, int ny, int pitch, int iters, float cx, float cy, int* cur_index,
                     void* stream);
/* One sweep per launch (the plain form). */
APPFIS_GB_API int appfis_gb_heat2d_sweep(const float* cur, float* next, int nx, int ny, int pitch, float cx, float cy, void* stream);
/* Whole run from host: field is the padded (nx+2)*(ny+2) dense array (ghost ring included), in
 * place.  stats (optional, 3 doubles): MAX, MIN, SUM of the interior at the end (reference seeds). */
APPFIS_GB_API int appfis_gb_heat2d_job(float* field, int nx, int ny, int iters, float cx, float cy, double* stats);

/* ----------------------------------------------------------------------------- Himeno */
/* Replaces the per-iteration Execute3D(config, omega, a0..wrk1, p, wrk2) of the Himeno functor
 * (Himeno/src/himeno_appfis.hpp:108-114,178-198) on a DUAL p grid with 12 SINGLE coefficient grids.
 * coef: host array of 12 device pointers (a0 a1 a2 a3 b0 b1 b2 c0 c1 c2 bnd wrk1), each a padded
 * (nx+2) x (ny+2) x (nz+2) FP32 field with row pitch `pitch`; p, wrk2: the two p buffers (zero
 * ghost ring, as after the reference's Scatter).  The FP32 update follows the reference's
 * summation order exactly (bit-identical to its CPU path).  dev_gosa (optional, `iters`
 * doubles): gosa of every sweep = sum over the interior of ss^2 with ss as in :195, reduced in
 * double inside the sweep (deterministic order); the reference computes no gosa. */
APPFIS_GB_API int appfis_gb_himeno(const float* const* coef, float* p, float* wrk2, int nx, int ny, int nz, int pitch,
                                   int iters, float omega, double* dev_gosa, int* cur_index, void* stream);
/* Mixed-precision defect correction: FP16 storage of the correction e, the defect D and the ten
 * neighbour/boundary coefficient fields, a3 read in FP32 (30 B per point per sweep instead of 56),
 * FP32 arithmetic, FP32 master p refreshed every `period` sweeps (the defect D = omega*ss(p) is
 * then recomputed from the FP32 coefficients).  Same iteration as appfis_gb_himeno in exact
 * arithmetic; the difference is the FP16 rounding inside one period.  p_work: a second FP32
 * field; half_work: 13 FP16 fields (13 * pitch*(ny+2)*(nz+2) halves).  gosa as above (from the
 * FP16 iterate, FP32 ss, double sum). */
APPFIS_GB_API int appfis_gb_himeno_mixed(const float* const* coef, float* p, float* p_work, void* half_work, int nx, int ny,
                                         int nz, int pitch, int iters, int period, float omega, double* dev_gosa,
                                         int* cur_index, void* stream);
/* appfis_gb_himeno_mixed with the number of inner sweeps per launch: 1 (the default, also for
 * 0) or 2: the coefficient, a3 and D tiles of a plane read once for two sweeps, the same bits as
 * two single sweeps (gosa summed in another order); it needs 16-byte aligned rows (pitch a
 * multiple of 8; EINVAL otherwise), and a period with an odd count of inner sweeps ends with a
 * single sweep.  On GB300 the two-sweep form is slower at every size measured (its one-point
 * ring is recomputed and each plane takes a second barrier), so it is an option, not a default. */
APPFIS_GB_API int appfis_gb_himeno_mixed_ex(const float* const* coef, float* p, float* p_work, void* half_work, int nx,
                                            int ny, int nz, int pitch, int iters, int period, float omega,
                                            int sweeps_per_pass, double* dev_gosa, int* cur_index, void* stream);
/* Whole run from host: coef_host = 12 dense padded fields back to back, p_host = dense padded p
 * (in place).  form 0 = plain FP32, 1 = defect correction with `period`.  gosa_host: `iters`
 * doubles or NULL. */
APPFIS_GB_API int appfis_gb_himeno_job(const float* coef_host, float* p_host, int nx, int ny, int nz, int iters,
                                       float omega, int form, int period, double* gosa_host);

/* ----------------------------------------------------------------------------- radius-4 star (FDTD3d) */
#define APPFIS_GB_STAR_AUTO 0
#define APPFIS_GB_STAR_SCALAR2 2 /* scalar tile, 2 rows per thread */
#define APPFIS_GB_STAR_SCALAR4 4 /* scalar tile, 4 rows per thread */
#define APPFIS_GB_STAR_TMA_X4 8  /* TMA-staged 64 x 16 tile, 4 x points x 2 rows per thread */
#define APPFIS_GB_STAR_TMA_X2 9  /* TMA-staged 32 x 16 tile, 2 x points x 2 rows per thread */
#define APPFIS_GB_STAR_VEC 10    /* register-staged 64 x 16 tile of 4-element vectors */
#define APPFIS_GB_STAR_TB2 11    /* TMA-staged, TWO time steps per launch (64 x 16 output tile, step-1 values kept on
                                    chip); an odd last step runs in the TMA_X4 tile */
#define APPFIS_GB_STAR_TB2_8 12  /* the same with a 64 x 8 output tile */
#define APPFIS_GB_STAR_TMA_X4R4 13 /* TMA-staged 64 x 32 tile, 4 x points x 4 rows per thread */
/* Replaces the per-step Execute3D(config, coeff, radius, cur, next) of the FDTD3d functor
 * (FDTD3d/src/fdtd3d_appfis.hpp:84-87,129-143) with radius 4 on a DUAL grid with a ghost halo of
 * width 4 (a, b: padded (nx+8) x (ny+8) x (nz+8), pitch >= nx+8, halo held at its values).
 * mode 0: the reference form  v = c + sum_{a=1..4} ((x-a + x+a) + (y-a + y+a) + (z-a + z+a)),
 *         v *= coeff  (same order; FP32 results bit-identical to the reference CPU path).
 * mode 1: weighted form  v = w[0]*c + sum_a w[a]*((x-a + x+a) + (y-a + y+a) + (z-a + z+a)).
 * dtype: APPFIS_GB_F32 or APPFIS_GB_F16 (storage).  tile selects the kernel (APPFIS_GB_STAR_*;
 * AUTO: the choice appfis_gb_star_r4_tune recorded for this device and shape, else the TMA-staged
 * tile when rows and fields are 16-byte aligned, else the vector tile when 4-element vectors are
 * aligned, else the scalar tile; all give the same results in the reference form and in FP32).  zchunk: z
 * planes per CTA (0 = the tile's default: TMA-staged 32-64 planes balanced over nz, the length that fills the
 * resident CTAs in the most nearly whole waves; 32 otherwise). */
APPFIS_GB_API int appfis_gb_star_r4(void* a, void* b, int dtype, int nx, int ny, int nz, int pitch, int iters, int mode,
                                    float coeff, const float* weights, int tile, int zchunk, int* cur_index,
                                    void* stream);

/* ----------------------------------------------------------------------------- FP64 sweeps */
/* The heat, Himeno and radius-4 star functors instantiated with double, every multiply and add
 * rounded separately in the reference's order: bit-identical to the reference's CPU path built
 * with double (its functors are templates on the element type; HeatDiffusion itself runs in
 * double, HeatDiffusion/src/heat_appfis.hpp:72,166-174).  Same layouts and arguments as the
 * FP32 entry points above (a, b: the two buffers; pitch in elements; ghost ring held in both).
 * They are also the precision reference that the FP32, FP16-storage, mixed-precision and
 * time-blocked forms state their error against.  Bounded by the FP64 pipe (not a fast path). */
APPFIS_GB_API int appfis_gb_heat2d_f64(double* a, double* b, int nx, int ny, int pitch, int iters, double cx, double cy,
                                       int* cur_index, void* stream);
/* Himeno/src/himeno_appfis.hpp:178-198 in double; coef: 12 device pointers as appfis_gb_himeno;
 * dev_gosa (optional, `iters` doubles): sum of ss^2 per sweep, fixed-order (deterministic). */
APPFIS_GB_API int appfis_gb_himeno_f64(const double* const* coef, double* p, double* wrk2, int nx, int ny, int nz, int pitch,
                                       int iters, double omega, double* dev_gosa, int* cur_index, void* stream);
/* FDTD3d/src/fdtd3d_appfis.hpp:129-143 (mode 0, coefficient `coeff`) or the weighted form
 * (mode 1, 5 double weights) in double, halo width 4. */
APPFIS_GB_API int appfis_gb_star_r4_f64(double* a, double* b, int nx, int ny, int nz, int pitch, int iters, int mode,
                                        double coeff, const double* weights, int* cur_index, void* stream);

/* Autotuner of the radius-4 star (no counterpart in the reference): times every candidate kernel
 * for this shape on `stream` — on 16-byte rows the TMA-staged tiles (4 or 2 x points per thread,
 * one step per launch) and the two-step time-blocked tiles (64 x 16 / 64 x 8 outputs), else the
 * vector / scalar tiles — with z chunks of the tile's default and 32 .. 256 planes, each run
 * from a into b (b's interior is overwritten; a and the halos are not), and keeps the fastest
 * per device and shape (dtype, form, nx, ny, nz, pitch) for the process; later calls with
 * tile = APPFIS_GB_STAR_AUTO use it (zchunk 0 = the tuned chunk).  With APPFIS_GB_TUNE_FILE set
 * in the environment, results are read from / appended to that text file.  Returns the choice
 * (tile id, z chunk; 0 = the tile's default) and its time per step; synchronises `stream`. */
APPFIS_GB_API int appfis_gb_star_r4_tune(void* a, void* b, int dtype, int nx, int ny, int nz, int pitch, int mode, float coeff,
                                         const float* weights, int* tile_out, int* zchunk_out, float* ms_per_step_out,
                                         void* stream);

/* ----------------------------------------------------------------------------- Triton flood model */
/* Replaces the reference's Triton time loop (Triton/src/triton_appfis.hpp:316-386: CFL dt functor +
 * Execute2DReduce(MIN) + host clamp, sqrt/RHS reset, X and Y Roe-type flux functors, update +
 * Manning friction, HaloExchange, wet/dry fix) for a BATCH of independent domains of uneven
 * sizes advanced in one persistent cooperative launch, each domain with its own dt, simulated
 * time and step count, until every domain reaches t_end (or max_steps).  Point sources
 * (:352-373): appfis_gb_flood_run_sources below.
 * A domain: padded (nx+2) x (ny+2) fields with row pitch `pitch`, element type `dtype`
 * (APPFIS_GB_F32 or APPFIS_GB_F64): h/qx/qy[0] = state at t_start, h/qx/qy[1] = second buffers
 * with the same ghost ring (0); dem with its ghost ring at the wall height (the reference uses
 * 1e6); n2 = Manning n^2.  After the run the newest state of domain d is in buffer
 * (steps[d] & 1), with the wet/dry fix of the last step applied. */
typedef struct {
    int nx, ny, pitch;
    void* h[2];
    void* qx[2];
    void* qy[2];
    const void* dem;
    const void* n2;
} appfis_gb_flood_domain;

typedef struct {
    double dx;             /* cell size (m) */
    double courant;        /* CFL number cn */
    double hextra;         /* wet threshold (m) */
    double t_end;          /* simulated end time (s) */
    double print_interval; /* dt is clamped so that the simulated time lands on multiples of it */
    double time_step;      /* dt used while no cell is wet */
    double t_start;        /* initial simulated time */
    int max_steps;         /* 0 = no limit; > 0 also enables the dt log */
    int flags;             /* APPFIS_GB_FLOOD_SKIP_DRY | APPFIS_GB_FLOOD_TWO_PHASE or _FUSED, or 0 */
} appfis_gb_flood_params;

/* flags: strips (28 or 30 x 32 cells) whose depth and momentum are exactly 0 and whose four neighbour
 * strips are dry as well are left out of a step: such cells cannot change (no face of theirs
 * has water on either side), so every field is bit-identical to the full sweep.  A strip is
 * skipped only after its output was dry for two consecutive steps (both state buffers hold the
 * dry state). */
#define APPFIS_GB_FLOOD_SKIP_DRY 1
/* FP32 runs without point sources take one fused pass per step (update, wet/dry fix and the
 * next step's CFL dt; 28-column strips whose one-cell ring is updated again by its neighbours),
 * with or without dry-strip skipping; FP64 runs and runs with point sources take two passes (fix
 * + dt, then update).  TWO_PHASE and FUSED (no point sources) select a form explicitly; the
 * fields, step counts and dt logs of the two forms are identical. */
#define APPFIS_GB_FLOOD_TWO_PHASE 2
#define APPFIS_GB_FLOOD_FUSED 4
/* The FP32 fused full sweep (no SKIP_DRY) streams each strip's rows into shared memory by TMA
 * (bulk tensor copies of 4-row stages, one stage ahead of the computation) when every domain's
 * arrays are 16-byte aligned and its pitch is a multiple of 4; UNSTAGED makes it load the rows
 * directly (the same fields). */
#define APPFIS_GB_FLOOD_UNSTAGED 8

#define APPFIS_GB_FLOOD_MAX_DOMAINS 64

/* Device entry: dev_dtlog (optional, ndom*max_steps doubles, needs max_steps > 0): dt of every
 * step; dev_steps / dev_simtime (optional, ndom each): steps taken and final time; dev_status
 * (optional int): APPFIS_GB_OK, APPFIS_GB_ETIMEOUT if a bounded grid-wide wait gave up, or
 * APPFIS_GB_ENUMERIC if a domain's time step collapsed to zero or NaN (the run stops).  With
 * max_steps = 0 each domain is capped at 1,000,000 steps. */
APPFIS_GB_API int appfis_gb_flood_run(const appfis_gb_flood_domain* doms, int ndom, int dtype,
                                      const appfis_gb_flood_params* prm, double* dev_dtlog, int* dev_steps,
                                      double* dev_simtime, int* dev_status, void* stream);
/* Point sources of one domain (the reference's hydrograph inflows, Triton/src/triton_appfis.hpp:
 * 218-293 set-up, 352-373 row search, 1115-1141 the Execute1D source functor): after every
 * step's update, before the wet/dry fix, h at each source cell grows by flow * dt / dx^2 with
 * flow interpolated in the hydrograph at the step's start time.  HOST arrays (copied per run):
 * cells[n] = the reference's padded sub-grid index row * (nx + 2) + col of an interior cell;
 * times[nt] in seconds, increasing; flows[nt * n] in m^3/s, row t holding the n sources at
 * times[t].  n = 0: no sources in that domain. */
typedef struct {
    int n, nt;
    const int* cells;
    const double* times;
    const double* flows;
} appfis_gb_flood_sources;

/* appfis_gb_flood_run with point sources: srcs[ndom] (one table per domain, n may be 0). */
APPFIS_GB_API int appfis_gb_flood_run_sources(const appfis_gb_flood_domain* doms, const appfis_gb_flood_sources* srcs, int ndom,
                                              int dtype, const appfis_gb_flood_params* prm, double* dev_dtlog, int* dev_steps,
                                              double* dev_simtime, int* dev_status, void* stream);
/* Initialises one domain's buffers (both state buffers, dem with a 1e6 ghost ring as the reference's
 * dem.SetBoundary(1e6), n2 = manning^2 everywhere) from FP64 DEVICE interiors dem, h, qx, qy
 * (nx*ny each; qx/qy may be NULL = 0). */
APPFIS_GB_API int appfis_gb_flood_setup(const appfis_gb_flood_domain* dom, int dtype, const double* dem, const double* h,
                                        const double* qx, const double* qy, double manning, void* stream);
/* Host-buffer job: per domain nx*ny FP64 interiors dem[d], h[d] (in/out), qx[d]/qy[d] (in/out,
 * may be NULL = zero initial momentum, not returned); computed in `dtype`.  steps_out (ndom),
 * mass_out (2*ndom: sum of h over the interior before and after, FP64), dtlog_host (ndom*max_steps)
 * are optional. */
APPFIS_GB_API int appfis_gb_flood_job(int ndom, const int* nx, const int* ny, const double* const* dem, double* const* h,
                                      double* const* qx, double* const* qy, double manning,
                                      const appfis_gb_flood_params* prm, int dtype, int* steps_out, double* mass_out,
                                      double* dtlog_host);

#ifdef __cplusplus
}
#endif

#endif /* APPFIS_GB_H */
