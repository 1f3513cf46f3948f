/*
 * tomography_gb300 -- C ABI of the GB300-native forward FDTD fitness path.
 *
 * The reference exposes its hot path as two C++ functions with the signature
 *     double FDTD_GPU(const std::vector<double>& arguments);   FDTD_GPU.cuh:8
 *     double FDTD_CPU(const std::vector<double>& arguments);   FDTD_CPU.h:8
 * which tao's particle-swarm / differential-evolution drivers call once per
 * candidate (test.cxx:94-121).  This header is the C boundary that replaces
 * them: plain pointers and sizes, integer status codes, no C++ or CUDA types.
 * The C++ drop-in with the reference's exact signature is declared in
 * include/tomography_fdtd.hpp and is a thin wrapper over tomo_fitness().
 *
 * All entry points return TOMO_OK (0) or a negative tomo_status; the message
 * of the last failure on the calling thread is returned by tomo_last_error().
 * A handle may be used from one thread at a time.
 */
#ifndef TOMOGRAPHY_GB300_H
#define TOMOGRAPHY_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum tomo_status {
    TOMO_OK = 0,
    TOMO_EINVAL = -1,          /* bad argument (the reference throws std::out_of_range) */
    TOMO_ENOMEM_BUDGET = -2,   /* request does not fit the device-memory budget          */
    TOMO_ETIMEOUT = -3,        /* a bounded wait ran out                                 */
    TOMO_ENUMERIC = -4,        /* non-finite field / fitness detected                    */
    TOMO_ECUDA = -5,           /* CUDA runtime error (the reference calls exit(-1))      */
    TOMO_ENOTREADY = -6,       /* serving ticket not finished yet                        */
    TOMO_ECANCELLED = -7,      /* serving ticket was cancelled                           */
    TOMO_ENOTARGET = -8,       /* fitness requested before a target was set              */
    TOMO_ENOMEM_HOST = -9      /* a host allocation failed (no C++ exception crosses the ABI) */
} tomo_status;

typedef enum tomo_mode {
    TOMO_MODE_REFERENCE_GPU = 0, /* FDTD_GPU.cu: 3x3 Debye patches, 27 args, 4 plane waves, |D| misfit   */
    TOMO_MODE_REFERENCE_CPU = 1, /* FDTD_CPU.cxx: 9x9 (eps_r, sigma) patches, 162 args, relative misfit  */
    TOMO_MODE_BREAST = 2         /* ellipse phantom, point transmitters, receiver traces, trace misfit    */
} tomo_mode;

typedef enum tomo_precision { TOMO_FP32 = 0, TOMO_FP64 = 1 } tomo_precision;

#define TOMO_MAX_FREQS 32

/* Runtime problem description; the reference fixes all of this at compile
 * time in FDTD_common.hxx:1-76.  tomo_spec_reference() fills the exact
 * reference values. */
typedef struct tomo_spec {
    int32_t mode;              /* tomo_mode                                          */
    int32_t precision;         /* tomo_precision of the field updates                */
    int32_t nx, ny;            /* H grid nx*ny; Ez grid (nx+1)*(ny+1)                */
    double dx;                 /* cell size [m] (dx = dy)                            */
    double dt;                 /* time step [s]                                      */
    int32_t steps;             /* time steps per solve                               */
    /* CPML (FDTD_GPU.cu:748-806) */
    int32_t ncpml;             /* CPML cells per side, 0..32                         */
    double cpml_grading, cpml_sigma_max, cpml_kappa_max, cpml_alpha_max, cpml_alpha_min;
    double tau;                /* Debye relaxation time [s]                          */
    /* reference plane-wave modes */
    double breast_radius;      /* [m]                                                */
    int32_t npatch;            /* patches per side (3 GPU path, 9 CPU path)          */
    int32_t n_excitations;     /* plane-wave angles 2*pi*k/n                         */
    double pw_tau, pw_t0, pw_l;/* fwf(): Gaussian width, delay, offset               */
    int32_t pw_centred;        /* 1: x - nx/2 (GPU path), 0: raw x (CPU path)        */
    int32_t nan_clamp;         /* 1: NaN -> 0 as FDTD_GPU.cu:335-350                 */
    /* breast-imaging phantom */
    double bg_eps_inf, bg_del_eps, bg_sigma;
    double disc_radius, disc_eps_inf, disc_del_eps, disc_sigma;
    int32_t n_ellipses;        /* 8 parameters each: cx, cy, a, b, angle, eps_inf, del_eps, sigma */
    int32_t n_antennas;        /* ring of point transmitters / receivers             */
    int32_t n_tx;              /* transmitters fired per candidate (<= n_antennas)   */
    double antenna_radius;     /* [m]                                                */
    double src_f0, src_tau, src_t0, src_amp;  /* modulated Gaussian current source; amp 0 = auto */
    /* near-to-far-field transform: in vacuum for the reference modes, in the
       background medium (k = sqrt(bg_eps_inf) k0, eta = eta0 / sqrt(bg_eps_inf))
       for the breast mode, whose contour lies in that lossless background */
    int32_t nf2ff_d;           /* contour distance from the grid edge [cells]        */
    int32_t nfreq;
    double freqs[TOMO_MAX_FREQS];
    int32_t n_angles;
    int32_t ff_norm;           /* 1: reference normalisation (Prad, 33.329), 0: plain */
    int32_t misfit;            /* 0: -sum (D-m)^2/(E F); 1: relative; 2: trace L2    */
    /* engine tuning: 0 = autotune */
    int32_t steps_per_launch;  /* temporal-blocking depth T; 0: autotuned            */
    int32_t cols_per_lane;     /* columns per lane; 0: autotuned                     */
    int32_t plain;             /* 1: one solve per launch sequence, one launch per
                                  step, no CUDA graph (the plain baseline path)      */
    int32_t total_field;       /* 1 (reference GPU mode only): the legacy total-field
                                  far field of oldFDTD_GPU.cu:425-482,655-717,762-824.
                                  Each batch also advances one incident vacuum grid
                                  driven at (nx/2, ny/2) by 100 (-dt/eps0) fwf(n, 0,0,0,0);
                                  the contour sums take H + H_inc and Ez plus the
                                  two-level average of Ez_inc, with M at (n - 1/2) dt.
                                  Not accepted by the serving loop.                  */
} tomo_spec;

typedef struct tomo_handle tomo_handle;

/* optional outputs of tomo_forward; any pointer may be NULL */
typedef struct tomo_outputs {
    float *traces;   /* [n_cand][n_tx][n_antennas][steps]  receiver Ez traces      */
    float *D;        /* [n_cand][n_exc][nfreq][n_angles]   far-field magnitude      */
    float *P;        /* [n_cand][n_exc][nfreq][n_angles]   far-field phase          */
    double *fitness; /* [n_cand] (requires a target)                                */
    double *traces_f64; /* as traces, in double (exact copy of FP64 state)         */
} tomo_outputs;

typedef struct tomo_stats {
    double advance_ms;        /* device time of the last batch's time loop (CUDA events)   */
    double total_ms;          /* device time of the last batch, set-up to misfit            */
    double cell_updates;      /* Ez cells x steps advanced in the last batch                */
    int64_t launches;         /* advance-kernel launches in the last batch                  */
    int64_t kernels;          /* all kernels launched in the last batch                     */
    int32_t steps_per_launch; /* T used                                                      */
    int32_t cols_per_lane;    /* COLS used                                                   */
    int64_t h2d_bytes, d2h_bytes;  /* host<->device bytes of the last batch                  */
    double tune_ms;           /* device time the autotuner spent in the last call (0 when
                                 the (T, COLS) choice for this batch size was cached)     */
    int32_t tuned_configs;    /* blockings the autotuner timed in the last call            */
    int32_t min_blocks_per_sm;/* register budget of the advance kernel used (2: 255 regs,
                                 3: 168, 4: 128 per thread)                               */
    /* serving loop, as of the end of the last tomo_serve_step */
    uint64_t serve_bytes_in_use;  /* device bytes held by admitted requests               */
    int32_t serve_running;        /* admitted requests still advancing                    */
    int32_t serve_queued;         /* requests waiting for memory or solve slots           */
    int32_t serve_running_solves; /* solves of the admitted requests                      */
} tomo_stats;

/* ---- presets */
/* Exactly FDTD_common.hxx: 401x401, 2000 steps, 10-cell CPML, 4 plane waves,
   10 frequencies, 100 angles; cpu_variant selects FDTD_CPU.cxx semantics.     */
int tomo_spec_reference(tomo_spec *spec, int cpu_variant);
/* Breast-imaging workloads 0..4 (plain forward solve, batched PSO, precision
   study, serving, large batch). */
int tomo_spec_breast(tomo_spec *spec, int config);
/* One request of the serving workload: the breast phantom (35 mm disc) at 70%
   of a 100 mm square domain of edge x edge cells (dx = 0.1 m / edge), steps =
   4 * edge, n_antennas antennas on the 42 mm ring, every antenna transmitting.
   No counterpart in the reference (its problem size is compiled in,
   FDTD_common.hxx:1-76). */
int tomo_spec_serving(tomo_spec *spec, int edge, int n_antennas);
/* number of candidate parameters the spec expects (27, 162 or 8*n_ellipses) */
int tomo_num_params(const tomo_spec *spec);
/* number of excitations (solves) per candidate */
int tomo_num_excitations(const tomo_spec *spec);

/* ---- lifetime (replaces the per-call cudaMalloc/cudaFree of FDTD_GPU.cu:858-1106) */
int tomo_create(const tomo_spec *spec, tomo_handle **out);
void tomo_destroy(tomo_handle *h);
/* run on this CUDA stream (cudaStream_t passed as void*); NULL = library stream */
int tomo_set_stream(tomo_handle *h, void *stream);
/* device-memory budget for batch and serving state, bytes (0 = 150 GB) */
int tomo_set_memory_budget(tomo_handle *h, uint64_t bytes);

/* ---- targets (the reference compiles them in: FDTD_GPU.cu:996, FDTD_CPU.cxx:789)
   reference modes: n = n_exc*nfreq*n_angles far-field magnitudes;
   breast mode: n = n_tx*n_antennas*steps receiver samples.                     */
int tomo_set_target(tomo_handle *h, const float *target, size_t n);

/* ---- fitness (FDTD_GPU.cu:650-1110 / FDTD_CPU.cxx:669-892)                   */
int tomo_fitness(tomo_handle *h, const double *args, size_t n_args, double *fitness);
/* a whole generation: args is [n_cand][n_param] row-major, fitness is [n_cand] */
int tomo_fitness_batch(tomo_handle *h, const double *args, size_t n_cand, size_t n_param, double *fitness);
/* forward solve with optional traces / far field / fitness */
int tomo_forward(tomo_handle *h, const double *args, size_t n_cand, size_t n_param, const tomo_outputs *out);

/* ---- serving: continuous batching of candidate requests.  There is no
   counterpart in the reference (tao farms candidates over MPI ranks, one
   blocking call per rank, test.cxx:82-121).  Requests are admitted in FIFO
   order as device memory (tomo_set_memory_budget) and solve slots free up;
   every admitted solve advances in the same kernel launches.               */
int tomo_submit(tomo_handle *h, const double *args, size_t n_cand, size_t n_param, uint64_t *ticket);
/* same with a per-request problem spec (e.g. another grid size; same precision) */
int tomo_submit_spec(tomo_handle *h, const tomo_spec *spec, const double *args, size_t n_cand, size_t n_param,
                     uint64_t *ticket);
/* target of requests that carry `spec` (NULL = the handle's spec) */
int tomo_set_target_spec(tomo_handle *h, const tomo_spec *spec, const float *target, size_t n);
/* device bytes a request of n_cand candidates with `spec` (NULL = the handle's
   spec) holds while admitted: what the HBM budget of tomo_set_memory_budget is
   charged.  No counterpart in the reference. */
int tomo_request_bytes(tomo_handle *h, const tomo_spec *spec, size_t n_cand, uint64_t *bytes);
/* advance every admitted solve by one launch; admits queued work first          */
int tomo_serve_step(tomo_handle *h, int *n_active);
/* fitness of a finished ticket (n_cand values), TOMO_ENOTREADY while running.
   A finished, failed or cancelled ticket is reported once (TOMO_OK or its
   status, TOMO_ECANCELLED), then forgotten: polling it again is TOMO_EINVAL.  */
int tomo_poll(tomo_handle *h, uint64_t ticket, double *fitness);
/* bounded wait for one ticket: runs tomo_serve_step until the ticket has
   finished (its result as tomo_poll) or timeout_ms has passed, checked before
   each step (TOMO_ETIMEOUT; the request stays queued or running and can be
   waited for again or cancelled).  The caller of a blocking evaluation per
   request, as tao's workers make one (test.cxx:82-121), uses this instead of
   its own poll loop.                                                           */
int tomo_wait(tomo_handle *h, uint64_t ticket, double timeout_ms, double *fitness);
int tomo_cancel(tomo_handle *h, uint64_t ticket);

/* ---- trace misfit without allocation.  No counterpart in the reference.
   For callers that cannot call cudaMalloc: a host framework whose caching
   allocator owns the device memory, or a latency-critical serving loop that
   must not take the device synchronisation of cudaMalloc/cudaFree.  Computes
   fitness[c] = -sum (s - t)^2 / sum t^2 of n_cand candidates from device
   buffers the caller owns -- traces [n_cand][n_tx][n_per_solve] and target
   [n_tx][n_per_solve] (float), fitness [n_cand] (double) -- asynchronously on
   `stream` (cudaStream_t as void*, NULL = default stream).  The scratch is a
   fixed device array of the library: at most 65536 solves (n_cand * n_tx)
   per call, about 1 MiB that every GPU loading the library holds until exit;
   larger problems return TOMO_EINVAL.  The first call on a device looks the
   array up, so make it before any stream capture; the address is kept for
   the life of the process, so do not call this across a cudaDeviceReset.
   All calls share the array: calls whose kernels overlap on the GPU race and
   must not be issued.  The call is asynchronous and reports no numeric
   status: a non-finite trace or target value gives a NaN or infinite
   fitness for that candidate (check the results; the batch path's
   tomo_forward returns TOMO_ENUMERIC instead). */
int tomo_trace_misfit_static(const float *traces, const float *target, size_t n_cand, size_t n_tx,
                             size_t n_per_solve, double *fitness, void *stream);

int tomo_get_stats(tomo_handle *h, tomo_stats *stats);

/* ---- field snapshots (headless stand-in for the reference's commented-out
   GL field view, FDTD_GPU.cu:23-25,418-422) */
#define TOMO_FIELD_EZ 0   /* (ny+1) x (nx+1) values */
#define TOMO_FIELD_HX 1   /* ny x nx values */
#define TOMO_FIELD_HY 2   /* ny x nx values */
/* Copy the final field `field` of solve (candidate, excitation) of the last
   tomo_forward / tomo_fitness / tomo_fitness_batch call on this handle into
   out (row-major, y then x, as float; n = capacity of out).  The state stays
   on the device until the handle's next batch.  TOMO_ENOTREADY before the
   first batch. */
int tomo_field_snapshot(tomo_handle *h, size_t candidate, int excitation, int field, float *out, size_t n);

/* ---- search drivers: synchronous particle swarm, differential evolution and
   a regression Newton method over whole generations, the drop-in for tao's
   ParticleSwarmMPI / DifferentialEvolutionMPI / AsynchronousNewtonMethod in
   the reference's driver (test.cxx:82-121, `ps(min_bound, max_bound,
   arguments); ps.go(FDTD_GPU)`, `anm(min_bound, max_bound, radius, arguments);
   anm.iterate(FDTD_GPU)`).  One call of the batch fitness function evaluates
   a whole generation; fitness is maximised.  Host code only: runs without a
   GPU when the fitness function needs none. */
enum { TOMO_SEARCH_PS = 0, TOMO_SEARCH_DE = 1, TOMO_SEARCH_ANM = 2 };
typedef struct tomo_search_params {
    int32_t type;                 /* TOMO_SEARCH_PS, TOMO_SEARCH_DE or TOMO_SEARCH_ANM  */
    int32_t population_size;      /* --population_size (>= 4)                            */
    int32_t maximum_iterations;   /* --maximum_iterations (generations after the first)  */
    int32_t number_pairs;         /* DE --number_pairs: difference vectors per donor     */
    uint64_t seed;                /* --seed                                              */
    double inertia;               /* PS --inertia                                        */
    double local_best_weight;     /* PS --local_best_weight                              */
    double global_best_weight;    /* PS --global_best_weight                             */
    double crossover_rate;        /* DE --crossover_rate                                 */
    double differential_scale;    /* DE --differential_scale                             */
    int32_t parent_best;          /* DE --parent_selection: 1 best, 0 random             */
    int32_t reserved;
    /* Newton method: each iteration samples regression_size points within
       radius of the best point so far (one batch), fits a quadratic model by
       least squares, and evaluates line_search_size points c + a s along the
       Newton step s, a from line_search_min to line_search_max (one batch).   */
    const double *radius;         /* ANM per-parameter sampling radius (n_param values);
                                     NULL: a tenth of max_bound - min_bound           */
    int32_t regression_size;      /* ANM --regression_size; 0: twice the model's unknowns */
    int32_t line_search_size;     /* ANM --line_search_size (>= 2)                       */
    double line_search_min;       /* ANM --line_search_min                               */
    double line_search_max;       /* ANM --line_search_max                               */
    int32_t hessian_diagonal;     /* ANM --hessian_diagonal 1: fit only the Hessian's
                                     diagonal (1 + 2k unknowns instead of
                                     1 + k + k(k+1)/2 for k free parameters)          */
    int32_t reserved2;
} tomo_search_params;
/* fitness[i] of population[i*n_param ...], i < n_cand; non-zero return aborts the
   search.  A NaN fitness ranks below every number (-infinity). */
typedef int (*tomo_batch_fitness_fn)(void *user, const double *population, size_t n_cand, size_t n_param,
                                     double *fitness);
/* called after every generation with the best fitness and parameters so far */
typedef void (*tomo_generation_fn)(void *user, int generation, double best_fitness, const double *best_params);
int tomo_search_defaults(tomo_search_params *p, int type);
/* tao-style "--name value" arguments over the defaults; unknown names are skipped */
int tomo_search_parse_args(tomo_search_params *p, int argc, const char *const *argv);
/* best_params: n_param doubles; history (may be NULL): maximum_iterations + 1
   best fitness values, the first after the initial generation (the Newton
   method: its starting point, the bounds' midpoint); evaluations (may be
   NULL): candidates evaluated */
int tomo_search_run(const tomo_search_params *p, const double *min_bound, const double *max_bound, size_t n_param,
                    tomo_batch_fitness_fn f, void *user, tomo_generation_fn report, void *report_user,
                    double *best_params, double *best_fitness, double *history, int64_t *evaluations);
/* the same with tomo_fitness_batch of the handle as f (tomo_num_params
   parameters).  A candidate whose solve diverges (non-finite fitness, which
   tomo_fitness_batch reports as TOMO_ENUMERIC) ranks below every number and
   the search goes on; best_fitness is -infinity when every candidate diverged. */
int tomo_search_fitness(tomo_handle *h, const tomo_search_params *p, const double *min_bound,
                        const double *max_bound, tomo_generation_fn report, void *report_user, double *best_params,
                        double *best_fitness, double *history);

const char *tomo_last_error(void);
const char *tomo_version(void);

#ifdef __cplusplus
}
#endif
#endif
