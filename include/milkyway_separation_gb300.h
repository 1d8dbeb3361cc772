/*
 * milkyway_separation_gb300.h -- C ABI of the GB300 (sm_103a) separation
 * likelihood library, libmwsep_gb300.so.
 *
 * The library is a drop-in for the evaluator slot of the Milkyway@Home
 * separation client: the reference registers an evaluator of type
 *
 *     typedef double (*EvalFunc)(double*, ASTRONOMY_PARAMETERS*,
 *                                EVALUATION_STATE*, STAR_POINTS*);
 *
 * (milkyway_separation/cpu/simple_evaluator.h:26) and calls it once from
 * worker() (src/milkyway_client_app.c:263-278).  mwsep_evaluate() below has
 * that signature and fills EVALUATION_STATE the way cpu_evaluate does.
 *
 * The problem structs are layout-compatible with the reference's
 * (cpu/parameters.h:27-71, cpu/star_points.h:27-31,
 * cpu/evaluation_state.h:30-58).  They are defined here under the reference
 * headers' own include guards, so a translation unit may include either the
 * reference headers or this one first; whichever comes first defines them.
 *
 * Every function except the EvalFunc-shaped ones returns an int status
 * (MWSEP_OK == 0).  The library never calls exit(); the EvalFunc-shaped
 * entry points return NaN on failure and record the status, readable with
 * mwsep_last_error().  All device work runs on one GPU.  There is no CPU
 * fallback: without a usable sm_103a device every call fails with
 * MWSEP_ERR_CUDA.
 */
#ifndef MILKYWAY_SEPARATION_GB300_H
#define MILKYWAY_SEPARATION_GB300_H

#include <stddef.h>
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ */
/* Reference problem structs (layout-compatible)                       */
/* ------------------------------------------------------------------ */

#ifndef ASTRONOMY_PARAMETERS_H
#define ASTRONOMY_PARAMETERS_H
/* cpu/parameters.h:27-35 */
typedef struct
{
    double r_min, r_max, r_step_size;
    double nu_min, nu_max, nu_step_size;
    double mu_min, mu_max, mu_step_size;
    int r_steps, nu_steps, mu_steps;

    long min_calculation, max_calculation;
} INTEGRAL;

/* cpu/parameters.h:37-71 */
typedef struct
{
    double parameters_version;

    int number_background_parameters;
    double background_weight;
    /* number_background_parameters values; at least 7 when aux_bg_profile
     * is 1, whose a, b, c are values 4..6 whatever
     * number_background_parameters says (as init_constants reads them) */
    double* background_parameters;
    double* background_step;
    double* background_min;
    double* background_max;
    int* background_optimize;

    int number_streams;
    int number_stream_parameters;

    double* stream_weights;
    double* stream_weight_step;
    double* stream_weight_min;
    double* stream_weight_max;
    int* stream_weight_optimize;

    double** stream_parameters;
    double** stream_step;
    double** stream_min;
    double** stream_max;
    int** stream_optimize;

    int convolve;
    int sgr_coordinates;
    int aux_bg_profile;
    int wedge;

    int number_integrals;
    INTEGRAL** integral;
} ASTRONOMY_PARAMETERS;
#endif

#ifndef _STAR_POINTS_H_
#define _STAR_POINTS_H_
/* cpu/star_points.h:27-31: stars[i] = {l (deg), b (deg), r (kpc)} */
typedef struct star_points
{
    int number_stars;
    double** stars;
} STAR_POINTS;
#endif

#ifndef _EVALUATION_STATE_H_
#define _EVALUATION_STATE_H_
/* cpu/evaluation_state.h:30-41 */
typedef struct integral_area
{
    int mu_steps, nu_steps, r_steps;
    double mu_min, nu_min, r_min;
    double mu_max, nu_max, r_max;
    double mu_step_size, nu_step_size, r_step_size;

    long min_calculation, max_calculation, current_calculation;

    int number_streams;
    double background_integral, *stream_integrals;
} INTEGRAL_AREA;

/* cpu/evaluation_state.h:43-58 */
typedef struct evaluation_state
{
    INTEGRAL_AREA** integral;
    int current_integral, number_streams, number_integrals;

    double background_integral;
    double* stream_integrals;

    int current_star_point, total_stars;
    int num_zero;
    int bad_jacobians;
    double prob_sum;
} EVALUATION_STATE;
#endif

#ifndef _SIMPLE_EVALUATOR_H_
/* cpu/simple_evaluator.h:26 */
typedef double (*EvalFunc)(double*, ASTRONOMY_PARAMETERS*, EVALUATION_STATE*, STAR_POINTS*);
#endif

/* ------------------------------------------------------------------ */
/* Status codes and limits                                             */
/* ------------------------------------------------------------------ */

enum
{
    MWSEP_OK = 0,
    MWSEP_ERR_ARG = 1,        /* NULL pointer, bad size, bad enum          */
    MWSEP_ERR_IO = 2,         /* file missing or unparsable                */
    MWSEP_ERR_PARAM_COUNT = 3,/* theta length != optimised-parameter count */
    MWSEP_ERR_UNSUPPORTED = 4,/* outside MWSEP_MAX_* limits                */
    MWSEP_ERR_CUDA = 5,       /* CUDA runtime error / no sm_103a device    */
    MWSEP_ERR_NOMEM = 6,      /* host or device allocation failed          */
    MWSEP_ERR_BUDGET = 7,     /* request exceeds the context HBM budget    */
    MWSEP_ERR_TIMEOUT = 8,    /* a bounded wait ran out                    */
    MWSEP_ERR_CANCELLED = 9,  /* serving request cancelled before launch   */
    MWSEP_ERR_STATE = 10,     /* call out of order (no problem / no stars) */
    MWSEP_ERR_BUSY = 11       /* serving: the admission queue is full      */
};

#define MWSEP_MAX_STREAMS 8
#define MWSEP_MAX_AREAS 8
#define MWSEP_MAX_CONVOLVE 512
#define MWSEP_MAX_BG_PARAMS 8
#define MWSEP_MAX_STREAM_PARAMS 8

/* Arithmetic of one evaluation. */
enum
{
    /* FP64 end to end, the reference's cell and convolution order.  The
     * drop-in form: within 1e-12 relative of the reference on each
     * integral and 1e-12 absolute on the log-likelihood. */
    MWSEP_PLAIN_F64 = 0,
    /* Densities and exp in FP32 (SFU) with compensated per-thread sums;
     * geometry, tables, cross-block sums, normalisation and the
     * log-likelihood in FP64.  Within 1e-7 absolute on the log-likelihood. */
    MWSEP_MIXED_F32 = 1,
    /* The plain form's accuracy (1e-12 relative on the integrals) computed in
     * double-float arithmetic -- pairs of FP32 values, about 48 bits -- on
     * the FP32 pipes, which GB300 runs ~74x faster than FP64.  Every
     * background form; the likelihood in double-float up to 4 streams, in
     * FP64 beyond.
     * Single-wedge evaluations and
     * batches, engine requests (each wedge's requests as one batch), the
     * server and the gradient/Hessian calls; the engine autotuner takes the
     * other two forms. */
    MWSEP_PLAIN_DF = 2
};

const char* mwsep_status_string(int status);
/* Status of the most recent failing call on this thread (0 if none). */
int mwsep_last_error(void);
/* Library build/version string. */
const char* mwsep_version(void);
/* ------------------------------------------------------------------ */
/* Problem I/O, same file formats and semantics as the reference        */
/* ------------------------------------------------------------------ */

/* Replaces read_astronomy_parameters (cpu/parameters.c:61-91) and
 * fread_astronomy_parameters (:107-228).  Fills *ap with heap arrays; free
 * them with mwsep_free_parameters. */
int mwsep_read_astronomy_parameters(const char* path, ASTRONOMY_PARAMETERS* ap);
/* Replaces write_astronomy_parameters (cpu/parameters.c:93-105, 230-305). */
int mwsep_write_astronomy_parameters(const char* path, const ASTRONOMY_PARAMETERS* ap);
/* Replaces free_parameters (cpu/parameters.c:27-59). */
void mwsep_free_parameters(ASTRONOMY_PARAMETERS* ap);
/* Replaces get_optimized_parameter_count (cpu/parameters.c:307-330). */
int mwsep_get_optimized_parameter_count(const ASTRONOMY_PARAMETERS* ap);
/* Replaces set_astronomy_parameters (cpu/parameters.c:332-363). */
int mwsep_set_astronomy_parameters(ASTRONOMY_PARAMETERS* ap, const double* parameters);
/* Replaces get_search_parameters (cpu/parameters.c:365-397); out holds
 * get_optimized_parameter_count doubles. */
int mwsep_get_search_parameters(const ASTRONOMY_PARAMETERS* ap, double* out);
/* Replace get_step, get_min_parameters, get_max_parameters
 * (cpu/parameters.c:399-500): the step / bounds of each optimised
 * parameter in theta order; out holds get_optimized_parameter_count doubles. */
int mwsep_get_step(const ASTRONOMY_PARAMETERS* ap, double* out);
int mwsep_get_min_parameters(const ASTRONOMY_PARAMETERS* ap, double* out);
int mwsep_get_max_parameters(const ASTRONOMY_PARAMETERS* ap, double* out);
/* Replaces split_astronomy_parameters (cpu/parameters.c:502-522), without
 * its printf. */
int mwsep_split_astronomy_parameters(ASTRONOMY_PARAMETERS* ap, int rank, int max_rank);

/* Replaces read_star_points (cpu/star_points.c:26-52, 69-81). */
int mwsep_read_star_points(const char* path, STAR_POINTS* sp);
/* Replaces write_star_points (cpu/star_points.c:54-67, 83-93). */
int mwsep_write_star_points(const char* path, const STAR_POINTS* sp);
/* Replaces free_star_points (cpu/star_points.c:95-103). */
void mwsep_free_star_points(STAR_POINTS* sp);
/* Replaces split_star_points (cpu/star_points.c:105-131). */
int mwsep_split_star_points(STAR_POINTS* sp, int rank, int max_rank);

/* Binary forms of the two input files (no reference counterpart: the
 * reference reads text only).  A star catalogue is a 64-byte header
 * ("MWSEPCAT", version 1, n, column offsets, file size) and three
 * 64-byte-aligned little-endian double columns l[n], b[n], r[n]; a parameter
 * file is "MWSEPPAR", version 1, the ASTRONOMY_PARAMETERS fields in
 * declaration order and an FNV-1a checksum.  Malformed or truncated files
 * give MWSEP_ERR_IO. */
typedef struct
{
    int number_stars;
    const double* l; /* degrees */
    const double* b; /* degrees */
    const double* r; /* kpc */
    void* map;       /* the read-only mapping; release with mwsep_unmap_star_catalogue */
    size_t map_bytes;
} mwsep_star_catalogue;

int mwsep_write_star_catalogue(const char* path, int n, const double* l, const double* b, const double* r);
int mwsep_write_star_points_binary(const char* path, const STAR_POINTS* sp);
/* Map a catalogue read-only: the columns point into the mapping. */
int mwsep_map_star_catalogue(const char* path, mwsep_star_catalogue* out);
int mwsep_unmap_star_catalogue(mwsep_star_catalogue* cat);
/* Read a binary catalogue into the reference's row layout. */
int mwsep_read_star_points_binary(const char* path, STAR_POINTS* sp);
int mwsep_write_astronomy_parameters_binary(const char* path, const ASTRONOMY_PARAMETERS* ap);
/* Free the result with mwsep_free_parameters. */
int mwsep_read_astronomy_parameters_binary(const char* path, ASTRONOMY_PARAMETERS* ap);

/* Replaces initialize_state (cpu/evaluation_state.c:153-176). */
int mwsep_initialize_state(const ASTRONOMY_PARAMETERS* ap, const STAR_POINTS* sp, EVALUATION_STATE* es);
/* Replaces free_state (cpu/evaluation_state.c:201-211). */
void mwsep_free_state(EVALUATION_STATE* es);

/* ------------------------------------------------------------------ */
/* EvalFunc drop-ins                                                    */
/* ------------------------------------------------------------------ */

/* Plain FP64 evaluation on the GPU.  Replaces cpu_evaluate
 * (cpu/evaluation_optimized.c:756-784) and cuda_evaluate
 * (cuda/evaluation_gpu6.cu:1058-1106, cuda/evaluation_gpu.h:34-37).
 * Applies parameters to *ap (set_astronomy_parameters), evaluates every
 * integral area and every star, writes es->integral[i]->*_integral,
 * es->background_integral, es->stream_integrals[], es->prob_sum,
 * es->num_zero, and returns prob_sum / number_stars.  The caller subtracts
 * 3.0 as worker() does (src/milkyway_client_app.c:278).  Does not need
 * init_constants.  Each call uploads the catalogue and rebuilds the wedge
 * tables (no state kept between calls besides device buffers).  Returns NaN
 * on failure (see mwsep_last_error). */
double mwsep_evaluate(double* parameters, ASTRONOMY_PARAMETERS* ap, EVALUATION_STATE* es, STAR_POINTS* sp);

/* Same contract in the compensated-FP32 form (MWSEP_MIXED_F32).  Replaces
 * the same reference entry points for callers that accept 1e-7 on the
 * log-likelihood. */
double mwsep_evaluate_mixed(double* parameters, ASTRONOMY_PARAMETERS* ap, EVALUATION_STATE* es, STAR_POINTS* sp);

/* Same contract in the double-float form (MWSEP_PLAIN_DF): the plain form's
 * bounds (1e-12 relative on the integrals, 1e-12 absolute on the
 * log-likelihood) at about 12x its speed; problems outside that form's
 * coverage are evaluated as mwsep_evaluate does. */
double mwsep_evaluate_df(double* parameters, ASTRONOMY_PARAMETERS* ap, EVALUATION_STATE* es, STAR_POINTS* sp);

/* The two per-rank steps of the reference's distributed evaluation, which
 * its MPI worker registers (cpu/mpi_astronomy.c:79-80), same signatures,
 * plain FP64.  mwsep_integral_f replaces integral_f
 * (cpu/astronomy_worker.c:33-64): applies parameters to *ap, integrates this
 * rank's cells of every area (es->integral[i]'s [min_calculation,
 * max_calculation), after split_astronomy_parameters and initialize_state)
 * and writes the cut-subtracted background and stream integrals to
 * results[0..S] and into es.  The ranks' results summed
 * (integral_compose, :67-92) are the whole evaluation's integrals.
 * mwsep_likelihood_f replaces likelihood_f (:94-121): calculate_likelihood of
 * this rank's stars (after split_star_points) at *ap's current parameters
 * against the given integrals[0..S]; results[0] = prob_sum, results[1] =
 * bad_jacobians (always 0).  likelihood_compose (:123-143) of every rank's
 * results is the whole evaluation's log-likelihood.  On failure the results
 * hold NaN and mwsep_last_error() says why. */
void mwsep_integral_f(double* parameters, double* results, ASTRONOMY_PARAMETERS* ap, EVALUATION_STATE* es,
                      STAR_POINTS* sp);
void mwsep_likelihood_f(double* integrals, double* results, ASTRONOMY_PARAMETERS* ap, EVALUATION_STATE* es,
                        STAR_POINTS* sp);

/* ------------------------------------------------------------------ */
/* Context API: resident wedges and catalogues, batches                 */
/* ------------------------------------------------------------------ */

typedef struct mwsep_ctx mwsep_ctx;

/* One evaluation's results.  likelihood = prob_sum/N - 3.0 (the value the
 * reference client prints as <search_likelihood>). */
typedef struct
{
    double likelihood;
    double prob_sum;
    int num_zero;
    int number_streams;
    int number_integrals;
    int status;
    double background_integral;
    double stream_integrals[MWSEP_MAX_STREAMS];
    double area_integrals[MWSEP_MAX_AREAS][1 + MWSEP_MAX_STREAMS];
    /* <background_only_likelihood>, <stream_only_likelihood> diagnostics
     * (cpu/evaluation_optimized.c:719-733), already minus 3.0 */
    double background_only_likelihood;
    double stream_only_likelihood[MWSEP_MAX_STREAMS];
} mwsep_result;

/* Create a context on CUDA device `device` (one stream, one GPU). */
int mwsep_ctx_create(int device, mwsep_ctx** out);
int mwsep_ctx_destroy(mwsep_ctx* ctx);

/* Make the wedge description of *ap resident: integral areas, convolve,
 * coordinate system, wedge, aux profile and the theta layout (optimize
 * flags).  Builds the per-(mu,nu) geometry and r-bin tables on the device.
 * Replaces any previous problem. */
int mwsep_ctx_set_problem(mwsep_ctx* ctx, const ASTRONOMY_PARAMETERS* ap);
/* Make a catalogue resident (rows {l, b, r_kpc}) and build its per-star
 * convolution tables on the device. */
int mwsep_ctx_set_stars(mwsep_ctx* ctx, const STAR_POINTS* sp);
int mwsep_ctx_set_stars_soa(mwsep_ctx* ctx, int n, const double* l, const double* b, const double* r);
/* Make a catalogue file resident: a binary catalogue is mapped and its
 * columns uploaded as they lie; anything else is read as the reference's
 * text star file. */
int mwsep_ctx_set_stars_file(mwsep_ctx* ctx, const char* path);

/* Number of theta values the resident problem expects. */
int mwsep_ctx_theta_count(const mwsep_ctx* ctx);

/* One evaluation of theta (mwsep_ctx_theta_count doubles) in `precision`. */
int mwsep_ctx_evaluate(mwsep_ctx* ctx, const double* theta, int precision, mwsep_result* out);

/* The two phases of one evaluation of wedge 0 separately, for an evaluation
 * sharded over ranks as the reference's distributed client does it
 * (integral_f / likelihood_f, cpu/astronomy_worker.c:33-121).
 * mwsep_ctx_integrals integrates the resident problem's cells (each area's
 * [min_calculation, max_calculation)) and needs no catalogue; out's
 * likelihood fields are NaN.  mwsep_ctx_likelihood evaluates the resident
 * catalogue against given cut-subtracted integrals (1 + S doubles:
 * background, then streams -- e.g. the sum of every rank's); out carries the
 * given integrals and zero area integrals.  Each gives the bits of the same
 * phase of mwsep_ctx_evaluate. */
int mwsep_ctx_integrals(mwsep_ctx* ctx, const double* theta, int precision, mwsep_result* out);
int mwsep_ctx_likelihood(mwsep_ctx* ctx, const double* theta, const double* integrals, int precision,
                         mwsep_result* out);

/* A population: n_theta vectors, row-major [n_theta][theta_count], evaluated
 * together (one batched launch per phase).  out[n_theta].  Each result is
 * the same as that theta evaluated alone. */
int mwsep_ctx_evaluate_batch(mwsep_ctx* ctx, int n_theta, const double* thetas, int precision, mwsep_result* out);

/* Bytes of device memory the context holds (tables, catalogue, scratch). */
int mwsep_ctx_device_bytes(const mwsep_ctx* ctx, size_t* out);

/* Per-phase device time of the last evaluate/evaluate_batch call, measured
 * with CUDA events on the context stream, in milliseconds:
 * out[0] integral kernels, out[1] integral reduction, out[2] likelihood
 * kernels, out[3] likelihood reduction, out[4] whole call. */
int mwsep_ctx_last_timings(const mwsep_ctx* ctx, double* out5);

/* Number of kernel launches issued by the last evaluate/evaluate_batch. */
int mwsep_ctx_last_launches(const mwsep_ctx* ctx, int* out);

/* ---- Many resident wedges, one launch per phase for a whole batch ---- */

/* Make another wedge (problem + catalogue) resident; *wedge_id receives its
 * id.  The single-problem calls above work on wedge 0.  Fails with
 * MWSEP_ERR_BUDGET when a device-memory budget is set and the wedge would
 * exceed it. */
int mwsep_ctx_add_wedge(mwsep_ctx* ctx, const ASTRONOMY_PARAMETERS* ap, const STAR_POINTS* sp, int* wedge_id);
/* theta length of a resident wedge (negative status on error). */
int mwsep_ctx_wedge_theta_count(const mwsep_ctx* ctx, int wedge_id);
/* Device bytes a resident wedge holds (tables + catalogue). */
int mwsep_ctx_wedge_bytes(const mwsep_ctx* ctx, int wedge_id, size_t* out);
/* Density points one evaluation of a resident wedge computes: cells x
 * convolve over the cells its areas integrate, plus stars x convolve (the
 * work unit of the throughput figures; a scheduler's cost estimate). */
int mwsep_ctx_wedge_points(const mwsep_ctx* ctx, int wedge_id, double* out);
/* Cap the context's device memory (0 = no cap). */
int mwsep_ctx_set_hbm_budget(mwsep_ctx* ctx, size_t bytes);

/* One evaluation request: a resident wedge and its parameter vector. */
typedef struct
{
    int wedge;
    const double* theta;
} mwsep_request;

/* Evaluate n requests over any resident wedges in `precision`.  All
 * requests of up to 4 streams run in one persistent launch per phase (5..8
 * streams in a second), blocks taking (request, area, item-run) tiles from a
 * global counter; the launch sequence is a captured CUDA graph, replayed
 * while the batch fits the engine's buffers.  Each result is the same as that
 * request evaluated alone (its reduction order depends on its wedge's tile
 * shape only).  out[n]. */
int mwsep_ctx_evaluate_requests(mwsep_ctx* ctx, int n, const mwsep_request* reqs, int precision, mwsep_result* out);

/* The autotuner: time candidate tile shapes (r-bins per item, items per
 * tile) for one wedge and precision and keep the fastest; *predicted_ms is
 * the predicted integral time of one evaluation with the chosen shape.  For
 * MWSEP_PLAIN_DF (whose requests run per wedge, not in the engine) it times
 * whole single evaluations over candidate r-chunks, and *predicted_ms is
 * the chosen one's measured integral time. */
int mwsep_ctx_autotune(mwsep_ctx* ctx, int wedge_id, int precision, double* predicted_ms);
/* The tile shape a wedge uses for one precision. */
int mwsep_ctx_wedge_tile_shape(const mwsep_ctx* ctx, int wedge_id, int precision, int* k_chunk, int* tile_items);
/* ---- Serving: continuous batching over the resident wedges ---- */

typedef struct mwsep_server mwsep_server;

typedef struct
{
    int lanes;             /* execution lanes (own stream + engine buffers each); default 2 */
    int max_batch;         /* requests per engine batch; default 256 */
    size_t lane_hbm_bytes; /* device-memory share of each lane's batch buffers (0 = no cap);
                              a batch that would exceed it is split until it fits */
    double target_batch_ms; /* a lane stops adding requests to a batch once their predicted
                               device time passes this (0 = no time cap); predictions are
                               points per evaluation x the time per point the lanes measure */
    long long max_queued;   /* admission: submit refuses with MWSEP_ERR_BUSY while this many
                               requests wait (0 = unbounded) */
} mwsep_server_config;

typedef struct
{
    long long completed, failed, cancelled, batches, queued;
    double mean_batch;
    double p50_latency_s, p99_latency_s, max_latency_s; /* submit -> result */
    double evals_per_s;                                 /* completed / (last result - first submit) */
    long long refused;                                  /* submits refused by admission (MWSEP_ERR_BUSY) */
    long long max_queue;                                /* most requests waiting at once */
} mwsep_server_stats;

/* Start serving the wedges resident in ctx (add them first; the server
 * snapshots the set).  cfg may be NULL for the defaults.  While the server
 * runs, ctx itself must not evaluate or change its wedges. */
int mwsep_server_create(mwsep_ctx* ctx, const mwsep_server_config* cfg, mwsep_server** out);
/* Queue one evaluation; returns at once with its id. */
int mwsep_server_submit(mwsep_server* s, int wedge_id, const double* theta, int precision, unsigned long long* id);
/* Wait up to timeout_s for a request's result (MWSEP_ERR_TIMEOUT when the
 * time runs out; the request stays pending and can be waited on again). */
int mwsep_server_wait(mwsep_server* s, unsigned long long id, double timeout_s, mwsep_result* out);
/* Cancel a request that has not started; its wait returns MWSEP_ERR_CANCELLED.
 * A request already on the GPU cannot be cancelled (MWSEP_ERR_STATE). */
int mwsep_server_cancel(mwsep_server* s, unsigned long long id);
int mwsep_server_get_stats(mwsep_server* s, mwsep_server_stats* out);
int mwsep_server_reset_stats(mwsep_server* s);
/* Stop: queued requests are cancelled, running batches finish. */
int mwsep_server_destroy(mwsep_server* s);

/* Bytes the context has copied host->device and device->host since it was
 * created (tables, catalogue, constants, results). */
int mwsep_ctx_transfer_bytes(const mwsep_ctx* ctx, size_t* h2d, size_t* d2h);

/* Bytes copied host->device and device->host by the most recent
 * mwsep_evaluate / _mixed / _df call on this process. */
int mwsep_evalfunc_transfer_bytes(size_t* h2d, size_t* d2h);

/* ------------------------------------------------------------------ */
/* Separation output                                                    */
/* ------------------------------------------------------------------ */

/* Totals of one separation (milkyway_separation/cpu/separation.c:37-254). */
typedef struct
{
    int number_streams;
    double likelihood;                            /* of the evaluation behind it */
    double background_integral;
    double stream_integrals[MWSEP_MAX_STREAMS];
    double expected[MWSEP_MAX_STREAMS];           /* sum over stars of sprob (:193-196) */
    long long assigned[MWSEP_MAX_STREAMS];        /* stars drawn into each stream */
    long long background_assigned;                /* stars drawn into the background */
} mwsep_separation_summary;

/* Separate wedge 0's catalogue at theta: replaces the per-star loop of
 * separation() (cpu/separation.c:150-234), which the reference builds no
 * more.  Evaluates the integrals (plain FP64), then per star:
 *   sprob[N][S]      psg_s / (sum psg + pbx), with epsilon_s = e^{w_s} /
 *                    (1 + sum e^{w}), epsilon_b = 1 / (1 + sum e^{w}) (:128-196);
 *   assignment[N]    0 for the background, k for stream k (1-based), drawn
 *                    against the cumulative sprob (probability.c:310-397 prob_ok);
 *                    the draw is SplitMix64(seed, star) / 2^53 instead of the
 *                    reference's clock-seeded drand48, so it repeats for a seed;
 *   xyz[N][3]        the star in the stripe frame: lbr -> xyz, to (l, b,
 *                    magnitude - 11), back to xyz, shifted by the Sun, rotated
 *                    by mwsep_stripe_transform (:75-116, :226-227).
 * Any output may be NULL.  Up to MWSEP_MAX_STREAMS streams. */
int mwsep_ctx_separation(mwsep_ctx* ctx, const double* theta, unsigned long long seed, double* sprob,
                         int* assignment, double* xyz, mwsep_separation_summary* summary);

/* The stripe-frame rotation (row-major 3x3) taking the stripe's normal onto
 * the z axis: stripe_normal or sgr_stripe_normal (cpu/stCoords.c:142-174),
 * then get_transform (cpu/stVector.c:109-137).  Host only. */
int mwsep_stripe_transform(int sgr_coordinates, int wedge, double* mat9);

/* Write separation()'s output file (cpu/separation.c:229): one line
 * "<stream> <x> <y> <z>" per star, stream 0 for the background. */
int mwsep_write_separation(const char* path, int n, const int* assignment, const double* xyz);

/* ------------------------------------------------------------------ */
/* Optimiser-side consumers: finite differences and parameter errors    */
/* ------------------------------------------------------------------ */

/* Central finite differences of f = likelihood (prob_sum/N - 3) of one
 * resident wedge at theta with per-parameter steps (mwsep_get_step), all
 * points evaluated as engine batches.  Replace get_hessian of the search
 * library that cpu/errors.c:47 and the gradient searches of
 * cpu/mpi_astronomy.c:96-124 call (that library is not part of the
 * reference):
 *   gradient[i]  = (f(x+h_i e_i) - f(x-h_i e_i)) / (2 h_i)
 *   hessian[i*P+i] = ((f(x+h_i e_i) - f0) + (f(x-h_i e_i) - f0)) / h_i^2
 *   hessian[i*P+j] = ((f(++) - f(+-)) - (f(-+) - f(--))) / (4 h_i h_j)
 * 2P+1 (gradient) or 2P^2+1 (Hessian) evaluations.  Outputs may be NULL. */
int mwsep_ctx_gradient(mwsep_ctx* ctx, int wedge, const double* theta, const double* step, int precision,
                       double* f0, double* gradient);
int mwsep_ctx_hessian(mwsep_ctx* ctx, int wedge, const double* theta, const double* step, int precision,
                      double* f0, double* gradient, double* hessian);

/* matrix_invert (util/matrix.c:234-319): LU with partial pivoting, one
 * solve per unit vector; row-major n x n.  MWSEP_ERR_ARG when singular. */
int mwsep_invert_matrix(int n, const double* a, double* inverse);
/* errors() (cpu/errors.c:38-84): sigma = hessian^-1 / number_stars,
 * stddev[i] = sqrt(|sigma_ii|).  Host only. */
int mwsep_errors_from_hessian(int n, const double* hessian, int number_stars, double* sigma, double* stddev);
/* errors()'s output file: the Hessian (" %.20lf"), SIGMA and the errors. */
int mwsep_write_errors(const char* path, int n, const double* hessian, const double* sigma, const double* stddev);

/* ------------------------------------------------------------------ */
/* Allocation-free area integral                                        */
/* ------------------------------------------------------------------ */

/* Device tables of one integral area, in the quantities the reference's
 * cpu__r_constants and calculate_probabilities use.  All pointers are device
 * memory on the calling thread's current device, owned by the caller,
 * 8-byte aligned; tables are row-major. */
typedef struct
{
    int mu_steps, nu_steps, r_steps, convolve;
    const double* geom;        /* [mu_steps*nu_steps][4]: sin(b), cos(b), sin(l), cos(l) of each
                                  (mu, nu) column centre, (l, b) in degrees divided by 180/pi */
    const double* r_point;     /* [r_steps][convolve] */
    const double* qw_r3_N;     /* [r_steps][convolve] */
    const double* r_in_mag;    /* [r_steps][convolve], read only when aux_bg_profile == 1 */
    const double* r_in_mag2;   /* [r_steps][convolve], read only when aux_bg_profile == 1 */
    const double* reff_xr_rp3; /* [r_steps] */
    const double* irv;         /* [r_steps] */
    const double* ids;         /* [nu_steps] */
    /* The cells integrated, as INTEGRAL_AREA's (cpu/evaluation_state.h:30-41):
     * [min_calculation, max_calculation) of the linearised index
     * (mu * nu_steps + nu) * r_steps + r -- 0 and mu_steps * nu_steps * r_steps
     * for the whole area, a rank's share after split_astronomy_parameters.
     * As calculate_integral does (cpu/evaluation_optimized.c:521-527), a
     * range with max_calculation <= min_calculation still integrates the cell
     * min_calculation; a negative min_calculation is MWSEP_ERR_ARG. */
    long min_calculation, max_calculation;
} mwsep_area_tables;

/* The density constants of one evaluation (init_constants' results). */
typedef struct
{
    double alpha, q, r0, delta;
    int aux_bg_profile;        /* 0 or 1 */
    double bg_a, bg_b, bg_c;   /* used when aux_bg_profile == 1 */
    int number_streams;        /* 0 .. MWSEP_MAX_STREAMS */
    double stream_sigma[MWSEP_MAX_STREAMS];
    double stream_a[MWSEP_MAX_STREAMS][3];
    double stream_c[MWSEP_MAX_STREAMS][3];
} mwsep_density_params;

/* Size of the fixed device array the allocation-free entry point works in. */
#define MWSEP_NOALLOC_SCRATCH_BYTES (256 * 1024)

/* Plain-FP64 background and stream integrals of one area (of its cells
 * [min_calculation, max_calculation)), written to d_integrals (device memory
 * on the current device, 8-byte aligned, 1 + number_streams doubles), for
 * callers that cannot
 * let a library allocate device memory: programs that give all device
 * memory to their own pool, hot paths where a cudaMalloc would synchronise
 * the device, loops that must not fail on allocation once running.  No
 * counterpart in the reference (its evaluators allocate per call).
 *
 * The call allocates nothing.  Its only working memory besides the caller's
 * buffers is a fixed MWSEP_NOALLOC_SCRATCH_BYTES array inside the library
 * image, which every GPU that loads the library holds until the process
 * exits.  The first call on a device looks that array up (once per device):
 * make that first call before any stream capture.  Calls share the array, so
 * calls that overlap on the GPU (different streams, or threads) race; order
 * them on one stream.  Work is queued on `stream` (a cudaStream_t; NULL is
 * the legacy default stream) and the call returns without waiting; the
 * result is in d_integrals when that stream reaches it.  number_streams above
 * MWSEP_MAX_STREAMS or convolve above MWSEP_MAX_CONVOLVE is rejected with
 * MWSEP_ERR_UNSUPPORTED. */
int mwsep_area_integrals_noalloc(const mwsep_area_tables* tables, const mwsep_density_params* params,
                                 double* d_integrals, void* stream);

/* ------------------------------------------------------------------ */
/* Pipe microbenchmark                                                  */
/* ------------------------------------------------------------------ */

/* Measured arithmetic-pipe throughput of one GPU: the denominators of the
 * kernels' roofline fractions (the plain form is bound by the FP64 pipe,
 * the compensated form by the FP32 pipe and the SFU). */
typedef struct
{
    double fp64_fma_tflops;  /* 2 flops per DFMA */
    double fp32_fma_tflops;  /* 2 flops per FFMA */
    double ex2_gops;         /* ex2.approx.f32 per second, 1e9 */
    double rsqrt_gops;       /* rsqrt.approx.f32 */
    double rcp_gops;         /* rcp.approx.f32 */
    int sm_count;
} mwsep_pipe_peaks;

int mwsep_measure_pipe_peaks(int device, mwsep_pipe_peaks* out);

#ifdef __cplusplus
}
#endif

#endif /* MILKYWAY_SEPARATION_GB300_H */
