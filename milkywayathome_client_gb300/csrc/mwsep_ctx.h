/* mwsep_ctx.h -- host-side state of a device context (internal).
 *
 * A context owns one CUDA stream on one GPU and any number of resident
 * wedges.  A wedge is one problem (its integral areas and the device tables
 * built from them) plus its catalogue (the per-star tables).  The plain
 * single-problem API works on wedge 0; the engine evaluates requests that
 * name any wedge.
 */
#ifndef MWSEP_CTX_H
#define MWSEP_CTX_H

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdio.h>
#include <stdlib.h>

#include <vector>

#include "milkyway_separation_gb300.h"
#include "mwsep_internal.h"
#include "mwsep_status.h"

#define CU(call)                                                                                           \
    do                                                                                                     \
    {                                                                                                      \
        cudaError_t e_ = (call);                                                                           \
        if (e_ != cudaSuccess)                                                                             \
        {                                                                                                  \
            if (getenv("MWSEP_DEBUG"))                                                                     \
                fprintf(stderr, "mwsep: %s failed: %s (%s:%d)\n", #call, cudaGetErrorString(e_), __FILE__, \
                        __LINE__);                                                                         \
            return mwsep_fail(MWSEP_ERR_CUDA);                                                             \
        }                                                                                                  \
    } while (0)

#define CK(expr)                                                                                           \
    do                                                                                                     \
    {                                                                                                      \
        int s_ = (expr);                                                                                   \
        if (s_ != 0)                                                                                       \
        {                                                                                                  \
            if (getenv("MWSEP_DEBUG"))                                                                     \
                fprintf(stderr, "mwsep: %s failed: %d (%s:%d)\n", #expr, s_, __FILE__, __LINE__);          \
            return mwsep_fail(MWSEP_ERR_CUDA);                                                             \
        }                                                                                                  \
    } while (0)

namespace mwsep {

/* An NVTX range over a host-side phase (a no-op unless a profiler listens). */
struct Range
{
    explicit Range(const char* name) { nvtxRangePushA(name); }
    ~Range() { nvtxRangePop(); }
    Range(const Range&) = delete;
    Range& operator=(const Range&) = delete;
};

/* A grow-only device buffer; `total` tracks the context's device bytes. */
struct DevBuf
{
    void* p = nullptr;
    size_t bytes = 0;
    int ensure(size_t want, size_t& total);
    void release(size_t& total);
    template <typename T> T* as() const { return (T*)p; }
};

/* A grow-only pinned host buffer. */
struct HostPinned
{
    void* p = nullptr;
    size_t bytes = 0;
    int ensure(size_t want);
    void release();
    template <typename T> T* as() const { return (T*)p; }
};

/* Host description of one integral area. */
struct AreaHost
{
    int mu_steps, nu_steps, r_steps;
    double mu_min, mu_max, nu_min, nu_max, r_min, r_max;
    double mu_step, nu_step, r_step;
    /* the cells integrated: [cell_begin, cell_end) of the linearised index,
     * from INTEGRAL's [min_calculation, max_calculation) (mwsep::effective_slice) */
    long long cell_begin, cell_end;
};

struct AreaDev
{
    DevBuf geom, r_point, qw, r_in_mag, r_in_mag2, reff, irv, ids, nus, pts, ptsdf;
    mwsep_area_dev view{};
};

/* The theta layout and the fixed values of a problem (a private copy of
 * the reference struct's values). */
struct ProblemHost
{
    int n_bg = 0, n_streams = 0, n_sparams = 0;
    double bg_weight = 0.0;
    double bg[MWSEP_MAX_BG_PARAMS] = {};
    int bg_opt[MWSEP_MAX_BG_PARAMS] = {};
    double st_weight[MWSEP_MAX_STREAMS] = {};
    int st_weight_opt[MWSEP_MAX_STREAMS] = {};
    double st[MWSEP_MAX_STREAMS][MWSEP_MAX_STREAM_PARAMS] = {};
    int st_opt[MWSEP_MAX_STREAMS][MWSEP_MAX_STREAM_PARAMS] = {};
    int convolve = 0, sgr = 0, aux = 0, wedge = 0;
    int n_areas = 0;
    AreaHost area[MWSEP_MAX_AREAS];
    int n_theta = 0;
};

/* Launch shapes of one precision for one wedge. */
struct Tune
{
    int block = 256;
    int grid = 0;       /* grid-stride kernels: persistent grid */
    int k_chunk = 0;    /* r-bins per item */
    int lk_block = 256;
    int lk_grid = 0;
    int tile_items = 0; /* engine: items per integral tile */
    int tile_stars = 0; /* engine: stars per likelihood tile */
    int warp_items = 0; /* integral items are warp tiles (compensated form) */
    bool tuned = false; /* chosen by the autotuner */
};

struct Wedge
{
    bool has_problem = false;
    ProblemHost prob;
    std::vector<double> gl_x, gl_w, dx, nfac;
    double coeff = 0.0;
    AreaDev areas[MWSEP_MAX_AREAS];
    DevBuf d_dx, d_glw, d_nfac; /* per convolution point: dx, gl_w, star-table factors */

    bool has_stars = false;
    int n_stars = 0;
    DevBuf s_l, s_b, s_r, s_geom, s_r_point, s_qw, s_r_in_mag, s_r_in_mag2, s_reff, s_pts;
    DevBuf s_head; /* per-star g' and distance factor, between the two star-table launches */
    /* double-float star table, built on the first double-float likelihood
     * of this catalogue */
    DevBuf s_ptsdf;
    bool has_star_df = false;
    /* the plain forms' FP64 star tables (r_point, qw, r_in_mag, r_in_mag2):
     * built with the catalogue, or on the first plain-form read after an
     * EvalFunc call's upload, which builds only what every form reads */
    bool has_star_f64 = false;
    mwsep_stars_dev stars_view{};
    HostPinned h_stars;

    Tune tune[3]; /* per precision: plain FP64, compensated FP32, double-float */
    unsigned tune_gen = 0; /* bumped whenever tune[] changes */
    size_t bytes = 0;      /* device bytes this wedge holds */
};

/* Buffers and graph of the tiled engine (mwsep_engine.cu). */
struct EngineState
{
    DevBuf d_areas, d_stars, d_reqs, d_itiles, d_ltiles, d_theta, d_ipart, d_lpart, d_out, d_counters;
    HostPinned h_areas, h_stars, h_reqs, h_itiles, h_ltiles, h_theta, h_out, h_counters;
    bool desc_dirty = true;
    int n_area_desc = 0, n_star_desc = 0;
    std::vector<int> area_base;     /* first area descriptor of each wedge */
    std::vector<unsigned> seen_gen; /* wedge tune generations the descriptors reflect */
    /* the captured graph of the last request shape */
    cudaGraphExec_t graph = nullptr;
    long long graph_key[5] = {-1, -1, -1, -1, -1};
    int graph_launches = 0;
};

} // namespace mwsep

struct mwsep_ctx
{
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[6] = {};
    /* The EvalFunc entries upload the catalogue on a side stream while the
     * integral runs; star-table readers on `stream` wait for ev_stars while
     * stars_pending (created on first use). */
    cudaStream_t side = nullptr;
    cudaEvent_t ev_main = nullptr, ev_stars = nullptr, ev_dens = nullptr;
    bool stars_pending = false;
    mwsep::Wedge* stars_build = nullptr;    /* its rows not yet gathered, uploaded and built from */
    const STAR_POINTS* stars_rows = nullptr;
    size_t dev_bytes = 0;
    size_t hbm_budget = 0; /* 0: no budget */

    std::vector<mwsep::Wedge*> wedges;
    bool shared_wedges = false; /* a serving lane: wedges belong to the parent context */

    /* single-problem path (wedge 0) */
    mwsep::DevBuf d_theta, d_partials, d_lkpartials, d_out;
    mwsep::DevBuf d_dens;    /* compensated likelihood: per-star densities of the batch */
    mwsep::DevBuf d_tilectr; /* compensated integral: tile counters per (theta, area) */
    mwsep::DevBuf d_segpart; /* and the first-level sums of its per-tile slots */
    mwsep::HostPinned h_theta, h_out;
    /* separation output of wedge 0 (mwsep_separation.cu) */
    mwsep::DevBuf d_sprob, d_assign, d_xyz;
    mwsep::HostPinned h_sep;

    mwsep::EngineState eng;

    double last_ms[5] = {};
    int last_launches = 0;
    size_t xfer_h2d = 0, xfer_d2h = 0;
};

namespace mwsep {

cudaError_t h2d(mwsep_ctx* c, void* dst, const void* src, size_t bytes, cudaStream_t st = nullptr);
cudaError_t d2h(mwsep_ctx* c, void* dst, const void* src, size_t bytes);
int check_problem(const ASTRONOMY_PARAMETERS* ap);
void theta_consts(const ProblemHost& base, const double* theta, mwsep_theta_consts& th);
long env_long(const char* name, long dflt);
/* (Re)build a wedge's problem tables from *ap. */
int wedge_set_problem(mwsep_ctx* c, Wedge& w, const ASTRONOMY_PARAMETERS* ap);
/* Upload a catalogue (SoA, host) and build all its star tables on stream st. */
int wedge_set_stars(mwsep_ctx* c, Wedge& w, int n, const double* l, const double* b, const double* r,
                    cudaStream_t st);
/* The plain forms' FP64 star tables on stream st, unless built (after the
 * catalogue's upload in stream order). */
int ensure_star_f64(mwsep_ctx* c, Wedge& w, cudaStream_t st);
/* From STAR_POINTS rows: synchronously on the context's stream, or (on_side)
 * deferred to launch_star_build with stars_pending set (sp must stay valid
 * until then). */
int wedge_set_stars_rows(mwsep_ctx* c, Wedge& w, const STAR_POINTS* sp, bool on_side);
/* The side stream and its events (created on first use). */
int ensure_side(mwsep_ctx* c);
/* Make st wait for a pending side-stream catalogue upload. */
int wait_stars(mwsep_ctx* c, cudaStream_t st);
/* Gather, upload and build from a deferred catalogue on the side stream
 * (the build after event `after`, if given) and record ev_stars. */
int launch_star_build(mwsep_ctx* c, cudaEvent_t after);
void wedge_release(mwsep_ctx* c, Wedge& w);
/* Integrate the cells [min_calculation, max_calculation) of each area of a
 * resident wedge (per area; the EvalFunc entries take them from
 * EVALUATION_STATE as calculate_integral does). */
int wedge_set_slices(mwsep_ctx* c, Wedge& w, const long* min_calc, const long* max_calc);
/* r-bins per warp tile that make a tile's points whole lane groups. */
int warp_tile_kstep(int convolve, int n_streams);
void default_tune(mwsep_ctx* c, Wedge& w);
/* One evaluation (or a batch) of wedge 0 through the grid-stride kernels;
 * leaves the integrals in c->d_out after the area block. */
int evaluate_impl(mwsep_ctx* c, int B, const double* thetas, int precision, mwsep_result* out);
/* Which phases of an evaluation run: both (the default), the integrals
 * alone (no catalogue needed; the likelihood fields come back NaN), or the
 * likelihood alone against given cut-subtracted integrals ([B][1 + S],
 * host), the two steps of the reference's distributed evaluation
 * (integral_f / likelihood_f, cpu/astronomy_worker.c:33-121). */
struct Phases
{
    bool integrals = true;
    bool likelihood = true;
    const double* given_integrals = nullptr;
};

/* The same for any resident wedge (wedge 0 is the one set_problem fills). */
int evaluate_wedge(mwsep_ctx* c, int wid, int B, const double* thetas, int precision, mwsep_result* out,
                   const Phases& ph = Phases());

} // namespace mwsep

#endif
