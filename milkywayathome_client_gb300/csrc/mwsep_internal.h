/* mwsep_internal.h -- shared between the host orchestration and the CUDA
 * kernels of libmwsep_gb300.  Not part of the public ABI. */
#ifndef MWSEP_INTERNAL_H
#define MWSEP_INTERNAL_H

#include <stdint.h>
#include "milkyway_separation_gb300.h"

#ifdef __CUDACC__
#define MWSEP_HD __host__ __device__
#define MWSEP_HDI __host__ __device__ __forceinline__
#else
#define MWSEP_HD
#define MWSEP_HDI inline
#endif

/* include/milkyway.h:46-52 (pi is M_PI on glibc; deg = 180/pi) and the
 * density-model constants of cpu/evaluation_optimized.c:41-46. */
#define MW_PI 3.1415926535897932384626433832795028841971693993751
#define MW_DEG (180.0 / MW_PI)
#define MW_D2PI 6.2831853071795864769252867665590057683943387987502
#define MW_STDEV 0.6
#define MW_LBR_R 8.5
#define MW_ABSM 4.2
#define MW_SIG0 0.9402
#define MW_SIG1 1.6171
#define MW_SIG2 23.5877

/* Kernels are specialised on an upper bound of the stream count. */
#define MWSEP_KMAX_STREAMS 8

/* Parameter-dependent constants of one evaluation, computed on the host in
 * FP64 with the reference's formulas (init_constants,
 * cpu/evaluation_optimized.c:54-133, and the weights of
 * calculate_likelihood :639-646). */
typedef struct
{
    double alpha, q, r0, delta;
    double bg_a, bg_b, bg_c;
    double alpha_delta3;
    int n_streams;
    int bg_mode;   /* 0: alpha=delta=1; 1: general pow branch; 2: q==0 */
    int aux;       /* aux_bg_profile (0/1) */
    int pad0;
    double sigma_sq2[MWSEP_KMAX_STREAMS];
    int stream_on[MWSEP_KMAX_STREAMS]; /* 0 when |sigma| < 1e-4 (:279-280) */
    double a[MWSEP_KMAX_STREAMS][3];
    double c[MWSEP_KMAX_STREAMS][3];
    double exp_bg_weight;
    double exp_stream_weight[MWSEP_KMAX_STREAMS];
    double sum_exp_weights;           /* already * 0.001 */
    /* single-precision copies for the compensated warp tiles' estimate of
     * each stream's exponent range: a_s, c_s + (Sun offset, 0, 0) and
     * -log2(e) / sigma2_s (0 for a switched-off stream) */
    float af[MWSEP_KMAX_STREAMS][3];
    float cf[MWSEP_KMAX_STREAMS][3];
    float kf[MWSEP_KMAX_STREAMS];
} mwsep_theta_consts;

/* A rectangular block of an area's cells: mu steps [mu0, mu0 + mu_n), nu
 * steps [nu0, nu0 + nu_n), r-bins [r0, r0 + r_n).  The cells an area
 * integrates -- all of them, or the slice [min_calculation, max_calculation)
 * of the linearised index (mu * nu_steps + nu) * r_steps + r that
 * calculate_integral walks (cpu/evaluation_optimized.c:461-530,
 * cpu/evaluation_state.c:129-151) -- are the union of at most
 * MWSEP_MAX_BOXES boxes, enumerated box after box. */
typedef struct
{
    int mu0, mu_n, nu0, nu_n, r0, r_n;
    int n_kchunks;       /* ceil(r_n / k_chunk) */
    int pad0;
    long long first;     /* the box's first item (or warp tile) in the area's enumeration */
} mwsep_box;
#define MWSEP_MAX_BOXES 5

/* One integral area on the device. */
typedef struct
{
    int mu_steps, nu_steps, r_steps, convolve; /* the grid the tables hold */
    int n_cols;          /* mu_steps * nu_steps */
    int k_chunk;         /* r-bins per item */
    int n_kchunks;       /* ceil(r_steps / k_chunk) */
    int warp_items;      /* 0: an item is (column, r-chunk), one thread;
                            1: an item is a warp tile (32 mu-columns at one nu, r-chunk) */
    long long n_items;   /* items over all boxes; for the whole area, thread items:
                            n_cols * n_kchunks; warp tiles: n_kchunks * nu_steps * ceil(mu_steps / 32) */
    long long cell_begin, cell_end; /* the cells integrated, [begin, end) of the linearised index */
    int n_boxes;         /* 0 (nothing to integrate) .. MWSEP_MAX_BOXES */
    int pad1;
    mwsep_box box[MWSEP_MAX_BOXES];
    const double* geom;      /* [mu][nu] x 4: bsin, bcos, lsin, lcos */
    const double* r_point;   /* [R][C] */
    const double* qw;        /* [R][C]  qw_r3_N */
    const double* r_in_mag;  /* [R][C] */
    const double* r_in_mag2; /* [R][C] */
    const double* reff;      /* [R] reff_xr_rp3 */
    const double* irv;       /* [R] */
    const double* ids;       /* [NU] */
    /* compensated-FP32 table: per (k, n) {r_hi, r_lo, qw*reff*irv, g}
     * where r = r_hi + r_lo to ~2^-48 and the weight is rounded once */
    const float4* pts;       /* [R][C] */
    /* double-float table: per (k, n) {r_hi, r_lo, w_hi, w_lo}, r and the
     * weight qw*reff*irv each as an unevaluated FP32 pair (~2^-48) */
    const float4* ptsdf;     /* [R][C] */
} mwsep_area_dev;

/* A resident catalogue on the device (tables are [C][N], star-minor). */
typedef struct
{
    int n_stars, convolve;
    const double* geom;      /* [N] x 4: bsin, bcos, lsin, lcos */
    const double* r_point;   /* [C][N] */
    const double* qw;        /* [C][N] */
    const double* r_in_mag;  /* [C][N] */
    const double* r_in_mag2; /* [C][N] */
    const double* reff;      /* [N] */
    const float4* pts;       /* [C][N] {r_hi, r_lo, qw*reff, g} */
    const double* l;         /* [N] the catalogue as given (degrees, degrees, kpc) */
    const double* b;
    const double* r;
} mwsep_stars_dev;

#ifdef __cplusplus
namespace mwsep {
/* Warp tiles of the compensated integral: 32 mu-columns at one nu and a run
 * of r-bins; lanes hold P convolution points each per group. */
constexpr int kTileCols = 32;
#ifndef MWSEP_F32_TILE_P
/* a multiple of 4 (pairs are taken two at a time); on the full-size wedge
 * 8 runs the integral in 16.25 ms, 12 in 16.56 ms, 4 in 17.7 ms, 16 in 16.7 ms */
#define MWSEP_F32_TILE_P 8
#endif
template <int S>
struct TileP
{
    static constexpr int P = S <= 4 ? MWSEP_F32_TILE_P : 6;
};
MWSEP_HD inline long long warp_tile_count(int mu_steps, int nu_steps, int n_kchunks)
{
    return (long long)n_kchunks * nu_steps * ((mu_steps + kTileCols - 1) / kTileCols);
}

/* The cells calculate_integral visits for an INTEGRAL_AREA with
 * [min_calculation, max_calculation) over a grid of `total` cells
 * (cpu/evaluation_optimized.c:461-530): it starts at min_calculation
 * (get_steps, cpu/evaluation_state.c:129-151) and stops after the first cell
 * that brings the count to max_calculation, so a slice with max <= min still
 * integrates the one cell min, and a start at or past the end integrates
 * nothing.  Returns false for a negative start (outside the reference's
 * domain: its get_steps would index before the grid). */
inline bool effective_slice(long long min_calc, long long max_calc, long long total, long long& begin,
                            long long& end)
{
    if (min_calc < 0) return false;
    begin = min_calc < total ? min_calc : total;
    end = max_calc > begin + 1 ? max_calc : begin + 1;
    if (end > total) end = total;
    return true;
}

/* The cells [begin, end) of the linearised index of an M x NU x R grid as
 * at most MWSEP_MAX_BOXES boxes in index order: the rest of the first
 * column, the rest of its mu row, the whole mu rows between, the start of
 * the last mu row, the start of the last column.  Returns the box count
 * (0 for an empty range); firsts and chunk counts are set by the caller. */
inline int slice_boxes(int M, int NU, int R, long long begin, long long end, mwsep_box* out)
{
    int n = 0;
    auto put = [&](int mu0, int mu_n, int nu0, int nu_n, int r0, int r_n) {
        if (mu_n <= 0 || nu_n <= 0 || r_n <= 0) return;
        mwsep_box& b = out[n++];
        b.mu0 = mu0, b.mu_n = mu_n, b.nu0 = nu0, b.nu_n = nu_n, b.r0 = r0, b.r_n = r_n;
        b.n_kchunks = 0, b.pad0 = 0, b.first = 0;
    };
    if (end <= begin) return 0;
    const long long rowc = (long long)NU * R; /* cells per mu row */
    const int ib = (int)(begin / rowc), jb = (int)((begin / R) % NU), kb = (int)(begin % R);
    const long long last = end - 1;
    const int ie = (int)(last / rowc), je = (int)((last / R) % NU), ke = (int)(last % R) + 1;
    if (ib == ie && jb == je)
    {
        put(ib, 1, jb, 1, kb, ke - kb);
        return n;
    }
    /* first column: [kb, R) unless it starts at 0 (then it joins its row) */
    int jrow = jb;
    if (kb > 0)
    {
        put(ib, 1, jb, 1, kb, R - kb);
        jrow = jb + 1;
    }
    /* the last column: [0, ke) unless it ends at R (then it joins its row) */
    int jend = je + 1; /* columns [.., jend) of the last row are whole */
    const bool last_partial = ke < R;
    if (last_partial) jend = je;
    if (ib == ie)
    {
        put(ib, 1, jrow, jend - jrow, 0, R);
    }
    else
    {
        /* the rest of the first row, whole rows between, the start of the last row */
        if (jrow > 0)
            put(ib, 1, jrow, NU - jrow, 0, R);
        const int mu_first_whole = jrow > 0 ? ib + 1 : ib;
        if (jend == NU)
            put(mu_first_whole, ie + 1 - mu_first_whole, 0, NU, 0, R);
        else
        {
            put(mu_first_whole, ie - mu_first_whole, 0, NU, 0, R);
            put(ie, 1, 0, jend, 0, R);
        }
    }
    if (last_partial) put(ie, 1, je, 1, 0, ke);
    return n;
}

/* The cells an area view integrates (set_chunking turns them into boxes). */
inline void set_slice(mwsep_area_dev& v, long long begin, long long end)
{
    v.cell_begin = begin;
    v.cell_end = end;
}

/* An area view's chunking -- k_chunk r-bins per item, warp tiles or thread
 * items -- and, from its [cell_begin, cell_end), its boxes, their first
 * items and the item count. */
inline void set_chunking(mwsep_area_dev& v, int k_chunk, int warp_items)
{
    v.k_chunk = k_chunk < 1 ? 1 : (k_chunk > v.r_steps ? v.r_steps : k_chunk);
    v.n_kchunks = (v.r_steps + v.k_chunk - 1) / v.k_chunk;
    v.warp_items = warp_items ? 1 : 0;
    v.n_boxes = slice_boxes(v.mu_steps, v.nu_steps, v.r_steps, v.cell_begin, v.cell_end, v.box);
    long long first = 0;
    for (int b = 0; b < v.n_boxes; ++b)
    {
        mwsep_box& x = v.box[b];
        x.n_kchunks = (x.r_n + v.k_chunk - 1) / v.k_chunk;
        x.first = first;
        first += warp_items ? warp_tile_count(x.mu_n, x.nu_n, x.n_kchunks) : (long long)x.mu_n * x.nu_n * x.n_kchunks;
    }
    for (int b = v.n_boxes; b < MWSEP_MAX_BOXES; ++b)
    {
        v.box[b] = mwsep_box{};
        v.box[b].first = first; /* past every item: never selected */
    }
    v.n_items = first;
}

/* Where an item or a warp tile of an area lies: its column (mu * nu_steps +
 * nu), nu step, first mu step and column count (warp tiles), r-bins [k0, k1). */
struct ItemPos
{
    int col, nu, k0, k1;
};
struct TilePos
{
    int mu0, ncols, nu, k0, k1;
};

/* The box holding item (or warp tile) idx: the last one starting at or
 * before it.  Fields are picked with constant indices, so the descriptor is
 * read where it lives (kernel parameters or shared memory). */
MWSEP_HDI mwsep_box box_of(const mwsep_area_dev& A, long long idx)
{
    mwsep_box b = A.box[0];
#pragma unroll
    for (int i = 1; i < MWSEP_MAX_BOXES; ++i)
        if (i < A.n_boxes && idx >= A.box[i].first) b = A.box[i];
    return b;
}

/* A thread item: a column of the box and a run of k_chunk of its r-bins;
 * consecutive items are consecutive columns of one r-run.  For a whole
 * area this is item = kc * n_cols + col. */
MWSEP_HDI ItemPos item_pos(const mwsep_area_dev& A, long long item)
{
    const mwsep_box b = box_of(A, item);
    const long long local = item - b.first;
    const long long cols = (long long)b.mu_n * b.nu_n;
    const int kc = (int)(local / cols);
    const int cl = (int)(local - kc * cols);
    const int il = cl / b.nu_n;
    ItemPos p;
    p.nu = b.nu0 + (cl - il * b.nu_n);
    p.col = (b.mu0 + il) * A.nu_steps + p.nu;
    p.k0 = b.r0 + kc * A.k_chunk;
    p.k1 = p.k0 + A.k_chunk < b.r0 + b.r_n ? p.k0 + A.k_chunk : b.r0 + b.r_n;
    return p;
}

/* A warp tile: up to 32 mu-columns of the box at one nu and a run of k_chunk
 * of its r-bins, mu blocks fastest, then nu, then r-chunks. */
MWSEP_HDI TilePos tile_pos(const mwsep_area_dev& A, long long wt)
{
    const mwsep_box b = box_of(A, wt);
    const long long local = wt - b.first;
    const int nmb = (b.mu_n + kTileCols - 1) / kTileCols;
    const long long rest = local / nmb;
    const int mb = (int)(local - rest * nmb);
    const int kc = (int)(rest / b.nu_n);
    TilePos p;
    p.nu = b.nu0 + (int)(rest - (long long)kc * b.nu_n);
    p.mu0 = b.mu0 + mb * kTileCols;
    p.ncols = kTileCols < b.mu0 + b.mu_n - p.mu0 ? kTileCols : b.mu0 + b.mu_n - p.mu0;
    p.k0 = b.r0 + kc * A.k_chunk;
    p.k1 = p.k0 + A.k_chunk < b.r0 + b.r_n ? p.k0 + A.k_chunk : b.r0 + b.r_n;
    return p;
}
} // namespace mwsep
#endif

/* Per-evaluation likelihood sums written by the reduction kernels:
 * [0] sum of log10 p (prob_sum), [1] zero-probability count, [2] bg-only
 * sum, [3..3+S) stream-only sums. */
#define MWSEP_LK_SLOTS (3 + MWSEP_KMAX_STREAMS)

/* Shape of one batched launch.  Partials are laid out
 * [theta][area][grid][ncomp] for integrals (ncomp = 1+S) and
 * [theta][grid][nslots] for the likelihood (nslots = 3+S). */
typedef struct
{
    int n_theta;     /* gridDim.y */
    int n_streams;   /* S, the same for every theta of a batch */
    int n_areas;     /* integral areas of the problem */
    int area_index;  /* which area this launch covers */
    int block;       /* threads per block */
    int grid;        /* blocks per theta (gridDim.x) */
    int bg_form;     /* compensated kernels: the background form this launch
                        evaluates (thetas of other forms are skipped) */
} mwsep_launch_shape;

/* Background form of one theta (the compensated kernels specialise on it):
 * 0 alpha=delta=1, 1 the same plus the aux profile, 2 general alpha/delta,
 * 3 q == 0. */
#ifdef __CUDACC__
__host__ __device__
#endif
static inline int mwsep_bg_form(const mwsep_theta_consts* th)
{
    return th->bg_mode == 2 ? 3 : th->bg_mode == 1 ? 2 : th->aux ? 1 : 0;
}

/* ---- tiled engine: many requests over many resident wedges ---- */

/* Components of one integral tile partial and one likelihood tile partial. */
#define MWSEP_ENG_ICOMP (1 + MWSEP_KMAX_STREAMS)
#define MWSEP_ENG_LCOMP (3 + MWSEP_KMAX_STREAMS)
/* Per-request output block: area integrals [MWSEP_MAX_AREAS][ICOMP], the
 * cut-subtracted integrals [ICOMP], the likelihood sums [LCOMP]. */
#define MWSEP_ENG_OUT_AREAS 0
#define MWSEP_ENG_OUT_INTS (MWSEP_MAX_AREAS * MWSEP_ENG_ICOMP)
#define MWSEP_ENG_OUT_LK (MWSEP_ENG_OUT_INTS + MWSEP_ENG_ICOMP)
#define MWSEP_ENG_OUT_STRIDE (MWSEP_ENG_OUT_LK + MWSEP_ENG_LCOMP)

/* One request of an engine batch. */
typedef struct
{
    int n_streams;                        /* S of its wedge */
    int n_areas;                          /* integral areas of its wedge */
    int stars;                            /* index of its catalogue descriptor */
    int pad0;
    int area_slot[MWSEP_MAX_AREAS + 1];   /* integral tiles of area a: [area_slot[a], area_slot[a+1]) */
    int lk_slot0, lk_slot1;               /* likelihood tiles: [lk_slot0, lk_slot1) */
} mwsep_req_dev;

/* A run of items of one area for one request (an integral tile). */
typedef struct
{
    int req;
    int area_desc;       /* index into the area descriptors */
    long long item_begin;
    long long item_end;
} mwsep_itile;

/* A run of stars for one request (a likelihood tile). */
typedef struct
{
    int req;
    int star_begin;
    int star_end;
    int pad0;
} mwsep_ltile;

/* Requests are split into kernel groups by stream count: group g = S for
 * S <= 4 (each kernel specialised on its exact S), group 5 for 5..8 streams.
 * Device-side counters of one engine launch, per group g: [4g+0] next
 * integral tile, [4g+1] next likelihood tile, [4g+2] end of the group's
 * integral tiles, [4g+3] end of its likelihood tiles; [24] requests.  A
 * group's tiles are contiguous and start where its "next" counters start. */
#define MWSEP_ENG_GROUPS 6
#define MWSEP_ENG_COUNTERS 28
#define MWSEP_ENG_NREQ 24

typedef struct
{
    const mwsep_area_dev* areas;
    const mwsep_stars_dev* stars;
    const mwsep_req_dev* reqs;
    const mwsep_theta_consts* thetas;     /* one per request */
    const mwsep_itile* itiles;
    const mwsep_ltile* ltiles;
    double2* ipart;                       /* [itiles][ICOMP] */
    double2* lpart;                       /* [ltiles][LCOMP] */
    double* out;                          /* [requests][OUT_STRIDE] */
    int* counters;
    int n_area_desc;                      /* descriptors in areas / stars */
    int n_star_desc;
} mwsep_engine_args;

#ifdef __cplusplus
extern "C" {
#endif
/* Engine launchers: persistent grids (grid = resident blocks x SMs). */
/* phase 0: integrals, 1: likelihood; group: the stream count (0..4) or 5 (5..8 streams) */
int mwsep_engine_f32_launch(int phase, int group, const mwsep_engine_args* a, int grid, void* stream);
int mwsep_engine_f64_launch(int phase, int group, const mwsep_engine_args* a, int grid, void* stream);
int mwsep_engine_f32_blocks_per_sm(int phase, int group);
int mwsep_engine_f64_blocks_per_sm(int phase, int group);
/* per-request fixed-order reductions: phase 0 integrals (+ cut
 * subtraction), phase 1 likelihood */
int mwsep_engine_reduce(int phase, const mwsep_engine_args* a, int grid, void* stream);
/* Launchers (defined in the .cu files).  All return cudaError_t as int. */
int mwsep_launch_geometry(double mu_min, double mu_step, int mu_steps, const double* nus, int nu_steps,
                          int sgr, int wedge, double* geom_out, void* stream);
/* The star tables every form reads (geom, reff, the compensated form's
 * pts) and head, 2n doubles per star (g', the distance factor) from which
 * mwsep_launch_star_f64 later builds the plain forms' FP64 tables.  nfac:
 * [C] 10^(dx_n/5), then [C] gl_w_n coeff e^{-dx_n^2 / 2 sigma^2}. */
int mwsep_launch_star_tables(int n, const double* l, const double* b, const double* r, int convolve,
                             const double* dx, const double* nfac, double* geom, double* reff, float4* pts,
                             double* head, void* stream);
int mwsep_launch_star_f64(int n, int convolve, const double* dx, const double* nfac, const double* head,
                          double* r_point, double* qw, double* r_in_mag, double* r_in_mag2, void* stream);
int mwsep_launch_integral_f64(const mwsep_area_dev* area, const mwsep_theta_consts* th_dev,
                              const mwsep_launch_shape* shape, double2* partials, void* stream);
int mwsep_launch_likelihood_f64(const mwsep_stars_dev* st, const mwsep_theta_consts* th_dev,
                                const mwsep_launch_shape* shape, const double* integrals,
                                double2* partials, void* stream);
int mwsep_launch_integral_f32(const mwsep_area_dev* area, const mwsep_theta_consts* th_dev,
                              const mwsep_launch_shape* shape, double2* partials, void* stream);
/* The warp-tile integral with tiles handed out by counters[theta * n_areas +
 * area] (zeroed before the launch): per (theta, area) n_slots tile slots of
 * 1 + S double2 (value, 0), tile-major, summed by mwsep_launch_reduce_integrals
 * with grid = n_slots; slots past an area's tile count must be zero. */
/* Sum per-tile slots (n_rows = theta * n_areas rows of n_slots x ncomp
 * double2) in fixed segments of seg_len into seg (rows x n_seg x ncomp,
 * n_seg = ceil(n_slots / seg_len)), for mwsep_launch_reduce_integrals with
 * grid = n_seg. */
int mwsep_launch_reduce_slots(const double2* slots, int n_rows, long long n_slots, int ncomp, int seg_len,
                              double2* seg, void* stream);
int mwsep_launch_integral_f32_dyn(const mwsep_area_dev* area, const mwsep_theta_consts* th_dev,
                                  const mwsep_launch_shape* shape, long long n_slots, double2* slots,
                                  int* counters, void* stream);
int mwsep_launch_likelihood_f32(const mwsep_stars_dev* st, const mwsep_theta_consts* th_dev,
                                const mwsep_launch_shape* shape, const double* integrals,
                                double2* partials, void* stream);
/* The same likelihood in two launches: per-star densities into
 * dens[theta][1 + S_max][star] (S_max = 8 beyond 4 streams), needing no
 * integral; then the epilogue and the per-block partials, bit for bit those
 * of mwsep_launch_likelihood_f32 on the same shape. */
int mwsep_launch_likelihood_f32_density(const mwsep_stars_dev* st, const mwsep_theta_consts* th_dev,
                                        const mwsep_launch_shape* shape, double* dens, void* stream);
int mwsep_launch_likelihood_f32_finish(int n_stars, const mwsep_theta_consts* th_dev,
                                       const mwsep_launch_shape* shape, const double* integrals,
                                       const double* dens, double2* partials, void* stream);
/* Resident blocks per SM of the integral kernels (persistent-grid sizing). */
int mwsep_integral_f32_blocks_per_sm(int n_streams, int warp_items);
/* double-float integral (mwsep_df.cu) */
#ifndef MWSEP_DF_TILE_P
/* points per lane, even; 8 / 12 / 16: 171.5 / 172.3 / 171.2 ms on the
 * full-size wedge, 6.55 / 6.26 / 6.72 ms on the 400 x 160 x 140 one */
#define MWSEP_DF_TILE_P 12
#endif
/* ... up to 4 streams; the 5-8 stream instances (4-warp blocks, 128
 * registers) take 8, which they hold without spilling */
MWSEP_HD constexpr int mwsep_df_tile_p(int n_streams) { return n_streams > 4 ? 8 : MWSEP_DF_TILE_P; }
int mwsep_df_prepare(int device);
int mwsep_integral_df_blocks_per_sm(int n_streams);
int mwsep_launch_integral_df(const mwsep_area_dev* area, const mwsep_theta_consts* th_dev,
                             const mwsep_launch_shape* sh, double2* partials, void* stream);
/* The double-float integral with a tile counter and per-tile slots, as
 * mwsep_launch_integral_f32_dyn. */
int mwsep_launch_integral_df_dyn(const mwsep_area_dev* area, const mwsep_theta_consts* th_dev,
                                 const mwsep_launch_shape* shape, long long n_slots, double2* slots,
                                 int* counters, void* stream);
/* Adds the aux profile's column-independent share of an area integral to
 * the double-float partials of the thetas that have it (after
 * mwsep_launch_integral_df for that area, same shape). */
int mwsep_launch_aux_area_df(const mwsep_area_dev* area, const mwsep_theta_consts* th_dev,
                             const mwsep_launch_shape* sh, double2* partials, void* stream);
/* Per-star double-float table [C][N] {r_hi, r_lo, qw_hi, qw_lo} from the
 * FP64 tables, and the likelihood over it (same partial layout as the FP64
 * likelihood; block <= 256, up to 4 streams). */
int mwsep_launch_star_df_table(int n, int convolve, const double* r_point, const double* qw, float4* out,
                               void* stream);
int mwsep_launch_likelihood_df(const mwsep_stars_dev* stars, const float4* star_df,
                               const mwsep_theta_consts* th_dev, const mwsep_launch_shape* sh,
                               const double* integrals, double2* partials, void* stream);
int mwsep_integral_f64_blocks_per_sm(int n_streams, int block);
/* Reduce per-block compensated partials of every area into area integrals
 * and subtract the cut areas (cpu/evaluation_optimized.c:584-593):
 * out_areas [n_theta][n_areas][1+S], out_integrals [n_theta][1+S]. */
int mwsep_launch_reduce_integrals(const double2* partials, const mwsep_launch_shape* shape,
                                  double* out_areas, double* out_integrals, void* stream);
/* Reduce likelihood partials into out [n_theta][3+S]. */
int mwsep_launch_reduce_likelihood(const double2* partials, const mwsep_launch_shape* shape,
                                   double* out, void* stream);
#ifdef __cplusplus
}
#endif

#endif
