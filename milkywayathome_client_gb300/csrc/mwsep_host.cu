/* mwsep_host.cu -- host orchestration of libmwsep_gb300.
 *
 * Owns the device context (one GPU, one stream), builds the resident wedge
 * and catalogue tables, computes the per-evaluation constants and issues the
 * kernel sequence of one evaluation or one batch:
 *
 *   H2D theta constants -> integral kernel per area -> integral reduction
 *   -> likelihood kernel -> likelihood reduction -> one D2H of the results.
 *
 * The integrals stay on the device between the two phases (the reference's
 * GPU backend copied per-cell partials back and summed on the host,
 * cuda/evaluation_gpu6.cu:639-767).
 *
 * Host-side formulas (r-bin tables, theta constants) are the reference's
 * (cpu/evaluation_optimized.c) evaluated with glibc libm, compiled with
 * -ffp-contract=off, so they equal the reference's doubles bit for bit.
 */
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <new>
#include <vector>

#include "milkyway_separation_gb300.h"
#include "milkyway_separation_gb300_test.h"
#include "mwsep_ctx.h"
#include "mwsep_geometry.cuh"
#include "mwsep_internal.h"
#include "mwsep_params.h"
#include "mwsep_checks.cuh"
#include "mwsep_status.h"

/* ---------------------------------------------------------------- status */

static thread_local int tl_last_error = 0;

extern "C" int mwsep_fail(int status)
{
    if (status != MWSEP_OK) tl_last_error = status;
    return status;
}

extern "C" int mwsep_last_error(void) { return tl_last_error; }

#if MWSEP_DEVICE_CHECKS
extern "C" int mwsep_checks_f32(unsigned long long*, unsigned long long*);
extern "C" int mwsep_checks_f64(unsigned long long*, unsigned long long*);
extern "C" int mwsep_checks_engine_f32(unsigned long long*, unsigned long long*);
extern "C" int mwsep_checks_engine_f64(unsigned long long*, unsigned long long*);
extern "C" int mwsep_checks_separation(unsigned long long*, unsigned long long*);
#endif

extern "C" int mwsep_device_checks(int device, int* enabled, unsigned long long* failures, unsigned long long* first)
{
    if (!enabled || !failures || !first) return mwsep_fail(MWSEP_ERR_ARG);
    *failures = 0;
    *first = 0;
#if MWSEP_DEVICE_CHECKS
    *enabled = 1;
    if (cudaSetDevice(device) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) return mwsep_fail(MWSEP_ERR_CUDA);
    int rc = 0;
    rc |= mwsep_checks_f32(failures, first);
    rc |= mwsep_checks_f64(failures, first);
    rc |= mwsep_checks_engine_f32(failures, first);
    rc |= mwsep_checks_engine_f64(failures, first);
    rc |= mwsep_checks_separation(failures, first);
    return rc ? mwsep_fail(MWSEP_ERR_CUDA) : MWSEP_OK;
#else
    (void)device;
    *enabled = 0;
    return MWSEP_OK;
#endif
}

extern "C" const char* mwsep_status_string(int s)
{
    switch (s)
    {
    case MWSEP_OK: return "ok";
    case MWSEP_ERR_ARG: return "invalid argument";
    case MWSEP_ERR_IO: return "file missing or unparsable";
    case MWSEP_ERR_PARAM_COUNT: return "parameter vector length does not match the optimised-parameter count";
    case MWSEP_ERR_UNSUPPORTED: return "problem outside the library limits";
    case MWSEP_ERR_CUDA: return "CUDA error or no sm_103 device";
    case MWSEP_ERR_NOMEM: return "out of memory";
    case MWSEP_ERR_BUDGET: return "request exceeds the device-memory budget";
    case MWSEP_ERR_TIMEOUT: return "bounded wait ran out";
    case MWSEP_ERR_CANCELLED: return "request cancelled";
    case MWSEP_ERR_STATE: return "call out of order";
    case MWSEP_ERR_BUSY: return "admission refused: the serving queue is full";
    default: return "unknown status";
    }
}

extern "C" const char* mwsep_version(void) { return "libmwsep_gb300 1.0 (sm_103a)"; }

namespace mwsep {

/* --------------------------------------------------------- device memory */

int DevBuf::ensure(size_t want, size_t& total)
{
    if (want <= bytes) return MWSEP_OK;
    if (p)
    {
        cudaFree(p);
        total -= bytes;
        p = nullptr;
        bytes = 0;
    }
    if (want == 0) return MWSEP_OK;
    if (cudaMalloc(&p, want) != cudaSuccess)
    {
        cudaGetLastError();
        return MWSEP_ERR_NOMEM;
    }
    bytes = want;
    total += bytes;
    return MWSEP_OK;
}

void DevBuf::release(size_t& total)
{
    if (p)
    {
        cudaFree(p);
        total -= bytes;
    }
    p = nullptr;
    bytes = 0;
}

int HostPinned::ensure(size_t want)
{
    if (want <= bytes) return MWSEP_OK;
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
    if (cudaMallocHost(&p, want) != cudaSuccess)
    {
        cudaGetLastError();
        return MWSEP_ERR_NOMEM;
    }
    bytes = want;
    return MWSEP_OK;
}

void HostPinned::release()
{
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
}

/* cudaMemcpyAsync with transfer accounting */
cudaError_t h2d(mwsep_ctx* c, void* dst, const void* src, size_t bytes, cudaStream_t st)
{
    c->xfer_h2d += bytes;
    return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st ? st : c->stream);
}
cudaError_t d2h(mwsep_ctx* c, void* dst, const void* src, size_t bytes)
{
    c->xfer_d2h += bytes;
    return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream);
}

namespace {

/* numericalIntegration.c:67-104 (Numerical Recipes gauleg on [-1, 1]). */
void gauss_legendre(int n, double* x, double* w)
{
    const double x1 = -1.0, x2 = 1.0, eps = 3.0e-11;
    const int m = (n + 1) / 2;
    const double xm = 0.5 * (x2 + x1), xl = 0.5 * (x2 - x1);
    for (int i = 1; i <= m; ++i)
    {
        double z = cos(MW_PI * (i - 0.25) / (n + 0.5)), z1, pp, p1, p2, p3;
        int guard = 0;
        do
        {
            p1 = 1.0;
            p2 = 0.0;
            for (int j = 1; j <= n; ++j)
            {
                p3 = p2;
                p2 = p1;
                p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
            }
            pp = n * (z * p1 - p2) / (z * z - 1.0);
            z1 = z;
            z = z1 - p1 / pp;
        } while (fabs(z - z1) > eps && ++guard < 1000);
        x[i - 1] = xm - xl * z;
        x[n - i] = xm + xl * z;
        w[i - 1] = 2.0 * xl / ((1.0 - z * z) * pp * pp);
        w[n - i] = w[i - 1];
    }
}

} // namespace

int check_problem(const ASTRONOMY_PARAMETERS* ap)
{
    if (!ap) return MWSEP_ERR_ARG;
    if (ap->number_streams < 0 || ap->number_streams > MWSEP_MAX_STREAMS) return MWSEP_ERR_UNSUPPORTED;
    if (ap->number_integrals < 1 || ap->number_integrals > MWSEP_MAX_AREAS) return MWSEP_ERR_UNSUPPORTED;
    if (ap->convolve < 1 || ap->convolve > MWSEP_MAX_CONVOLVE) return MWSEP_ERR_UNSUPPORTED;
    if (ap->number_background_parameters < 4 || ap->number_background_parameters > MWSEP_MAX_BG_PARAMS)
        return MWSEP_ERR_UNSUPPORTED;
    if (ap->aux_bg_profile != 0 && ap->aux_bg_profile != 1) return MWSEP_ERR_UNSUPPORTED;
    if (ap->sgr_coordinates != 0 && ap->sgr_coordinates != 1) return MWSEP_ERR_UNSUPPORTED;
    if (ap->number_streams > 0 &&
        (ap->number_stream_parameters < 5 || ap->number_stream_parameters > MWSEP_MAX_STREAM_PARAMS))
        return MWSEP_ERR_UNSUPPORTED;
    for (int i = 0; i < ap->number_integrals; ++i)
    {
        const INTEGRAL* in = ap->integral[i];
        if (!in || in->mu_steps < 1 || in->nu_steps < 1 || in->r_steps < 1) return MWSEP_ERR_ARG;
        if ((long long)in->mu_steps * in->nu_steps > (1LL << 30)) return MWSEP_ERR_UNSUPPORTED;
        if (in->min_calculation < 0) return MWSEP_ERR_ARG;
    }
    return MWSEP_OK;
}

namespace {

/* Copy the reference struct's values into the context's private copy. */
void copy_problem(const ASTRONOMY_PARAMETERS* ap, ProblemHost& p)
{
    p = ProblemHost();
    p.n_bg = ap->number_background_parameters;
    p.n_streams = ap->number_streams;
    p.n_sparams = ap->number_stream_parameters;
    p.bg_weight = ap->background_weight;
    for (int i = 0; i < p.n_bg; ++i)
    {
        p.bg[i] = ap->background_parameters[i];
        p.bg_opt[i] = ap->background_optimize[i];
    }
    /* the aux profile's a, b, c beyond the searched values */
    for (int i = p.n_bg; i < mwsep_background_values(ap); ++i) p.bg[i] = ap->background_parameters[i];
    for (int s = 0; s < p.n_streams; ++s)
    {
        p.st_weight[s] = ap->stream_weights[s];
        p.st_weight_opt[s] = ap->stream_weight_optimize[s];
        for (int j = 0; j < p.n_sparams; ++j)
        {
            p.st[s][j] = ap->stream_parameters[s][j];
            p.st_opt[s][j] = ap->stream_optimize[s][j];
        }
    }
    p.convolve = ap->convolve;
    p.sgr = ap->sgr_coordinates;
    p.aux = ap->aux_bg_profile;
    p.wedge = ap->wedge;
    p.n_areas = ap->number_integrals;
    for (int a = 0; a < p.n_areas; ++a)
    {
        const INTEGRAL* in = ap->integral[a];
        AreaHost& A = p.area[a];
        A.mu_steps = in->mu_steps;
        A.nu_steps = in->nu_steps;
        A.r_steps = in->r_steps;
        A.mu_min = in->mu_min;
        A.mu_max = in->mu_max;
        A.nu_min = in->nu_min;
        A.nu_max = in->nu_max;
        A.r_min = in->r_min;
        A.r_max = in->r_max;
        /* INTEGRAL_AREA step sizes (cpu/evaluation_state.c:247-249) */
        A.mu_step = (A.mu_max - A.mu_min) / A.mu_steps;
        A.nu_step = (A.nu_max - A.nu_min) / A.nu_steps;
        A.r_step = (A.r_max - A.r_min) / A.r_steps;
        mwsep::effective_slice(in->min_calculation, in->max_calculation,
                               (long long)A.mu_steps * A.nu_steps * A.r_steps, A.cell_begin, A.cell_end);
    }
    int n = 0;
    for (int i = 0; i < p.n_bg; ++i) n += p.bg_opt[i] ? 1 : 0;
    for (int s = 0; s < p.n_streams; ++s)
    {
        n += p.st_weight_opt[s] ? 1 : 0;
        for (int j = 0; j < p.n_sparams; ++j) n += p.st_opt[s][j] ? 1 : 0;
    }
    p.n_theta = n;
}

} // namespace

/* theta -> constants: set_astronomy_parameters (cpu/parameters.c:332-363),
 * init_constants (cpu/evaluation_optimized.c:54-133) and the likelihood
 * weights (:639-646). */
void theta_consts(const ProblemHost& base, const double* theta, mwsep_theta_consts& th)
{
    ProblemHost p = base;
    int k = 0;
    for (int i = 0; i < p.n_bg; ++i)
        if (p.bg_opt[i]) p.bg[i] = theta[k++];
    for (int s = 0; s < p.n_streams; ++s)
    {
        if (p.st_weight_opt[s]) p.st_weight[s] = theta[k++];
        for (int j = 0; j < p.n_sparams; ++j)
            if (p.st_opt[s][j]) p.st[s][j] = theta[k++];
    }
    memset(&th, 0, sizeof(th));
    th.alpha = p.bg[0];
    th.q = p.bg[1];
    th.r0 = p.bg[2];
    th.delta = p.bg[3];
    if (p.aux == 1)
    {
        th.bg_a = p.bg[4];
        th.bg_b = p.bg[5];
        th.bg_c = p.bg[6];
    }
    th.aux = p.aux;
    th.alpha_delta3 = 3 - th.alpha + th.delta;
    th.bg_mode = (th.q == 0) ? 2 : ((th.alpha == 1 && th.delta == 1) ? 0 : 1);
    th.n_streams = p.n_streams;
    for (int s = 0; s < p.n_streams; ++s)
    {
        const double sigma = p.st[s][4];
        th.sigma_sq2[s] = 2.0 * sigma * sigma;
        th.stream_on[s] = !(sigma > -0.0001 && sigma < 0.0001);
        double l, b;
        mwsep::wedge_point_lb(p.sgr, p.wedge, p.st[s][0], 0, l, b);
        mwsep::lbr_to_xyz(l, b, p.st[s][1], th.c[s]);
        th.a[s][0] = sin(p.st[s][2]) * cos(p.st[s][3]);
        th.a[s][1] = sin(p.st[s][2]) * sin(p.st[s][3]);
        th.a[s][2] = cos(p.st[s][2]);
        for (int i = 0; i < 3; ++i)
        {
            th.af[s][i] = (float)th.a[s][i];
            th.cf[s][i] = (float)(th.c[s][i] + (i == 0 ? MW_LBR_R : 0.0));
        }
        th.kf[s] = th.stream_on[s] ? (float)(-1.4426950408889634 / th.sigma_sq2[s]) : 0.f;
    }
    th.exp_bg_weight = exp(p.bg_weight);
    double sum = th.exp_bg_weight;
    for (int s = 0; s < p.n_streams; ++s)
    {
        th.exp_stream_weight[s] = exp(p.st_weight[s]);
        sum += exp(p.st_weight[s]);
    }
    th.sum_exp_weights = sum * 0.001;
}

namespace {

int occupancy_grid(mwsep_ctx* c, int block, long long items)
{
    long long g = (items + block - 1) / block;
    const long long cap = (long long)c->sm_count * (2048 / block);
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

} // namespace

long env_long(const char* name, long dflt)
{
    const char* v = getenv(name);
    return (v && *v) ? strtol(v, nullptr, 10) : dflt;
}

/* Default launch shapes for a resident wedge.  The shape depends only on the
 * wedge, never on the batch, so a theta gives the same bits alone and inside
 * any batch.  Grid-stride kernels run a persistent grid (resident blocks per
 * SM x SMs); items (column x r-run) are sized so each thread gets ~48, which
 * keeps the static tail near 2%.  The engine uses the same items, in tiles of
 * tile_items.  MWSEP_TUNE_{KCHUNK,GRID_F32,GRID_F64} override the choice. */
/* Warp-tile r-chunk for a wedge too small to fill the GPU: over chunks of
 * 1..kc_max bins, the modelled time is the larger of the per-SM work and one
 * warp's chain of tiles at the speed of a lone warp (an SM saturates at about
 * half its warp slots).  Work is counted in lane groups (ceil of the chunk's
 * points over the group size, ragged last chunk included) plus `prologue`
 * groups per tile for the column constants. */
int fill_kchunk(int max_r, int convolve, int group, long long tiles_per_chunk, int sms, long long slots,
                double prologue, int kc_max)
{
    const double wsat = std::max(1.0, 0.5 * (double)slots / std::max(sms, 1));
    int best = kc_max;
    double best_cost = 1e300;
    for (int kc = 1; kc <= kc_max; ++kc)
    {
        const int nk = (max_r + kc - 1) / kc;
        double work = 0.0, gmax = 0.0;
        for (int k = 0; k < nk; ++k)
        {
            const long long pts = (long long)std::min(kc, max_r - k * kc) * std::max(convolve, 1);
            const double g = (double)((pts + group - 1) / group) + prologue;
            work += g;
            gmax = std::max(gmax, g);
        }
        const long long tiles = tiles_per_chunk * nk;
        const double per_sm = work * (double)tiles_per_chunk / std::max(sms, 1);
        const double chain = wsat * gmax * (double)((tiles + slots - 1) / slots);
        const double cost = std::max(per_sm, chain);
        if (cost <= best_cost)
        {
            best_cost = cost;
            best = kc;
        }
    }
    return best;
}

/* Modelled time of one warp-tile launch of the compensated kernel, which
 * strides statically (warp w of W takes tiles w, w + W, ...; tiles in
 * r-chunk-major order; block b on SM b % sms): the largest per-SM sum of
 * tile costs, a tile costing its lane groups of points plus a per-tile
 * column prologue of `prologue` groups.  With prologue 0.5 it reproduces
 * the measured full-size integral (1600 x 640 x 140 cells, convolve 120,
 * 3 streams) within 0.6% for r-chunks of 28 to 140 bins. */
double static_tile_cost(int max_r, int convolve, int group, long long tiles_per_chunk, int kc, int sms,
                        int blocks_per_sm, int warps_per_block, double prologue)
{
    const long long W = (long long)sms * blocks_per_sm * warps_per_block;
    const int nk = (max_r + kc - 1) / kc;
    std::vector<double> sm(sms, 0.0);
    double all = 0.0; /* added to every SM */
    for (int k = 0; k < nk; ++k)
    {
        const long long pts = (long long)std::min(kc, max_r - k * kc) * std::max(convolve, 1);
        const double cost = (double)((pts + group - 1) / group) + prologue;
        const long long lo = (long long)k * tiles_per_chunk;
        const long long full = tiles_per_chunk / W, rem = tiles_per_chunk - full * W;
        all += (double)full * cost * blocks_per_sm * warps_per_block;
        for (long long i = 0; i < rem; ++i)
            sm[(size_t)((((lo + full * W + i) % W) / warps_per_block) % sms)] += cost;
    }
    return all + *std::max_element(sm.begin(), sm.end());
}

/* The compensated form's r-chunk: the least modelled time (static_tile_cost,
 * a 0.5-group column prologue) for chunks from kmin up to max_r bins. */
int model_kchunk(int max_r, int convolve, int group, long long tiles_per_chunk, int kmin, int sms,
                 int blocks_per_sm, int warps_per_block, double* cost_out)
{
    double best = 1e300;
    int kc = max_r;
    for (int k = std::max(1, std::min(max_r, kmin)); k <= max_r; ++k)
    {
        const double cost =
            static_tile_cost(max_r, convolve, group, tiles_per_chunk, k, sms, blocks_per_sm, warps_per_block, 0.5);
        if (cost < best * (1.0 - 1e-12))
        {
            best = cost;
            kc = k;
        }
    }
    if (cost_out) *cost_out = best;
    return kc;
}

/* Warp-tile chunking inputs: points per lane group and the least chunk. */
void warp_tile_groups(int prec, int n_streams, int convolve, int max_r, int& group, int& ks, int& kmin)
{
    group = prec == MWSEP_PLAIN_DF ? 32 * mwsep_df_tile_p(n_streams)
                                   : 32 * (n_streams <= 4 ? mwsep::TileP<4>::P : mwsep::TileP<8>::P);
    ks = group;
    for (int a = group, b = std::max(convolve, 1); b;)
    {
        const int t2 = a % b;
        a = b;
        b = t2;
        ks = group / a;
    }
    /* at least four lane groups of points per column of a tile, so the
     * column prologue and the last group's padding stay small */
    kmin = std::min(max_r, ((4 * group + convolve - 1) / std::max(convolve, 1) + ks - 1) / ks * ks);
}

void default_tune(mwsep_ctx* c, Wedge& w)
{
    const ProblemHost& p = w.prob;
    long long max_cols = 0;
    int max_r = 1;
    for (int a = 0; a < p.n_areas; ++a)
    {
        max_cols = std::max<long long>(max_cols, (long long)p.area[a].mu_steps * p.area[a].nu_steps);
        max_r = std::max(max_r, p.area[a].r_steps);
    }
    for (int prec = 0; prec < 3; ++prec)
    {
        Tune& t = w.tune[prec];
        t.block = (prec == MWSEP_PLAIN_DF && p.n_streams >= 4) ? 128 : 256; /* the DF kernel's own blocks */
        t.warp_items = (prec == MWSEP_PLAIN_DF ||
                        (prec == MWSEP_MIXED_F32 && env_long("MWSEP_F32_WARP_TILES", 1) != 0)) ? 1 : 0;
        const int per_sm = prec == MWSEP_PLAIN_F64   ? mwsep_integral_f64_blocks_per_sm(p.n_streams, t.block)
                           : prec == MWSEP_PLAIN_DF ? mwsep_integral_df_blocks_per_sm(p.n_streams)
                                                    : mwsep_integral_f32_blocks_per_sm(p.n_streams, t.warp_items);
        const long long threads = (long long)c->sm_count * per_sm * t.block;
        if (t.warp_items)
        {
            /* warp tiles: ~32 per warp, r-chunks of whole lane groups */
            long long tiles_per_chunk = 0;
            for (int a = 0; a < p.n_areas; ++a)
                tiles_per_chunk = std::max(tiles_per_chunk,
                                           mwsep::warp_tile_count(p.area[a].mu_steps, p.area[a].nu_steps, 1));
            const long long want = threads / 32 * 32;
            long long nk = (want + tiles_per_chunk - 1) / std::max<long long>(tiles_per_chunk, 1);
            nk = std::max<long long>(1, std::min<long long>(nk, max_r));
            int kc = (int)((max_r + nk - 1) / nk);
            int group, ks, kmin;
            warp_tile_groups(prec, p.n_streams, p.convolve, max_r, group, ks, kmin);
            kc = std::max(kc, kmin);
            if (kc >= ks) kc = kc / ks * ks;
            /* a small wedge whose tiles would leave warps idle: the chunk that
             * minimises the modelled time instead (lane groups per tile, a
             * per-tile prologue, and one warp's sequential chain) */
            const long long slots = threads / 32;
            if (prec == MWSEP_MIXED_F32)
                kc = model_kchunk(max_r, p.convolve, group, tiles_per_chunk, kmin, c->sm_count, per_sm, t.block / 32,
                                  nullptr);
            else if (tiles_per_chunk * ((max_r + kc - 1) / kc) < slots)
                kc = fill_kchunk(max_r, p.convolve, group, tiles_per_chunk, c->sm_count, slots, 0.1, kc);
            t.k_chunk = (int)env_long("MWSEP_TUNE_KCHUNK", kc);
            long long g = (long long)c->sm_count * per_sm;
            g = env_long("MWSEP_TUNE_GRID_F32", g);
            t.grid = (int)std::max<long long>(1, g);
            t.lk_block = 256;
            t.lk_grid = occupancy_grid(c, t.lk_block, std::max(w.n_stars, 1));
            /* engine: warp tiles per integral tile (the compensated engine
             * hands a tile to one warp) */
            t.tile_items = prec == MWSEP_MIXED_F32 ? 4 : 8 * 4;
            t.tile_stars = 1024;
            t.tuned = false;
            continue;
        }
        const long long want_items = threads * 48;
        long long chunks = (want_items + max_cols - 1) / std::max<long long>(max_cols, 1);
        chunks = std::max<long long>(1, std::min<long long>(chunks, max_r));
        t.k_chunk = (int)((max_r + chunks - 1) / chunks);
        t.k_chunk = (int)env_long("MWSEP_TUNE_KCHUNK", t.k_chunk);
        const long long items = max_cols * ((max_r + t.k_chunk - 1) / t.k_chunk);
        long long g = std::min<long long>((long long)c->sm_count * per_sm, (items + t.block - 1) / t.block);
        g = env_long(prec == MWSEP_PLAIN_F64 ? "MWSEP_TUNE_GRID_F64" : "MWSEP_TUNE_GRID_F32", g);
        t.grid = (int)std::max<long long>(1, g);
        t.lk_block = 256;
        t.lk_grid = occupancy_grid(c, t.lk_block, std::max(w.n_stars, 1));
        /* engine: thread items per integral tile (the compensated engine's
         * tiles go to one warp, the plain engine's to a block) */
        t.tile_items = (prec == MWSEP_MIXED_F32 ? 32 : t.block) * 8;
        t.tile_stars = 1024;
        t.tuned = false;
    }
    ++w.tune_gen;
}

namespace {

int build_area(mwsep_ctx* c, Wedge& w, int a)
{
    const ProblemHost& p = w.prob;
    const AreaHost& A = p.area[a];
    AreaDev& D = w.areas[a];
    const int R = A.r_steps, C = p.convolve, NU = A.nu_steps;
    const size_t RC = (size_t)R * C;

    /* cpu__r_constants (cpu/evaluation_optimized.c:360-422) on the host */
    std::vector<double> irv(R), reff(R), rp(RC), qw(RC), gm(RC), gm2(RC), ids(NU), nus(NU);
    std::vector<float4> pts(RC), ptsdf(RC);
    for (int i = 0; i < R; ++i)
    {
        const double log_r = A.r_min + (i * A.r_step);
        const double r = pow(10.0, (log_r - 14.2) / 5.0);
        const double next_r = pow(10.0, (log_r + A.r_step - 14.2) / 5.0);
        irv[i] = (((next_r * next_r * next_r) - (r * r * r)) / 3.0) * A.mu_step / MW_DEG;
        const double rPrime = (next_r + r) / 2.0;
        double gPrime;
        mwsep::prob_consts_head(rPrime, gPrime, reff[i]);
        for (int n = 0; n < C; ++n)
        {
            const size_t o = (size_t)i * C + n;
            double g;
            mwsep::prob_consts_point(gPrime, w.dx[n], w.gl_w[n], w.coeff, g, rp[o], qw[o]);
            gm[o] = g;
            gm2[o] = g * g;
            const float hi = (float)rp[o];
            pts[o] = make_float4(hi, (float)(rp[o] - (double)hi), (float)(qw[o] * (reff[i] * irv[i])), (float)g);
            const double wd = qw[o] * (reff[i] * irv[i]);
            const float whi = (float)wd;
            ptsdf[o] = make_float4(hi, (float)(rp[o] - (double)hi), whi, (float)(wd - (double)whi));
        }
    }
    for (int j = 0; j < NU; ++j)
    {
        nus[j] = A.nu_min + (j * A.nu_step);
        ids[j] = cos((90 - nus[j] - A.nu_step) / MW_DEG) - cos((90 - nus[j]) / MW_DEG);
        nus[j] += 0.5 * A.nu_step;
    }

    const size_t cols = (size_t)A.mu_steps * NU;
    size_t& tot = c->dev_bytes;
    const size_t before = tot;
    int rc = 0;
    rc |= D.geom.ensure(cols * 4 * sizeof(double), tot);
    rc |= D.r_point.ensure(RC * 8, tot);
    rc |= D.qw.ensure(RC * 8, tot);
    rc |= D.r_in_mag.ensure(RC * 8, tot);
    rc |= D.r_in_mag2.ensure(RC * 8, tot);
    rc |= D.reff.ensure(R * 8, tot);
    rc |= D.irv.ensure(R * 8, tot);
    rc |= D.ids.ensure(NU * 8, tot);
    rc |= D.nus.ensure(NU * 8, tot);
    rc |= D.pts.ensure(RC * sizeof(float4), tot);
    rc |= D.ptsdf.ensure(RC * sizeof(float4), tot);
    w.bytes += tot - before;
    if (rc) return mwsep_fail(MWSEP_ERR_NOMEM);

    cudaStream_t st = c->stream;
    CU(h2d(c, D.r_point.p, rp.data(), RC * 8));
    CU(h2d(c, D.qw.p, qw.data(), RC * 8));
    CU(h2d(c, D.r_in_mag.p, gm.data(), RC * 8));
    CU(h2d(c, D.r_in_mag2.p, gm2.data(), RC * 8));
    CU(h2d(c, D.reff.p, reff.data(), R * 8));
    CU(h2d(c, D.irv.p, irv.data(), R * 8));
    CU(h2d(c, D.ids.p, ids.data(), NU * 8));
    CU(h2d(c, D.nus.p, nus.data(), NU * 8));
    CU(h2d(c, D.pts.p, pts.data(), RC * sizeof(float4)));
    CU(h2d(c, D.ptsdf.p, ptsdf.data(), RC * sizeof(float4)));
    CK(mwsep_launch_geometry(A.mu_min, A.mu_step, A.mu_steps, D.nus.as<double>(), NU, p.sgr, p.wedge,
                             D.geom.as<double>(), st));
    /* the host vectors die with this frame: wait for the copies */
    CU(cudaStreamSynchronize(st));

    mwsep_area_dev& v = D.view;
    v.mu_steps = A.mu_steps;
    v.nu_steps = NU;
    v.r_steps = R;
    v.convolve = C;
    v.n_cols = (int)cols;
    v.geom = D.geom.as<double>();
    v.r_point = D.r_point.as<double>();
    v.qw = D.qw.as<double>();
    v.r_in_mag = D.r_in_mag.as<double>();
    v.r_in_mag2 = D.r_in_mag2.as<double>();
    v.reff = D.reff.as<double>();
    v.irv = D.irv.as<double>();
    v.ids = D.ids.as<double>();
    v.pts = D.pts.as<float4>();
    v.ptsdf = D.ptsdf.as<float4>();
    set_slice(v, A.cell_begin, A.cell_end);
    return MWSEP_OK;
}

} // namespace

int wedge_set_slices(mwsep_ctx* c, Wedge& w, const long* min_calc, const long* max_calc)
{
    for (int a = 0; a < w.prob.n_areas; ++a)
    {
        AreaHost& A = w.prob.area[a];
        long long b, e;
        if (!mwsep::effective_slice(min_calc[a], max_calc[a], (long long)A.mu_steps * A.nu_steps * A.r_steps, b, e))
            return mwsep_fail(MWSEP_ERR_ARG);
        A.cell_begin = b;
        A.cell_end = e;
        mwsep_area_dev& v = w.areas[a].view;
        if (v.cell_begin != b || v.cell_end != e)
        {
            set_slice(v, b, e);
            c->eng.desc_dirty = true;
        }
    }
    return MWSEP_OK;
}

int warp_tile_kstep(int convolve, int n_streams)
{
    const int group = 32 * (n_streams <= 4 ? mwsep::TileP<4>::P : mwsep::TileP<8>::P);
    int a = group, b = std::max(convolve, 1);
    while (b)
    {
        const int t = a % b;
        a = b;
        b = t;
    }
    return group / a;
}

/* Device buffers and views of an n-star catalogue (contents uploaded by
 * upload_stars). */
int prepare_stars(mwsep_ctx* c, Wedge& w, int n)
{
    if (!w.has_problem) return mwsep_fail(MWSEP_ERR_STATE);
    if (n < 1) return mwsep_fail(MWSEP_ERR_ARG);
    const int C = w.prob.convolve;
    const size_t NC = (size_t)n * C;
    size_t& tot = c->dev_bytes;
    const size_t before = tot;
    int rc = 0;
    rc |= w.s_l.ensure((size_t)n * 8, tot);
    rc |= w.s_b.ensure((size_t)n * 8, tot);
    rc |= w.s_r.ensure((size_t)n * 8, tot);
    rc |= w.s_geom.ensure((size_t)n * 32, tot);
    rc |= w.s_r_point.ensure(NC * 8, tot);
    rc |= w.s_qw.ensure(NC * 8, tot);
    rc |= w.s_r_in_mag.ensure(NC * 8, tot);
    rc |= w.s_r_in_mag2.ensure(NC * 8, tot);
    rc |= w.s_reff.ensure((size_t)n * 8, tot);
    rc |= w.s_pts.ensure(NC * sizeof(float4), tot);
    rc |= w.s_head.ensure((size_t)n * 2 * sizeof(double), tot);
    w.bytes += tot - before;
    if (rc) return mwsep_fail(MWSEP_ERR_NOMEM);
    mwsep_stars_dev& v = w.stars_view;
    v.n_stars = n;
    v.convolve = C;
    v.geom = w.s_geom.as<double>();
    v.r_point = w.s_r_point.as<double>();
    v.qw = w.s_qw.as<double>();
    v.r_in_mag = w.s_r_in_mag.as<double>();
    v.r_in_mag2 = w.s_r_in_mag2.as<double>();
    v.reff = w.s_reff.as<double>();
    v.pts = w.s_pts.as<float4>();
    v.l = w.s_l.as<double>();
    v.b = w.s_b.as<double>();
    v.r = w.s_r.as<double>();
    w.n_stars = n;
    w.has_stars = true;
    w.has_star_df = false; /* rebuilt from these tables when first needed */
    w.has_star_f64 = false;
    for (int prec = 0; prec < 3; ++prec)
        w.tune[prec].lk_grid = occupancy_grid(c, w.tune[prec].lk_block, n);
    return MWSEP_OK;
}

/* The catalogue's columns to the device and the star tables built from
 * them, on stream st (the build after event `after`, if given); the plain
 * forms' FP64 tables too when with_f64. */
int upload_stars(mwsep_ctx* c, Wedge& w, const double* l, const double* b, const double* r, cudaStream_t st,
                 cudaEvent_t after, bool with_f64)
{
    const size_t bytes = (size_t)w.n_stars * 8;
    CU(h2d(c, w.s_l.p, l, bytes, st));
    CU(h2d(c, w.s_b.p, b, bytes, st));
    CU(h2d(c, w.s_r.p, r, bytes, st));
    if (after) CU(cudaStreamWaitEvent(st, after, 0));
    CK(mwsep_launch_star_tables(w.n_stars, w.s_l.as<double>(), w.s_b.as<double>(), w.s_r.as<double>(),
                                w.prob.convolve, w.d_dx.as<double>(), w.d_nfac.as<double>(), w.s_geom.as<double>(),
                                w.s_reff.as<double>(), w.s_pts.as<float4>(), w.s_head.as<double>(), st));
    w.has_star_f64 = false;
    return with_f64 ? ensure_star_f64(c, w, st) : MWSEP_OK;
}

int ensure_star_f64(mwsep_ctx* c, Wedge& w, cudaStream_t st)
{
    (void)c;
    if (w.has_star_f64 || !w.has_stars) return MWSEP_OK;
    CK(mwsep_launch_star_f64(w.n_stars, w.prob.convolve, w.d_dx.as<double>(), w.d_nfac.as<double>(),
                             w.s_head.as<double>(), w.s_r_point.as<double>(), w.s_qw.as<double>(),
                             w.s_r_in_mag.as<double>(), w.s_r_in_mag2.as<double>(), st));
    w.has_star_f64 = true;
    return MWSEP_OK;
}

int wedge_set_stars(mwsep_ctx* c, Wedge& w, int n, const double* l, const double* b, const double* r,
                    cudaStream_t st)
{
    mwsep::Range nvtx_range("mwsep.set_stars");
    int rc = prepare_stars(c, w, n);
    if (rc) return rc;
    return upload_stars(c, w, l, b, r, st, nullptr, true);
}

/* STAR_POINTS rows (l, b, r) into the wedge's pinned staging columns. */
static void gather_rows(Wedge& w, const STAR_POINTS* sp)
{
    const int n = sp->number_stars;
    double* l = w.h_stars.as<double>();
    double* b = l + n;
    double* r = b + n;
    for (int i = 0; i < n; ++i)
    {
        const double* row = sp->stars[i];
        l[i] = row[0];
        b[i] = row[1];
        r[i] = row[2];
    }
}

int wedge_set_stars_rows(mwsep_ctx* c, Wedge& w, const STAR_POINTS* sp, bool on_side)
{
    if (!sp || !sp->stars || sp->number_stars < 1) return mwsep_fail(MWSEP_ERR_ARG);
    const int n = sp->number_stars;
    for (int i = 0; i < n; ++i)
        if (!sp->stars[i]) return mwsep_fail(MWSEP_ERR_ARG);
    /* an earlier side-stream upload may still read the staging buffer or
     * write the star tables */
    if (c->ev_stars) CU(cudaEventSynchronize(c->ev_stars));
    if (w.h_stars.ensure((size_t)n * 3 * sizeof(double))) return mwsep_fail(MWSEP_ERR_NOMEM);
    if (!on_side)
    {
        gather_rows(w, sp);
        const double* l = w.h_stars.as<double>();
        int rc = wedge_set_stars(c, w, n, l, l + n, l + 2 * (size_t)n, c->stream);
        if (rc) return rc;
        /* the pinned staging buffer is reused: wait for the copies */
        CU(cudaStreamSynchronize(c->stream));
        return MWSEP_OK;
    }
    /* on the side stream, after everything already queued on the context's
     * stream (the problem tables the star tables are built from, earlier
     * readers of the star tables); the rows are gathered, copied and built
     * from when launch_star_build is called, and the readers of this upload
     * wait for ev_stars */
    int rc = ensure_side(c);
    if (rc) return rc;
    rc = prepare_stars(c, w, n);
    if (rc) return rc;
    CU(cudaEventRecord(c->ev_main, c->stream));
    CU(cudaStreamWaitEvent(c->side, c->ev_main, 0));
    c->stars_build = &w;
    c->stars_rows = sp;
    c->stars_pending = true;
    return MWSEP_OK;
}

int ensure_side(mwsep_ctx* c)
{
    if (c->side) return MWSEP_OK;
    CU(cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking));
    CU(cudaEventCreateWithFlags(&c->ev_main, cudaEventDisableTiming));
    CU(cudaEventCreateWithFlags(&c->ev_stars, cudaEventDisableTiming));
    CU(cudaEventCreateWithFlags(&c->ev_dens, cudaEventDisableTiming));
    return MWSEP_OK;
}

int launch_star_build(mwsep_ctx* c, cudaEvent_t after)
{
    if (!c->stars_build) return MWSEP_OK;
    Wedge& w = *c->stars_build;
    const STAR_POINTS* sp = c->stars_rows;
    c->stars_build = nullptr;
    c->stars_rows = nullptr;
    gather_rows(w, sp);
    const double* l = w.h_stars.as<double>();
    const size_t n = (size_t)w.n_stars;
    /* the tables every form reads; a plain form builds its FP64 ones on
     * its first read (ensure_star_f64) */
    int rc = upload_stars(c, w, l, l + n, l + 2 * n, c->side, after, false);
    if (rc) return rc;
    CU(cudaEventRecord(c->ev_stars, c->side));
    return MWSEP_OK;
}

/* Readers of the star tables on the context's stream: wait for a pending
 * side-stream upload (launching its table build first if nothing has). */
int wait_stars(mwsep_ctx* c, cudaStream_t st)
{
    if (!c->stars_pending) return MWSEP_OK;
    int rc = launch_star_build(c, nullptr);
    if (rc) return rc;
    CU(cudaStreamWaitEvent(st, c->ev_stars, 0));
    return MWSEP_OK;
}

namespace {

/* The device tables of a wedge depend on these fields only (never on the
 * parameter values): equal fields give the same tables. */
bool same_tables(const ProblemHost& a, const ProblemHost& b)
{
    if (a.convolve != b.convolve || a.wedge != b.wedge || a.sgr != b.sgr || a.n_areas != b.n_areas ||
        a.n_streams != b.n_streams)
        return false;
    for (int i = 0; i < a.n_areas; ++i)
    {
        const AreaHost &x = a.area[i], &y = b.area[i];
        if (x.mu_steps != y.mu_steps || x.nu_steps != y.nu_steps || x.r_steps != y.r_steps ||
            x.mu_min != y.mu_min || x.mu_max != y.mu_max || x.nu_min != y.nu_min || x.nu_max != y.nu_max ||
            x.r_min != y.r_min || x.r_max != y.r_max || x.mu_step != y.mu_step || x.nu_step != y.nu_step ||
            x.r_step != y.r_step)
            return false;
    }
    return true;
}

} // namespace

int wedge_set_problem(mwsep_ctx* c, Wedge& w, const ASTRONOMY_PARAMETERS* ap)
{
    mwsep::Range nvtx_range("mwsep.set_problem");
    int rc = check_problem(ap);
    if (rc) return mwsep_fail(rc);
    if (w.has_problem)
    {
        /* the same grids, convolution, wedge and frame: the resident tables
         * (and the wedge's tuned shape) stand; only the values change */
        ProblemHost next;
        copy_problem(ap, next);
        if (same_tables(next, w.prob))
        {
            w.prob = next;
            for (int a = 0; a < w.prob.n_areas; ++a)
            {
                mwsep_area_dev& v = w.areas[a].view;
                if (v.cell_begin != w.prob.area[a].cell_begin || v.cell_end != w.prob.area[a].cell_end)
                {
                    set_slice(v, w.prob.area[a].cell_begin, w.prob.area[a].cell_end);
                    c->eng.desc_dirty = true;
                }
            }
            return MWSEP_OK;
        }
    }
    const int old_convolve = w.has_problem ? w.prob.convolve : -1;
    copy_problem(ap, w.prob);
    w.has_problem = false;
    const int C = w.prob.convolve;
    w.gl_x.assign(C, 0.0);
    w.gl_w.assign(C, 0.0);
    w.dx.assign(C, 0.0);
    gauss_legendre(C, w.gl_x.data(), w.gl_w.data());
    for (int i = 0; i < C; ++i) w.dx[i] = 3 * MW_STDEV * w.gl_x[i]; /* evaluation_optimized.c:131 */
    w.coeff = 1 / (MW_STDEV * sqrt(2 * MW_PI));                      /* :84 */
    const size_t before = c->dev_bytes;
    if (w.d_dx.ensure((size_t)C * 8, c->dev_bytes) || w.d_glw.ensure((size_t)C * 8, c->dev_bytes) ||
        w.d_nfac.ensure((size_t)C * 16, c->dev_bytes))
        return mwsep_fail(MWSEP_ERR_NOMEM);
    w.bytes += c->dev_bytes - before;
    /* star-table factors (the separable form of set_probability_constants) */
    w.nfac.assign((size_t)2 * C, 0.0);
    for (int i = 0; i < C; ++i)
    {
        w.nfac[(size_t)i] = pow(10.0, w.dx[i] / 5.0);
        w.nfac[(size_t)C + i] = w.gl_w[i] * (w.coeff * exp(-(w.dx[i] * w.dx[i]) / (2 * MW_STDEV * MW_STDEV)));
    }
    CU(h2d(c, w.d_dx.p, w.dx.data(), (size_t)C * 8));
    CU(h2d(c, w.d_glw.p, w.gl_w.data(), (size_t)C * 8));
    CU(h2d(c, w.d_nfac.p, w.nfac.data(), (size_t)C * 16));
    for (int a = 0; a < w.prob.n_areas; ++a)
    {
        rc = build_area(c, w, a);
        if (rc) return rc;
    }
    /* a catalogue built for another convolve count is stale */
    if (old_convolve != C) w.has_stars = false;
    w.has_problem = true;
    default_tune(c, w);
    c->eng.desc_dirty = true;
    return MWSEP_OK;
}

void wedge_release(mwsep_ctx* c, Wedge& w)
{
    size_t& t = c->dev_bytes;
    for (int a = 0; a < MWSEP_MAX_AREAS; ++a)
    {
        AreaDev& D = w.areas[a];
        DevBuf* bufs[] = {&D.geom, &D.r_point, &D.qw, &D.r_in_mag, &D.r_in_mag2, &D.reff, &D.irv,
                          &D.ids, &D.nus, &D.pts, &D.ptsdf};
        for (DevBuf* b : bufs) b->release(t);
    }
    DevBuf* bufs[] = {&w.d_dx, &w.d_glw, &w.d_nfac, &w.s_l, &w.s_b, &w.s_r, &w.s_geom, &w.s_r_point, &w.s_qw,
                      &w.s_r_in_mag, &w.s_r_in_mag2, &w.s_reff, &w.s_pts, &w.s_ptsdf, &w.s_head};
    for (DevBuf* b : bufs) b->release(t);
    w.has_star_df = false;
    w.has_star_f64 = false;
    w.h_stars.release();
    w.bytes = 0;
    w.has_problem = w.has_stars = false;
}

int evaluate_impl(mwsep_ctx* c, int B, const double* thetas, int precision, mwsep_result* out)
{
    return evaluate_wedge(c, 0, B, thetas, precision, out);
}

int evaluate_wedge(mwsep_ctx* c, int wid, int B, const double* thetas, int precision, mwsep_result* out,
                   const Phases& ph)
{
    mwsep::Range nvtx_range("mwsep.evaluate");
    if (wid < 0 || wid >= (int)c->wedges.size() || !c->wedges[wid]->has_problem ||
        (ph.likelihood && !c->wedges[wid]->has_stars))
        return mwsep_fail(MWSEP_ERR_STATE);
    if (!ph.integrals && (!ph.likelihood || !ph.given_integrals)) return mwsep_fail(MWSEP_ERR_ARG);
    Wedge& w = *c->wedges[wid];
    if (B < 1 || B > 65535 || !thetas || !out) return mwsep_fail(MWSEP_ERR_ARG);
    if (precision != MWSEP_PLAIN_F64 && precision != MWSEP_MIXED_F32 && precision != MWSEP_PLAIN_DF)
        return mwsep_fail(MWSEP_ERR_ARG);
    const ProblemHost& p = w.prob;
    const int S = p.n_streams, A = p.n_areas, P = p.n_theta;
    const int ncomp = 1 + S, nslots = 3 + S;

    size_t& tot = c->dev_bytes;
    const size_t th_bytes = sizeof(mwsep_theta_consts) * (size_t)B;
    if (c->h_theta.ensure(th_bytes)) return mwsep_fail(MWSEP_ERR_NOMEM);
    mwsep_theta_consts* hth = c->h_theta.as<mwsep_theta_consts>();
    for (int i = 0; i < B; ++i) theta_consts(p, thetas + (size_t)i * P, hth[i]);
    /* the double-float kernels cover every background form (alpha = delta
     * = 1 with or without the aux profile, general alpha/delta, q = 0) and
     * any stream count (the likelihood kernel up to 4 streams, the FP64
     * likelihood beyond).  One launch per form present, each skipping the
     * other forms' thetas. */
    bool df_aux = false, df_hern = false, df_general = false, df_none = false;
    if (precision == MWSEP_PLAIN_DF)
        for (int i = 0; i < B; ++i)
        {
            const int form = mwsep_bg_form(&hth[i]);
            df_aux = df_aux || form == 1;
            df_hern = df_hern || form <= 1;
            df_general = df_general || form == 2;
            df_none = df_none || form == 3;
        }
    const bool df_likelihood = precision == MWSEP_PLAIN_DF && S <= 4 && ph.likelihood;
    if (precision == MWSEP_PLAIN_DF && mwsep_df_prepare(c->device)) return mwsep_fail(MWSEP_ERR_CUDA);
    const Tune& t = w.tune[precision];
    /* the compensated warp tiles with a tile counter write one slot per tile
     * (per theta and area); batches go through in theta chunks whose slots
     * fit kDynSlotBytes (each theta's sum is its own, whatever the chunk) */
    long long n_slots = 0;
    if ((precision == MWSEP_MIXED_F32 || precision == MWSEP_PLAIN_DF) && t.warp_items)
        for (int a = 0; a < A; ++a)
        {
            mwsep_area_dev v = w.areas[a].view;
            set_chunking(v, t.k_chunk, t.warp_items);
            n_slots = std::max(n_slots, v.n_items);
        }
    const bool dyn = n_slots > 0 && n_slots < (1LL << 30) &&
                     env_long(precision == MWSEP_PLAIN_DF ? "MWSEP_DF_DYNAMIC" : "MWSEP_F32_DYNAMIC", 1) != 0;
    constexpr size_t kDynSlotBytes = (size_t)512 << 20;
    const size_t slot_bytes_theta = sizeof(double2) * (size_t)A * n_slots * ncomp;
    constexpr int kSegLen = 1024; /* slots per first-level reduction block */
    const long long n_seg = (n_slots + kSegLen - 1) / kSegLen;
    const long chunk_cap = env_long("MWSEP_F32_DYN_CHUNK", 65535); /* at most this many theta per chunk */
    const int dyn_chunk =
        dyn ? (int)std::max<size_t>(1, std::min<size_t>({(size_t)B, kDynSlotBytes / slot_bytes_theta,
                                                         (size_t)(65535 / A), (size_t)std::max(1L, chunk_cap)}))
            : B;
    const size_t part_bytes =
        dyn ? slot_bytes_theta * dyn_chunk : sizeof(double2) * (size_t)B * A * t.grid * ncomp;
    const size_t lkpart_bytes = sizeof(double2) * (size_t)B * t.lk_grid * nslots;
    const size_t out_doubles = (size_t)B * (A * ncomp + ncomp + nslots);
    int rc = 0;
    rc |= c->d_theta.ensure(th_bytes, tot);
    rc |= c->d_partials.ensure(part_bytes, tot);
    rc |= c->d_lkpartials.ensure(lkpart_bytes, tot);
    rc |= c->d_out.ensure(out_doubles * 8, tot);
    rc |= c->h_out.ensure(out_doubles * 8);
    /* the compensated likelihood's densities need no integral: computed on
     * the side stream beside the integral kernel */
    const bool split_lk =
        precision == MWSEP_MIXED_F32 && ph.likelihood && env_long("MWSEP_SPLIT_LIKELIHOOD", 1) != 0;
    if (split_lk) rc |= c->d_dens.ensure((size_t)B * (1 + (S <= 4 ? S : 8)) * w.n_stars * sizeof(double), tot);
    if (dyn)
    {
        rc |= c->d_tilectr.ensure((size_t)dyn_chunk * A * sizeof(int), tot);
        rc |= c->d_segpart.ensure(sizeof(double2) * (size_t)dyn_chunk * A * n_seg * ncomp, tot);
    }
    if (rc) return mwsep_fail(MWSEP_ERR_NOMEM);
    if (split_lk)
    {
        rc = ensure_side(c);
        if (rc) return rc;
    }
    if (df_likelihood && !w.has_star_df)
    {
        const size_t before = tot, need = (size_t)w.n_stars * p.convolve * sizeof(float4);
        if (c->hbm_budget && tot + need > c->hbm_budget) return mwsep_fail(MWSEP_ERR_BUDGET);
        if (w.s_ptsdf.ensure(need, tot)) return mwsep_fail(MWSEP_ERR_NOMEM);
        w.bytes += tot - before;
    }

    double* d_areas = c->d_out.as<double>();
    double* d_ints = d_areas + (size_t)B * A * ncomp;
    double* d_lk = d_ints + (size_t)B * ncomp;

    cudaStream_t st = c->stream;
    int launches = 0;
    CU(cudaEventRecord(c->ev[0], st));
    CU(h2d(c, c->d_theta.p, hth, th_bytes));
    CU(cudaEventRecord(c->ev[1], st));
    mwsep_launch_shape sh;
    sh.n_theta = B;
    sh.n_streams = S;
    sh.n_areas = A;
    sh.block = t.block;
    sh.grid = t.grid;
    /* background forms present in the batch (the compensated integral is
     * specialised on the form) */
    bool forms[4] = {false, false, false, false};
    for (int i = 0; i < B; ++i) forms[mwsep_bg_form(&hth[i])] = true;
    sh.bg_form = 0;
    if (!ph.integrals)
    {
        /* the likelihood alone: the given (composed) integrals stand in for
         * the reduction's output; no area results */
        CU(cudaMemsetAsync(d_areas, 0, sizeof(double) * (size_t)B * A * ncomp, st));
        CU(h2d(c, d_ints, ph.given_integrals, sizeof(double) * (size_t)B * ncomp, st));
    }
    for (int a = 0; a < (ph.integrals ? A : 0); ++a)
    {
        mwsep_area_dev v = w.areas[a].view;
        set_chunking(v, t.k_chunk, t.warp_items);
        sh.area_index = a;
        if (precision == MWSEP_PLAIN_F64)
        {
            CK(mwsep_launch_integral_f64(&v, c->d_theta.as<mwsep_theta_consts>(), &sh,
                                         c->d_partials.as<double2>(), st));
            ++launches;
        }
        else if (precision == MWSEP_PLAIN_DF && !dyn)
        {
            for (int form : {0, 2, 3})
            {
                if (!(form == 0 ? df_hern : form == 2 ? df_general : df_none)) continue;
                sh.bg_form = form;
                CK(mwsep_launch_integral_df(&v, c->d_theta.as<mwsep_theta_consts>(), &sh,
                                            c->d_partials.as<double2>(), st));
                ++launches;
            }
            if (df_aux || df_none)
            {
                CK(mwsep_launch_aux_area_df(&v, c->d_theta.as<mwsep_theta_consts>(), &sh,
                                            c->d_partials.as<double2>(), st));
                ++launches;
            }
        }
        else if (!dyn)
        {
            for (int form = 0; form < 4; ++form)
            {
                if (!forms[form]) continue;
                sh.bg_form = form;
                CK(mwsep_launch_integral_f32(&v, c->d_theta.as<mwsep_theta_consts>(), &sh,
                                             c->d_partials.as<double2>(), st));
                ++launches;
            }
        }
    }
    if (dyn && ph.integrals)
    {
        for (int b0 = 0; b0 < B; b0 += dyn_chunk)
        {
            const int nb = std::min(dyn_chunk, B - b0);
            CU(cudaMemsetAsync(c->d_tilectr.p, 0, (size_t)nb * A * sizeof(int), st));
            if (A > 1) CU(cudaMemsetAsync(c->d_partials.p, 0, slot_bytes_theta * nb, st)); /* unused slots */
            mwsep_launch_shape ds = sh;
            ds.n_theta = nb;
            for (int a = 0; a < A; ++a)
            {
                mwsep_area_dev v = w.areas[a].view;
                set_chunking(v, t.k_chunk, t.warp_items);
                ds.area_index = a;
                const mwsep_theta_consts* thb = c->d_theta.as<mwsep_theta_consts>() + b0;
                if (precision == MWSEP_PLAIN_DF)
                {
                    for (int form : {0, 2, 3})
                    {
                        if (!(form == 0 ? df_hern : form == 2 ? df_general : df_none)) continue;
                        ds.bg_form = form;
                        CK(mwsep_launch_integral_df_dyn(&v, thb, &ds, n_slots, c->d_partials.as<double2>(),
                                                        c->d_tilectr.as<int>(), st));
                        ++launches;
                    }
                    if (df_aux || df_none)
                    {
                        /* into each (theta, area)'s slot 0, after the tiles wrote it */
                        mwsep_launch_shape as = ds;
                        as.grid = (int)n_slots;
                        CK(mwsep_launch_aux_area_df(&v, thb, &as, c->d_partials.as<double2>(), st));
                        ++launches;
                    }
                    continue;
                }
                for (int form = 0; form < 4; ++form)
                {
                    bool present = false;
                    for (int i = b0; i < b0 + nb; ++i) present |= mwsep_bg_form(&hth[i]) == form;
                    if (!present) continue;
                    ds.bg_form = form;
                    CK(mwsep_launch_integral_f32_dyn(&v, thb, &ds, n_slots, c->d_partials.as<double2>(),
                                                     c->d_tilectr.as<int>(), st));
                    ++launches;
                }
            }
            CK(mwsep_launch_reduce_slots(c->d_partials.as<double2>(), nb * A, n_slots, (int)ncomp, kSegLen,
                                         c->d_segpart.as<double2>(), st));
            mwsep_launch_shape rs = sh;
            rs.n_theta = nb;
            rs.grid = (int)n_seg;
            CK(mwsep_launch_reduce_integrals(c->d_segpart.as<double2>(), &rs, d_areas + (size_t)b0 * A * ncomp,
                                             d_ints + (size_t)b0 * ncomp, st));
            launches += 2;
        }
    }
    /* a catalogue uploaded on the side stream: its table build released
     * with the integral (after the parameter upload), so it fills SMs the
     * integral's blocks leave */
    if (ph.likelihood)
    {
        rc = launch_star_build(c, c->ev[1]);
        if (rc) return rc;
    }
    mwsep_launch_shape lk = sh;
    lk.block = t.lk_block;
    lk.grid = t.lk_grid;
    lk.area_index = 0;
    if (split_lk)
    {
        /* after the parameter upload (and everything before it on the
         * context's stream, e.g. the last reader of the densities) */
        CU(cudaStreamWaitEvent(c->side, c->ev[1], 0));
        CK(mwsep_launch_likelihood_f32_density(&w.stars_view, c->d_theta.as<mwsep_theta_consts>(), &lk,
                                               c->d_dens.as<double>(), c->side));
        CU(cudaEventRecord(c->ev_dens, c->side));
        ++launches;
    }
    CU(cudaEventRecord(c->ev[2], st));
    if (!dyn && ph.integrals)
    {
        CK(mwsep_launch_reduce_integrals(c->d_partials.as<double2>(), &sh, d_areas, d_ints, st));
        ++launches;
    }
    CU(cudaEventRecord(c->ev[3], st));
    if (ph.likelihood)
    {
        /* from here on the star tables are read */
        rc = wait_stars(c, st);
        if (rc) return rc;
        if (precision != MWSEP_MIXED_F32)
        {
            rc = ensure_star_f64(c, w, st);
            if (rc) return rc;
        }
        if (df_likelihood && !w.has_star_df)
        {
            CK(mwsep_launch_star_df_table(w.n_stars, p.convolve, w.stars_view.r_point, w.stars_view.qw,
                                          w.s_ptsdf.as<float4>(), st));
            w.has_star_df = true;
        }
        if (df_likelihood)
        {
            int n_forms = 0;
            for (int form : {0, 2, 3})
            {
                if (!(form == 0 ? df_hern : form == 2 ? df_general : df_none)) continue;
                lk.bg_form = form;
                CK(mwsep_launch_likelihood_df(&w.stars_view, w.s_ptsdf.as<float4>(), c->d_theta.as<mwsep_theta_consts>(),
                                              &lk, d_ints, c->d_lkpartials.as<double2>(), st));
                if (n_forms++) ++launches; /* the first one is counted below */
            }
        }
        else if (precision != MWSEP_MIXED_F32)
            CK(mwsep_launch_likelihood_f64(&w.stars_view, c->d_theta.as<mwsep_theta_consts>(), &lk, d_ints,
                                           c->d_lkpartials.as<double2>(), st));
        else if (split_lk)
        {
            CU(cudaStreamWaitEvent(st, c->ev_dens, 0));
            CK(mwsep_launch_likelihood_f32_finish(w.n_stars, c->d_theta.as<mwsep_theta_consts>(), &lk, d_ints,
                                                  c->d_dens.as<double>(), c->d_lkpartials.as<double2>(), st));
        }
        else
            CK(mwsep_launch_likelihood_f32(&w.stars_view, c->d_theta.as<mwsep_theta_consts>(), &lk, d_ints,
                                           c->d_lkpartials.as<double2>(), st));
        ++launches;
        CU(cudaEventRecord(c->ev[4], st));
        CK(mwsep_launch_reduce_likelihood(c->d_lkpartials.as<double2>(), &lk, d_lk, st));
        ++launches;
    }
    else
        CU(cudaEventRecord(c->ev[4], st));
    CU(d2h(c, c->h_out.p, c->d_out.p, out_doubles * 8));
    CU(cudaEventRecord(c->ev[5], st));
    CU(cudaStreamSynchronize(st));

    float ms;
    cudaEventElapsedTime(&ms, c->ev[1], c->ev[2]);
    c->last_ms[0] = ms;
    cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]);
    c->last_ms[1] = ms;
    cudaEventElapsedTime(&ms, c->ev[3], c->ev[4]);
    c->last_ms[2] = ms;
    cudaEventElapsedTime(&ms, c->ev[4], c->ev[5]);
    c->last_ms[3] = ms;
    cudaEventElapsedTime(&ms, c->ev[0], c->ev[5]);
    c->last_ms[4] = ms;
    c->last_launches = launches;

    const double* h_areas = c->h_out.as<double>();
    const double* h_ints = h_areas + (size_t)B * A * ncomp;
    const double* h_lk = h_ints + (size_t)B * ncomp;
    const double N = (double)w.n_stars;
    for (int i = 0; i < B; ++i)
    {
        mwsep_result& r = out[i];
        memset(&r, 0, sizeof(r));
        r.number_streams = S;
        r.number_integrals = A;
        for (int a = 0; a < A; ++a)
            for (int k = 0; k < ncomp; ++k) r.area_integrals[a][k] = h_areas[((size_t)i * A + a) * ncomp + k];
        r.background_integral = h_ints[(size_t)i * ncomp];
        for (int s = 0; s < S; ++s) r.stream_integrals[s] = h_ints[(size_t)i * ncomp + 1 + s];
        r.status = MWSEP_OK;
        if (!ph.likelihood)
        {
            r.prob_sum = r.likelihood = r.background_only_likelihood = NAN;
            for (int s = 0; s < S; ++s) r.stream_only_likelihood[s] = NAN;
            continue;
        }
        const double* lkv = h_lk + (size_t)i * nslots;
        r.prob_sum = lkv[0];
        r.num_zero = (int)llround(lkv[1]);
        /* cpu_evaluate returns prob_sum/(N - bad_jacobians) (:783); the app
         * subtracts 3.0 (src/milkyway_client_app.c:278) */
        r.likelihood = lkv[0] / N - 3.0;
        r.background_only_likelihood = lkv[2] / N - 3.0;
        for (int s = 0; s < S; ++s) r.stream_only_likelihood[s] = lkv[3 + s] / N - 3.0;
    }
    return MWSEP_OK;
}

namespace {

Wedge* wedge0(mwsep_ctx* c)
{
    if (c->wedges.empty())
    {
        Wedge* w = new (std::nothrow) Wedge();
        if (!w) return nullptr;
        c->wedges.push_back(w);
    }
    return c->wedges[0];
}

} // namespace
} // namespace mwsep

using namespace mwsep;

/* ------------------------------------------------------------ public API */

extern "C" int mwsep_ctx_create(int device, mwsep_ctx** out)
{
    if (!out) return mwsep_fail(MWSEP_ERR_ARG);
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0)
    {
        cudaGetLastError();
        return mwsep_fail(MWSEP_ERR_CUDA);
    }
    if (device < 0 || device >= ndev) return mwsep_fail(MWSEP_ERR_ARG);
    cudaDeviceProp prop;
    CU(cudaGetDeviceProperties(&prop, device));
    /* the kernels are built for sm_103a only */
    if (prop.major != 10 || prop.minor != 3) return mwsep_fail(MWSEP_ERR_CUDA);
    CU(cudaSetDevice(device));
    mwsep_ctx* c = new (std::nothrow) mwsep_ctx();
    if (!c) return mwsep_fail(MWSEP_ERR_NOMEM);
    c->device = device;
    c->sm_count = prop.multiProcessorCount;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess)
    {
        delete c;
        return mwsep_fail(MWSEP_ERR_CUDA);
    }
    for (int i = 0; i < 6; ++i)
    {
        if (cudaEventCreate(&c->ev[i]) != cudaSuccess)
        {
            mwsep_ctx_destroy(c);
            return mwsep_fail(MWSEP_ERR_CUDA);
        }
    }
    *out = c;
    return MWSEP_OK;
}

extern "C" void mwsep_engine_release(mwsep_ctx* c);

extern "C" int mwsep_ctx_destroy(mwsep_ctx* c)
{
    if (!c) return mwsep_fail(MWSEP_ERR_ARG);
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->side) cudaStreamSynchronize(c->side);
    mwsep_engine_release(c);
    if (!c->shared_wedges)
        for (Wedge* w : c->wedges)
        {
            wedge_release(c, *w);
            delete w;
        }
    c->wedges.clear();
    size_t& t = c->dev_bytes;
    DevBuf* bufs[] = {&c->d_theta, &c->d_partials, &c->d_lkpartials, &c->d_out,
                      &c->d_sprob, &c->d_assign, &c->d_xyz, &c->d_dens, &c->d_tilectr, &c->d_segpart};
    for (DevBuf* b : bufs) b->release(t);
    c->h_theta.release();
    c->h_out.release();
    c->h_sep.release();
    for (int i = 0; i < 6; ++i)
        if (c->ev[i]) cudaEventDestroy(c->ev[i]);
    if (c->ev_main) cudaEventDestroy(c->ev_main);
    if (c->ev_stars) cudaEventDestroy(c->ev_stars);
    if (c->ev_dens) cudaEventDestroy(c->ev_dens);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return MWSEP_OK;
}

/* A serving lane: a context on the parent's device with its own stream and
 * engine state that shares (does not own) the parent's resident wedges. */
extern "C" mwsep_ctx* mwsep_ctx_lane(mwsep_ctx* parent)
{
    if (!parent) return nullptr;
    mwsep_ctx* c = nullptr;
    if (mwsep_ctx_create(parent->device, &c) != MWSEP_OK) return nullptr;
    c->wedges = parent->wedges;
    c->shared_wedges = true;
    return c;
}

extern "C" int mwsep_ctx_set_problem(mwsep_ctx* c, const ASTRONOMY_PARAMETERS* ap)
{
    if (!c || !ap) return mwsep_fail(MWSEP_ERR_ARG);
    if (c->shared_wedges) return mwsep_fail(MWSEP_ERR_STATE);
    CU(cudaSetDevice(c->device));
    Wedge* w = wedge0(c);
    if (!w) return mwsep_fail(MWSEP_ERR_NOMEM);
    return wedge_set_problem(c, *w, ap);
}

extern "C" int mwsep_ctx_set_stars_soa(mwsep_ctx* c, int n, const double* l, const double* b, const double* r)
{
    if (!c || !l || !b || !r) return mwsep_fail(MWSEP_ERR_ARG);
    CU(cudaSetDevice(c->device));
    if (c->wedges.empty()) return mwsep_fail(MWSEP_ERR_STATE);
    if (c->ev_stars) CU(cudaStreamWaitEvent(c->stream, c->ev_stars, 0));
    int rc = wedge_set_stars(c, *c->wedges[0], n, l, b, r, c->stream);
    if (rc) return rc;
    c->eng.desc_dirty = true;
    CU(cudaStreamSynchronize(c->stream));
    return MWSEP_OK;
}

extern "C" int mwsep_ctx_set_stars(mwsep_ctx* c, const STAR_POINTS* sp)
{
    if (!c || !sp || !sp->stars || sp->number_stars < 1) return mwsep_fail(MWSEP_ERR_ARG);
    CU(cudaSetDevice(c->device));
    if (c->wedges.empty()) return mwsep_fail(MWSEP_ERR_STATE);
    int rc = wedge_set_stars_rows(c, *c->wedges[0], sp, false);
    if (rc) return rc;
    c->eng.desc_dirty = true;
    return MWSEP_OK;
}

extern "C" int mwsep_ctx_theta_count(const mwsep_ctx* c)
{
    if (!c || c->wedges.empty() || !c->wedges[0]->has_problem) return -mwsep_fail(MWSEP_ERR_STATE);
    return c->wedges[0]->prob.n_theta;
}

extern "C" int mwsep_ctx_evaluate(mwsep_ctx* c, const double* theta, int precision, mwsep_result* out)
{
    if (!c) return mwsep_fail(MWSEP_ERR_ARG);
    CU(cudaSetDevice(c->device));
    return evaluate_impl(c, 1, theta, precision, out);
}

extern "C" int mwsep_ctx_integrals(mwsep_ctx* c, const double* theta, int precision, mwsep_result* out)
{
    if (!c) return mwsep_fail(MWSEP_ERR_ARG);
    CU(cudaSetDevice(c->device));
    Phases ph;
    ph.likelihood = false;
    return evaluate_wedge(c, 0, 1, theta, precision, out, ph);
}

extern "C" int mwsep_ctx_likelihood(mwsep_ctx* c, const double* theta, const double* integrals, int precision,
                                    mwsep_result* out)
{
    if (!c || !integrals) return mwsep_fail(MWSEP_ERR_ARG);
    CU(cudaSetDevice(c->device));
    Phases ph;
    ph.integrals = false;
    ph.given_integrals = integrals;
    return evaluate_wedge(c, 0, 1, theta, precision, out, ph);
}

extern "C" int mwsep_ctx_evaluate_batch(mwsep_ctx* c, int n_theta, const double* thetas, int precision,
                                        mwsep_result* out)
{
    if (!c) return mwsep_fail(MWSEP_ERR_ARG);
    CU(cudaSetDevice(c->device));
    return evaluate_impl(c, n_theta, thetas, precision, out);
}

extern "C" int mwsep_ctx_device_bytes(const mwsep_ctx* c, size_t* out)
{
    if (!c || !out) return mwsep_fail(MWSEP_ERR_ARG);
    *out = c->dev_bytes;
    return MWSEP_OK;
}

extern "C" int mwsep_ctx_last_timings(const mwsep_ctx* c, double* out5)
{
    if (!c || !out5) return mwsep_fail(MWSEP_ERR_ARG);
    for (int i = 0; i < 5; ++i) out5[i] = c->last_ms[i];
    return MWSEP_OK;
}

extern "C" int mwsep_ctx_last_launches(const mwsep_ctx* c, int* out)
{
    if (!c || !out) return mwsep_fail(MWSEP_ERR_ARG);
    *out = c->last_launches;
    return MWSEP_OK;
}

extern "C" double mwsep_model_tile_cost(int r_steps, int convolve, int group, long long tiles_per_chunk, int k_chunk,
                                        int sms, int blocks_per_sm, int warps_per_block, double prologue)
{
    if (r_steps < 1 || convolve < 1 || group < 1 || tiles_per_chunk < 1 || k_chunk < 1 || sms < 1 ||
        blocks_per_sm < 1 || warps_per_block < 1)
        return -1.0;
    return static_tile_cost(r_steps, convolve, group, tiles_per_chunk, k_chunk, sms, blocks_per_sm, warps_per_block,
                            prologue);
}

extern "C" int mwsep_model_kchunk(int r_steps, int convolve, int n_streams, long long mu_steps, long long nu_steps,
                                  int sms, int blocks_per_sm, int* k_chunk, double* cost)
{
    if (r_steps < 1 || convolve < 1 || n_streams < 0 || n_streams > 8 || mu_steps < 1 || nu_steps < 1 || sms < 1 ||
        blocks_per_sm < 1 || !k_chunk)
        return mwsep_fail(MWSEP_ERR_ARG);
    int group, ks, kmin;
    warp_tile_groups(MWSEP_MIXED_F32, n_streams, convolve, r_steps, group, ks, kmin);
    const long long tiles_per_chunk = mwsep::warp_tile_count((int)mu_steps, (int)nu_steps, 1);
    *k_chunk = model_kchunk(r_steps, convolve, group, tiles_per_chunk, kmin, sms, blocks_per_sm, 256 / 32, cost);
    return MWSEP_OK;
}

extern "C" int mwsep_ctx_transfer_bytes(const mwsep_ctx* c, size_t* h2d_out, size_t* d2h_out)
{
    if (!c || !h2d_out || !d2h_out) return mwsep_fail(MWSEP_ERR_ARG);
    *h2d_out = c->xfer_h2d;
    *d2h_out = c->xfer_d2h;
    return MWSEP_OK;
}

/* --------------------------------------------------------- EvalFunc path */

namespace {

std::mutex g_default_mu;
mwsep_ctx* g_default = nullptr;
size_t g_last_h2d = 0, g_last_d2h = 0;

double evalfunc_impl(double* parameters, ASTRONOMY_PARAMETERS* ap, EVALUATION_STATE* es, STAR_POINTS* sp,
                     int precision)
{
    const double nan = NAN;
    if (!parameters || !ap || !es || !sp)
    {
        mwsep_fail(MWSEP_ERR_ARG);
        return nan;
    }
    std::lock_guard<std::mutex> lock(g_default_mu);
    if (!g_default)
    {
        int dev = 0;
        if (const char* e = getenv("MWSEP_DEVICE")) dev = atoi(e);
        if (mwsep_ctx_create(dev, &g_default) != MWSEP_OK) return nan;
    }
    /* cpu_evaluate: set_astronomy_parameters (:763), then integrals and
     * likelihood. */
    const size_t h2d0 = g_default->xfer_h2d, d2h0 = g_default->xfer_d2h;
    if (mwsep_set_astronomy_parameters(ap, parameters) != MWSEP_OK) return nan;
    if (mwsep_ctx_set_problem(g_default, ap) != MWSEP_OK) return nan;
    if (es->number_integrals != ap->number_integrals || es->number_streams != ap->number_streams || !es->integral)
    {
        mwsep_fail(MWSEP_ERR_STATE);
        return nan;
    }
    /* calculate_integral walks each area from the state's min_calculation
     * (reset_evaluation_state, cpu/evaluation_state.c:197) to its
     * max_calculation (cpu/evaluation_optimized.c:521-527) */
    mwsep_ctx* c = g_default;
    {
        long mn[MWSEP_MAX_AREAS], mx[MWSEP_MAX_AREAS];
        for (int a = 0; a < ap->number_integrals; ++a)
        {
            if (!es->integral[a])
            {
                mwsep_fail(MWSEP_ERR_STATE);
                return nan;
            }
            mn[a] = es->integral[a]->min_calculation;
            mx[a] = es->integral[a]->max_calculation;
        }
        if (wedge_set_slices(c, *c->wedges[0], mn, mx) != MWSEP_OK) return nan;
    }
    /* the catalogue goes up on the side stream while the integral (which
     * does not read it) runs; the likelihood waits for it */
    if (!sp->stars || sp->number_stars < 1)
    {
        mwsep_fail(MWSEP_ERR_ARG);
        return nan;
    }
    if (cudaSetDevice(c->device) != cudaSuccess)
    {
        mwsep_fail(MWSEP_ERR_CUDA);
        return nan;
    }
    int rc = wedge_set_stars_rows(c, *c->wedges[0], sp, true);
    c->eng.desc_dirty = true;
    mwsep_result r;
    if (rc == MWSEP_OK) rc = mwsep_ctx_evaluate(c, parameters, precision, &r);
    if (c->stars_pending)
    {
        /* an evaluation that stopped early still leaves valid star tables */
        const int rc2 = launch_star_build(c, nullptr);
        if (cudaEventSynchronize(c->ev_stars) != cudaSuccess || rc2) rc = rc ? rc : mwsep_fail(MWSEP_ERR_CUDA);
        c->stars_pending = false;
    }
    if (rc != MWSEP_OK) return nan;
    g_last_h2d = g_default->xfer_h2d - h2d0;
    g_last_d2h = g_default->xfer_d2h - d2h0;

    const int S = ap->number_streams;
    for (int a = 0; a < ap->number_integrals; ++a)
    {
        INTEGRAL_AREA* ia = es->integral[a];
        ia->background_integral = r.area_integrals[a][0];
        for (int s = 0; s < S; ++s) ia->stream_integrals[s] = r.area_integrals[a][1 + s];
        /* where calculate_integral's walk stopped: after its last cell */
        const AreaHost& A = c->wedges[0]->prob.area[a];
        ia->current_calculation = A.cell_begin < A.cell_end ? (long)A.cell_end : ia->min_calculation;
    }
    es->current_integral = ap->number_integrals;
    es->background_integral = r.background_integral;
    for (int s = 0; s < S; ++s) es->stream_integrals[s] = r.stream_integrals[s];
    es->current_star_point = sp->number_stars;
    es->total_stars = sp->number_stars;
    es->num_zero = r.num_zero;
    es->bad_jacobians = 0;
    es->prob_sum = r.prob_sum;
    return es->prob_sum / (sp->number_stars - es->bad_jacobians);
}

/* The library's default context for the process-wide entries (created on
 * first use; the caller holds g_default_mu). */
mwsep_ctx* default_ctx()
{
    if (!g_default)
    {
        int dev = 0;
        if (const char* e = getenv("MWSEP_DEVICE")) dev = atoi(e);
        if (mwsep_ctx_create(dev, &g_default) != MWSEP_OK) return nullptr;
    }
    return g_default;
}

/* Writes NaN into the n results of a failed worker step. */
void worker_fail(double* results, int n)
{
    if (results)
        for (int i = 0; i < n; ++i) results[i] = NAN;
}

} // namespace

/* integral_f (cpu/astronomy_worker.c:33-64): theta applied to *ap, this
 * rank's cells of every area integrated (es->integral[i]'s
 * [min_calculation, max_calculation), as calculate_integral walks them),
 * the cut-subtracted background and stream integrals into results[0..S]
 * and into es, as the reference leaves them. */
extern "C" void mwsep_integral_f(double* parameters, double* results, ASTRONOMY_PARAMETERS* ap, EVALUATION_STATE* es,
                                 STAR_POINTS* sp)
{
    (void)sp; /* the integrals read no catalogue */
    const int S = ap ? ap->number_streams : 0;
    if (!parameters || !results || !ap || !es || S < 0 || S > MWSEP_MAX_STREAMS)
    {
        mwsep_fail(MWSEP_ERR_ARG);
        worker_fail(results, S >= 0 && S <= MWSEP_MAX_STREAMS ? 1 + S : 0);
        return;
    }
    std::lock_guard<std::mutex> lock(g_default_mu);
    mwsep_ctx* c = default_ctx();
    if (!c || mwsep_set_astronomy_parameters(ap, parameters) != MWSEP_OK || mwsep_ctx_set_problem(c, ap) != MWSEP_OK)
        return worker_fail(results, 1 + S);
    if (es->number_integrals != ap->number_integrals || es->number_streams != S || !es->integral)
    {
        mwsep_fail(MWSEP_ERR_STATE);
        return worker_fail(results, 1 + S);
    }
    long mn[MWSEP_MAX_AREAS], mx[MWSEP_MAX_AREAS];
    for (int a = 0; a < ap->number_integrals; ++a)
    {
        if (!es->integral[a])
        {
            mwsep_fail(MWSEP_ERR_STATE);
            return worker_fail(results, 1 + S);
        }
        mn[a] = es->integral[a]->min_calculation;
        mx[a] = es->integral[a]->max_calculation;
    }
    mwsep_result r;
    if (wedge_set_slices(c, *c->wedges[0], mn, mx) != MWSEP_OK ||
        mwsep_ctx_integrals(c, parameters, MWSEP_PLAIN_F64, &r) != MWSEP_OK)
        return worker_fail(results, 1 + S);
    for (int a = 0; a < ap->number_integrals; ++a)
    {
        INTEGRAL_AREA* ia = es->integral[a];
        ia->background_integral = r.area_integrals[a][0];
        for (int s = 0; s < S; ++s) ia->stream_integrals[s] = r.area_integrals[a][1 + s];
        const AreaHost& A = c->wedges[0]->prob.area[a];
        ia->current_calculation = A.cell_begin < A.cell_end ? (long)A.cell_end : ia->min_calculation;
    }
    es->current_integral = ap->number_integrals;
    es->background_integral = results[0] = r.background_integral;
    for (int s = 0; s < S; ++s) es->stream_integrals[s] = results[1 + s] = r.stream_integrals[s];
}

/* likelihood_f (cpu/astronomy_worker.c:94-121): calculate_likelihood of
 * this rank's stars at *ap's current parameters against the given
 * (composed) integrals[0..S]; results[0] = prob_sum, results[1] =
 * bad_jacobians (always 0), and es as the reference leaves it. */
extern "C" void mwsep_likelihood_f(double* integrals, double* results, ASTRONOMY_PARAMETERS* ap, EVALUATION_STATE* es,
                                   STAR_POINTS* sp)
{
    if (!integrals || !results || !ap || !es || !sp || ap->number_streams < 0 ||
        ap->number_streams > MWSEP_MAX_STREAMS)
    {
        mwsep_fail(MWSEP_ERR_ARG);
        return worker_fail(results, 2);
    }
    const int S = ap->number_streams;
    std::lock_guard<std::mutex> lock(g_default_mu);
    mwsep_ctx* c = default_ctx();
    const int P = mwsep_get_optimized_parameter_count(ap);
    if (!c || P < 0) return worker_fail(results, 2);
    std::vector<double> theta((size_t)std::max(P, 1));
    if (mwsep_get_search_parameters(ap, theta.data()) != MWSEP_OK || mwsep_ctx_set_problem(c, ap) != MWSEP_OK)
        return worker_fail(results, 2);
    if (cudaSetDevice(c->device) != cudaSuccess)
    {
        mwsep_fail(MWSEP_ERR_CUDA);
        return worker_fail(results, 2);
    }
    if (wedge_set_stars_rows(c, *c->wedges[0], sp, false) != MWSEP_OK) return worker_fail(results, 2);
    c->eng.desc_dirty = true;
    mwsep_result r;
    if (mwsep_ctx_likelihood(c, theta.data(), integrals, MWSEP_PLAIN_F64, &r) != MWSEP_OK)
        return worker_fail(results, 2);
    es->background_integral = integrals[0];
    if (es->stream_integrals)
        for (int s = 0; s < S && s < es->number_streams; ++s) es->stream_integrals[s] = integrals[1 + s];
    es->current_star_point = sp->number_stars;
    es->num_zero = r.num_zero;
    es->bad_jacobians = 0;
    es->prob_sum = r.prob_sum;
    results[0] = r.prob_sum;
    results[1] = 0.0;
}

extern "C" int mwsep_evalfunc_transfer_bytes(size_t* h2d_out, size_t* d2h_out)
{
    if (!h2d_out || !d2h_out) return mwsep_fail(MWSEP_ERR_ARG);
    std::lock_guard<std::mutex> lock(g_default_mu);
    *h2d_out = g_last_h2d;
    *d2h_out = g_last_d2h;
    return MWSEP_OK;
}

extern "C" double mwsep_evaluate(double* parameters, ASTRONOMY_PARAMETERS* ap, EVALUATION_STATE* es,
                                 STAR_POINTS* sp)
{
    return evalfunc_impl(parameters, ap, es, sp, MWSEP_PLAIN_F64);
}

extern "C" double mwsep_evaluate_mixed(double* parameters, ASTRONOMY_PARAMETERS* ap, EVALUATION_STATE* es,
                                       STAR_POINTS* sp)
{
    return evalfunc_impl(parameters, ap, es, sp, MWSEP_MIXED_F32);
}

extern "C" double mwsep_evaluate_df(double* parameters, ASTRONOMY_PARAMETERS* ap, EVALUATION_STATE* es,
                                    STAR_POINTS* sp)
{
    return evalfunc_impl(parameters, ap, es, sp, MWSEP_PLAIN_DF);
}
