/* mwsep_df.cu -- the plain form's integral in double-float arithmetic
 * (MWSEP_PLAIN_DF): FP64-level accuracy computed on the FP32 pipes.
 *
 * Same decomposition as the compensated warp tiles (32 mu-columns at one nu
 * and a run of r-bins per warp; each lane holds DFP points of a group, the
 * columns' constants are broadcast from shared memory), with every quantity
 * carried as a double-float pair (mwsep_df.cuh):
 *   t = r - rb,  rg = sqrt(B2 t^2 + Db),  bg += w / (rg (rg + r0)^3),
 *   stream s:  st_s += w 2^(k2_s (r - rs_s)^2 + k0_s),
 * where w = qw_r3_N * reff_xr_rp3 * irv is the table weight (as a pair), the
 * completed-square constants are formed per column in FP64 (as in the plain
 * FP64 kernel) and the stream exponent is in base 2.  FP32 has an exponent
 * range of 2^+-126, so before each lane group the warp finds, in FP32, the
 * largest stream exponent over the group's points and the tile's columns
 * (a cheap pass: per column and stream the point nearest the stream's
 * closest approach, 2 operations per point), and each column
 * writes its k0 shifted by floor of that maximum, formed in FP64.  The
 * group's largest term is then about 1 and its sums are scaled back in FP64,
 * so integrals far below FP32 range keep their FP64 magnitude; terms more
 * than 2^126 below the group's largest are dropped, far below FP64
 * resolution of the sum.
 *
 * Per lane the group sums are double-float; per group they go to FP64
 * (times ids), across blocks the usual compensated FP64 reduction.
 *
 * Background forms: alpha = delta = 1 with or without the aux profile,
 * general alpha/delta, and q = 0 (the aux share and the q = 0 background
 * are column-independent: aux_area_kernel adds them), up to 8 streams (the
 * likelihood kernel below up to 4; the host runs the FP64 likelihood
 * beyond).
 */
#include <cuda_runtime.h>
#include <math.h>

#include <atomic>
#include <mutex>

#include "milkyway_separation_gb300.h"
#include "milkyway_separation_gb300_test.h"
#include "mwsep_checks.cuh"
#include "mwsep_df.cuh"
#include "mwsep_f64_point.cuh"
#include "mwsep_internal.h"
#include "mwsep_reduce.cuh"


namespace {

using mwsep::dfl::df;
namespace D = mwsep::dfl;

/* Integral blocks: 8 warps up to 3 streams, 4 warps for 4-8 streams (the
 * columns' constants and the log2 table of the general form then fit the
 * static shared memory). */
template <int S>
struct DfShape
{
    static constexpr int block = S >= 4 ? 128 : 256;
    static constexpr int min_blocks = S >= 4 ? 4 : 2;
};
/* Background forms of the double-float kernels: alpha = delta = 1 (the aux
 * profile's share added separately), general alpha/delta, or none (q = 0:
 * the background is -1 per cell, added separately); each launch skips the
 * thetas of the other forms. */
constexpr int kFormHern = 0, kFormGeneral = 2, kFormNone = 3;
__device__ __forceinline__ bool df_form_is(const mwsep_theta_consts& th, int form)
{
    const int f = mwsep_bg_form(&th);
    return form == kFormHern ? f <= 1 : f == form;
}
static_assert(MWSEP_DF_TILE_P % 2 == 0, "points are taken in pairs");

/* Column constants, as pairs: B2, rb, Db, then per stream rs, k2, k0 - eref. */
template <int S>
struct ColDF
{
    static constexpr int W = 2 * (3 + 3 * S); /* floats */
};
__host__ __device__ constexpr int kSP(int S) { return S > 0 ? S : 1; }

/* 2^(j/1024) as pairs (host-built). */
__constant__ float2 c_exp2_tab[D::kExp2Table];
/* {log2 c, 1/c} as pairs for c = 1 + j/256 (host-built). */
__constant__ float4 c_log2_tab[D::kLog2Table];

template <int S>
__device__ __forceinline__ void put(float* dst, int i, double v)
{
    const df x = D::from_double(v);
    dst[2 * i] = x.hi;
    dst[2 * i + 1] = x.lo;
}

template <int S>
__device__ __forceinline__ df get(const float* src, int i)
{
    const float2 v = reinterpret_cast<const float2*>(src)[i];
    return D::mk(v.x, v.y);
}

/* One warp tile of the double-float integral (all 32 lanes). */
template <int S, int FORM>
__device__ __forceinline__ void warp_tile_df(const mwsep_area_dev& A, const mwsep_theta_consts& th, long long wt,
                                             float* __restrict__ cs, float* __restrict__ kf,
                                             const float* __restrict__ thi, const float* __restrict__ tlo,
                                             const float4* __restrict__ ltab, double (&acc)[1 + S])
{
    constexpr int CW = ColDF<S>::W;
    constexpr int DFP = mwsep_df_tile_p(S); /* points per lane per group */
    constexpr int NPR = DFP / 2;            /* ... as pairs of points */
    const int lane = threadIdx.x & 31;
    const mwsep::TilePos tp = mwsep::tile_pos(A, wt);
    const int nu = tp.nu;
    const int mu0 = tp.mu0;
    const int ncols = tp.ncols;

    /* column constants (FP64); the stream exponents in base 2 */
    mwsep::f64::ColF64<kSP(S)> cc;
    double k0b[kSP(S)];
    const bool live = lane < ncols;
    if (live)
    {
        const double* g = A.geom + 4 * (size_t)MWSEP_IDX((size_t)(mu0 + lane) * A.nu_steps + nu, A.n_cols, 1);
        mwsep::f64::column_consts_f64<kSP(S)>(g[0], g[1], g[2], g[3], th, cc);
        constexpr double kLog2e = 1.4426950408889634073599246810018921;
        float* c = cs + lane * CW;
        put<S>(c, 0, cc.B2);
        put<S>(c, 1, cc.rb);
        put<S>(c, 2, cc.Db);
#pragma unroll
        for (int s = 0; s < S; ++s)
        {
            const bool on = s < th.n_streams && th.stream_on[s];
            k0b[s] = on ? cc.k0[s] * kLog2e : -1.0e300;
            put<S>(c, 3 + 3 * s, cc.rs[s]);
            put<S>(c, 4 + 3 * s, on ? cc.k2[s] * kLog2e : 0.0);
            put<S>(c, 5 + 3 * s, -1.0e30); /* set per group */
            kf[lane * kSP(S) + s] = on ? (float)fmax(k0b[s], -1.0e30) : -1.0e30f;
        }
    }
    __syncwarp();

    const D::df2 r0 = D::dup(D::from_double(th.r0));
    const D::df2 al = D::dup(D::from_double(th.alpha)), ad3 = D::dup(D::from_double(th.alpha_delta3));
    const int C = A.convolve;
    const int k0 = tp.k0;
    const int k1 = tp.k1;
    const int nf = (k1 - k0) * C;
    const double idsv = A.ids[MWSEP_IDX(nu, A.nu_steps, 3)];
    for (int g0 = 0; g0 < nf; g0 += 32 * DFP)
    {
        /* the lane's points as pairs of points: pair q holds points 2q and
         * 2q + 1 in the two halves of each register pair */
        D::df2 r[NPR], w[NPR];
#pragma unroll
        for (int q = 0; q < NPR; ++q)
        {
            const int fa = g0 + 32 * (2 * q) + lane, fb = fa + 32;
            /* past the tile's end: a copy of its first point with zero weight */
            const float4 va = A.ptsdf[MWSEP_IDX((size_t)k0 * C + (fa < nf ? fa : 0), (size_t)A.r_steps * C, 2)];
            const float4 vb = A.ptsdf[MWSEP_IDX((size_t)k0 * C + (fb < nf ? fb : 0), (size_t)A.r_steps * C, 2)];
            r[q] = D::mk2(make_float2(va.x, vb.x), make_float2(va.y, vb.y));
            w[q] = D::mk2(make_float2(fa < nf ? va.z : 0.f, fb < nf ? vb.z : 0.f),
                          make_float2(fa < nf ? va.w : 0.f, fb < nf ? vb.w : 0.f));
        }
        /* the group's largest stream exponent (FP32 estimate, error far
         * below 1 for |k0| < 2^20), and the columns' k0 shifted by its floor */
        double scale[kSP(S)];
        if constexpr (S > 0)
        {
            float mx[S];
#pragma unroll
            for (int s = 0; s < S; ++s) mx[s] = -3.0e38f;
            for (int j = 0; j < ncols; ++j)
            {
                const float* c = cs + j * CW;
#pragma unroll
                for (int s = 0; s < S; ++s)
                {
                    /* k2 <= 0: the largest exponent is at the point nearest rs */
                    const float rs = c[2 * (3 + 3 * s)], k2 = c[2 * (4 + 3 * s)], k0 = kf[j * S + s];
                    float um = 3.0e38f;
#pragma unroll
                    for (int q = 0; q < NPR; ++q)
                        um = fminf(um, fminf(fabsf(__fsub_rn(r[q].hi.x, rs)), fabsf(__fsub_rn(r[q].hi.y, rs))));
                    mx[s] = fmaxf(mx[s], __fmaf_rn(k2, __fmul_rn(um, um), k0));
                }
            }
            int eref[S];
#pragma unroll
            for (int s = 0; s < S; ++s)
            {
                for (int o = 16; o > 0; o >>= 1) mx[s] = fmaxf(mx[s], __shfl_xor_sync(0xffffffffu, mx[s], o));
                eref[s] = (int)floorf(fmaxf(mx[s], -1100.0f));
                scale[s] = eref[s] > -1100 ? ldexp(1.0, eref[s]) : 0.0;
            }
            __syncwarp(); /* every lane is done with the previous group's constants */
#pragma unroll
            for (int s = 0; s < S; ++s)
                if (live && s < th.n_streams && th.stream_on[s])
                    put<S>(cs + lane * CW, 5 + 3 * s, fmax(k0b[s] - (double)eref[s], -1.0e30));
            __syncwarp();
        }
        /* Per column: the background over the lane's points, then one
         * stream at a time (a rolled loop: the unrolled body of every stream
         * over every point overflows the instruction cache).  Each stream's
         * terms are summed as a run (two halves of four), then added to its
         * lane sums (two halves, joined in FP64 at the end of the group). */
        D::df2 bg = D::mk2(D::pd(0.f), D::pd(0.f)), st[kSP(S)];
#pragma unroll
        for (int s = 0; s < S; ++s) st[s] = D::mk2(D::pd(0.f), D::pd(0.f));
        for (int j = 0; j < ncols; ++j)
        {
            const float* c = cs + j * CW;
            const D::df2 B2 = D::dup(get<S>(c, 0)), nrb = D::dup(D::neg(get<S>(c, 1))), Db = D::dup(get<S>(c, 2));
            if constexpr (FORM != kFormNone)
            {
            D::lazy_sum2 pb;
#pragma unroll
            for (int q = 0; q < NPR; ++q)
            {
                const D::df2 rg = D::sqrt2(D::sq_scale_add2(B2, D::add_fast2(r[q], nrb), Db));
                const D::df2 sum = D::add_fast2(rg, r0);
                D::df2 v;
                if constexpr (FORM == kFormHern)
                    v = D::div2(w[q], D::mul2(rg, D::mul2(sum, D::sqr2(sum))));
                else /* w / (rg^alpha (rg + r0)^(3 - alpha + delta)) = w 2^-(alpha log2 rg + ad3 log2(rg + r0)) */
                {
                    const D::df2 E = D::add_fast2(D::mul2(al, D::log2_2(rg, ltab)), D::mul2(ad3, D::log2_2(sum, ltab)));
                    v = D::mul_raw2(w[q], D::exp2_2(D::mk2(D::pneg(E.hi), D::pneg(E.lo)), thi, tlo));
                }
                if (q == 0)
                    pb = D::lazy_start2(v);
                else
                    D::lazy_add2(pb, v);
            }
            bg = D::add_fast2(bg, D::lazy_end2(pb));
            }
#pragma unroll 1
            for (int s = 0; s < S; ++s)
            {
                const D::df2 nrs = D::dup(D::neg(get<S>(c, 3 + 3 * s))), k2 = D::dup(get<S>(c, 4 + 3 * s)),
                             k0 = D::dup(get<S>(c, 5 + 3 * s));
                D::lazy_sum2 ps;
#pragma unroll
                for (int q = 0; q < NPR; ++q)
                {
                    const D::df2 a = D::sq_scale_add2(k2, D::add_fast2(r[q], nrs), k0);
                    const D::df2 e = D::mul_raw2(w[q], D::exp2_2(a, thi, tlo));
                    if (q == 0)
                        ps = D::lazy_start2(e);
                    else
                        D::lazy_add2(ps, e);
                }
                st[s] = D::add_fast2(st[s], D::lazy_end2(ps));
            }
        }
        acc[0] += (((double)bg.hi.x + (double)bg.lo.x) + ((double)bg.hi.y + (double)bg.lo.y)) * idsv;
#pragma unroll
        for (int s = 0; s < S; ++s)
            acc[1 + s] += (((double)st[s].hi.x + (double)st[s].lo.x) + ((double)st[s].hi.y + (double)st[s].lo.y)) *
                          scale[s] * idsv;
    }
    __syncwarp();
}

/* DYN: tiles handed out by counters[theta * counter_stride] instead of a
 * fixed share per warp (the warp scheduler favours an SM's older block), each
 * tile's sums added across the warp in a fixed order into the tile's own
 * slot of `partials` (tile-major, 1 + S components) for the fixed-order slot
 * reduction. */
template <int S, int FORM, bool DYN>
__global__ void __launch_bounds__(DfShape<S>::block, DfShape<S>::min_blocks) integral_df_kernel(const mwsep_area_dev A,
                                                                const mwsep_theta_consts* __restrict__ thetas,
                                                                double2* __restrict__ partials, long long theta_stride,
                                                                int* __restrict__ counters, int counter_stride)
{
    __shared__ mwsep_theta_consts th;
    constexpr int kBlock = DfShape<S>::block;
    __shared__ __align__(16) float cs[kBlock / 32][mwsep::kTileCols * ColDF<S>::W];
    static_assert(sizeof(cs) >= 2 * (1 + S) * 32 * sizeof(double), "the block reduction reuses cs");
    __shared__ float kf[kBlock / 32][mwsep::kTileCols * kSP(S)];
    __shared__ float thi[D::kExp2Table], tlo[D::kExp2Table];
    __shared__ float4 ltab[FORM == kFormGeneral ? D::kLog2Table : 1];
    mwsep::f64::load_theta(th, thetas + blockIdx.y);
    for (int j = threadIdx.x; j < D::kExp2Table; j += kBlock)
    {
        thi[j] = c_exp2_tab[j].x;
        tlo[j] = c_exp2_tab[j].y;
    }
    if (FORM == kFormGeneral)
        for (int j = threadIdx.x; j < D::kLog2Table; j += kBlock) ltab[j] = c_log2_tab[j];
    __syncthreads();
    if (!df_form_is(th, FORM)) return; /* the other form's launch covers this theta (whole block) */
    const int warp = threadIdx.x >> 5;
    if constexpr (DYN)
    {
        const int lane = threadIdx.x & 31;
        const int NC = 1 + th.n_streams;
        int* ctr = counters + (size_t)blockIdx.y * counter_stride;
        double2* out = partials + (size_t)blockIdx.y * theta_stride;
        for (;;)
        {
            int wt = 0;
            if (lane == 0) wt = atomicAdd(ctr, 1);
            wt = __shfl_sync(0xffffffffu, wt, 0);
            if ((long long)wt >= A.n_items) break;
            double acc[1 + S];
#pragma unroll
            for (int k = 0; k < 1 + S; ++k) acc[k] = 0.0;
            warp_tile_df<S, FORM>(A, th, wt, cs[warp], kf[warp], thi, tlo, ltab, acc);
#pragma unroll
            for (int k = 0; k < 1 + S; ++k)
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], off);
            if (lane == 0)
            {
#pragma unroll
                for (int k = 0; k < 1 + S; ++k)
                    if (k < NC) out[(size_t)wt * NC + k] = make_double2(acc[k], 0.0);
            }
        }
        return;
    }
    double acc[1 + S];
#pragma unroll
    for (int k = 0; k < 1 + S; ++k) acc[k] = 0.0;
    const long long warps = (long long)gridDim.x * (kBlock / 32);
    for (long long wt = (long long)blockIdx.x * (kBlock / 32) + warp; wt < A.n_items; wt += warps)
        warp_tile_df<S, FORM>(A, th, wt, cs[warp], kf[warp], thi, tlo, ltab, acc);
    /* block reduction into compensated pairs, in cs once every warp is done
     * with its tiles */
    __syncthreads();
    double* red = reinterpret_cast<double*>(&cs[0][0]);
    mwsep::comp_sum cacc[1 + S];
#pragma unroll
    for (int k = 0; k < 1 + S; ++k)
    {
        cacc[k].s = acc[k];
        cacc[k].c = 0.0;
    }
    mwsep::block_reduce<1 + S>(cacc, red);
    if (threadIdx.x == 0)
    {
        double2* out = partials + (size_t)blockIdx.y * theta_stride + (size_t)blockIdx.x * (1 + th.n_streams);
#pragma unroll
        for (int k = 0; k < 1 + S; ++k)
            if (k < 1 + th.n_streams) out[k] = make_double2(cacc[k].s, cacc[k].c);
    }
}

template <int S>
int launch(const mwsep_area_dev* A, const mwsep_theta_consts* th, const mwsep_launch_shape* sh, double2* partials,
           cudaStream_t st)
{
    const long long ncomp = 1 + sh->n_streams;
    const long long theta_stride = (long long)sh->n_areas * sh->grid * ncomp;
    double2* base = partials + (size_t)sh->area_index * sh->grid * ncomp;
    dim3 g(sh->grid, sh->n_theta);
    if (sh->bg_form == kFormGeneral)
        integral_df_kernel<S, kFormGeneral, false>
            <<<g, DfShape<S>::block, 0, st>>>(*A, th, base, theta_stride, nullptr, 0);
    else if (sh->bg_form == kFormNone)
        integral_df_kernel<S, kFormNone, false><<<g, DfShape<S>::block, 0, st>>>(*A, th, base, theta_stride, nullptr, 0);
    else
        integral_df_kernel<S, kFormHern, false><<<g, DfShape<S>::block, 0, st>>>(*A, th, base, theta_stride, nullptr, 0);
    return (int)cudaGetLastError();
}

template <int S>
int launch_dyn(const mwsep_area_dev* A, const mwsep_theta_consts* th, const mwsep_launch_shape* sh,
               long long n_slots, double2* slots, int* counters, cudaStream_t st)
{
    const long long ncomp = 1 + sh->n_streams;
    const long long theta_stride = (long long)sh->n_areas * n_slots * ncomp;
    double2* base = slots + (size_t)sh->area_index * n_slots * ncomp;
    int* ctr = counters + sh->area_index;
    dim3 g(sh->grid, sh->n_theta);
    if (sh->bg_form == kFormGeneral)
        integral_df_kernel<S, kFormGeneral, true>
            <<<g, DfShape<S>::block, 0, st>>>(*A, th, base, theta_stride, ctr, sh->n_areas);
    else if (sh->bg_form == kFormNone)
        integral_df_kernel<S, kFormNone, true>
            <<<g, DfShape<S>::block, 0, st>>>(*A, th, base, theta_stride, ctr, sh->n_areas);
    else
        integral_df_kernel<S, kFormHern, true>
            <<<g, DfShape<S>::block, 0, st>>>(*A, th, base, theta_stride, ctr, sh->n_areas);
    return (int)cudaGetLastError();
}

/* Resident blocks per SM: the smallest of the forms' (one grid serves all). */
template <int S>
cudaError_t occupancy(int* b)
{
    int b0 = 0, b2 = 0, b3 = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b0, integral_df_kernel<S, kFormHern, false>,
                                                                  DfShape<S>::block, 0);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b2, integral_df_kernel<S, kFormGeneral, false>, DfShape<S>::block, 0);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b3, integral_df_kernel<S, kFormNone, false>, DfShape<S>::block, 0);
    *b = b0 < b2 ? b0 : b2;
    *b = *b < b3 ? *b : b3;
    return e;
}

/* Per-star double-float table [C][N]: {r_hi, r_lo, qw_hi, qw_lo}. */
__global__ void star_df_table_kernel(long long total, const double* __restrict__ r_point,
                                     const double* __restrict__ qw, float4* __restrict__ out)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x)
    {
        const df r = D::from_double(r_point[i]), q = D::from_double(qw[i]);
        out[i] = make_float4(r.hi, r.lo, q.hi, q.lo);
    }
}

/* calculate_likelihood for one star per thread (cpu/evaluation_optimized.c:
 * 665-717) with the convolution in double-float: the star's completed-square
 * constants in FP64 (as the integral's columns), each stream's exponent
 * shifted by floor of its largest value over the star's points (the point
 * nearest the stream's closest approach, found in FP32), the points' terms
 * summed in runs of eight, and the mixture weights and log10 sums in FP64
 * (likelihood_finish, shared with the FP64 kernel). */
template <int S, int FORM>
__global__ void __launch_bounds__(256) likelihood_df_kernel(const mwsep_stars_dev St, const float4* __restrict__ pdf,
                                                            const mwsep_theta_consts* __restrict__ thetas,
                                                            const double* __restrict__ integrals,
                                                            double2* __restrict__ partials, long long theta_stride)
{
    constexpr int SP = kSP(S);
    __shared__ mwsep_theta_consts th;
    __shared__ double red[2 * (3 + SP) * 32];
    __shared__ float2 tab[D::kExp2Table];
    __shared__ float4 ltab[FORM == kFormGeneral ? D::kLog2Table : 1];
    mwsep::f64::load_theta(th, thetas + blockIdx.y);
    for (int j = threadIdx.x; j < D::kExp2Table; j += blockDim.x) tab[j] = c_exp2_tab[j];
    if (FORM == kFormGeneral)
        for (int j = threadIdx.x; j < D::kLog2Table; j += blockDim.x) ltab[j] = c_log2_tab[j];
    __syncthreads();
    if (!df_form_is(th, FORM)) return; /* the other form's launch covers this theta (whole block) */
    const double* I = integrals + (size_t)blockIdx.y * (1 + th.n_streams);
    mwsep::comp_sum acc[3 + SP];
#pragma unroll
    for (int k = 0; k < 3 + SP; ++k) acc[k].zero();
    constexpr double kLog2e = 1.4426950408889634073599246810018921;
    const int N = St.n_stars, C = St.convolve;
    const df r0 = D::from_double(th.r0);
    const df al = D::from_double(th.alpha), ad3 = D::from_double(th.alpha_delta3);
    for (int s0 = blockIdx.x * blockDim.x + threadIdx.x; s0 < N; s0 += gridDim.x * blockDim.x)
    {
        const double* g = St.geom + 4 * (size_t)s0;
        mwsep::f64::ColF64<SP> cc;
        mwsep::f64::column_consts_f64<SP>(g[0], g[1], g[2], g[3], th, cc);
        const df B2 = D::from_double(cc.B2), nrb = D::from_double(-cc.rb), Db = D::from_double(cc.Db);
        df nrs[SP], k2[SP], k0[SP];
        double scale[SP];
        float rsf[SP], umin[SP];
#pragma unroll
        for (int s = 0; s < S; ++s)
        {
            rsf[s] = (float)cc.rs[s];
            umin[s] = 3.0e38f;
        }
        if constexpr (S > 0)
        {
            for (int n = 0; n < C; ++n)
            {
                const float rh = pdf[(size_t)MWSEP_IDX((size_t)n * N + s0, (size_t)C * N, 8)].x;
#pragma unroll
                for (int s = 0; s < S; ++s) umin[s] = fminf(umin[s], fabsf(__fsub_rn(rh, rsf[s])));
            }
        }
#pragma unroll
        for (int s = 0; s < S; ++s)
        {
            const bool on = s < th.n_streams && th.stream_on[s];
            const double k2b = on ? cc.k2[s] * kLog2e : 0.0, k0b = cc.k0[s] * kLog2e;
            const double um = (double)umin[s];
            const int eref = on ? (int)floor(fmax(k2b * um * um + k0b, -1100.0)) : -1100;
            nrs[s] = D::from_double(-cc.rs[s]);
            k2[s] = D::from_double(k2b);
            k0[s] = D::from_double(on ? fmax(k0b - (double)eref, -1.0e30) : -1.0e30);
            scale[s] = eref > -1100 ? ldexp(1.0, eref) : 0.0;
        }
        df bg = D::mk(0.f, 0.f), st[SP];
#pragma unroll
        for (int s = 0; s < S; ++s) st[s] = D::mk(0.f, 0.f);
        for (int n0 = 0; n0 < C; n0 += 8)
        {
            D::lazy_sum pb = {0.f, 0.f}, ps[SP];
#pragma unroll
            for (int s = 0; s < S; ++s) ps[s] = {0.f, 0.f};
            const int n1 = min(n0 + 8, C);
#pragma unroll 1
            for (int n = n0; n < n1; ++n)
            {
                const float4 v = pdf[(size_t)MWSEP_IDX((size_t)n * N + s0, (size_t)C * N, 8)];
                const df r = D::mk(v.x, v.y), w = D::mk(v.z, v.w);
                const df rg = D::sqrt(D::sq_scale_add(B2, D::add_fast(r, nrb), Db));
                const df sum = D::add_fast(rg, r0);
                if constexpr (FORM == kFormHern)
                    D::lazy_add(pb, D::div(w, D::mul(rg, D::mul(sum, D::sqr(sum)))));
                else if constexpr (FORM == kFormGeneral)
                {
                    const df E = D::add_fast(D::mul(al, D::log2(rg, ltab)), D::mul(ad3, D::log2(sum, ltab)));
                    D::lazy_add(pb, D::mul_raw(w, D::exp2(D::neg(E), tab)));
                }
#pragma unroll
                for (int s = 0; s < S; ++s)
                {
                    const df a = D::sq_scale_add(k2[s], D::add_fast(r, nrs[s]), k0[s]);
                    D::lazy_add(ps[s], D::mul_raw(w, D::exp2(a, tab)));
                }
            }
            bg = D::add_fast(bg, D::lazy_end(pb));
#pragma unroll
            for (int s = 0; s < S; ++s) st[s] = D::add_fast(st[s], D::lazy_end(ps[s]));
        }
        /* the aux profile, point by point in FP64 as the reference adds it;
         * q = 0: the background is -1 (cpu/evaluation_optimized.c:213-216) */
        double bgd = FORM == kFormNone ? -1.0 : (double)bg.hi + (double)bg.lo;
        if (th.aux && th.bg_mode == 0)
        {
            double v = 0.0;
            for (int n = 0; n < C; ++n)
            {
                const size_t o = (size_t)MWSEP_IDX((size_t)n * N + s0, (size_t)C * N, 8);
                v += St.qw[o] * (th.bg_a * St.r_in_mag2[o] + th.bg_b * St.r_in_mag[o] + th.bg_c);
            }
            bgd += v;
        }
        double stv[SP];
        stv[0] = 0.0;
#pragma unroll
        for (int s = 0; s < S; ++s) stv[s] = ((double)st[s].hi + (double)st[s].lo) * scale[s];
        mwsep::f64::likelihood_finish<SP>(th, I, St.reff[s0], bgd, stv, acc);
    }
    mwsep::block_reduce<3 + SP>(acc, red);
    if (threadIdx.x == 0)
    {
        double2* out = partials + (size_t)blockIdx.y * theta_stride + (size_t)blockIdx.x * (3 + th.n_streams);
#pragma unroll
        for (int k = 0; k < 3 + SP; ++k)
            if (k < 3 + th.n_streams) out[k] = make_double2(acc[k].s, acc[k].c);
    }
}

template <int S>
int launch_likelihood(const mwsep_stars_dev* St, const float4* pdf, const mwsep_theta_consts* th,
                      const mwsep_launch_shape* sh, const double* integrals, double2* partials, cudaStream_t st)
{
    const long long theta_stride = (long long)sh->grid * (3 + sh->n_streams);
    dim3 g(sh->grid, sh->n_theta);
    if (sh->bg_form == kFormGeneral)
        likelihood_df_kernel<S, kFormGeneral><<<g, sh->block, 0, st>>>(*St, pdf, th, integrals, partials, theta_stride);
    else if (sh->bg_form == kFormNone)
        likelihood_df_kernel<S, kFormNone><<<g, sh->block, 0, st>>>(*St, pdf, th, integrals, partials, theta_stride);
    else
        likelihood_df_kernel<S, kFormHern><<<g, sh->block, 0, st>>>(*St, pdf, th, integrals, partials, theta_stride);
    return (int)cudaGetLastError();
}

/* The column-independent background shares of an area integral, summed
 * over the area's cells as cpu/evaluation_optimized.c:498-520 does (times
 * V = irv_k ids_j), box by box (the whole area is one box):
 *  - the aux profile (form 1: alpha = delta = 1 plus qw (a g^2 + b g + c),
 *    :234-239, times reff):
 *      mu_n * sum_j ids_j * sum_k irv_k reff_k sum_n qw_kn (a g2_kn + b g_kn + c);
 *  - q = 0 (form 3: bg = -1 per cell, no reff, :213-216):
 *      mu_n * sum_j ids_j * sum_k irv_k * (-1),
 * j and k over the box's nu steps and r-bins.  O(R C) work in FP64, added
 * (TwoSum) to block 0's background partial of the area after the
 * double-float kernel has written it.  One block per theta; thetas of the
 * other forms are left alone. */
__global__ void aux_area_kernel(const mwsep_area_dev A, const mwsep_theta_consts* __restrict__ thetas,
                                double2* __restrict__ partials, long long theta_stride)
{
    __shared__ double red[2 * 2 * 32];
    const mwsep_theta_consts* th = thetas + blockIdx.y;
    const int form = mwsep_bg_form(th);
    if (form != 1 && form != 3) return; /* uniform per block */
    const double a = th->bg_a, b = th->bg_b, c = th->bg_c;
    const int C = A.convolve;
    double total = 0.0;
#pragma unroll 1
    for (int bi = 0; bi < A.n_boxes; ++bi)
    {
        mwsep_box bx = A.box[0];
#pragma unroll
        for (int i = 1; i < MWSEP_MAX_BOXES; ++i)
            if (i == bi) bx = A.box[i];
        mwsep::comp_sum acc[2];
        acc[0].zero();
        acc[1].zero();
        for (int k = bx.r0 + threadIdx.x; k < bx.r0 + bx.r_n; k += blockDim.x)
        {
            if (form == 3)
            {
                acc[0].add(-A.irv[k]);
                continue;
            }
            const size_t row = (size_t)k * C;
            double v = 0.0;
            for (int n = 0; n < C; ++n)
                v += A.qw[row + n] * (a * A.r_in_mag2[row + n] + b * A.r_in_mag[row + n] + c);
            acc[0].add(v * A.reff[k] * A.irv[k]);
        }
        for (int j = bx.nu0 + threadIdx.x; j < bx.nu0 + bx.nu_n; j += blockDim.x) acc[1].add(A.ids[j]);
        mwsep::block_reduce<2>(acc, red);
        if (threadIdx.x == 0) total += (acc[0].s + acc[0].c) * (acc[1].s + acc[1].c) * (double)bx.mu_n;
        __syncthreads(); /* red is reused by the next box */
    }
    if (threadIdx.x == 0 && A.n_boxes > 0)
    {
        const double v = total;
        double2* p = partials + (size_t)blockIdx.y * theta_stride;
        const double s = p->x + v;
        const double bb = s - p->x;
        const double e = (p->x - (s - bb)) + (v - bb);
        p->x = s;
        p->y += e;
    }
}

/* Element-wise evaluation of the double-float primitives for the tests:
 * op 0 exp2(x), 1 sqrt(x), 2 x / y, 3 x * y, 4 x + y (Dekker), 5 x y^2 + z,
 * 6 log2(x); ops 10-16 the same through the packed (two values at once)
 * versions;
 * inputs are doubles split into pairs, results returned as hi + lo in FP64. */
__global__ void df_eval_kernel(int op, int n, const double* __restrict__ x, const double* __restrict__ y,
                               const double* __restrict__ z, double* __restrict__ out)
{
    __shared__ float2 tab[D::kExp2Table];
    __shared__ float thi[D::kExp2Table], tlo[D::kExp2Table];
    __shared__ float4 ltab[D::kLog2Table];
    for (int j = threadIdx.x; j < D::kExp2Table; j += blockDim.x)
    {
        tab[j] = c_exp2_tab[j];
        thi[j] = c_exp2_tab[j].x;
        tlo[j] = c_exp2_tab[j].y;
    }
    for (int j = threadIdx.x; j < D::kLog2Table; j += blockDim.x) ltab[j] = c_log2_tab[j];
    __syncthreads();
    if (op >= 10)
    {
        /* element pairs (2i, 2i + 1); an odd last element is paired with itself */
        const int np = (n + 1) / 2;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x)
        {
            const int ia = 2 * i, ib = (2 * i + 1 < n) ? 2 * i + 1 : 2 * i;
            auto pair = [&](const double* v) {
                const df a = D::from_double(v[ia]), b = D::from_double(v[ib]);
                return D::mk2(make_float2(a.hi, b.hi), make_float2(a.lo, b.lo));
            };
            const D::df2 a = pair(x), b = pair(y), c = pair(z);
            D::df2 r;
            switch (op)
            {
            case 10: r = D::exp2_2(a, thi, tlo); break;
            case 11: r = D::sqrt2(a); break;
            case 12: r = D::div2(a, b); break;
            case 13: r = D::mul2(a, b); break;
            case 14: r = D::add_fast2(a, b); break;
            case 15: r = D::sq_scale_add2(a, b, c); break;
            default: r = D::log2_2(a, ltab); break;
            }
            out[ia] = (double)r.hi.x + (double)r.lo.x;
            out[ib] = (double)r.hi.y + (double)r.lo.y;
        }
        return;
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const df a = D::from_double(x[i]), b = D::from_double(y[i]);
        df r;
        switch (op)
        {
        case 0: r = D::exp2(a, tab); break;
        case 1: r = D::sqrt(a); break;
        case 2: r = D::div(a, b); break;
        case 3: r = D::mul(a, b); break;
        case 4: r = D::add_fast(a, b); break;
        case 5: r = D::sq_scale_add(a, b, D::from_double(z[i])); break;
        default: r = D::log2(a, ltab); break;
        }
        out[i] = (double)r.hi + (double)r.lo;
    }
}

/* The FP64 integral kernel's own exp (op 20) and reciprocal (op 21). */
__global__ void f64_eval_kernel(int op, int n, const double* __restrict__ x, double* __restrict__ out)
{
    __shared__ double etab[mwsep::f64::kExpTable];
    mwsep::f64::exp_tang_table(etab);
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = (op == 20) ? mwsep::f64::exp_tang(x[i], etab) : mwsep::f64::rcp_nr(x[i]);
}

std::atomic<bool> g_table_ready[64];
std::mutex g_table_mu;

} // namespace

/* Upload the 2^(j/1024) and log2 tables to `device` (once per device;
 * contexts on other threads may ask at the same time). */
extern "C" int mwsep_df_prepare(int device)
{
    if (device < 0 || device >= 64) return 1;
    if (g_table_ready[device].load(std::memory_order_acquire)) return 0;
    std::lock_guard<std::mutex> lock(g_table_mu);
    if (g_table_ready[device].load(std::memory_order_relaxed)) return 0;
    float2 t[D::kExp2Table];
    for (int j = 0; j < D::kExp2Table; ++j)
    {
        const mwsep::dfl::df v = mwsep::dfl::from_double(exp2((double)j / D::kExp2Table));
        t[j] = make_float2(v.hi, v.lo);
    }
    float4 lt[D::kLog2Table];
    for (int j = 0; j < D::kLog2Table; ++j)
    {
        const double c = 1.0 + (double)j / D::kLog2Table;
        const mwsep::dfl::df l = mwsep::dfl::from_double(log2(c)), r = mwsep::dfl::from_double(1.0 / c);
        lt[j] = make_float4(l.hi, l.lo, r.hi, r.lo);
    }
    int prev = 0;
    if (cudaGetDevice(&prev) != cudaSuccess || cudaSetDevice(device) != cudaSuccess) return 1;
    cudaError_t e = cudaMemcpyToSymbol(c_exp2_tab, t, sizeof(t));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_log2_tab, lt, sizeof(lt));
    cudaSetDevice(prev);
    if (e != cudaSuccess) return 1;
    g_table_ready[device].store(true, std::memory_order_release);
    return 0;
}

extern "C" int mwsep_integral_df_blocks_per_sm(int n_streams)
{
    int b = 0;
    cudaError_t e;
    switch (n_streams)
    {
    case 0: e = occupancy<0>(&b); break;
    case 1: e = occupancy<1>(&b); break;
    case 2: e = occupancy<2>(&b); break;
    case 3: e = occupancy<3>(&b); break;
    case 4: e = occupancy<4>(&b); break;
    case 5: e = occupancy<5>(&b); break;
    case 6: e = occupancy<6>(&b); break;
    case 7: e = occupancy<7>(&b); break;
    default: e = occupancy<8>(&b); break;
    }
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        return 1;
    }
    return b > 0 ? b : 1;
}

extern "C" int mwsep_launch_integral_df(const mwsep_area_dev* area, const mwsep_theta_consts* th_dev,
                                        const mwsep_launch_shape* sh, double2* partials, void* stream)
{
    cudaStream_t st = (cudaStream_t)stream;
    switch (sh->n_streams)
    {
    case 0: return launch<0>(area, th_dev, sh, partials, st);
    case 1: return launch<1>(area, th_dev, sh, partials, st);
    case 2: return launch<2>(area, th_dev, sh, partials, st);
    case 3: return launch<3>(area, th_dev, sh, partials, st);
    case 4: return launch<4>(area, th_dev, sh, partials, st);
    case 5: return launch<5>(area, th_dev, sh, partials, st);
    case 6: return launch<6>(area, th_dev, sh, partials, st);
    case 7: return launch<7>(area, th_dev, sh, partials, st);
    case 8: return launch<8>(area, th_dev, sh, partials, st);
    default: return (int)cudaErrorInvalidValue;
    }
}

extern "C" int mwsep_launch_integral_df_dyn(const mwsep_area_dev* area, const mwsep_theta_consts* th_dev,
                                            const mwsep_launch_shape* sh, long long n_slots, double2* slots,
                                            int* counters, void* stream)
{
    cudaStream_t st = (cudaStream_t)stream;
    switch (sh->n_streams)
    {
    case 0: return launch_dyn<0>(area, th_dev, sh, n_slots, slots, counters, st);
    case 1: return launch_dyn<1>(area, th_dev, sh, n_slots, slots, counters, st);
    case 2: return launch_dyn<2>(area, th_dev, sh, n_slots, slots, counters, st);
    case 3: return launch_dyn<3>(area, th_dev, sh, n_slots, slots, counters, st);
    case 4: return launch_dyn<4>(area, th_dev, sh, n_slots, slots, counters, st);
    case 5: return launch_dyn<5>(area, th_dev, sh, n_slots, slots, counters, st);
    case 6: return launch_dyn<6>(area, th_dev, sh, n_slots, slots, counters, st);
    case 7: return launch_dyn<7>(area, th_dev, sh, n_slots, slots, counters, st);
    case 8: return launch_dyn<8>(area, th_dev, sh, n_slots, slots, counters, st);
    default: return (int)cudaErrorInvalidValue;
    }
}

/* Diagnostics entry (declared in the public header): host arrays in and
 * out, synchronous, on the default stream of `device`. */
extern "C" int mwsep_df_eval(int device, int op, int n, const double* x, const double* y, const double* z,
                             double* out)
{
    if (op < 0 || (op > 6 && op < 10) || (op > 16 && op < 20) || op > 21 || n < 0 ||
        (n > 0 && (!x || !y || !z || !out)))
        return MWSEP_ERR_ARG;
    if (n == 0) return MWSEP_OK;
    if (cudaSetDevice(device) != cudaSuccess || mwsep_df_prepare(device)) return MWSEP_ERR_CUDA;
    const size_t bytes = (size_t)n * sizeof(double);
    double* d = nullptr;
    if (cudaMalloc(&d, 4 * bytes) != cudaSuccess)
    {
        cudaGetLastError();
        return MWSEP_ERR_NOMEM;
    }
    cudaError_t e = cudaMemcpy(d, x, bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d + n, y, bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d + 2 * (size_t)n, z, bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
    {
        const int grid = (n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024;
        if (op >= 20)
            f64_eval_kernel<<<grid, 256>>>(op, n, d, d + 3 * (size_t)n);
        else
            df_eval_kernel<<<grid, 256>>>(op, n, d, d + n, d + 2 * (size_t)n, d + 3 * (size_t)n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, d + 3 * (size_t)n, bytes, cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e == cudaSuccess ? MWSEP_OK : MWSEP_ERR_CUDA;
}

extern "C" int mwsep_launch_aux_area_df(const mwsep_area_dev* area, const mwsep_theta_consts* th_dev,
                                        const mwsep_launch_shape* sh, double2* partials, void* stream)
{
    const long long ncomp = 1 + sh->n_streams;
    const long long theta_stride = (long long)sh->n_areas * sh->grid * ncomp;
    double2* base = partials + (size_t)sh->area_index * sh->grid * ncomp;
    aux_area_kernel<<<dim3(1, sh->n_theta), 256, 0, (cudaStream_t)stream>>>(*area, th_dev, base, theta_stride);
    return (int)cudaGetLastError();
}

extern "C" int mwsep_launch_star_df_table(int n, int convolve, const double* r_point, const double* qw,
                                         float4* out, void* stream)
{
    const long long total = (long long)n * convolve;
    if (total <= 0) return 0;
    long long grid = (total + 255) / 256;
    if (grid > 152 * 16) grid = 152 * 16;
    star_df_table_kernel<<<(int)grid, 256, 0, (cudaStream_t)stream>>>(total, r_point, qw, out);
    return (int)cudaGetLastError();
}

extern "C" int mwsep_launch_likelihood_df(const mwsep_stars_dev* stars, const float4* star_df,
                                          const mwsep_theta_consts* th_dev, const mwsep_launch_shape* sh,
                                          const double* integrals, double2* partials, void* stream)
{
    cudaStream_t st = (cudaStream_t)stream;
    if (sh->block > 256) return (int)cudaErrorInvalidValue;
    switch (sh->n_streams)
    {
    case 0: return launch_likelihood<0>(stars, star_df, th_dev, sh, integrals, partials, st);
    case 1: return launch_likelihood<1>(stars, star_df, th_dev, sh, integrals, partials, st);
    case 2: return launch_likelihood<2>(stars, star_df, th_dev, sh, integrals, partials, st);
    case 3: return launch_likelihood<3>(stars, star_df, th_dev, sh, integrals, partials, st);
    case 4: return launch_likelihood<4>(stars, star_df, th_dev, sh, integrals, partials, st);
    default: return (int)cudaErrorInvalidValue; /* 5..8 streams run in native FP64 */
    }
}

MWSEP_CHECKS_READER(mwsep_checks_df)
