/* mwsep_f64_point.cuh -- the plain-FP64 density evaluation shared by every
 * FP64 kernel (single evaluation, batches, the tiled engine).
 *
 * Two forms of calculate_probabilities (cpu/evaluation_optimized.c:190-299):
 *  - convolve_f64, used per star by the likelihood and separation kernels:
 *    every operation in the reference's association order, IEEE division,
 *    square root and exp;
 *  - convolve_f64_cs, used per cell by the integral kernels: the same
 *    densities with the geometry rewritten as completed squares in r
 *    (column_consts_f64), e^x by Tang's table method (exp_tang) and the
 *    Hernquist divide as a Newton-Raphson reciprocal (rcp_nr), with explicit
 *    FMAs.  Its rounding differs from the reference's; measured against the
 *    reference's own outputs it stays within 4e-15 relative per integral on
 *    the reference's test fixtures and 6.4e-16 on the full-size wedge
 *    (1.72e10 points), against the 1e-12 bound of the plain form.
 * Translation units that include this compile with -fmad=false, so only the
 * written FMAs are fused.  Per cell the convolution points are summed in
 * order n = 0..C-1, then multiplied by reff_xr_rp3 and by the cell volume
 * V = irv[k]*ids[j] (:500-504, :513), and each thread Kahan-sums its cells
 * as the reference does.
 */
#ifndef MWSEP_F64_POINT_CUH
#define MWSEP_F64_POINT_CUH

#include <cuda_runtime.h>
#include <math.h>
#include "mwsep_internal.h"
#include "mwsep_checks.cuh"
#include "mwsep_reduce.cuh"

namespace mwsep {
namespace f64 {

using mwsep::comp_sum;

__device__ __forceinline__ void load_theta(mwsep_theta_consts& dst, const mwsep_theta_consts* src)
{
    static_assert(sizeof(mwsep_theta_consts) % 8 == 0, "theta consts must be 8-byte sized");
    const unsigned long long* s = reinterpret_cast<const unsigned long long*>(src);
    unsigned long long* d = reinterpret_cast<unsigned long long*>(&dst);
    for (int i = threadIdx.x; i < (int)(sizeof(mwsep_theta_consts) / 8); i += blockDim.x) d[i] = s[i];
}

/* The convolution loop of calculate_probabilities for one point (a cell's
 * r-bin or a star): tables are read at p[n*stride].  Returns bg and st[]
 * before the reff_xr_rp3 factor. */
template <int SMAX>
__device__ __forceinline__ void convolve_f64(const double* __restrict__ rp, const double* __restrict__ qwt,
                                             const double* __restrict__ gm, const double* __restrict__ gm2,
                                             size_t stride, int C, double bsin, double bcos, double lsin,
                                             double lcos, const mwsep_theta_consts& th, double& bg,
                                             double (&st)[SMAX])
{
    const int S = th.n_streams;
    const double qq = th.q * th.q;
    bg = (th.bg_mode == 2) ? -1.0 : 0.0;
#pragma unroll
    for (int s = 0; s < SMAX; ++s) st[s] = 0.0;

    for (int n = 0; n < C; ++n)
    {
        const size_t o = (size_t)n * stride;
        const double r = rp[o];
        const double qw = qwt[o];
        const double x2 = r * bsin;
        const double zp = r * bcos;
        const double x0 = zp * lcos - MW_LBR_R;
        const double x1 = zp * lsin;
        if (th.bg_mode == 0)
        {
            const double rg = sqrt(x0 * x0 + x1 * x1 + (x2 * x2) / qq);
            const double rs = rg + th.r0;
            if (th.aux)
            {
                const double h_prob = qw / (rg * rs * rs * rs);
                const double aux_prob = qw * (th.bg_a * gm2[o] + th.bg_b * gm[o] + th.bg_c);
                bg += h_prob + aux_prob;
            }
            else
            {
                bg += qw / (rg * rs * rs * rs);
            }
        }
        else if (th.bg_mode == 1)
        {
            const double rg = sqrt(x0 * x0 + x1 * x1 + (x2 * x2) / qq);
            bg += qw / (pow(rg, th.alpha) * pow(rg + th.r0, th.alpha_delta3));
        }
#pragma unroll
        for (int s = 0; s < SMAX; ++s)
        {
            if (s < S && th.stream_on[s])
            {
                double d0 = x0 - th.c[s][0];
                double d1 = x1 - th.c[s][1];
                double d2 = x2 - th.c[s][2];
                const double dotted = th.a[s][0] * d0 + th.a[s][1] * d1 + th.a[s][2] * d2;
                d0 = d0 - dotted * th.a[s][0];
                d1 = d1 - dotted * th.a[s][1];
                d2 = d2 - dotted * th.a[s][2];
                const double norm = d0 * d0 + d1 * d1 + d2 * d2;
                st[s] += qw * exp(-norm / th.sigma_sq2[s]);
            }
        }
    }
}

/* e^x for x <= 709 in FP64 by Tang's table-driven method (ACM TOMS
 * 15(2), 1989): m = rint(4096 x / ln2), r = x - m ln2/4096 with ln2/4096
 * split Cody-Waite style (a 29-bit high part, so m times it is exact for
 * |m| < 2^24), then e^x = 2^(m >> 12) 2^((m & 4095)/4096) e^r with
 * |r| <= ln2/8192 and e^r - 1 = r + r^2 (1/2 + r/6) (remainder below
 * 3e-18 relative).  Eight FP64 operations; within 1 ulp of 2^-52 relative
 * on a CPU restatement over [-745, 0].  tab[j] = 2^(j/4096) (kExpTable
 * doubles, 32 KB of shared memory).  The range check is on the integer
 * bits (|x| > 745.2 or NaN): NaN stays NaN, below -745.2 the result is 0
 * as FP64 underflows there, above +745.2 it is +inf. */
constexpr int kExpBits = 12;
constexpr int kExpTable = 1 << kExpBits;

__device__ __forceinline__ double exp_tang(double x, const double* __restrict__ tab)
{
    constexpr unsigned long long kMaxMag = 0x408749999999999aull; /* bits of 745.2 */
    if ((__double_as_longlong(x) & 0x7fffffffffffffffll) > (long long)kMaxMag)
        return (x != x) ? x : (x < 0.0 ? 0.0 : __longlong_as_double(0x7ff0000000000000ll));
    constexpr double kInvL = 5909.278887481194;           /* 4096 / ln2 */
    constexpr double kL1 = 0x1.62e42ff000000p-13;         /* ln2/4096, high part */
    constexpr double kL2 = -0x1.718432a1b0e26p-47;        /* ln2/4096 - kL1 */
    constexpr double kShift = 6755399441055744.0;         /* 1.5 * 2^52 */
    const double t = fma(x, kInvL, kShift);
    const long long m = __double_as_longlong(t) - __double_as_longlong(kShift);
    const double md = t - kShift;
    const double r = fma(-md, kL2, fma(-md, kL1, x));
    const double em1 = fma(r * r, fma(r, 1.0 / 6.0, 0.5), r);
    const double T = tab[m & (kExpTable - 1)];
    const double v = fma(T, em1, T);
    const int n = (int)(m >> kExpBits);
    return n >= -1021 ? __longlong_as_double(__double_as_longlong(v) + ((long long)n << 52)) : ldexp(v, n);
}

/* 1/x for positive x with x and 1/x normal, by two Newton-Raphson steps
 * y' = y + y (1 - x y) (each squares the relative error; Markstein, IBM J.
 * Res. Dev. 34(1), 1990) from the hardware's approximate FP64 reciprocal:
 * four FMAs and one SFU operation, within 1 ulp of the quotient.  No
 * special-case handling: the approximation flushes subnormals to zero, so
 * x or 1/x subnormal, zero, infinite or NaN is outside its domain (in the
 * halo term x = rg (rg + r0)^3 lies between about 1e-3 and 1e12). */
__device__ __forceinline__ double rcp_nr(double x)
{
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    double e = fma(-x, y, 1.0);
    y = fma(y, e, y);
    e = fma(-x, y, 1.0);
    return fma(y, e, y);
}

/* The 2^(j/4096) table for exp_tang, filled by a block into its shared memory. */
__device__ __forceinline__ void exp_tang_table(double* tab)
{
    for (int j = threadIdx.x; j < kExpTable; j += blockDim.x) tab[j] = exp2((double)j / (double)kExpTable);
}

/* Per-column constants of the integral's density in completed-square form,
 * in FP64.  With u = (cos b cos l, cos b sin l, sin b) the column's unit
 * vector, a point at distance r sits at x = r u - (R, 0, 0)
 * (cpu/evaluation_optimized.c:222-227), and
 *   background  x0^2 + x1^2 + x2^2/q^2 = B2 (r - rb)^2 + Db,
 *   stream s    |x - c - ((x - c).a) a|^2 = A2 (r - rs)^2 + Ds,
 * both sums of non-negative terms (no cancellation), so the stream exponent
 * -|.|^2 / sigma2_s is k2 (r - rs)^2 + k0.  The same quantities as the
 * reference's x0, x1, x2 and perpendicular-distance arithmetic, in about
 * half the FP64 operations (no per-point divide by q^2 or sigma2). */
template <int SMAX>
struct ColF64
{
    double B2, rb, Db;
    double rs[SMAX], k2[SMAX], k0[SMAX];
};

template <int SMAX>
__device__ __forceinline__ void column_consts_f64(double bsin, double bcos, double lsin, double lcos,
                                                  const mwsep_theta_consts& th, ColF64<SMAX>& cc)
{
    const double u0 = bcos * lcos, u1 = bcos * lsin, u2 = bsin;
    const double perp = u1 * u1 + u2 * u2 / (th.q * th.q);
    cc.B2 = u0 * u0 + perp;
    cc.rb = MW_LBR_R * u0 / cc.B2;
    cc.Db = (MW_LBR_R * MW_LBR_R) * perp / cc.B2;
#pragma unroll
    for (int s = 0; s < SMAX; ++s)
    {
        cc.rs[s] = 0.0;
        cc.k2[s] = 0.0;
        cc.k0[s] = 0.0;
        if (s < th.n_streams && th.stream_on[s])
        {
            const double a0 = th.a[s][0], a1 = th.a[s][1], a2 = th.a[s][2];
            /* c' = c + (R, 0, 0) so that x - c = r u - c' */
            const double c0 = th.c[s][0] + MW_LBR_R, c1 = th.c[s][1], c2 = th.c[s][2];
            const double au = a0 * u0 + a1 * u1 + a2 * u2;
            const double p0 = u0 - au * a0, p1 = u1 - au * a1, p2 = u2 - au * a2;
            const double ac = a0 * c0 + a1 * c1 + a2 * c2;
            const double q0 = c0 - ac * a0, q1 = c1 - ac * a1, q2 = c2 - ac * a2;
            const double A2 = p0 * p0 + p1 * p1 + p2 * p2;
            const double rs = (A2 > 1e-300) ? (p0 * q0 + p1 * q1 + p2 * q2) / A2 : 0.0;
            const double e0 = q0 - rs * p0, e1 = q1 - rs * p1, e2 = q2 - rs * p2;
            const double Ds = e0 * e0 + e1 * e1 + e2 * e2;
            const double f = -1.0 / th.sigma_sq2[s];
            cc.rs[s] = rs;
            cc.k2[s] = A2 * f;
            cc.k0[s] = Ds * f;
        }
    }
}

/* One cell's convolution with the completed-square constants (the
 * integral's counterpart of convolve_f64). */
template <int SMAX>
__device__ __forceinline__ void convolve_f64_cs(const double* __restrict__ rp, const double* __restrict__ qwt,
                                                const double* __restrict__ gm, const double* __restrict__ gm2,
                                                int C, const ColF64<SMAX>& cc, const mwsep_theta_consts& th,
                                                const double* __restrict__ etab, double& bg, double (&st)[SMAX])
{
    const int S = th.n_streams;
    bg = (th.bg_mode == 2) ? -1.0 : 0.0;
#pragma unroll
    for (int s = 0; s < SMAX; ++s) st[s] = 0.0;
    for (int n = 0; n < C; ++n)
    {
        const double r = rp[n];
        const double qw = qwt[n];
        if (th.bg_mode != 2)
        {
            const double t = r - cc.rb;
            const double rg = sqrt(fma(cc.B2 * t, t, cc.Db));
            if (th.bg_mode == 0)
            {
                const double rs = rg + th.r0;
                bg = fma(qw, rcp_nr(rg * rs * rs * rs), bg);
                if (th.aux) bg += qw * (th.bg_a * gm2[n] + th.bg_b * gm[n] + th.bg_c);
            }
            else
                bg += qw / (pow(rg, th.alpha) * pow(rg + th.r0, th.alpha_delta3));
        }
#pragma unroll
        for (int s = 0; s < SMAX; ++s)
        {
            if (s < S && th.stream_on[s])
            {
                const double u = r - cc.rs[s];
                st[s] = fma(qw, exp_tang(fma(cc.k2[s] * u, u, cc.k0[s]), etab), st[s]);
            }
        }
    }
}

/* One item of an integral (a column and its run of r-bins): Kahan-adds
 * each cell's bg*V and st*V into acc (cpu/evaluation_optimized.c:498-520). */
template <int SMAX>
__device__ __forceinline__ void integral_item(const mwsep_area_dev& A, const mwsep_theta_consts& th,
                                              const double* __restrict__ etab, long long item,
                                              comp_sum (&acc)[1 + SMAX])
{
    const int S = th.n_streams;
    const int C = A.convolve;
    const mwsep::ItemPos ip = mwsep::item_pos(A, item);
    const double* g = A.geom + 4 * (size_t)MWSEP_IDX(ip.col, A.n_cols, 1);
    ColF64<SMAX> cc;
    column_consts_f64<SMAX>(g[0], g[1], g[2], g[3], th, cc);
    const double idsj = A.ids[MWSEP_IDX(ip.nu, A.nu_steps, 3)];
    for (int k = ip.k0; k < ip.k1; ++k)
    {
        const double V = A.irv[MWSEP_IDX(k, A.r_steps, 4)] * idsj;
        double bg, st[SMAX];
        const size_t row = (size_t)MWSEP_IDX(k, A.r_steps, 5) * C;
        convolve_f64_cs<SMAX>(A.r_point + row, A.qw + row, A.r_in_mag + row, A.r_in_mag2 + row, C, cc, th, etab, bg,
                              st);
        const double rf = A.reff[MWSEP_IDX(k, A.r_steps, 6)];
        if (th.bg_mode != 2) bg *= rf;
        bg *= V;
        acc[0].add(bg);
#pragma unroll
        for (int s = 0; s < SMAX; ++s)
        {
            if (s < S)
            {
                double v = st[s];
                if (th.stream_on[s]) v *= rf;
                v *= V;
                acc[1 + s].add(v);
            }
        }
    }
}

template <int SMAX>
__device__ __forceinline__ void likelihood_finish(const mwsep_theta_consts& th, const double* I, double rf,
                                                  double bg, const double (&st)[SMAX], comp_sum (&acc)[3 + SMAX]);

/* calculate_likelihood for one star (cpu/evaluation_optimized.c:665-717).
 * acc slots: [0] log10 p, [1] zero count, [2] bg-only, [3+s] stream-only. */
template <int SMAX>
__device__ __forceinline__ void likelihood_star(const mwsep_stars_dev& St, const mwsep_theta_consts& th,
                                                const double* I, int s0, comp_sum (&acc)[3 + SMAX])
{
    const int N = St.n_stars;
    s0 = (int)MWSEP_IDX(s0, N, 7);
    const double* g = St.geom + 4 * (size_t)s0;
    double bg, st[SMAX];
    convolve_f64<SMAX>(St.r_point + s0, St.qw + s0, St.r_in_mag + s0, St.r_in_mag2 + s0, (size_t)N, St.convolve,
                       g[0], g[1], g[2], g[3], th, bg, st);
    likelihood_finish<SMAX>(th, I, St.reff[s0], bg, st, acc);
}

/* The rest of calculate_likelihood for one star from its convolved bg and
 * st[] before the reff_xr_rp3 factor rf (cpu/evaluation_optimized.c:679-716):
 * the mixture weights, the -238 sentinel and the log10 sums. */
template <int SMAX>
__device__ __forceinline__ void likelihood_finish(const mwsep_theta_consts& th, const double* I, double rf,
                                                  double bg, const double (&st)[SMAX], comp_sum (&acc)[3 + SMAX])
{
    const int S = th.n_streams;
    if (th.bg_mode != 2) bg *= rf;

    double bg_only = (bg / I[0]) * th.exp_bg_weight;
    double star_prob = bg_only;
    bg_only = (bg_only == 0.0) ? -238.0 : log10(bg_only / th.sum_exp_weights);
    acc[2].add(bg_only);
#pragma unroll
    for (int s = 0; s < SMAX; ++s)
    {
        if (s < S)
        {
            double v = st[s];
            if (th.stream_on[s]) v *= rf;
            double st_only = v / I[1 + s] * th.exp_stream_weight[s];
            star_prob += st_only;
            st_only = (st_only == 0.0) ? -238.0 : log10(st_only / th.sum_exp_weights);
            acc[3 + s].add(st_only);
        }
    }
    star_prob /= th.sum_exp_weights;
    if (star_prob != 0.0)
        acc[0].add(log10(star_prob));
    else
    {
        acc[0].add(-238.0);
        acc[1].add(1.0);
    }
}

} // namespace f64
} // namespace mwsep

#endif
