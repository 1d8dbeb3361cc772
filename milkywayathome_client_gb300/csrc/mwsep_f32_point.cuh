/* mwsep_f32_point.cuh -- the compensated-FP32 density evaluation shared by
 * every compensated kernel (single evaluation, batches, the tiled engine).
 *
 * Split of precision:
 *   FP64 or float pairs (~2^-44): the per-column (or per-star) coordinate
 *         transform with the Sun offset -- in pairs on the FP32 pipe for warp
 *         tiles and stars (column_consts_df), in FP64 for thread items -- the
 *         r-bin volume and convolution weight tables (built in FP64, rounded
 *         to FP32 once), the per-item and cross-block sums, the
 *         normalisation and the log-likelihood;
 *   FP32: the density at each convolution point, on the FMA pipe and the
 *         SFU (ex2 / rsqrt / rcp approximations), with Kahan-compensated
 *         per-thread sums across cells.
 *
 * Reformulation (exact in real arithmetic).  A point at distance r along the
 * column's unit vector u = (cos b cos l, cos b sin l, sin b) sits at
 * x = r u - (8.5, 0, 0) (cpu/evaluation_optimized.c:224-227).  Then
 *   background: x0^2 + x1^2 + x2^2/q^2 = B2 (r - rb)^2 + Db
 *   stream s:   |x - c - ((x - c).a) a|^2 = A2 (r - rs)^2 + Ds
 * with B2, rb, Db, A2, rs, Ds >= 0 computed per column (FP64 or pairs).  Both forms
 * are sums of non-negative terms, so FP32 evaluation has no cancellation.
 * t = r - rb is formed from (hi, lo) float pairs, so it keeps full relative
 * accuracy even where r and rb are close, and each stream reuses it:
 * r - rs = t + (rb - rs) with the offset split into (hi, lo) too.
 * The stream exponent -|.|^2/(2 sigma^2) becomes k2 ts^2 + k0 in base 2.
 */
#ifndef MWSEP_F32_POINT_CUH
#define MWSEP_F32_POINT_CUH

#include <cuda_runtime.h>
#include <math.h>
#include "mwsep_internal.h"
#include "mwsep_reduce.cuh"
#include "mwsep_checks.cuh"
#include "mwsep_df.cuh"

namespace mwsep {
namespace f32 {

using mwsep::comp_sum;

constexpr double kLog2e = 1.4426950408889634073599246810018921;

/* background forms */
enum BgForm
{
    BG_HERNQUIST = 0,     /* alpha = delta = 1 (:220-258) */
    BG_HERNQUIST_AUX = 1, /* ... plus the quadratic-in-g aux profile (:234-239) */
    BG_GENERAL = 2,       /* pow(rg, alpha) pow(rg + r0, 3 - alpha + delta) (:259-272) */
    BG_NONE = 3           /* q == 0: bg = -1 per point set, no reff (:213-216) */
};

__device__ __forceinline__ float ex2a(float x)
{
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rsqa(float x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcpa(float x)
{
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float lg2a(float x)
{
    float y;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

/* FP32 Kahan accumulator (value = s - c). */
struct fkahan
{
    float s, c;
    __device__ __forceinline__ void zero() { s = 0.f; c = 0.f; }
    __device__ __forceinline__ void add(float x)
    {
        const float y = __fsub_rn(x, c);
        const float t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

__device__ __forceinline__ void split(double v, float& hi, float& lo)
{
    hi = (float)v;
    lo = (float)(v - (double)hi);
}

template <int S>
struct SArr
{
    static constexpr int N = S > 0 ? S : 1;
};

/* Per-column (or per-star) constants of one theta.  Stream s: with
 * u = t + d_hi and d = rb - rs = d_hi + d_lo, the base-2 exponent is
 *   k2 (u + d_lo)^2 + k0 = u (k2 u + k2dl) + k0c,
 * k2dl = 2 k2 d_lo, k0c = k0 + k2 d_lo^2 (two FMAs per point). */
template <int S>
struct Col
{
    float B2, Db, rb_hi, rb_lo;
    float k2[SArr<S>::N], k2dl[SArr<S>::N], k0c[SArr<S>::N], d_hi[SArr<S>::N];
};

/* FROM_HI = true gives the constants of the packed form, where t is
 * measured from the float rb_hi (t' = r - rb_hi = t + rb_lo):
 *   background  B2 (t' - rb_lo)^2 + Db = t' (B2 t' + L) + D,
 *               L = -2 B2 rb_lo (kept in the rb_lo slot), D = Db + B2 rb_lo^2;
 *   streams     offsets d = rb_hi - rs.
 * The same quadratics, with the small rb_lo folded into the constants. */
/* Range of the stream exponents: FP32 holds 2^+-126, an FP64 integral goes
 * far lower, and a stream whose closest approach is far from a wedge has
 * every term below 2^-126 (a zero integral, a NaN likelihood).  So per item
 * (a column run, a warp tile or a star) each stream's base-2 exponent is
 * shifted by eref = floor of its largest value over the item's r range --
 * k2 (r* - rs)^2 + k0 at r* = rs clamped into [r_lo, r_hi] -- formed in FP64
 * before the constant is rounded to float, and the item's sums are scaled
 * back by 2^eref in FP64.  StreamExp carries the two FP64 values. */
template <int S>
struct StreamExp
{
    double amax[SArr<S>::N], k0c[SArr<S>::N];
};

constexpr int kErefFloor = -1100; /* 2^-1100 is 0 in FP64 */

/* floor(a) clamped at kErefFloor (also for -inf and NaN) */
__device__ __forceinline__ int exp_ref(double a) { return (a > (double)kErefFloor) ? (int)floor(a) : kErefFloor; }
/* 2^e: a normal double from its exponent bits, ldexp below that */
__device__ __forceinline__ double exp_scale(int e)
{
    return e > -1023 ? __longlong_as_double((long long)(e + 1023) << 52) : (e > kErefFloor ? ldexp(1.0, e) : 0.0);
}

/* The shifted constants into cc (switched-off streams keep -1e30). */
template <int S>
__device__ __forceinline__ void shift_exponents(const mwsep_theta_consts& th, const StreamExp<S>& se,
                                                const int (&eref)[SArr<S>::N], Col<S>& cc)
{
#pragma unroll
    for (int s = 0; s < S; ++s)
        if (s < th.n_streams && th.stream_on[s]) cc.k0c[s] = (float)fmax(se.k0c[s] - (double)eref[s], -1.0e30);
}

/* r range of the convolution points of r-bins [k0, k1) of an area: the
 * points increase with the bin and, within a bin, with the Gauss-Legendre
 * node, so the chunk's corner points bound it. */
__device__ __forceinline__ void chunk_r_range(const mwsep_area_dev& A, int k0, int k1, double& lo, double& hi)
{
    const int C = A.convolve;
    const size_t n = (size_t)A.r_steps * C;
    (void)n; /* used by the index checks only */
    const double a = A.r_point[MWSEP_IDX((size_t)k0 * C, n, 5)];
    const double b = A.r_point[MWSEP_IDX((size_t)k0 * C + C - 1, n, 5)];
    const double c = A.r_point[MWSEP_IDX((size_t)(k1 - 1) * C, n, 5)];
    const double d = A.r_point[MWSEP_IDX((size_t)(k1 - 1) * C + C - 1, n, 5)];
    lo = fmin(fmin(a, b), fmin(c, d));
    hi = fmax(fmax(a, b), fmax(c, d));
}

/* The warp tiles' estimate of each stream's largest exponent over an r
 * range, in FP32: the stream geometry of column_consts below at single
 * precision (error well below 1 in the exponent for |k0| < 2^20; only its
 * floor is used, and a term up to 2^5 stays in range). */
template <int S>
__device__ __forceinline__ void stream_amax_f32(const double* g, const mwsep_theta_consts& th, float r_lo,
                                                float r_hi, float (&amax)[SArr<S>::N])
{
    const float bsin = (float)g[0], bcos = (float)g[1], lsin = (float)g[2], lcos = (float)g[3];
    const float u0 = bcos * lcos, u1 = bcos * lsin, u2 = bsin;
#pragma unroll
    for (int s = 0; s < S; ++s)
    {
        amax[s] = -INFINITY;
        if (s < th.n_streams && th.stream_on[s])
        {
            const float a0 = th.af[s][0], a1 = th.af[s][1], a2 = th.af[s][2];
            const float c0 = th.cf[s][0], c1 = th.cf[s][1], c2 = th.cf[s][2];
            const float au = a0 * u0 + a1 * u1 + a2 * u2;
            const float p0 = u0 - au * a0, p1 = u1 - au * a1, p2 = u2 - au * a2;
            const float ac = a0 * c0 + a1 * c1 + a2 * c2;
            const float q0 = c0 - ac * a0, q1 = c1 - ac * a1, q2 = c2 - ac * a2;
            const float A2 = p0 * p0 + p1 * p1 + p2 * p2;
            const float rs = (A2 > 1e-30f) ? (p0 * q0 + p1 * q1 + p2 * q2) / A2 : 0.f;
            const float e0 = q0 - rs * p0, e1 = q1 - rs * p1, e2 = q2 - rs * p2;
            const float rc = fminf(fmaxf(rs, r_lo), r_hi) - rs;
            amax[s] = th.kf[s] * (A2 * rc * rc + (e0 * e0 + e1 * e1 + e2 * e2));
        }
    }
}

/* A warp tile's per-stream eref: the FP32 estimate on each live column (one
 * per lane), the warp's maximum, floored; lane 0 also leaves ids_nu 2^eref
 * in shared memory for the group hand-offs. */
template <int S>
__device__ __forceinline__ void tile_erefs(const mwsep_area_dev& A, const mwsep_theta_consts& th, int k0, int k1,
                                           const double* g, bool live, int lane, double idsv, double* tscale,
                                           int (&eref)[SArr<S>::N])
{
    double r_lo, r_hi;
    chunk_r_range(A, k0, k1, r_lo, r_hi);
    float am[SArr<S>::N];
#pragma unroll
    for (int s = 0; s < S; ++s) am[s] = -INFINITY;
    if (live) stream_amax_f32<S>(g, th, (float)r_lo, (float)r_hi, am);
#pragma unroll
    for (int s = 0; s < S; ++s)
    {
        float m = am[s];
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        eref[s] = exp_ref((double)m);
        if (lane == 0) tscale[s] = idsv * exp_scale(eref[s]);
    }
}

/* eref: when given, each stream's exponent constant is shifted by it
 * (formed in FP64 before the rounding to float). */
template <int S, bool FROM_HI = false>
__device__ __forceinline__ void column_consts(const double* g, const mwsep_theta_consts& th, Col<S>& cc,
                                              StreamExp<S>* se = nullptr, double r_lo = 0.0, double r_hi = 0.0,
                                              const int* eref = nullptr)
{
    const double bsin = g[0], bcos = g[1], lsin = g[2], lcos = g[3];
    const double u0 = bcos * lcos, u1 = bcos * lsin, u2 = bsin;
    const double iq2 = 1.0 / (th.q * th.q);
    const double perp = u1 * u1 + u2 * u2 * iq2;
    const double B2 = u0 * u0 + perp;
    const double rb_exact = MW_LBR_R * u0 / B2;
    const double Db = (MW_LBR_R * MW_LBR_R) * perp / B2;
    cc.B2 = (float)B2;
    split(rb_exact, cc.rb_hi, cc.rb_lo);
    double rb = rb_exact;
    if (FROM_HI)
    {
        const double dl = rb_exact - (double)cc.rb_hi;
        cc.rb_lo = (float)(-2.0 * B2 * dl);
        cc.Db = (float)(Db + B2 * dl * dl);
        rb = (double)cc.rb_hi;
    }
    else
        cc.Db = (float)Db;
#pragma unroll
    for (int s = 0; s < S; ++s)
    {
        if (s < th.n_streams)
        {
            const double a0 = th.a[s][0], a1 = th.a[s][1], a2 = th.a[s][2];
            /* c' = c + Sun offset so that x - c = r u - c' */
            const double c0 = th.c[s][0] + MW_LBR_R, c1 = th.c[s][1], c2 = th.c[s][2];
            const double au = a0 * u0 + a1 * u1 + a2 * u2;
            const double p0 = u0 - au * a0, p1 = u1 - au * a1, p2 = u2 - au * a2;
            const double ac = a0 * c0 + a1 * c1 + a2 * c2;
            const double q0 = c0 - ac * a0, q1 = c1 - ac * a1, q2 = c2 - ac * a2;
            const double A2 = p0 * p0 + p1 * p1 + p2 * p2;
            const double rs = (A2 > 1e-300) ? (p0 * q0 + p1 * q1 + p2 * q2) / A2 : 0.0;
            const double e0 = q0 - rs * p0, e1 = q1 - rs * p1, e2 = q2 - rs * p2;
            const double Ds = e0 * e0 + e1 * e1 + e2 * e2;
            const double f = th.stream_on[s] ? -kLog2e / th.sigma_sq2[s] : 0.0;
            const double k2 = A2 * f;
            float d_lo;
            split(rb - rs, cc.d_hi[s], d_lo);
            cc.k2[s] = (float)k2;
            cc.k2dl[s] = (float)(2.0 * k2 * (double)d_lo);
            /* a switched-off stream gets an exponent far below the FTZ range */
            const double k0c = Ds * f + k2 * (double)d_lo * (double)d_lo;
            cc.k0c[s] = th.stream_on[s] ? (float)fmax(k0c - (eref ? (double)eref[s] : 0.0), -1.0e30) : -1.0e30f;
            if (se)
            {
                const double rc = fmin(fmax(rs, r_lo), r_hi) - rs;
                se->amax[s] = th.stream_on[s] ? k2 * rc * rc + Ds * f : -INFINITY;
                se->k0c[s] = k0c;
            }
        }
        else
        {
            cc.k2[s] = 0.f;
            cc.k2dl[s] = 0.f;
            cc.k0c[s] = -1.0e30f;
            cc.d_hi[s] = 0.f;
            if (se)
            {
                se->amax[s] = -INFINITY;
                se->k0c[s] = -1.0e30;
            }
        }
    }
}

/* ---- the column (or star) prologue in double-float ----
 * The same constants as column_consts, formed in pairs of floats (about 2^-44
 * relative, mwsep_df.cuh) on the FP32 pipe: GB300 runs FP64 at ~1/70 of
 * FP32, so the ~190 FP64 operations of a column prologue held a warp for as
 * long as thousands of FP32 ones.  Each constant is rounded to float as
 * before; the exponent constants k2 (r - rs)^2 + k0 need rs and Ds to ~1e-9
 * absolute, which the pairs give with margin under the cancellation of
 * e = q - rs p (|q| / |e| up to ~1e4). */

/* theta-only constants, formed once per block in FP64 and split into pairs:
 * 1/q^2 (0 when q = 0: no background is evaluated then, and the streams do
 * not depend on rb), each stream's axis a, its centre's offset from the
 * axis q = c' - (a.c') a with c' = c + (8.5, 0, 0), and
 * f = -log2(e) / (2 sigma^2) (0 for a switched-off stream). */
template <int S>
struct ThetaDF
{
    dfl::df iq2;
    dfl::df a[SArr<S>::N][3], q[SArr<S>::N][3], f[SArr<S>::N];
};

/* Part i of the theta pairs: stream i's for i < S, 1/q^2 for i == S (parts
 * are independent, so S + 1 threads form them at once; callers sync after). */
template <int S>
__device__ __forceinline__ void theta_df_part(const mwsep_theta_consts& th, ThetaDF<S>& td, int i)
{
    if (i == S)
    {
        td.iq2 = dfl::from_double(th.q != 0.0 ? 1.0 / (th.q * th.q) : 0.0);
        return;
    }
    if (i < 0 || i >= S) return;
    const int s = i;
    const bool on = s < th.n_streams && th.stream_on[s];
    const double a0 = th.a[s][0], a1 = th.a[s][1], a2 = th.a[s][2];
    const double c0 = th.c[s][0] + MW_LBR_R, c1 = th.c[s][1], c2 = th.c[s][2];
    const double ac = a0 * c0 + a1 * c1 + a2 * c2;
    td.a[s][0] = dfl::from_double(on ? a0 : 0.0);
    td.a[s][1] = dfl::from_double(on ? a1 : 0.0);
    td.a[s][2] = dfl::from_double(on ? a2 : 0.0);
    td.q[s][0] = dfl::from_double(on ? c0 - ac * a0 : 0.0);
    td.q[s][1] = dfl::from_double(on ? c1 - ac * a1 : 0.0);
    td.q[s][2] = dfl::from_double(on ? c2 - ac * a2 : 0.0);
    td.f[s] = dfl::from_double(on ? -kLog2e / th.sigma_sq2[s] : 0.0);
}

__device__ __forceinline__ dfl::df df_norm(dfl::df x)
{
    float h, l;
    dfl::fast_two_sum(x.hi, x.lo, h, l);
    return dfl::mk(h, l);
}

__device__ __forceinline__ dfl::df df_sub(dfl::df x, dfl::df y) { return dfl::add_fast(x, dfl::neg(y)); }

__device__ __forceinline__ dfl::df df_dot3(const dfl::df (&x)[3], const dfl::df (&y)[3])
{
    return dfl::add_fast(dfl::add_fast(dfl::mul(x[0], y[0]), dfl::mul(x[1], y[1])), dfl::mul(x[2], y[2]));
}

/* floor of a pair, clamped at kErefFloor (also for NaN) */
__device__ __forceinline__ int df_floor(dfl::df x)
{
    if (!(x.hi > (float)kErefFloor)) return kErefFloor;
    float f = floorf(x.hi);
    if (f == x.hi && x.lo < 0.f) f -= 1.f;
    return (int)f;
}

/* column_consts from pairs.  FROM_HI as there.  STAR: eref is computed here
 * (each stream's largest exponent over [r_lo, r_hi], floored) instead of
 * given; either way each stream's k0c comes out shifted by it. */
template <int S, bool FROM_HI, bool STAR>
__device__ __forceinline__ void column_consts_df(const double* g, const mwsep_theta_consts& th, const ThetaDF<S>& td,
                                                 Col<S>& cc, int (&eref)[SArr<S>::N], double r_lo = 0.0,
                                                 double r_hi = 0.0)
{
    using namespace dfl;
    df u[3];
    u[0] = from_double(g[1] * g[3]);
    u[1] = from_double(g[1] * g[2]);
    u[2] = from_double(g[0]);
    const df perp = add_fast(sqr(u[1]), mul(sqr(u[2]), td.iq2));
    const df B2 = add_fast(sqr(u[0]), perp);
    df rb = df_norm(div(mul(mk((float)MW_LBR_R, 0.f), u[0]), B2));
    const df Db = df_norm(div(mul(mk((float)(MW_LBR_R * MW_LBR_R), 0.f), perp), B2));
    cc.B2 = B2.hi;
    cc.rb_hi = rb.hi;
    if (FROM_HI)
    {
        /* t' = r - rb_hi; the pair's low part is rb - rb_hi */
        const float dl = rb.lo;
        cc.rb_lo = -2.f * B2.hi * dl;
        cc.Db = add_fast(Db, mk(B2.hi * dl * dl, 0.f)).hi;
        rb = mk(rb.hi, 0.f);
    }
    else
    {
        cc.rb_lo = rb.lo;
        cc.Db = Db.hi;
    }
    const df rlo = from_double(r_lo), rhi = from_double(r_hi);
#pragma unroll
    for (int s = 0; s < S; ++s)
    {
        cc.k2[s] = 0.f;
        cc.k2dl[s] = 0.f;
        cc.k0c[s] = -1.0e30f; /* far below the FTZ range: a stream that is off or absent */
        cc.d_hi[s] = 0.f;
        if (STAR) eref[s] = kErefFloor;
        if (s < th.n_streams && th.stream_on[s])
        {
            const df au = df_dot3(td.a[s], u);
            df p[3], e[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) p[i] = df_sub(u[i], mul(au, td.a[s][i]));
            const df A2 = add_fast(add_fast(sqr(p[0]), sqr(p[1])), sqr(p[2]));
            const df rs = (A2.hi > 1e-30f) ? df_norm(div(df_dot3(p, td.q[s]), A2)) : mk(0.f, 0.f);
#pragma unroll
            for (int i = 0; i < 3; ++i) e[i] = df_sub(td.q[s][i], mul(rs, p[i]));
            const df Dsf = mul(add_fast(add_fast(sqr(e[0]), sqr(e[1])), sqr(e[2])), td.f[s]);
            const df k2 = mul(A2, td.f[s]);
            const df d = df_sub(rb, rs);
            cc.d_hi[s] = d.hi;
            cc.k2[s] = k2.hi;
            cc.k2dl[s] = 2.f * k2.hi * d.lo;
            const df k0c = add_fast(Dsf, mk(k2.hi * d.lo * d.lo, 0.f));
            if (STAR)
            {
                /* the largest exponent over the star's points: at rs clamped
                 * into [r_lo, r_hi] */
                const df rc = (rs.hi < rlo.hi) ? df_sub(rlo, rs) : (rs.hi > rhi.hi) ? df_sub(rhi, rs) : mk(0.f, 0.f);
                eref[s] = df_floor(add_fast(mul(k2, sqr(rc)), Dsf));
            }
            cc.k0c[s] = fmaxf(add_fast(k0c, mk(-(float)eref[s], 0.f)).hi, -1.0e30f);
        }
    }
}

struct BgConsts
{
    float r0, aux_a, aux_b, aux_c, alpha, ad3;
};

/* One convolution point v = {r_hi, r_lo, weight, g}: adds its weighted
 * background and stream densities into bgacc and sacc[]. */
template <int S, int FORM>
__device__ __forceinline__ void point(const float4 v, const Col<S>& cc, const BgConsts& bc, float& bgacc,
                                      float (&sacc)[SArr<S>::N])
{
    const float t = (v.x - cc.rb_hi) + (v.y - cc.rb_lo);
    if (FORM == BG_HERNQUIST || FORM == BG_HERNQUIST_AUX)
    {
        const float rg2 = fmaf(cc.B2 * t, t, cc.Db);
        const float y = rsqa(rg2);           /* 1 / rg */
        const float rs = fmaf(rg2, y, bc.r0); /* rg + r0 */
        const float den = rs * rs * rs;
        bgacc = fmaf(v.z * y, rcpa(den), bgacc);
        if (FORM == BG_HERNQUIST_AUX)
            bgacc = fmaf(v.z, fmaf(fmaf(bc.aux_a, v.w, bc.aux_b), v.w, bc.aux_c), bgacc);
    }
    else if (FORM == BG_GENERAL)
    {
        const float rg2 = fmaf(cc.B2 * t, t, cc.Db);
        const float rg = rg2 * rsqa(rg2);
        const float l2 = fmaf(bc.alpha, lg2a(rg), bc.ad3 * lg2a(rg + bc.r0));
        bgacc = fmaf(v.z, ex2a(-l2), bgacc);
    }
#pragma unroll
    for (int s = 0; s < S; ++s)
    {
        const float u = t + cc.d_hi[s];
        const float arg = fmaf(u, fmaf(cc.k2[s], u, cc.k2dl[s]), cc.k0c[s]);
        sacc[s] = fmaf(v.z, ex2a(arg), sacc[s]);
    }
}

/* The density sums of one cell (or star) over its C convolution points:
 * points at p[n * stride], {r_hi, r_lo, weight, g}.  Plain FP32 sums in two
 * interleaved halves (more independent chains, smaller rounding). */
template <int S, int FORM>
__device__ __forceinline__ void convolve(const float4* __restrict__ p, int stride, int C, const Col<S>& cc,
                                         const BgConsts& bc, float& bg, float (&st)[SArr<S>::N])
{
    float bga = 0.f, bgb = 0.f;
    float sa[SArr<S>::N], sb[SArr<S>::N];
#pragma unroll
    for (int s = 0; s < S; ++s) sa[s] = sb[s] = 0.f;
    auto pt = [&](const float4 v, float& bgacc, float (&sacc)[SArr<S>::N]) { point<S, FORM>(v, cc, bc, bgacc, sacc); };

    /* four points per trip, loads issued before any arithmetic */
    int n = 0;
    for (; n + 3 < C; n += 4)
    {
        const float4 v0 = p[(size_t)n * stride];
        const float4 v1 = p[(size_t)(n + 1) * stride];
        const float4 v2 = p[(size_t)(n + 2) * stride];
        const float4 v3 = p[(size_t)(n + 3) * stride];
        pt(v0, bga, sa);
        pt(v1, bgb, sb);
        pt(v2, bga, sa);
        pt(v3, bgb, sb);
    }
    for (; n < C; ++n) pt(p[(size_t)n * stride], bga, sa);
    bg = bga + bgb;
#pragma unroll
    for (int s = 0; s < S; ++s) st[s] = sa[s] + sb[s];
}

__device__ __forceinline__ void load_theta(mwsep_theta_consts& dst, const mwsep_theta_consts* src)
{
    const unsigned long long* s = reinterpret_cast<const unsigned long long*>(src);
    unsigned long long* d = reinterpret_cast<unsigned long long*>(&dst);
    for (int i = threadIdx.x; i < (int)(sizeof(mwsep_theta_consts) / 8); i += blockDim.x) d[i] = s[i];
}

__device__ __forceinline__ BgConsts bg_consts(const mwsep_theta_consts& th)
{
    BgConsts b;
    b.r0 = (float)th.r0;
    b.aux_a = (float)th.bg_a;
    b.aux_b = (float)th.bg_b;
    b.aux_c = (float)th.bg_c;
    b.alpha = (float)th.alpha;
    b.ad3 = (float)th.alpha_delta3;
    return b;
}

/* Block-level reduction of plain per-thread doubles into compensated pairs. */
template <int NC>
__device__ __forceinline__ void reduce_and_store(const double (&v)[NC], int ncomp, double* smem, double2* out)
{
    comp_sum acc[NC];
#pragma unroll
    for (int k = 0; k < NC; ++k)
    {
        acc[k].s = v[k];
        acc[k].c = 0.0;
    }
    mwsep::block_reduce<NC>(acc, smem);
    if (threadIdx.x == 0)
    {
#pragma unroll
        for (int k = 0; k < NC; ++k)
            if (k < ncomp) out[k] = make_double2(acc[k].s, acc[k].c);
    }
}


/* A thread item's column constants with each stream's exponent shifted by
 * the item's own eref, out of line (once per item) so its FP64
 * temporaries do not add to the register pressure of the kernels that
 * inline the point loops. */
template <int S>
__device__ __noinline__ void item_prologue(const mwsep_area_dev& A, const mwsep_theta_consts& th, int col, int k0,
                                           int k1, Col<S>& cc, int (&eref)[SArr<S>::N])
{
    StreamExp<S> se;
    double r_lo, r_hi;
    chunk_r_range(A, k0, k1, r_lo, r_hi);
    column_consts<S>(A.geom + 4 * (size_t)MWSEP_IDX(col, A.n_cols, 1), th, cc, &se, r_lo, r_hi);
#pragma unroll
    for (int s = 0; s < S; ++s) eref[s] = exp_ref(se.amax[s]);
    shift_exponents<S>(th, se, eref, cc);
}

/* One item of an integral: a (mu, nu) column and its run of k_chunk r-bins.
 * Adds the item's background and stream integrals (FP64) into acc. */
template <int S, int FORM>
__device__ __forceinline__ void integral_item(const mwsep_area_dev& A, const mwsep_theta_consts& th,
                                              const BgConsts& bc, long long item, double (&acc)[1 + S])
{
    const int C = A.convolve;
    const mwsep::ItemPos ip = mwsep::item_pos(A, item);
    const int col = ip.col;
    const int k0 = ip.k0;
    const int k1 = ip.k1;
    Col<S> cc;
    int eref[SArr<S>::N];
    item_prologue<S>(A, th, col, k0, k1, cc, eref);
    fkahan kb, ks[SArr<S>::N];
    kb.zero();
#pragma unroll
    for (int s = 0; s < S; ++s) ks[s].zero();
    for (int k = k0; k < k1; ++k)
    {
        float bg, st[SArr<S>::N];
        convolve<S, FORM>(A.pts + (size_t)MWSEP_IDX(k, A.r_steps, 2) * C, 1, C, cc, bc, bg, st);
        /* q == 0: bg = -1, times V but not reff (:213-216, :504) */
        if (FORM == BG_NONE) bg = -(float)A.irv[MWSEP_IDX(k, A.r_steps, 4)];
        kb.add(bg);
#pragma unroll
        for (int s = 0; s < S; ++s) ks[s].add(st[s]);
    }
    /* the table weights carry reff*irv; the nu-slab factor ids[j] and the
     * hand-off to FP64 happen once per item */
    const double idsj = A.ids[MWSEP_IDX(ip.nu, A.nu_steps, 3)];
    acc[0] += kb.value() * idsj;
#pragma unroll
    for (int s = 0; s < S; ++s) acc[1 + s] += ks[s].value() * (idsj * exp_scale(eref[s]));
}

/* ---- warp tiles ----
 * A warp tile is 32 mu-columns at one nu (one ids factor) and a run of
 * r-bins.  The tile's convolution points, in the table's own (k, n) order,
 * are dealt to the lanes in groups of 32 P: lane l holds points
 * g + 32 i + l (i < P) of a group in registers, and the warp walks the
 * tile's columns with each column's constants broadcast from shared memory.
 * Every point is then evaluated against every column with no load in the
 * inner loop.  The column constants are computed once per tile, one column
 * per lane, in FP64. */
template <int S>
struct ColWords
{
    static constexpr int N = ((4 + 4 * S) + 3) / 4 * 4; /* floats, whole float4s */
};

template <int S>
__device__ __forceinline__ void store_col(float* dst, const Col<S>& cc)
{
    dst[0] = cc.B2;
    dst[1] = cc.Db;
    dst[2] = cc.rb_hi;
    dst[3] = cc.rb_lo;
#pragma unroll
    for (int s = 0; s < S; ++s)
    {
        dst[4 + s] = cc.k2[s];
        dst[4 + S + s] = cc.k2dl[s];
        dst[4 + 2 * S + s] = cc.k0c[s];
        dst[4 + 3 * S + s] = cc.d_hi[s];
    }
}

template <int S>
__device__ __forceinline__ void load_col(const float* src, Col<S>& cc)
{
    constexpr int N = ColWords<S>::N;
    float w[N];
#pragma unroll
    for (int q = 0; q < N / 4; ++q)
    {
        const float4 x = reinterpret_cast<const float4*>(src)[q];
        w[4 * q] = x.x;
        w[4 * q + 1] = x.y;
        w[4 * q + 2] = x.z;
        w[4 * q + 3] = x.w;
    }
    cc.B2 = w[0];
    cc.Db = w[1];
    cc.rb_hi = w[2];
    cc.rb_lo = w[3];
#pragma unroll
    for (int s = 0; s < S; ++s)
    {
        cc.k2[s] = w[4 + s];
        cc.k2dl[s] = w[4 + S + s];
        cc.k0c[s] = w[4 + 2 * S + s];
        cc.d_hi[s] = w[4 + 3 * S + s];
    }
}

/* One warp tile of an integral, called by all 32 lanes of a warp.  cs is
 * this warp's shared scratch of mwsep::kTileCols * ColWords<S>::N floats (16-byte
 * aligned).  Adds the tile's integrals (each lane its share, FP64) into
 * acc. */
template <int S, int FORM>
__device__ __forceinline__ void warp_tile(const mwsep_area_dev& A, const mwsep_theta_consts& th,
                                          const ThetaDF<S>& td, const BgConsts& bc, long long wt,
                                          float* __restrict__ cs, double (&acc)[1 + S])
{
    constexpr int P = mwsep::TileP<S>::P;
    constexpr int CW = ColWords<S>::N;
    const int lane = threadIdx.x & 31;
    const mwsep::TilePos tp = mwsep::tile_pos(A, wt);
    const int nu = tp.nu;
    const int mu0 = tp.mu0;
    const int ncols = tp.ncols;
    const int C = A.convolve;
    const int k0 = tp.k0;
    const int k1 = tp.k1;
    /* the column constants, each stream's exponent shifted by the tile's
     * eref; ids_nu 2^eref goes after the constants in shared memory */
    const double idsv = A.ids[MWSEP_IDX(nu, A.nu_steps, 3)];
    double* const tscale = reinterpret_cast<double*>(cs + mwsep::kTileCols * CW);
    {
        const bool live = lane < ncols;
        const double* g =
            A.geom + 4 * (size_t)MWSEP_IDX((size_t)(mu0 + (live ? lane : 0)) * A.nu_steps + nu, A.n_cols, 1);
        int eref[SArr<S>::N];
        tile_erefs<S>(A, th, k0, k1, g, live, lane, idsv, tscale, eref);
        if (live)
        {
            Col<S> cc;
            column_consts_df<S, false, false>(g, th, td, cc, eref);
            store_col<S>(cs + lane * CW, cc);
        }
    }
    __syncwarp();
    const int nf = (k1 - k0) * C;
    for (int g0 = 0; g0 < nf; g0 += 32 * P)
    {
        /* this lane's points of the group; past the tile's end a copy of its
         * first point with zero weight */
        float4 v[P];
#pragma unroll
        for (int i = 0; i < P; ++i)
        {
            const int f = g0 + 32 * i + lane;
            v[i] = A.pts[MWSEP_IDX((size_t)k0 * C + (f < nf ? f : 0), (size_t)A.r_steps * C, 2)];
            if (f >= nf) v[i].z = 0.f;
        }
        float gb0 = 0.f, gb1 = 0.f, gs0[SArr<S>::N], gs1[SArr<S>::N];
#pragma unroll
        for (int s = 0; s < S; ++s) gs0[s] = gs1[s] = 0.f;
        for (int j = 0; j < ncols; ++j)
        {
            Col<S> cc;
            load_col<S>(cs + j * CW, cc);
#pragma unroll
            for (int i = 0; i < P; i += 2)
            {
                point<S, FORM>(v[i], cc, bc, gb0, gs0);
                if (i + 1 < P) point<S, FORM>(v[i + 1], cc, bc, gb1, gs1);
            }
        }
        if (FORM != BG_NONE) acc[0] += (double)(gb0 + gb1) * idsv;
#pragma unroll
        for (int s = 0; s < S; ++s) acc[1 + s] += (double)(gs0[s] + gs1[s]) * tscale[s];
    }
    /* q == 0: every cell's background is -irv[k] (times ids, not reff;
     * :213-216, :504), the same for all the tile's columns */
    if (FORM == BG_NONE && lane == 0)
    {
        double sum = 0.0;
        for (int k = k0; k < k1; ++k) sum += (double)(-(float)A.irv[MWSEP_IDX(k, A.r_steps, 4)]);
        acc[0] += sum * (double)ncols * idsv;
    }
    __syncwarp();
}

/* ---- packed warp tiles (FP32x2) ----
 * The same warp tile with each lane's points taken two at a time in float2
 * registers, so the FP32 arithmetic runs as packed f32x2 FMA/ADD/MUL
 * (__ffma2_rn, __fadd2_rn, __fmul2_rn): half the FP32 instructions.  The
 * column constants are kept duplicated ({c, c} pairs) in shared memory so
 * they load as ready pairs.  The four Hernquist terms w_i / (rg_i d_i),
 * d_i = (rg_i + r0)^3, of two pairs A = (1, 2), B = (3, 4) are added as one
 * fraction
 *   N / D,  N = (wy1 d3 + wy3 d1) D24 + (wy2 d4 + wy4 d2) D13,  D = D13 D24,
 * with one SFU reciprocal instead of four, which moves work from the SFU to
 * the FMA pipe (the two are the bound of this kernel).  D is clamped at
 * FLT_MIN (a scale radius below ~1e-3 kpc would otherwise flush it). */
typedef float2 f2;
__device__ __forceinline__ f2 add2(f2 a, f2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ f2 mul2(f2 a, f2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ f2 dup2(float a) { return make_float2(a, a); }

/* Packed tiles are used up to 4 streams (their constants fit the registers). */
template <int S>
struct PackedTile
{
    static constexpr bool ok = S <= 4;
    static constexpr int W = 2 * (4 + 4 * S); /* floats per column: every constant twice */
    static constexpr int P = mwsep::TileP<S>::P; /* points per lane per group */
};

/* Floats of shared memory per warp for one tile: the columns' constants,
 * then the tile's per-stream factors ids_nu 2^eref (doubles), read at each
 * group's hand-off to FP64 instead of held in registers or recomputed (an
 * FP64 multiply costs ~64 FP32 operations here). */
template <int S>
struct TileSmem
{
    static constexpr int CW = PackedTile<S>::ok ? PackedTile<S>::W : ColWords<S>::N;
    static constexpr int N = mwsep::kTileCols * CW + (2 * SArr<S>::N + 3) / 4 * 4;
};

template <int S>
struct Col2
{
    f2 B2, D, nrb_hi, L; /* column_consts<S, true>: D and L of t' (B2 t' + L) + D */
    f2 k2[SArr<S>::N], k2dl[SArr<S>::N], k0c[SArr<S>::N], d_hi[SArr<S>::N];
};

template <int S>
__device__ __forceinline__ void store_col2(float* dst, const Col<S>& cc)
{
    auto put = [&](int i, float v) {
        dst[2 * i] = v;
        dst[2 * i + 1] = v;
    };
    put(0, cc.B2);
    put(1, cc.Db);
    put(2, -cc.rb_hi);
    put(3, cc.rb_lo);
#pragma unroll
    for (int s = 0; s < S; ++s)
    {
        put(4 + 4 * s, cc.k2[s]);
        put(5 + 4 * s, cc.k2dl[s]);
        put(6 + 4 * s, cc.k0c[s]);
        put(7 + 4 * s, cc.d_hi[s]);
    }
}

template <int S>
__device__ __forceinline__ void load_col2(const float* src, Col2<S>& c)
{
    const float4* q = reinterpret_cast<const float4*>(src);
    float4 x = q[0];
    c.B2 = make_float2(x.x, x.y);
    c.D = make_float2(x.z, x.w);
    x = q[1];
    c.nrb_hi = make_float2(x.x, x.y);
    c.L = make_float2(x.z, x.w);
#pragma unroll
    for (int s = 0; s < S; ++s)
    {
        x = q[2 + 2 * s];
        c.k2[s] = make_float2(x.x, x.y);
        c.k2dl[s] = make_float2(x.z, x.w);
        x = q[3 + 2 * s];
        c.k0c[s] = make_float2(x.x, x.y);
        c.d_hi[s] = make_float2(x.z, x.w);
    }
}

/* The four points' stream terms against one column.  ARGS_FIRST: every
 * stream's exponent arguments before the first ex2 (the single-evaluation
 * kernels: -0.15% on the full-size integral, -1.5% on config 2; the engine's
 * kernel, +1% there, keeps each stream's ex2 after its own arguments). */
template <int S, bool ARGS_FIRST>
__device__ __forceinline__ void stream_terms4(const f2 tA, const f2 tB, const f2 WA, const f2 WB, const Col2<S>& c,
                                              f2 (&stA)[SArr<S>::N], f2 (&stB)[SArr<S>::N])
{
    if (ARGS_FIRST)
    {
        f2 aA[SArr<S>::N], aB[SArr<S>::N];
#pragma unroll
        for (int s = 0; s < S; ++s)
        {
            const f2 uA = add2(tA, c.d_hi[s]);
            const f2 uB = add2(tB, c.d_hi[s]);
            aA[s] = fma2(uA, fma2(c.k2[s], uA, c.k2dl[s]), c.k0c[s]);
            aB[s] = fma2(uB, fma2(c.k2[s], uB, c.k2dl[s]), c.k0c[s]);
        }
#pragma unroll
        for (int s = 0; s < S; ++s)
        {
            stA[s] = fma2(WA, make_float2(ex2a(aA[s].x), ex2a(aA[s].y)), stA[s]);
            stB[s] = fma2(WB, make_float2(ex2a(aB[s].x), ex2a(aB[s].y)), stB[s]);
        }
        return;
    }
#pragma unroll
    for (int s = 0; s < S; ++s)
    {
        const f2 uA = add2(tA, c.d_hi[s]);
        const f2 uB = add2(tB, c.d_hi[s]);
        const f2 aA = fma2(uA, fma2(c.k2[s], uA, c.k2dl[s]), c.k0c[s]);
        const f2 aB = fma2(uB, fma2(c.k2[s], uB, c.k2dl[s]), c.k0c[s]);
        stA[s] = fma2(WA, make_float2(ex2a(aA.x), ex2a(aA.y)), stA[s]);
        stB[s] = fma2(WB, make_float2(ex2a(aB.x), ex2a(aB.y)), stB[s]);
    }
}

/* Two pairs of points (four points) against one column.  SF: the stream
 * terms before the halo's in the source (the instruction schedule follows:
 * measured -1.8% on the full-size single-evaluation integral and +1.9% in
 * the engine's kernel, whose registers fall differently). */
template <int S, int FORM, bool SF>
__device__ __forceinline__ void points4(const f2 XA, const f2 YA, const f2 WA, const f2 GA, const f2 XB, const f2 YB,
                                        const f2 WB, const f2 GB, const Col2<S>& c, const BgConsts& bc, f2& bg,
                                        f2 (&stA)[SArr<S>::N], f2 (&stB)[SArr<S>::N])
{
    /* t' = (r_hi - rb_hi) + r_lo */
    const f2 tA = add2(add2(XA, c.nrb_hi), YA);
    const f2 tB = add2(add2(XB, c.nrb_hi), YB);
    if (SF) stream_terms4<S, true>(tA, tB, WA, WB, c, stA, stB);
    if (FORM == BG_HERNQUIST || FORM == BG_HERNQUIST_AUX)
    {
        const f2 r0 = dup2(bc.r0);
        const f2 gA = fma2(tA, fma2(c.B2, tA, c.L), c.D);
        const f2 gB = fma2(tB, fma2(c.B2, tB, c.L), c.D);
        const f2 yA = make_float2(rsqa(gA.x), rsqa(gA.y));
        const f2 yB = make_float2(rsqa(gB.x), rsqa(gB.y));
        const f2 sA = fma2(gA, yA, r0);
        const f2 sB = fma2(gB, yB, r0);
        const f2 dA = mul2(mul2(sA, sA), sA);
        const f2 dB = mul2(mul2(sB, sB), sB);
        /* sum_i w_i y_i / d_i over the four points as one fraction N / D:
         * one reciprocal and one accumulation per four points */
        const f2 wyA = mul2(WA, yA), wyB = mul2(WB, yB);
        /* packed first: the two-term fractions of points (A.x, B.x) and
         * (A.y, B.y) in one pair, then their two halves -- the same products
         * as pairing within A and within B, in 3 packed and 5 scalar
         * instructions instead of 11 scalar */
        const f2 n2 = fma2(wyA, dB, mul2(wyB, dA));
        const f2 D2 = mul2(dA, dB);
        const float num = fmaf(n2.x, D2.y, n2.y * D2.x);
        bg.x = fmaf(num, rcpa(fmaxf(D2.x * D2.y, 1.17549435e-38f)), bg.x);
        if (FORM == BG_HERNQUIST_AUX)
        {
            const f2 a = dup2(bc.aux_a), b = dup2(bc.aux_b), cc = dup2(bc.aux_c);
            bg = fma2(WA, fma2(fma2(a, GA, b), GA, cc), bg);
            bg = fma2(WB, fma2(fma2(a, GB, b), GB, cc), bg);
        }
    }
    else if (FORM == BG_GENERAL)
    {
        const f2 r0 = dup2(bc.r0), al = dup2(bc.alpha), ad = dup2(bc.ad3);
        const f2 gA = fma2(tA, fma2(c.B2, tA, c.L), c.D);
        const f2 gB = fma2(tB, fma2(c.B2, tB, c.L), c.D);
        const f2 rA = mul2(gA, make_float2(rsqa(gA.x), rsqa(gA.y)));
        const f2 rB = mul2(gB, make_float2(rsqa(gB.x), rsqa(gB.y)));
        const f2 sA = add2(rA, r0), sB = add2(rB, r0);
        const f2 lA = fma2(al, make_float2(lg2a(rA.x), lg2a(rA.y)), mul2(ad, make_float2(lg2a(sA.x), lg2a(sA.y))));
        const f2 lB = fma2(al, make_float2(lg2a(rB.x), lg2a(rB.y)), mul2(ad, make_float2(lg2a(sB.x), lg2a(sB.y))));
        bg = fma2(WA, make_float2(ex2a(-lA.x), ex2a(-lA.y)), bg);
        bg = fma2(WB, make_float2(ex2a(-lB.x), ex2a(-lB.y)), bg);
    }
    if (!SF) stream_terms4<S, false>(tA, tB, WA, WB, c, stA, stB);
}

/* A packed tile's column constants (one column per lane) and per-stream
 * factors (inline: out of line, the call's register saves cost 1.5% of the
 * full-size integral). */
template <int S>
__device__ __forceinline__ void tile_prologue2(const mwsep_area_dev& A, const mwsep_theta_consts& th,
                                            const ThetaDF<S>& td, int k0, int k1, int mu0, int nu, int ncols,
                                            int lane, double idsv, float* cs, double* tscale)
{
    constexpr int CW = PackedTile<S>::W;
    const bool live = lane < ncols;
    const double* g =
        A.geom + 4 * (size_t)MWSEP_IDX((size_t)(mu0 + (live ? lane : 0)) * A.nu_steps + nu, A.n_cols, 1);
    int eref[SArr<S>::N];
    tile_erefs<S>(A, th, k0, k1, g, live, lane, idsv, tscale, eref);
    if (live)
    {
        Col<S> cc;
        column_consts_df<S, true, false>(g, th, td, cc, eref);
        store_col2<S>(cs + lane * CW, cc);
    }
}

/* warp_tile with packed arithmetic; cs holds TileSmem<S>::N floats for
 * this warp. */
template <int S, int FORM, bool SF = false>
__device__ __forceinline__ void warp_tile2(const mwsep_area_dev& A, const mwsep_theta_consts& th,
                                           const ThetaDF<S>& td, const BgConsts& bc, long long wt,
                                           float* __restrict__ cs, double (&acc)[1 + S])
{
    constexpr int P = PackedTile<S>::P;
    constexpr int NP = P / 2;
    constexpr int CW = PackedTile<S>::W;
    static_assert(NP % 2 == 0, "pairs are taken two at a time");
    const int lane = threadIdx.x & 31;
    const mwsep::TilePos tp = mwsep::tile_pos(A, wt);
    const int nu = tp.nu;
    const int mu0 = tp.mu0;
    const int ncols = tp.ncols;
    const int C = A.convolve;
    const int k0 = tp.k0;
    const int k1 = tp.k1;
    /* the column constants, each stream's exponent shifted by the tile's
     * eref; ids_nu 2^eref goes after the constants in shared memory */
    const double idsv = A.ids[MWSEP_IDX(nu, A.nu_steps, 3)];
    double* const tscale = reinterpret_cast<double*>(cs + mwsep::kTileCols * CW);
    tile_prologue2<S>(A, th, td, k0, k1, mu0, nu, ncols, lane, idsv, cs, tscale);
    __syncwarp();
    const int nf = (k1 - k0) * C;
    for (int g0 = 0; g0 < nf; g0 += 32 * P)
    {
        /* pair m = this lane's points g0 + 64 m + lane and g0 + 64 m + 32 + lane;
         * past the tile's end a copy of its first point with zero weight */
        f2 X[NP], Y[NP], Wt[NP], G[NP];
#pragma unroll
        for (int m = 0; m < NP; ++m)
        {
            const int fa = g0 + 64 * m + lane, fb = fa + 32;
            float4 a = A.pts[MWSEP_IDX((size_t)k0 * C + (fa < nf ? fa : 0), (size_t)A.r_steps * C, 2)];
            float4 b = A.pts[MWSEP_IDX((size_t)k0 * C + (fb < nf ? fb : 0), (size_t)A.r_steps * C, 2)];
            if (fa >= nf) a.z = 0.f;
            if (fb >= nf) b.z = 0.f;
            X[m] = make_float2(a.x, b.x);
            Y[m] = make_float2(a.y, b.y);
            Wt[m] = make_float2(a.z, b.z);
            G[m] = make_float2(a.w, b.w);
        }
        f2 gb = make_float2(0.f, 0.f), gs[SArr<S>::N];
#pragma unroll
        for (int s = 0; s < S; ++s) gs[s] = make_float2(0.f, 0.f);
        f2 gs2[SArr<S>::N]; /* the B pairs' stream sums: two independent chains */
#pragma unroll
        for (int s = 0; s < S; ++s) gs2[s] = make_float2(0.f, 0.f);
        /* columns two or four at a time for up to three streams (measured:
         * -1.7% on the full-size three-stream wedge, -8..-12% on one-stream
         * wedges); four streams keep the rolled loop (their registers spill) */
#pragma unroll(S <= 2 ? 4 : S == 3 ? 2 : 1)
        for (int j = 0; j < ncols; ++j)
        {
            Col2<S> c;
            load_col2<S>(cs + j * CW, c);
#pragma unroll
            for (int m = 0; m < NP; m += 2)
                points4<S, FORM, SF>(X[m], Y[m], Wt[m], G[m], X[m + 1], Y[m + 1], Wt[m + 1], G[m + 1], c, bc, gb,
                                     gs, gs2);
        }
#pragma unroll
        for (int s = 0; s < S; ++s) gs[s] = add2(gs[s], gs2[s]);
        if (FORM != BG_NONE) acc[0] += (double)(gb.x + gb.y) * idsv;
#pragma unroll
        for (int s = 0; s < S; ++s) acc[1 + s] += (double)(gs[s].x + gs[s].y) * tscale[s];
    }
    if (FORM == BG_NONE && lane == 0)
    {
        double sum = 0.0;
        for (int k = k0; k < k1; ++k) sum += (double)(-(float)A.irv[MWSEP_IDX(k, A.r_steps, 4)]);
        acc[0] += sum * (double)ncols * idsv;
    }
    __syncwarp();
}

/* The per-evaluation factors of the likelihood's mixture: w_b / I_b,
 * w_s / I_s and 1 / (0.001 sum w), formed once per block so the per-star
 * epilogue multiplies instead of dividing. */
template <int S>
struct LkScale
{
    double bg, st[SArr<S>::N], inv_sw;
};

template <int S>
__device__ __forceinline__ void lk_scale(const mwsep_theta_consts& th, const double* I, LkScale<S>& k)
{
    k.bg = th.exp_bg_weight / I[0];
#pragma unroll
    for (int s = 0; s < S; ++s) k.st[s] = (s < th.n_streams) ? th.exp_stream_weight[s] / I[1 + s] : 0.0;
    k.inv_sw = 1.0 / th.sum_exp_weights;
}

/* One star's densities (cpu/evaluation_optimized.c:672-690): the
 * background's (-1 for q = 0) and each stream's, summed over the star's
 * convolution points in FP32 and returned in FP64 with the stream's exponent
 * shift undone (the star weights carry its reff_xr_rp3). */
template <int S>
__device__ __forceinline__ void star_density(const mwsep_stars_dev& St, const mwsep_theta_consts& th,
                                             const ThetaDF<S>& td, const BgConsts& bc, int s0, double& bg,
                                             double (&st)[SArr<S>::N])
{
    const int N = St.n_stars;
    Col<S> cc;
    s0 = (int)MWSEP_IDX(s0, N, 7);
    /* the star's convolution points span [r_0, r_{C-1}] (their float parts
     * suffice: the range only places each stream's exponent shift) */
    const double ra = St.pts[s0].x, rb = St.pts[(size_t)(St.convolve - 1) * N + s0].x;
    int eref[SArr<S>::N];
    column_consts_df<S, false, true>(St.geom + 4 * (size_t)s0, th, td, cc, eref, fmin(ra, rb), fmax(ra, rb));
    float bgf = 0.f, stf[SArr<S>::N];
    switch (mwsep_bg_form(&th))
    {
    case BG_HERNQUIST: convolve<S, BG_HERNQUIST>(St.pts + s0, N, St.convolve, cc, bc, bgf, stf); break;
    case BG_HERNQUIST_AUX: convolve<S, BG_HERNQUIST_AUX>(St.pts + s0, N, St.convolve, cc, bc, bgf, stf); break;
    case BG_GENERAL: convolve<S, BG_GENERAL>(St.pts + s0, N, St.convolve, cc, bc, bgf, stf); break;
    default: convolve<S, BG_NONE>(St.pts + s0, N, St.convolve, cc, bc, bgf, stf); break;
    }
    bg = (th.bg_mode == 2) ? -1.0 : (double)bgf;
#pragma unroll
    for (int s = 0; s < S; ++s) st[s] = (double)stf[s] * exp_scale(eref[s]);
}

/* A sum of log10 terms without a log10 per term.  A positive normal term
 * x = m 2^e (m in [1, 2)) adds e to an integer sum and multiplies m into a
 * running FP64 product kept in [1, 2) the same way; log10 is taken once, of
 * the product, plus e log10(2).  Each factor rounds by at most 2^-53
 * relative, 2^-53 / ln 10 ~ 5e-17 in the sum per term -- below the rounding
 * of the per-term log10 sum it replaces -- while the FP64 work per term is
 * one multiply.  Terms follow log10: 0 gives -inf, a negative or NaN term
 * NaN, +inf +inf.  The -238 of a zero star probability
 * (cpu/evaluation_optimized.c:700-716) is counted apart (sentinels). */
struct Log10Sum
{
    double m;      /* product of the mantissas, in [1, 2) */
    long long e;   /* sum of the binary exponents */
    int sentinels; /* -238 terms */
    int special;   /* 1: NaN, 2: +inf, 4: -inf */
};

/* One thread's sum: the same with a 32-bit exponent sum (a thread adds at
 * most a few thousand terms of |e| <= 1128; the block's merge widens it). */
struct Log10Acc
{
    double m;
    int e;
    int sentinels;
    int special;
};

constexpr double kLog10Two_hi = 0.3010299956639812;     /* log10(2) rounded to double */
constexpr double kLog10Two_lo = -2.8037281277851704e-18; /* log10(2) - kLog10Two_hi */
constexpr long long kMantissa = 0x000fffffffffffffLL, kOne = 0x3ff0000000000000LL;

__device__ __forceinline__ void lsum_init(Log10Acc& a)
{
    a.m = 1.0;
    a.e = 0;
    a.sentinels = 0;
    a.special = 0;
}

/* a *= m 2^e for m in [1, 2), renormalised into [1, 2) */
template <typename T, typename E>
__device__ __forceinline__ void lsum_mul(T& a, double m, E e)
{
    const long long b = __double_as_longlong(a.m * m);
    const int k = (int)(b >> 52) - 1023; /* 0 or 1 */
    a.m = __longlong_as_double(b - ((long long)k << 52));
    a.e += e + k;
}

__device__ __forceinline__ void lsum_add(Log10Acc& a, double x)
{
    const long long b = __double_as_longlong(x);
    if (b >= 0x0010000000000000LL && b < 0x7ff0000000000000LL) /* positive normal */
        lsum_mul(a, __longlong_as_double((b & kMantissa) | kOne), (int)(b >> 52) - 1023);
    else if (x == 0.0)
        a.special |= 4;
    else if (!(x > 0.0))
        a.special |= 1;
    else if (x == INFINITY)
        a.special |= 2;
    else /* positive subnormal */
    {
        const long long s = __double_as_longlong(x * 0x1p54);
        lsum_mul(a, __longlong_as_double((s & kMantissa) | kOne), (int)(s >> 52) - 1023 - 54);
    }
}

template <typename T>
__device__ __forceinline__ void lsum_merge(Log10Sum& a, const T& b)
{
    lsum_mul(a, b.m, (long long)b.e);
    a.sentinels += b.sentinels;
    a.special |= b.special;
}

/* the sum: NaN if a term was NaN (or both infinities occurred) */
__device__ __forceinline__ double lsum_value(const Log10Sum& a)
{
    if ((a.special & 1) || (a.special & 6) == 6) return NAN;
    if (a.special & 2) return INFINITY;
    if (a.special & 4) return -INFINITY;
    const double e = (double)a.e;
    const double hi = e * kLog10Two_hi;
    const double lo = fma(e, kLog10Two_hi, -hi) + fma(e, kLog10Two_lo, log10(a.m));
    return (hi + -238.0 * (double)a.sentinels) + lo;
}

/* The likelihood's log10 sums of one thread: [0] the star probabilities,
 * [1] the background alone, [2 + s] stream s alone. */
template <int S>
struct LkAcc
{
    Log10Acc c[2 + S];
    __device__ __forceinline__ void init()
    {
#pragma unroll
        for (int k = 0; k < 2 + S; ++k) lsum_init(c[k]);
    }
};

/* The rest of calculate_likelihood for one star (cpu/evaluation_optimized.c:
 * 692-717), in FP64: the mixture weights over the integrals, the log10
 * terms. */
template <int S>
__device__ __forceinline__ void star_epilogue(const mwsep_theta_consts& th, const LkScale<S>& ks, double bg,
                                              const double (&st)[SArr<S>::N], LkAcc<S>& acc)
{
    const int NS = th.n_streams;
    const double bg_only = bg * ks.bg;
    double star_prob = bg_only;
    if (bg_only == 0.0)
        ++acc.c[1].sentinels;
    else
        lsum_add(acc.c[1], bg_only * ks.inv_sw);
#pragma unroll
    for (int s = 0; s < S; ++s)
    {
        if (s < NS)
        {
            const double st_only = st[s] * ks.st[s];
            star_prob += st_only;
            if (st_only == 0.0)
                ++acc.c[2 + s].sentinels;
            else
                lsum_add(acc.c[2 + s], st_only * ks.inv_sw);
        }
    }
    star_prob *= ks.inv_sw;
    if (star_prob != 0.0)
        lsum_add(acc.c[0], star_prob);
    else
        ++acc.c[0].sentinels;
}

/* calculate_likelihood for one star (cpu/evaluation_optimized.c:665-717):
 * the density sums in FP32, everything after them in FP64. */
template <int S>
__device__ __forceinline__ void likelihood_star(const mwsep_stars_dev& St, const mwsep_theta_consts& th,
                                                const ThetaDF<S>& td, const BgConsts& bc, const LkScale<S>& ks,
                                                int s0, LkAcc<S>& acc)
{
    double bg, st[SArr<S>::N];
    star_density<S>(St, th, td, bc, s0, bg, st);
    star_epilogue<S>(th, ks, bg, st, acc);
}

/* Shared memory of lk_block_store: one Log10Sum per warp and sum. */
template <int S, int BLOCK>
struct LkSmem
{
    static constexpr int N = (BLOCK / 32) * (2 + S);
};

/* The block's sums, combined in a fixed order (warps by butterfly, then
 * warp after warp), as the likelihood partial slots: [0] log10 p, [1] the
 * zero-probability count, [2] background alone, [3 + s] stream s alone,
 * each (value, 0); n_out = 3 + streams. */
template <int S>
__device__ __forceinline__ void lk_block_store(LkAcc<S>& acc, int n_out, Log10Sum* smem, double2* out)
{
    constexpr int NC = 2 + S;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NC; ++k)
    {
        Log10Sum a;
        a.m = acc.c[k].m;
        a.e = acc.c[k].e;
        a.sentinels = acc.c[k].sentinels;
        a.special = acc.c[k].special;
        for (int off = 16; off > 0; off >>= 1)
        {
            Log10Sum b;
            b.m = __shfl_xor_sync(0xffffffffu, a.m, off);
            b.e = __shfl_xor_sync(0xffffffffu, a.e, off);
            b.sentinels = __shfl_xor_sync(0xffffffffu, a.sentinels, off);
            b.special = __shfl_xor_sync(0xffffffffu, a.special, off);
            lsum_merge(a, b);
        }
        if (lane == 0) smem[warp * NC + k] = a;
    }
    __syncthreads();
    if (warp == 0 && lane < NC)
    {
        Log10Sum t = smem[lane];
        for (int w = 1; w < nw; ++w) lsum_merge(t, smem[w * NC + lane]);
        const int slot = lane == 0 ? 0 : lane + 1;
        if (slot < n_out) out[slot] = make_double2(lsum_value(t), 0.0);
        if (lane == 0) out[1] = make_double2((double)t.sentinels, 0.0);
    }
}

} // namespace f32
} // namespace mwsep

#endif
