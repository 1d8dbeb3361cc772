/* mwsep_f32_point.cuh -- the compensated-FP32 density evaluation shared by
 * every compensated kernel (single evaluation, batches, the tiled engine).
 *
 * Split of precision:
 *   FP64: the per-column (or per-star) coordinate transform with the Sun
 *         offset, the r-bin volume and convolution weight tables (built in
 *         FP64, rounded to FP32 once), the per-item and cross-block sums, the
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
 * with B2, rb, Db, A2, rs, Ds >= 0 computed per column in FP64.  Both forms
 * are sums of non-negative terms, so FP32 evaluation has no cancellation.
 * t = r - rb is formed from (hi, lo) float pairs, so it keeps full relative
 * accuracy even where r and rb are close, and each stream reuses it:
 * r - rs = t + (rb - rs) with the FP64 offset split into (hi, lo) too.
 * The stream exponent -|.|^2/(2 sigma^2) becomes k2 ts^2 + k0 in base 2.
 */
#ifndef MWSEP_F32_POINT_CUH
#define MWSEP_F32_POINT_CUH

#include <cuda_runtime.h>
#include <math.h>
#include "mwsep_internal.h"
#include "mwsep_reduce.cuh"

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

template <int S>
__device__ __forceinline__ void column_consts(const double* g, const mwsep_theta_consts& th, Col<S>& cc)
{
    const double bsin = g[0], bcos = g[1], lsin = g[2], lcos = g[3];
    const double u0 = bcos * lcos, u1 = bcos * lsin, u2 = bsin;
    const double iq2 = 1.0 / (th.q * th.q);
    const double perp = u1 * u1 + u2 * u2 * iq2;
    const double B2 = u0 * u0 + perp;
    const double rb = MW_LBR_R * u0 / B2;
    cc.B2 = (float)B2;
    cc.Db = (float)((MW_LBR_R * MW_LBR_R) * perp / B2);
    split(rb, cc.rb_hi, cc.rb_lo);
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
            cc.k0c[s] = th.stream_on[s] ? (float)(Ds * f + k2 * (double)d_lo * (double)d_lo) : -1.0e30f;
        }
        else
        {
            cc.k2[s] = 0.f;
            cc.k2dl[s] = 0.f;
            cc.k0c[s] = -1.0e30f;
            cc.d_hi[s] = 0.f;
        }
    }
}

struct BgConsts
{
    float r0, aux_a, aux_b, aux_c, alpha, ad3;
};

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

    auto point = [&](const float4 v, float& bgacc, float (&sacc)[SArr<S>::N]) {
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
    };

    /* four points per trip, loads issued before any arithmetic */
    int n = 0;
    for (; n + 3 < C; n += 4)
    {
        const float4 v0 = p[(size_t)n * stride];
        const float4 v1 = p[(size_t)(n + 1) * stride];
        const float4 v2 = p[(size_t)(n + 2) * stride];
        const float4 v3 = p[(size_t)(n + 3) * stride];
        point(v0, bga, sa);
        point(v1, bgb, sb);
        point(v2, bga, sa);
        point(v3, bgb, sb);
    }
    for (; n < C; ++n) point(p[(size_t)n * stride], bga, sa);
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


/* One item of an integral: a (mu, nu) column and its run of k_chunk r-bins.
 * Adds the item's background and stream integrals (FP64) into acc. */
template <int S, int FORM>
__device__ __forceinline__ void integral_item(const mwsep_area_dev& A, const mwsep_theta_consts& th,
                                              const BgConsts& bc, long long item, double (&acc)[1 + S])
{
    const int C = A.convolve;
    const int kc = (int)(item / A.n_cols);
    const int col = (int)(item - (long long)kc * A.n_cols);
    Col<S> cc;
    column_consts<S>(A.geom + 4 * (size_t)col, th, cc);
    const int k0 = kc * A.k_chunk;
    const int k1 = min(k0 + A.k_chunk, A.r_steps);
    fkahan kb, ks[SArr<S>::N];
    kb.zero();
#pragma unroll
    for (int s = 0; s < S; ++s) ks[s].zero();
    for (int k = k0; k < k1; ++k)
    {
        float bg, st[SArr<S>::N];
        convolve<S, FORM>(A.pts + (size_t)k * C, 1, C, cc, bc, bg, st);
        /* q == 0: bg = -1, times V but not reff (:213-216, :504) */
        if (FORM == BG_NONE) bg = -(float)A.irv[k];
        kb.add(bg);
#pragma unroll
        for (int s = 0; s < S; ++s) ks[s].add(st[s]);
    }
    /* the table weights carry reff*irv; the nu-slab factor ids[j] and the
     * hand-off to FP64 happen once per item */
    const double idsj = A.ids[col % A.nu_steps];
    acc[0] += kb.value() * idsj;
#pragma unroll
    for (int s = 0; s < S; ++s) acc[1 + s] += ks[s].value() * idsj;
}

/* calculate_likelihood for one star (cpu/evaluation_optimized.c:665-717):
 * the density sums in FP32, everything after them in FP64.  acc slots:
 * [0] log10 p, [1] zero count, [2] bg-only, [3+s] stream-only. */
template <int S>
__device__ __forceinline__ void likelihood_star(const mwsep_stars_dev& St, const mwsep_theta_consts& th,
                                                const BgConsts& bc, const double* I, int s0, double (&acc)[3 + S])
{
    const int NS = th.n_streams;
    const int N = St.n_stars;
    Col<S> cc;
    column_consts<S>(St.geom + 4 * (size_t)s0, th, cc);
    float bgf = 0.f, stf[SArr<S>::N];
    switch (mwsep_bg_form(&th))
    {
    case BG_HERNQUIST: convolve<S, BG_HERNQUIST>(St.pts + s0, N, St.convolve, cc, bc, bgf, stf); break;
    case BG_HERNQUIST_AUX: convolve<S, BG_HERNQUIST_AUX>(St.pts + s0, N, St.convolve, cc, bc, bgf, stf); break;
    case BG_GENERAL: convolve<S, BG_GENERAL>(St.pts + s0, N, St.convolve, cc, bc, bgf, stf); break;
    default: convolve<S, BG_NONE>(St.pts + s0, N, St.convolve, cc, bc, bgf, stf); break;
    }
    /* the star weights carry its reff_xr_rp3 */
    const double bg = (th.bg_mode == 2) ? -1.0 : (double)bgf;
    double bg_only = (bg / I[0]) * th.exp_bg_weight;
    double star_prob = bg_only;
    acc[2] += (bg_only == 0.0) ? -238.0 : log10(bg_only / th.sum_exp_weights);
#pragma unroll
    for (int s = 0; s < S; ++s)
    {
        if (s < NS)
        {
            double st_only = (double)stf[s] / I[1 + s] * th.exp_stream_weight[s];
            star_prob += st_only;
            acc[3 + s] += (st_only == 0.0) ? -238.0 : log10(st_only / th.sum_exp_weights);
        }
    }
    star_prob /= th.sum_exp_weights;
    if (star_prob != 0.0)
        acc[0] += log10(star_prob);
    else
    {
        acc[0] += -238.0;
        acc[1] += 1.0;
    }
}

} // namespace f32
} // namespace mwsep

#endif
