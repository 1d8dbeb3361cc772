/* mwsep_f32.cu -- compensated-FP32 integral and likelihood kernels
 * (MWSEP_MIXED_F32).
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
 * are sums of non-negative terms, so FP32 evaluation has no cancellation;
 * r - rb is formed from (hi, lo) float pairs so it keeps full relative
 * accuracy even when r and rb are close.  The stream exponent
 * -|.|^2/(2 sigma^2) becomes a base-2 polynomial k2 t^2 + k0 fed to ex2.
 */
#include <cuda_runtime.h>
#include <math.h>
#include "mwsep_internal.h"
#include "mwsep_reduce.cuh"

using mwsep::comp_sum;

namespace {

constexpr double kLog2e = 1.4426950408889634073599246810018921;

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

/* FP32 Kahan accumulator. */
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

/* Per-column (or per-star) constants of one theta, FP64 -> FP32. */
template <int SMAX>
struct ColumnConsts
{
    float B2, Db, rb_hi, rb_lo;
    float k2[SMAX], k0[SMAX], rs_hi[SMAX], rs_lo[SMAX];
};

template <int SMAX>
__device__ __forceinline__ void column_consts(double bsin, double bcos, double lsin, double lcos,
                                              const mwsep_theta_consts& th, ColumnConsts<SMAX>& cc)
{
    const double u0 = bcos * lcos, u1 = bcos * lsin, u2 = bsin;
    const double iq2 = 1.0 / (th.q * th.q);
    const double perp = u1 * u1 + u2 * u2 * iq2;
    const double B2 = u0 * u0 + perp;
    const double rb = MW_LBR_R * u0 / B2;
    const double Db = (MW_LBR_R * MW_LBR_R) * perp / B2;
    cc.B2 = (float)B2;
    cc.Db = (float)Db;
    split(rb, cc.rb_hi, cc.rb_lo);
#pragma unroll
    for (int s = 0; s < SMAX; ++s)
    {
        if (s < th.n_streams)
        {
            const double a0 = th.a[s][0], a1 = th.a[s][1], a2 = th.a[s][2];
            /* c' = c + Sun offset: x - c = r u - c' */
            const double c0 = th.c[s][0] + MW_LBR_R, c1 = th.c[s][1], c2 = th.c[s][2];
            const double au = a0 * u0 + a1 * u1 + a2 * u2;
            const double p0 = u0 - au * a0, p1 = u1 - au * a1, p2 = u2 - au * a2;
            const double ac = a0 * c0 + a1 * c1 + a2 * c2;
            const double q0 = c0 - ac * a0, q1 = c1 - ac * a1, q2 = c2 - ac * a2;
            const double A2 = p0 * p0 + p1 * p1 + p2 * p2;
            const double rs = (A2 > 1e-300) ? (p0 * q0 + p1 * q1 + p2 * q2) / A2 : 0.0;
            const double e0 = q0 - rs * p0, e1 = q1 - rs * p1, e2 = q2 - rs * p2;
            const double Ds = e0 * e0 + e1 * e1 + e2 * e2;
            const double f = -kLog2e / th.sigma_sq2[s];
            cc.k2[s] = (float)(A2 * f);
            cc.k0[s] = (float)(Ds * f);
            split(rs, cc.rs_hi[s], cc.rs_lo[s]);
        }
        else
        {
            cc.k2[s] = 0.f;
            cc.k0[s] = 0.f;
            cc.rs_hi[s] = 0.f;
            cc.rs_lo[s] = 0.f;
        }
    }
}

/* Sum over the C convolution points of one cell or star.  rh/rl/qv/gm are
 * read at [n*stride].  Returns plain FP32 sums (bg, st[]), each already
 * weighted by the folded table factor qv. */
template <int SMAX>
__device__ __forceinline__ void convolve_f32(const float* __restrict__ rh, const float* __restrict__ rl,
                                             const float* __restrict__ qv, const float* __restrict__ gm,
                                             size_t stride, int C, const ColumnConsts<SMAX>& cc,
                                             const mwsep_theta_consts& th, float r0f, float auxa, float auxb,
                                             float auxc, float alpha, float ad3, float& bg, float (&st)[SMAX])
{
    const int S = th.n_streams;
    float bgs = 0.f;
    float sts[SMAX];
#pragma unroll
    for (int s = 0; s < SMAX; ++s) sts[s] = 0.f;
    const int mode = th.bg_mode;
    const bool aux = th.aux != 0;

#pragma unroll 4
    for (int n = 0; n < C; ++n)
    {
        const size_t o = (size_t)n * stride;
        const float r_hi = rh[o], r_lo = rl[o], q = qv[o];
        if (mode == 0)
        {
            const float t = (r_hi - cc.rb_hi) + (r_lo - cc.rb_lo);
            const float rg2 = fmaf(cc.B2 * t, t, cc.Db);
            const float y = rsqa(rg2);            /* 1/rg */
            const float rs = fmaf(rg2, y, r0f);    /* rg + r0 */
            const float den = rs * rs * rs;
            float term = q * y * rcpa(den);
            if (aux)
            {
                const float g = gm[o];
                term = fmaf(q, fmaf(fmaf(auxa, g, auxb), g, auxc), term);
            }
            bgs += term;
        }
        else if (mode == 1)
        {
            const float t = (r_hi - cc.rb_hi) + (r_lo - cc.rb_lo);
            const float rg2 = fmaf(cc.B2 * t, t, cc.Db);
            const float rg = rg2 * rsqa(rg2);
            /* rg^alpha (rg + r0)^(3 - alpha + delta) in base 2 */
            const float l2 = fmaf(alpha, lg2a(rg), ad3 * lg2a(rg + r0f));
            bgs += q * ex2a(-l2);
        }
#pragma unroll
        for (int s = 0; s < SMAX; ++s)
        {
            if (s < S)
            {
                const float t = (r_hi - cc.rs_hi[s]) + (r_lo - cc.rs_lo[s]);
                const float e = ex2a(fmaf(cc.k2[s] * t, t, cc.k0[s]));
                sts[s] = fmaf(q, e, sts[s]);
            }
        }
    }
    bg = bgs;
#pragma unroll
    for (int s = 0; s < SMAX; ++s) st[s] = sts[s];
}

__device__ __forceinline__ void load_theta(mwsep_theta_consts& dst, const mwsep_theta_consts* src)
{
    const unsigned long long* s = reinterpret_cast<const unsigned long long*>(src);
    unsigned long long* d = reinterpret_cast<unsigned long long*>(&dst);
    for (int i = threadIdx.x; i < (int)(sizeof(mwsep_theta_consts) / 8); i += blockDim.x) d[i] = s[i];
}

template <int SMAX>
__global__ void __launch_bounds__(256) integral_f32_kernel(const mwsep_area_dev A,
                                                           const mwsep_theta_consts* __restrict__ thetas,
                                                           double2* __restrict__ partials,
                                                           long long theta_stride)
{
    __shared__ mwsep_theta_consts th;
    __shared__ double red[2 * (1 + SMAX) * 32];
    load_theta(th, thetas + blockIdx.y);
    __syncthreads();

    comp_sum acc[1 + SMAX];
#pragma unroll
    for (int k = 0; k < 1 + SMAX; ++k) acc[k].zero();

    const int S = th.n_streams;
    const int C = A.convolve;
    const float r0f = (float)th.r0;
    const float auxa = (float)th.bg_a, auxb = (float)th.bg_b, auxc = (float)th.bg_c;
    const float alpha = (float)th.alpha, ad3 = (float)th.alpha_delta3;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long item = (long long)blockIdx.x * blockDim.x + threadIdx.x; item < A.n_items; item += stride)
    {
        const int kc = (int)(item / A.n_cols);
        const int col = (int)(item - (long long)kc * A.n_cols);
        const int j = col % A.nu_steps;
        const double* g = A.geom + 4 * (size_t)col;
        ColumnConsts<SMAX> cc;
        column_consts<SMAX>(g[0], g[1], g[2], g[3], th, cc);
        const int k0 = kc * A.k_chunk;
        const int k1 = min(k0 + A.k_chunk, A.r_steps);
        fkahan kb, ks[SMAX];
        kb.zero();
#pragma unroll
        for (int s = 0; s < SMAX; ++s) ks[s].zero();
        for (int k = k0; k < k1; ++k)
        {
            float bg, st[SMAX];
            const size_t row = (size_t)k * C;
            convolve_f32<SMAX>(A.r_hi + row, A.r_lo + row, A.qwv + row, A.gmag + row, 1, C, cc, th, r0f, auxa,
                               auxb, auxc, alpha, ad3, bg, st);
            if (th.bg_mode == 2) bg = -(float)A.irv[k]; /* bg = -1 times V, no reff (:213-216) */
            kb.add(bg);
#pragma unroll
            for (int s = 0; s < SMAX; ++s)
                if (s < S && th.stream_on[s]) ks[s].add(st[s]);
        }
        /* the folded qwv carries reff*irv; the nu-slab factor ids[j] and the
         * hand-off to FP64 happen once per item */
        const double idsj = A.ids[j];
        acc[0].add(kb.value() * idsj);
#pragma unroll
        for (int s = 0; s < SMAX; ++s)
            if (s < S) acc[1 + s].add(ks[s].value() * idsj);
    }
    mwsep::block_reduce<1 + SMAX>(acc, red);
    if (threadIdx.x == 0)
    {
        double2* out = partials + (size_t)blockIdx.y * theta_stride + (size_t)blockIdx.x * (1 + S);
        out[0] = make_double2(acc[0].s, acc[0].c);
#pragma unroll
        for (int s = 0; s < SMAX; ++s)
            if (s < S) out[1 + s] = make_double2(acc[1 + s].s, acc[1 + s].c);
    }
}

template <int SMAX>
__global__ void __launch_bounds__(256) likelihood_f32_kernel(const mwsep_stars_dev St,
                                                             const mwsep_theta_consts* __restrict__ thetas,
                                                             const double* __restrict__ integrals,
                                                             double2* __restrict__ partials,
                                                             long long theta_stride)
{
    __shared__ mwsep_theta_consts th;
    __shared__ double red[2 * (3 + SMAX) * 32];
    load_theta(th, thetas + blockIdx.y);
    __syncthreads();
    const int S = th.n_streams;
    const double* I = integrals + (size_t)blockIdx.y * (1 + S);
    const double Ibg = I[0];
    const float r0f = (float)th.r0;
    const float auxa = (float)th.bg_a, auxb = (float)th.bg_b, auxc = (float)th.bg_c;
    const float alpha = (float)th.alpha, ad3 = (float)th.alpha_delta3;

    comp_sum acc[3 + SMAX];
#pragma unroll
    for (int k = 0; k < 3 + SMAX; ++k) acc[k].zero();

    const int N = St.n_stars;
    for (int s0 = blockIdx.x * blockDim.x + threadIdx.x; s0 < N; s0 += gridDim.x * blockDim.x)
    {
        const double* g = St.geom + 4 * (size_t)s0;
        ColumnConsts<SMAX> cc;
        column_consts<SMAX>(g[0], g[1], g[2], g[3], th, cc);
        float bgf, stf[SMAX];
        convolve_f32<SMAX>(St.r_hi + s0, St.r_lo + s0, St.qwv + s0, St.gmag + s0, (size_t)N, St.convolve, cc,
                           th, r0f, auxa, auxb, auxc, alpha, ad3, bgf, stf);
        /* qwv already carries the star's reff_xr_rp3 */
        const double bg = (th.bg_mode == 2) ? -1.0 : (double)bgf;

        double bg_only = (bg / Ibg) * th.exp_bg_weight;
        double star_prob = bg_only;
        bg_only = (bg_only == 0.0) ? -238.0 : log10(bg_only / th.sum_exp_weights);
        acc[2].add(bg_only);
#pragma unroll
        for (int s = 0; s < SMAX; ++s)
        {
            if (s < S)
            {
                const double v = th.stream_on[s] ? (double)stf[s] : 0.0;
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
    mwsep::block_reduce<3 + SMAX>(acc, red);
    if (threadIdx.x == 0)
    {
        double2* out = partials + (size_t)blockIdx.y * theta_stride + (size_t)blockIdx.x * (3 + S);
#pragma unroll
        for (int k = 0; k < 3 + SMAX; ++k)
            if (k < 3 + S) out[k] = make_double2(acc[k].s, acc[k].c);
    }
}

template <int SMAX>
int launch_integral(const mwsep_area_dev* A, const mwsep_theta_consts* th, const mwsep_launch_shape* sh,
                    double2* partials, cudaStream_t st)
{
    const long long ncomp = 1 + sh->n_streams;
    const long long theta_stride = (long long)sh->n_areas * sh->grid * ncomp;
    dim3 g(sh->grid, sh->n_theta);
    integral_f32_kernel<SMAX><<<g, sh->block, 0, st>>>(*A, th, partials + (size_t)sh->area_index * sh->grid * ncomp,
                                                        theta_stride);
    return (int)cudaGetLastError();
}

template <int SMAX>
int launch_likelihood(const mwsep_stars_dev* S, const mwsep_theta_consts* th, const mwsep_launch_shape* sh,
                      const double* integrals, double2* partials, cudaStream_t st)
{
    const long long theta_stride = (long long)sh->grid * (3 + sh->n_streams);
    dim3 g(sh->grid, sh->n_theta);
    likelihood_f32_kernel<SMAX><<<g, sh->block, 0, st>>>(*S, th, integrals, partials, theta_stride);
    return (int)cudaGetLastError();
}

} // namespace

extern "C" int mwsep_launch_integral_f32(const mwsep_area_dev* area, const mwsep_theta_consts* th_dev,
                                         const mwsep_launch_shape* sh, double2* partials, void* stream)
{
    cudaStream_t st = (cudaStream_t)stream;
    if (sh->n_streams <= 1) return launch_integral<1>(area, th_dev, sh, partials, st);
    if (sh->n_streams <= 2) return launch_integral<2>(area, th_dev, sh, partials, st);
    if (sh->n_streams <= 4) return launch_integral<4>(area, th_dev, sh, partials, st);
    return launch_integral<8>(area, th_dev, sh, partials, st);
}

extern "C" int mwsep_launch_likelihood_f32(const mwsep_stars_dev* stars, const mwsep_theta_consts* th_dev,
                                           const mwsep_launch_shape* sh, const double* integrals,
                                           double2* partials, void* stream)
{
    cudaStream_t st = (cudaStream_t)stream;
    if (sh->n_streams <= 1) return launch_likelihood<1>(stars, th_dev, sh, integrals, partials, st);
    if (sh->n_streams <= 2) return launch_likelihood<2>(stars, th_dev, sh, integrals, partials, st);
    if (sh->n_streams <= 4) return launch_likelihood<4>(stars, th_dev, sh, integrals, partials, st);
    return launch_likelihood<8>(stars, th_dev, sh, integrals, partials, st);
}
