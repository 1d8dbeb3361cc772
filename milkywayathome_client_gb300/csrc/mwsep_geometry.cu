/* mwsep_geometry.cu -- parameter-independent device tables.
 *
 *  - per-(mu, nu) column of a wedge: Galactic (l, b) of the column centre
 *    and the four sines/cosines the density loop uses;
 *  - per-star convolution tables (the per-star set_probability_constants).
 *
 * Compiled with -fmad=false; transcendentals are CUDA's double-precision
 * libm (<= 2 ulp), so these tables agree with the reference's host tables
 * to a few ulp rather than bit for bit; the tests bound that.
 */
#include <cuda_runtime.h>
#include <math.h>
#include "mwsep_internal.h"
#include "mwsep_geometry.cuh"
#include "mwsep_df.cuh"

namespace {

/* One (mu, nu) column: cpu/evaluation_optimized.c:463 and :480-491, then
 * the per-point sines/cosines of calculate_probabilities :205-208. */
__global__ void geometry_kernel(double mu_min, double mu_step, int mu_steps, const double* __restrict__ nus,
                                int nu_steps, int sgr, int wedge, double* __restrict__ geom)
{
    const int n = mu_steps * nu_steps;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x)
    {
        const int i = idx / nu_steps;
        const int j = idx - i * nu_steps;
        const double mu = mu_min + (i * mu_step);
        const double nu = nus[j];
        double l, b;
        mwsep::wedge_point_lb(sgr, wedge, mu + 0.5 * mu_step, nu, l, b);
        double* g = geom + 4 * (size_t)idx;
        g[0] = sin(b / MW_DEG);
        g[1] = cos(b / MW_DEG);
        g[2] = sin(l / MW_DEG);
        g[3] = cos(l / MW_DEG);
    }
}

/* Per-star tables: cpu/evaluation_optimized.c:159-188 applied to the
 * star's distance, plus its sines/cosines (:205-208).  Tables are [C][N].
 * The per-point pow and exp separate into a per-star and a per-point factor:
 *   r_point = 10^((g' - M)/5 + 1) / 1000 * 10^(dx_n / 5),
 *   qw_r3_N = (gl_w_n coeff e^{-dx_n^2 / 2 sigma^2}) r_point^3,
 * with nfac = {10^(dx_n/5)} then {gl_w_n coeff e^{-dx_n^2/2 sigma^2}} built
 * once per problem on the host: one multiply per point instead of a pow and
 * an exp, equal to the reference's values within a few ulp. */
/* Per star: g', reff_xr_rp3, the distance factor 10^((g' - M)/5 + 1)/1000 and
 * the star's sines/cosines; head[s] = g', head[n + s] = the factor. */
__global__ void star_head_kernel(int n, const double* __restrict__ l, const double* __restrict__ b,
                                 const double* __restrict__ r, double* __restrict__ geom, double* __restrict__ reff,
                                 double* __restrict__ head)
{
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x)
    {
        double gPrime, rf;
        mwsep::prob_consts_head(r[s], gPrime, rf);
        reff[s] = rf;
        head[s] = gPrime;
        head[(size_t)n + s] = pow(10.0, (gPrime - MW_ABSM) / 5.0 + 1.0) / 1000.0;
        double* gg = geom + 4 * (size_t)s;
        gg[0] = sin(b[s] / MW_DEG);
        gg[1] = cos(b[s] / MW_DEG);
        gg[2] = sin(l[s] / MW_DEG);
        gg[3] = cos(l[s] / MW_DEG);
    }
}

/* The plain forms' FP64 tables at [i][s] (convolution point i =
 * blockIdx.y, one thread per star): r_point, qw_r3_N, r_in_mag,
 * r_in_mag2.  Built when a plain form first reads them. */
__global__ void star_f64_kernel(int n, const double* __restrict__ dx, const double* __restrict__ nfac,
                                const double* __restrict__ head, double* __restrict__ r_point,
                                double* __restrict__ qw, double* __restrict__ r_in_mag,
                                double* __restrict__ r_in_mag2)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int i = blockIdx.y, C = gridDim.y;
    const double g = head[s] + dx[i];
    const double rp = head[(size_t)n + s] * nfac[i];
    const size_t o = (size_t)i * n + s;
    r_in_mag[o] = g;
    r_in_mag2[o] = g * g;
    r_point[o] = rp;
    qw[o] = nfac[C + i] * (rp * rp * rp);
}

/* The compensated form's table pts[i][s] = {r_hi, r_lo, qw * reff, g}, one
 * thread per star over its C points, in float pairs on the FP32 pipe (the
 * FP64 tables took ~0.25 ms of FP64 work per 100k x 120 points): the same
 * factors r = r' F_i, qw = wq_i r^3, g = g' + dx_i (r', g' per star from
 * star_head_kernel; F_i = nfac[i], wq_i = nfac[C + i]), each rounded to
 * float once from its pair (~2^-44 relative before the rounding).  kc holds
 * the per-point pairs F_i, wq_i and dx_i, built by the block. */
__global__ void star_pts_kernel(int n, int C, const double* __restrict__ dx, const double* __restrict__ nfac,
                                const double* __restrict__ head, const double* __restrict__ reff,
                                float4* __restrict__ pts)
{
    using namespace mwsep::dfl;
    extern __shared__ float2 kc[]; /* [C] x {F, wq, dx} pairs */
    for (int i = threadIdx.x; i < C; i += blockDim.x)
    {
        const df f = from_double(nfac[i]), w = from_double(nfac[C + i]), d = from_double(dx[i]);
        kc[3 * i] = make_float2(f.hi, f.lo);
        kc[3 * i + 1] = make_float2(w.hi, w.lo);
        kc[3 * i + 2] = make_float2(d.hi, d.lo);
    }
    __syncthreads();
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const df rs = from_double(head[(size_t)n + s]), gs = from_double(head[s]), rf = from_double(reff[s]);
    for (int i = 0; i < C; ++i)
    {
        const float2 f = kc[3 * i], w = kc[3 * i + 1], d = kc[3 * i + 2];
        const df r = mul(rs, mk(f.x, f.y));
        const df q = mul(mk(w.x, w.y), mul(sqr(r), r));
        pts[(size_t)i * n + s] = make_float4(r.hi, r.lo, mul(q, rf).hi, add_fast(gs, mk(d.x, d.y)).hi);
    }
}

} // namespace

extern "C" int mwsep_launch_geometry(double mu_min, double mu_step, int mu_steps, const double* nus, int nu_steps,
                                     int sgr, int wedge, double* geom_out, void* stream)
{
    const int n = mu_steps * nu_steps;
    if (n <= 0) return 0;
    int grid = (n + 255) / 256;
    if (grid > 152 * 32) grid = 152 * 32;
    geometry_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(mu_min, mu_step, mu_steps, nus,
                                                            nu_steps, sgr, wedge, geom_out);
    return (int)cudaGetLastError();
}

extern "C" int mwsep_launch_star_tables(int n, const double* l, const double* b, const double* r, int convolve,
                                        const double* dx, const double* nfac, double* geom, double* reff,
                                        float4* pts, double* head, void* stream)
{
    if (n <= 0) return 0;
    if (convolve < 1 || convolve > MWSEP_MAX_CONVOLVE) return (int)cudaErrorInvalidValue;
    cudaStream_t st = (cudaStream_t)stream;
    int grid = (n + 127) / 128;
    if (grid > 152 * 32) grid = 152 * 32;
    star_head_kernel<<<grid, 128, 0, st>>>(n, l, b, r, geom, reff, head);
    star_pts_kernel<<<(n + 127) / 128, 128, (size_t)convolve * 3 * sizeof(float2), st>>>(n, convolve, dx, nfac, head,
                                                                                        reff, pts);
    return (int)cudaGetLastError();
}

extern "C" int mwsep_launch_star_f64(int n, int convolve, const double* dx, const double* nfac, const double* head,
                                     double* r_point, double* qw, double* r_in_mag, double* r_in_mag2, void* stream)
{
    if (n <= 0) return 0;
    if (convolve < 1 || convolve > MWSEP_MAX_CONVOLVE) return (int)cudaErrorInvalidValue;
    star_f64_kernel<<<dim3((n + 255) / 256, convolve), 256, 0, (cudaStream_t)stream>>>(n, dx, nfac, head, r_point, qw,
                                                                                      r_in_mag, r_in_mag2);
    return (int)cudaGetLastError();
}
