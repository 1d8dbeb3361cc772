/* mwsep_separation.cu -- the per-star separation output.
 *
 * What the reference's separation program computed after an evaluation
 * (milkyway_separation/cpu/separation.c:37-254; it no longer builds: MPI and
 * headers that are gone), on the GPU for a resident catalogue:
 *
 *   epsilon_s = e^{w_s} / (1 + sum e^{w}),  epsilon_b = 1 / (1 + sum e^{w})   (:128-140)
 *   pbx = epsilon_b psi_b / I_b,  psg_s = epsilon_s psi_s / I_s               (:170-175)
 *   sprob_s = psg_s / (sum psg + pbx),  expected_s = sum over stars           (:186-196)
 *   assignment: a uniform draw r per star, stream k when r falls in the k-th
 *     cumulative sprob interval, background (0) beyond their sum               (probability.c:310-397)
 *   xyz: the star in the stripe frame, magnitude as the radial coordinate    (:75-116, :226-227)
 *
 * psi are the same per-star densities the likelihood uses (plain FP64,
 * mwsep_f64_point.cuh).  The reference drew r with drand48 seeded by the
 * clock; here r = SplitMix64(seed, star) / 2^53, so an assignment is
 * reproducible from its seed.  Up to 8 streams (the reference stopped at 4).
 */
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include "milkyway_separation_gb300.h"
#include "mwsep_ctx.h"
#include "mwsep_f64_point.cuh"
#include "mwsep_geometry.cuh"
#include "mwsep_internal.h"
#include "mwsep_status.h"

using namespace mwsep;

namespace {

struct SepConsts
{
    double eps_b;
    double eps_s[MWSEP_KMAX_STREAMS];
    double m[9]; /* stripe-frame rotation */
    unsigned long long seed;
};

MWSEP_HD inline double uniform01(unsigned long long seed, unsigned long long i)
{
    unsigned long long z = seed + (i + 1ULL) * 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

/* stVector.c:155-169 with stCoords.c:52-65, :188-201 */
MWSEP_HD inline void transform_point(const double* point, const double* m, double* out)
{
    const double r0 = 8.5;
    const double xsun = point[0] + r0;
    const double temp = xsun * xsun + point[1] * point[1];
    double l = atan2(point[1], xsun) * MW_DEG;
    const double b = atan2(point[2], sqrt(temp)) * MW_DEG;
    double g = sqrt(temp + point[2] * point[2]);
    if (l < 0) l += 360;
    g = 5.0 * (log(100.0 * g) / log(10.0)) + 4.2 - 11.0;
    double v[3];
    mwsep::lbr_to_xyz(l, b, g, v);
    v[0] = v[0] - (-8.5);
    out[0] = m[0] * v[0] + m[1] * v[1] + m[2] * v[2];
    out[1] = m[3] * v[0] + m[4] * v[1] + m[5] * v[2];
    out[2] = m[6] * v[0] + m[7] * v[1] + m[8] * v[2];
}

template <int SMAX>
__global__ void __launch_bounds__(256) separation_kernel(const mwsep_stars_dev St,
                                                         const mwsep_theta_consts* __restrict__ thp,
                                                         const double* __restrict__ I, const SepConsts sc,
                                                         double* __restrict__ sprob, int* __restrict__ assign,
                                                         double* __restrict__ xyz)
{
    __shared__ mwsep_theta_consts th;
    f64::load_theta(th, thp);
    __syncthreads();
    const int S = th.n_streams;
    const int N = St.n_stars;
    for (int s0 = blockIdx.x * blockDim.x + threadIdx.x; s0 < N; s0 += gridDim.x * blockDim.x)
    {
        const int si = (int)MWSEP_IDX(s0, N, 7);
        const double* g = St.geom + 4 * (size_t)si;
        double bg, st[SMAX];
        f64::convolve_f64<SMAX>(St.r_point + si, St.qw + si, St.r_in_mag + si, St.r_in_mag2 + si, (size_t)N,
                                St.convolve, g[0], g[1], g[2], g[3], th, bg, st);
        const double rf = St.reff[si];
        if (th.bg_mode != 2) bg *= rf;
        const double pbx = sc.eps_b * bg / I[0];
        double psg[SMAX], sum = 0.0;
#pragma unroll
        for (int j = 0; j < SMAX; ++j)
        {
            psg[j] = 0.0;
            if (j < S)
            {
                const double v = th.stream_on[j] ? st[j] * rf : st[j];
                psg[j] = sc.eps_s[j] * v / I[1 + j];
                sum += psg[j];
            }
        }
        const double r = uniform01(sc.seed, (unsigned long long)s0);
        double cum = 0.0, total = 0.0;
        int k = 0;
#pragma unroll
        for (int j = 0; j < SMAX; ++j)
            if (j < S)
            {
                const double sp = psg[j] / (sum + pbx);
                if (sprob) sprob[(size_t)s0 * S + j] = sp;
                total += sp;
            }
        if (r <= total)
        {
#pragma unroll
            for (int j = 0; j < SMAX; ++j)
                if (j < S && k == 0)
                {
                    cum += psg[j] / (sum + pbx);
                    if (r <= cum) k = j + 1;
                }
        }
        if (assign) assign[s0] = k;
        if (xyz)
        {
            double p[3];
            mwsep::lbr_to_xyz(St.l[si], St.b[si], St.r[si], p);
            transform_point(p, sc.m, xyz + 3 * (size_t)s0);
        }
    }
}

/* The stripe frame: stripe_normal (stCoords.c:142-150, atSurveyGeometry.c:415-459)
 * or sgr_stripe_normal (stCoords.c:153-174), then get_transform onto the z
 * axis (stVector.c:109-137). */
void stripe_transform(int sgr, int wedge, double* m)
{
    double n[3];
    auto lb_to_xyz = [](double l, double b, double* v) {
        l = l / MW_DEG;
        b = b / MW_DEG;
        v[0] = cos(l) * cos(b);
        v[1] = sin(l) * cos(b);
        v[2] = sin(b);
    };
    if (sgr == 0)
    {
        const double eta = (wedge <= 46) ? wedge * 2.5 - 57.5 : wedge * 2.5 - 57.5 - 180.0;
        double slong = 0, slat = 90.0 + eta, ra, dec, l, b;
        slong = slong * MW_PI / 180.0;
        slat = slat * MW_PI / 180.0;
        double anode = 185.0 - 90.0;
        anode = anode * MW_PI / 180.0;
        const double etaPole = 32.5 * MW_PI / 180.0;
        const double x1 = -sin(slong), y1 = cos(slat + etaPole) * cos(slong), z1 = sin(slat + etaPole) * cos(slong);
        ra = atan2(y1, x1) + anode;
        dec = asin(z1);
        ra = ra * 180.0 / MW_PI;
        dec = dec * 180.0 / MW_PI;
        mwsep::bound2(dec, ra);
        mwsep::eq_to_gal(ra, dec, l, b);
        lb_to_xyz(l, b, n);
    }
    else
    {
        double l1, b1, l2, b2, a1[3], a2[3], rot[9];
        mwsep::sgr_rotation_ratio_form(rot);
        mwsep::sgr_to_gal(wedge * 2.5, 0, rot, l1, b1);
        mwsep::sgr_to_gal(wedge * 2.5, 90, rot, l2, b2);
        lb_to_xyz(l1, b1, a1);
        lb_to_xyz(l2, b2, a2);
        n[0] = a1[1] * a2[2] - a1[2] * a2[1];
        n[1] = a1[2] * a2[0] - a1[0] * a2[2];
        n[2] = a1[0] * a2[1] - a1[1] * a2[0];
    }
    const double t[3] = {0.0, 0.0, 1.0};
    double axis[3] = {n[1] * t[2] - n[2] * t[1], n[2] * t[0] - n[0] * t[2], n[0] * t[1] - n[1] * t[0]};
    const double an = sqrt(axis[0] * axis[0] + axis[1] * axis[1] + axis[2] * axis[2]);
    axis[0] /= an;
    axis[1] /= an;
    axis[2] /= an;
    const double nn = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    const double tn = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
    const double angle = acos((n[0] * t[0] + n[1] * t[1] + n[2] * t[2]) / (nn * tn));
    const double sin_a = sin(angle / 2);
    const double x = axis[0] * sin_a, y = axis[1] * sin_a, z = axis[2] * sin_a, w = cos(angle / 2);
    m[0] = 1 - 2 * (y * y + z * z);
    m[1] = 2 * (x * y - z * w);
    m[2] = 2 * (x * z + y * w);
    m[3] = 2 * (x * y + z * w);
    m[4] = 1 - 2 * (x * x + z * z);
    m[5] = 2 * (y * z - x * w);
    m[6] = 2 * (x * z - y * w);
    m[7] = 2 * (y * z + x * w);
    m[8] = 1 - 2 * (x * x + y * y);
}

} // namespace

extern "C" int mwsep_stripe_transform(int sgr_coordinates, int wedge, double* mat9)
{
    if (!mat9 || (sgr_coordinates != 0 && sgr_coordinates != 1)) return mwsep_fail(MWSEP_ERR_ARG);
    stripe_transform(sgr_coordinates, wedge, mat9);
    return MWSEP_OK;
}

extern "C" int mwsep_ctx_separation(mwsep_ctx* c, const double* theta, unsigned long long seed, double* sprob,
                                    int* assignment, double* xyz, mwsep_separation_summary* summary)
{
    mwsep::Range nvtx_range("mwsep.separation");
    if (!c || !theta) return mwsep_fail(MWSEP_ERR_ARG);
    if (c->wedges.empty() || !c->wedges[0]->has_problem || !c->wedges[0]->has_stars)
        return mwsep_fail(MWSEP_ERR_STATE);
    CU(cudaSetDevice(c->device));
    Wedge& w = *c->wedges[0];
    const int S = w.prob.n_streams, A = w.prob.n_areas, N = w.n_stars;
    mwsep_result res;
    int rc = evaluate_impl(c, 1, theta, MWSEP_PLAIN_F64, &res);
    if (rc) return rc;
    /* evaluate_impl leaves theta constants in d_theta and the integrals
     * after the area block of d_out */
    const double* d_ints = c->d_out.as<double>() + (size_t)A * (1 + S);

    SepConsts sc;
    memset(&sc, 0, sizeof(sc));
    double denom = 1.0;
    {
        /* stream weights of this theta (set_astronomy_parameters) */
        ProblemHost p = w.prob;
        int k = 0;
        for (int i = 0; i < p.n_bg; ++i)
            if (p.bg_opt[i]) ++k;
        for (int s = 0; s < p.n_streams; ++s)
        {
            if (p.st_weight_opt[s]) p.st_weight[s] = theta[k++];
            for (int j = 0; j < p.n_sparams; ++j)
                if (p.st_opt[s][j]) ++k;
        }
        for (int j = 0; j < S; ++j) denom += exp(p.st_weight[j]);
        for (int j = 0; j < S; ++j) sc.eps_s[j] = exp(p.st_weight[j]) / denom;
    }
    sc.eps_b = 1.0 / denom;
    stripe_transform(w.prob.sgr, w.prob.wedge, sc.m);
    sc.seed = seed;

    size_t& tot = c->dev_bytes;
    const size_t sp_bytes = sizeof(double) * (size_t)N * (size_t)S;
    const size_t as_bytes = sizeof(int) * (size_t)N;
    const size_t xyz_bytes = sizeof(double) * 3 * (size_t)N;
    int rc2 = 0;
    rc2 |= c->d_sprob.ensure(sp_bytes > 0 ? sp_bytes : 8, tot);
    rc2 |= c->d_assign.ensure(as_bytes, tot);
    rc2 |= c->d_xyz.ensure(xyz_bytes, tot);
    rc2 |= c->h_sep.ensure(sp_bytes + as_bytes + 8);
    if (rc2) return mwsep_fail(MWSEP_ERR_NOMEM);

    int grid = (N + 255) / 256;
    if (grid > c->sm_count * 8) grid = c->sm_count * 8;
    const mwsep_theta_consts* d_th = c->d_theta.as<mwsep_theta_consts>();
    double* d_sp = c->d_sprob.as<double>();
    int* d_as = c->d_assign.as<int>();
    double* d_xyz = xyz ? c->d_xyz.as<double>() : nullptr;
    cudaStream_t st = c->stream;
    int rc3 = wait_stars(c, st);
    if (!rc3) rc3 = ensure_star_f64(c, w, st);
    if (rc3) return rc3;
    if (S <= 1)
        separation_kernel<1><<<grid, 256, 0, st>>>(w.stars_view, d_th, d_ints, sc, d_sp, d_as, d_xyz);
    else if (S <= 2)
        separation_kernel<2><<<grid, 256, 0, st>>>(w.stars_view, d_th, d_ints, sc, d_sp, d_as, d_xyz);
    else if (S <= 4)
        separation_kernel<4><<<grid, 256, 0, st>>>(w.stars_view, d_th, d_ints, sc, d_sp, d_as, d_xyz);
    else
        separation_kernel<8><<<grid, 256, 0, st>>>(w.stars_view, d_th, d_ints, sc, d_sp, d_as, d_xyz);
    CU(cudaGetLastError());
    double* h_sp = c->h_sep.as<double>();
    int* h_as = (int*)(h_sp + (size_t)N * S);
    if (sp_bytes) CU(d2h(c, h_sp, d_sp, sp_bytes));
    CU(d2h(c, h_as, d_as, as_bytes));
    if (xyz) CU(d2h(c, xyz, d_xyz, xyz_bytes));
    CU(cudaStreamSynchronize(st));
    c->last_launches += 1;
    if (sprob) memcpy(sprob, h_sp, sp_bytes);
    if (assignment) memcpy(assignment, h_as, as_bytes);
    if (summary)
    {
        memset(summary, 0, sizeof(*summary));
        summary->number_streams = S;
        summary->likelihood = res.likelihood;
        summary->background_integral = res.background_integral;
        for (int j = 0; j < S; ++j) summary->stream_integrals[j] = res.stream_integrals[j];
        /* separation.c:193-196: expected counts as the running sum over stars */
        for (int s = 0; s < N; ++s)
            for (int j = 0; j < S; ++j) summary->expected[j] += h_sp[(size_t)s * S + j];
        for (int s = 0; s < N; ++s)
        {
            if (h_as[s] == 0)
                ++summary->background_assigned;
            else
                ++summary->assigned[h_as[s] - 1];
        }
    }
    return MWSEP_OK;
}

MWSEP_CHECKS_READER(mwsep_checks_separation)
