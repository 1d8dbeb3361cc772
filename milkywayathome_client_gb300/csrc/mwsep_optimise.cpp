/* mwsep_optimise.cpp -- optimiser-side consumers of batched evaluations.
 *
 * The reference's parameter-error program (milkyway_separation/cpu/errors.c:38-84)
 * takes the Hessian of the likelihood at the best point by finite
 * differences (get_hessian, from the Milkyway@Home search library, which the
 * reference does not carry), inverts it (util/matrix.c:234-331), divides by
 * the number of stars and reports sqrt|Sigma_ii|.  Its searches (gradient
 * descent, Newton, cpu/mpi_astronomy.c:96-124) consume gradients the same way.
 * Every finite-difference point is an independent evaluation of one wedge, so
 * here all of them go to the engine as batches of requests
 * (mwsep_ctx_evaluate_requests) instead of one evaluation at a time.
 *
 * Differences, with f = the evaluation's likelihood (prob_sum/N - 3):
 *   gradient  g_i  = (f(x + h_i e_i) - f(x - h_i e_i)) / (2 h_i)
 *   diagonal  H_ii = ((f(x + h_i e_i) - f0) + (f(x - h_i e_i) - f0)) / (h_i h_i)
 *   off-diag  H_ij = ((f(x+h_i e_i+h_j e_j) - f(x+h_i e_i-h_j e_j))
 *                    - (f(x-h_i e_i+h_j e_j) - f(x-h_i e_i-h_j e_j))) / (4 h_i h_j)
 * 2P^2 + 1 evaluations for P parameters.  Results do not depend on how the
 * points are batched: an evaluation's bits depend on its wedge only.
 */
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <new>
#include <vector>

#include "milkyway_separation_gb300.h"
#include "mwsep_status.h"

namespace {

constexpr int kChunk = 256; /* requests per engine batch */

/* Evaluate f at every point (rows of P doubles) of one wedge. */
int evaluate_points(mwsep_ctx* ctx, int wedge, int P, const std::vector<double>& pts, int precision,
                    std::vector<double>& f)
{
    const int n = (int)(pts.size() / (size_t)P);
    f.assign((size_t)n, 0.0);
    std::vector<mwsep_request> reqs;
    std::vector<mwsep_result> out;
    for (int b = 0; b < n; b += kChunk)
    {
        const int m = (n - b < kChunk) ? n - b : kChunk;
        reqs.resize((size_t)m);
        out.resize((size_t)m);
        for (int i = 0; i < m; ++i)
        {
            reqs[(size_t)i].wedge = wedge;
            reqs[(size_t)i].theta = pts.data() + (size_t)(b + i) * P;
        }
        int rc = mwsep_ctx_evaluate_requests(ctx, m, reqs.data(), precision, out.data());
        if (rc) return rc;
        for (int i = 0; i < m; ++i) f[(size_t)(b + i)] = out[(size_t)i].likelihood;
    }
    return MWSEP_OK;
}

int check_inputs(mwsep_ctx* ctx, int wedge, const double* theta, const double* step, int precision, int& P)
{
    if (!ctx || !theta || !step) return MWSEP_ERR_ARG;
    if (precision != MWSEP_PLAIN_F64 && precision != MWSEP_MIXED_F32 && precision != MWSEP_PLAIN_DF)
        return MWSEP_ERR_ARG;
    P = mwsep_ctx_wedge_theta_count(ctx, wedge);
    if (P < 1) return MWSEP_ERR_ARG;
    for (int i = 0; i < P; ++i)
        if (!(step[i] > 0.0) || !isfinite(step[i])) return MWSEP_ERR_ARG;
    return MWSEP_OK;
}

/* util/matrix.c:234-269: LU decomposition with partial pivoting (first
 * largest |a_ik| wins), rows swapped in place. */
int lup_decompose(int n, std::vector<double>& lu, std::vector<int>& perm)
{
    perm.resize((size_t)n);
    for (int i = 0; i < n; ++i) perm[(size_t)i] = i;
    for (int k = 0; k < n; ++k)
    {
        double best = 0.0;
        int kp = 0;
        for (int i = k; i < n; ++i)
        {
            const double a = fabs(lu[(size_t)i * n + k]);
            if (a > best)
            {
                best = a;
                kp = i;
            }
        }
        if (best == 0.0) return -1; /* singular */
        const int t = perm[(size_t)k];
        perm[(size_t)k] = perm[(size_t)kp];
        perm[(size_t)kp] = t;
        for (int j = 0; j < n; ++j)
        {
            const double v = lu[(size_t)k * n + j];
            lu[(size_t)k * n + j] = lu[(size_t)kp * n + j];
            lu[(size_t)kp * n + j] = v;
        }
        const double pivot = lu[(size_t)k * n + k];
        for (int i = k + 1; i < n; ++i)
        {
            double& lik = lu[(size_t)i * n + k];
            lik = lik / pivot;
            for (int j = k + 1; j < n; ++j) lu[(size_t)i * n + j] = lu[(size_t)i * n + j] - lik * lu[(size_t)k * n + j];
        }
    }
    return 0;
}

/* util/matrix.c:277-296: forward then back substitution for one column. */
void lup_solve(int n, const std::vector<double>& lu, const std::vector<int>& perm, const double* b, double* x)
{
    std::vector<double> y((size_t)n);
    for (int i = 0; i < n; ++i)
    {
        double v = b[perm[(size_t)i]];
        for (int j = 0; j < i; ++j) v -= lu[(size_t)i * n + j] * y[(size_t)j];
        y[(size_t)i] = v;
    }
    for (int i = n - 1; i >= 0; --i)
    {
        double v = y[(size_t)i];
        for (int j = i + 1; j < n; ++j) v -= lu[(size_t)i * n + j] * x[j];
        x[i] = v / lu[(size_t)i * n + i];
    }
}

} // namespace

extern "C" int mwsep_invert_matrix(int n, const double* a, double* inverse)
{
    if (n < 1 || !a || !inverse) return mwsep_fail(MWSEP_ERR_ARG);
    std::vector<double> lu(a, a + (size_t)n * n);
    std::vector<int> perm;
    if (lup_decompose(n, lu, perm)) return mwsep_fail(MWSEP_ERR_ARG);
    /* util/matrix.c:298-319: solve for each unit vector, then transpose */
    std::vector<double> e((size_t)n, 0.0), col((size_t)n);
    for (int c = 0; c < n; ++c)
    {
        e[(size_t)c] = 1.0;
        lup_solve(n, lu, perm, e.data(), col.data());
        e[(size_t)c] = 0.0;
        for (int r = 0; r < n; ++r) inverse[(size_t)r * n + c] = col[(size_t)r];
    }
    return MWSEP_OK;
}

extern "C" int mwsep_errors_from_hessian(int n, const double* hessian, int number_stars, double* sigma,
                                         double* stddev)
{
    if (n < 1 || !hessian || number_stars < 1) return mwsep_fail(MWSEP_ERR_ARG);
    std::vector<double> inv((size_t)n * n);
    const int rc = mwsep_invert_matrix(n, hessian, inv.data());
    if (rc) return rc;
    /* cpu/errors.c:56-80 */
    for (size_t i = 0; i < inv.size(); ++i) inv[i] /= (double)number_stars;
    if (sigma) memcpy(sigma, inv.data(), inv.size() * sizeof(double));
    if (stddev)
        for (int i = 0; i < n; ++i) stddev[i] = sqrt(fabs(inv[(size_t)i * n + i]));
    return MWSEP_OK;
}

extern "C" int mwsep_ctx_gradient(mwsep_ctx* ctx, int wedge, const double* theta, const double* step, int precision,
                                  double* f0, double* gradient)
{
    int P = 0;
    int rc = check_inputs(ctx, wedge, theta, step, precision, P);
    if (rc) return mwsep_fail(rc);
    std::vector<double> pts;
    try
    {
        pts.resize((size_t)(2 * P + 1) * P);
    }
    catch (const std::bad_alloc&)
    {
        return mwsep_fail(MWSEP_ERR_NOMEM);
    }
    for (int k = 0; k < 2 * P + 1; ++k) memcpy(&pts[(size_t)k * P], theta, sizeof(double) * P);
    for (int i = 0; i < P; ++i)
    {
        pts[(size_t)(1 + 2 * i) * P + i] += step[i];
        pts[(size_t)(2 + 2 * i) * P + i] -= step[i];
    }
    std::vector<double> f;
    rc = evaluate_points(ctx, wedge, P, pts, precision, f);
    if (rc) return rc;
    if (f0) *f0 = f[0];
    if (gradient)
        for (int i = 0; i < P; ++i) gradient[i] = (f[(size_t)(1 + 2 * i)] - f[(size_t)(2 + 2 * i)]) / (2.0 * step[i]);
    return MWSEP_OK;
}

extern "C" int mwsep_ctx_hessian(mwsep_ctx* ctx, int wedge, const double* theta, const double* step, int precision,
                                 double* f0, double* gradient, double* hessian)
{
    int P = 0;
    int rc = check_inputs(ctx, wedge, theta, step, precision, P);
    if (rc) return mwsep_fail(rc);
    /* points: [0] centre, [1+2i] +h_i, [2+2i] -h_i, then for each i<j the
     * four corners (++, +-, -+, --) */
    const int n_pairs = P * (P - 1) / 2;
    const int n = 1 + 2 * P + 4 * n_pairs;
    std::vector<double> pts;
    try
    {
        pts.resize((size_t)n * P);
    }
    catch (const std::bad_alloc&)
    {
        return mwsep_fail(MWSEP_ERR_NOMEM);
    }
    for (int k = 0; k < n; ++k) memcpy(&pts[(size_t)k * P], theta, sizeof(double) * P);
    for (int i = 0; i < P; ++i)
    {
        pts[(size_t)(1 + 2 * i) * P + i] += step[i];
        pts[(size_t)(2 + 2 * i) * P + i] -= step[i];
    }
    int k = 1 + 2 * P;
    for (int i = 0; i < P; ++i)
        for (int j = i + 1; j < P; ++j)
        {
            const double si[4] = {+1, +1, -1, -1}, sj[4] = {+1, -1, +1, -1};
            for (int c = 0; c < 4; ++c, ++k)
            {
                pts[(size_t)k * P + i] += si[c] * step[i];
                pts[(size_t)k * P + j] += sj[c] * step[j];
            }
        }
    std::vector<double> f;
    rc = evaluate_points(ctx, wedge, P, pts, precision, f);
    if (rc) return rc;
    const double fc = f[0];
    if (f0) *f0 = fc;
    if (gradient)
        for (int i = 0; i < P; ++i) gradient[i] = (f[(size_t)(1 + 2 * i)] - f[(size_t)(2 + 2 * i)]) / (2.0 * step[i]);
    if (hessian)
    {
        for (int i = 0; i < P; ++i)
            hessian[(size_t)i * P + i] =
                ((f[(size_t)(1 + 2 * i)] - fc) + (f[(size_t)(2 + 2 * i)] - fc)) / (step[i] * step[i]);
        k = 1 + 2 * P;
        for (int i = 0; i < P; ++i)
            for (int j = i + 1; j < P; ++j, k += 4)
            {
                const double h = ((f[(size_t)k] - f[(size_t)k + 1]) - (f[(size_t)k + 2] - f[(size_t)k + 3])) /
                                 (4.0 * step[i] * step[j]);
                hessian[(size_t)i * P + j] = h;
                hessian[(size_t)j * P + i] = h;
            }
    }
    return MWSEP_OK;
}

extern "C" int mwsep_write_errors(const char* path, int n, const double* hessian, const double* sigma,
                                  const double* stddev)
{
    if (!path || n < 1 || !hessian || !sigma || !stddev) return mwsep_fail(MWSEP_ERR_ARG);
    FILE* f = fopen(path, "w");
    if (!f) return mwsep_fail(MWSEP_ERR_IO);
    /* cpu/errors.c:49-82 with util/matrix.c:75-85 */
    fprintf(f, "hessian [%d x %d]:\n", n, n);
    for (int i = 0; i < n; ++i)
    {
        for (int j = 0; j < n; ++j) fprintf(f, " %.20lf", hessian[(size_t)i * n + j]);
        fprintf(f, "\n");
    }
    fprintf(f, "\n");
    fprintf(f, "SIGMA:\n");
    for (int i = 0; i < n; ++i)
    {
        for (int j = 0; j < n; ++j) fprintf(f, " %lf", sigma[(size_t)i * n + j]);
        fprintf(f, "\n");
    }
    fprintf(f, "\nErrors: q, r0, epsilon, mu, r, theta, phi, sigma\n");
    for (int i = 0; i < n; ++i) fprintf(f, " %lf", stddev[i]);
    fprintf(f, "\n");
    if (fclose(f) != 0) return mwsep_fail(MWSEP_ERR_IO);
    return MWSEP_OK;
}
