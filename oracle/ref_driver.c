/* Driver around the reference's own CPU separation evaluator, compiled from
 * the reference sources by oracle/Makefile into oracle/_ref/.  It stands in
 * for worker() in src/milkyway_client_app.c:197-288 without popt or BOINC:
 *
 *   read_astronomy_parameters / read_star_points   (app :214-215)
 *   optional split_astronomy_parameters / split_star_points (the reference's
 *     own rank slicing, cpu/parameters.c:502-522, cpu/star_points.c:105-131)
 *   initialize_state                                (app :242)
 *   get_optimized_parameter_count check             (app :244-259)
 *   set_astronomy_parameters + init_constants       (app :261-265)
 *   cpu_evaluate(...) - 3.0                         (app :278)
 *
 * Test infrastructure only: the checker, never the thing measured as the
 * product.  Output is one "key value" pair per line, values printed %.17g.
 *
 * Usage:  mw_ref -a params.txt -p stars.txt [-r rank -n nranks] [-k repeats]
 *                [-t] [-I i0,i1,...] theta0 theta1 ...
 *   -t : print wall seconds of the evaluation(s) (integral+likelihood)
 *   -k : evaluate k times (θ reapplied, constants re-initialised each time)
 *   -I : no integrals: the likelihood alone against the given background
 *        and stream integrals (1 + S values), as the distributed client's
 *        likelihood_f does with the composed integrals
 *        (cpu/astronomy_worker.c:94-121): set_astronomy_parameters,
 *        init_constants, then the reference's calculate_likelihood
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "milkyway.h"
#include "milkyway_priv.h"
#include "parameters.h"
#include "star_points.h"
#include "evaluation_state.h"
#include "evaluation_optimized.h"
#include "simple_evaluator.h"

static double now_seconds(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* One evaluation of the reference path on files.  Returns 0 on success.
 * area_out receives (1+S) doubles per integral area, in area order. */
/* The likelihood alone of a whole catalogue against given integrals
 * (likelihood_f, cpu/astronomy_worker.c:94-121, with the reference's own
 * calculate_likelihood).  Returns 0 on success. */
int mwref_likelihood_files(const char* param_path, const char* star_path, const double* theta, int n_theta,
                           const double* integrals, double* prob_sum, int* num_zero, double* likelihood)
{
    ASTRONOMY_PARAMETERS ap;
    STAR_POINTS sp;
    EVALUATION_STATE es;
    double* params;
    int i;

    memset(&ap, 0, sizeof(ap));
    memset(&sp, 0, sizeof(sp));
    memset(&es, 0, sizeof(es));
    if (read_astronomy_parameters(param_path, &ap))
        return 1;
    if (read_star_points(star_path, &sp))
        return 2;
    initialize_state(&ap, &sp, &es);
    if (n_theta < 1 || n_theta != get_optimized_parameter_count(&ap))
        return 3;
    params = (double*)malloc(sizeof(double) * (size_t)n_theta);
    memcpy(params, theta, sizeof(double) * (size_t)n_theta);
    set_astronomy_parameters(&ap, params);
    init_constants(&ap);
    es.background_integral = integrals[0];
    for (i = 0; i < ap.number_streams; ++i)
        es.stream_integrals[i] = integrals[1 + i];
    if (calculate_likelihood(&ap, &es, &sp))
        return 4;
    free_constants(&ap);
    *prob_sum = es.prob_sum;
    *num_zero = es.num_zero;
    /* likelihood_compose (:123-143) over one rank: prob_sum / N - 3 */
    *likelihood = es.prob_sum / (sp.number_stars - es.bad_jacobians) - 3.0;
    free(params);
    free_state(&es);
    free_star_points(&sp);
    free_parameters(&ap);
    return 0;
}

int mwref_evaluate_files(const char* param_path, const char* star_path,
                         const double* theta, int n_theta,
                         int rank, int nranks, int repeats,
                         double* bg_integral, double* stream_integrals,
                         double* area_out, double* prob_sum, int* num_zero,
                         double* likelihood, double* seconds)
{
    ASTRONOMY_PARAMETERS ap;
    STAR_POINTS sp;
    EVALUATION_STATE es;
    double* params;
    double t0, result = 0.0;
    int i, j, k;

    memset(&ap, 0, sizeof(ap));
    memset(&sp, 0, sizeof(sp));
    memset(&es, 0, sizeof(es));

    if (read_astronomy_parameters(param_path, &ap))
        return 1;
    if (read_star_points(star_path, &sp))
        return 2;
    if (nranks > 1)
    {
        split_astronomy_parameters(&ap, rank, nranks);
        split_star_points(&sp, rank, nranks);
    }
    initialize_state(&ap, &sp, &es);
    if (n_theta < 1 || n_theta != get_optimized_parameter_count(&ap))
    {
        fprintf(stderr, "mw_ref: %d parameters given, %d expected\n",
                n_theta, get_optimized_parameter_count(&ap));
        return 3;
    }
    params = (double*)malloc(sizeof(double) * (size_t)n_theta);
    memcpy(params, theta, sizeof(double) * (size_t)n_theta);
    if (repeats < 1)
        repeats = 1;

    init_simple_evaluator(cpu_evaluate);
    t0 = now_seconds();
    for (k = 0; k < repeats; ++k)
    {
        set_astronomy_parameters(&ap, params);
        init_constants(&ap); /* cpu_evaluate frees them on return */
        result = evaluate(params, &ap, &es, &sp);
    }
    if (seconds)
        *seconds = now_seconds() - t0;

    if (bg_integral)
        *bg_integral = es.background_integral;
    for (i = 0; i < ap.number_streams; ++i)
        if (stream_integrals)
            stream_integrals[i] = es.stream_integrals[i];
    if (area_out)
    {
        for (j = 0; j < ap.number_integrals; ++j)
        {
            area_out[j * (1 + ap.number_streams)] = es.integral[j]->background_integral;
            for (i = 0; i < ap.number_streams; ++i)
                area_out[j * (1 + ap.number_streams) + 1 + i] = es.integral[j]->stream_integrals[i];
        }
    }
    if (prob_sum)
        *prob_sum = es.prob_sum;
    if (num_zero)
        *num_zero = es.num_zero;
    if (likelihood)
        *likelihood = result - 3.0; /* src/milkyway_client_app.c:278 */

    free(params);
    free_state(&es);
    free_star_points(&sp);
    free_parameters(&ap);
    return 0;
}

#ifndef MWREF_NO_MAIN
int main(int argc, char** argv)
{
    const char* pfile = NULL;
    const char* sfile = NULL;
    int rank = 0, nranks = 1, repeats = 1, timing = 0;
    double theta[256];
    int n_theta = 0;
    double bg = 0.0, st[64], areas[64 * 65], psum = 0.0, logl = 0.0, secs = 0.0;
    double given[65];
    int n_given = 0;
    int nz = 0, i, rc;
    ASTRONOMY_PARAMETERS probe;

    for (i = 1; i < argc; ++i)
    {
        if (!strcmp(argv[i], "-a") && i + 1 < argc) pfile = argv[++i];
        else if (!strcmp(argv[i], "-p") && i + 1 < argc) sfile = argv[++i];
        else if (!strcmp(argv[i], "-r") && i + 1 < argc) rank = atoi(argv[++i]);
        else if (!strcmp(argv[i], "-n") && i + 1 < argc) nranks = atoi(argv[++i]);
        else if (!strcmp(argv[i], "-k") && i + 1 < argc) repeats = atoi(argv[++i]);
        else if (!strcmp(argv[i], "-t")) timing = 1;
        else if (!strcmp(argv[i], "-I") && i + 1 < argc)
        {
            char* p = argv[++i];
            while (*p && n_given < 65)
            {
                char* end;
                given[n_given++] = strtod(p, &end);
                p = (*end == ',') ? end + 1 : end;
                if (end == p && *p) break;
            }
        }
        else if (n_theta < 256) theta[n_theta++] = strtod(argv[i], NULL);
    }
    if (!pfile || !sfile)
    {
        fprintf(stderr, "usage: mw_ref -a params -p stars [-r rank -n nranks] [-k reps] [-t] theta...\n");
        return 2;
    }
    memset(&probe, 0, sizeof(probe));
    if (read_astronomy_parameters(pfile, &probe))
        return 1;
    if (probe.number_streams > 64 || probe.number_integrals > 64)
        return 1;

    if (n_given)
    {
        if (n_given != 1 + probe.number_streams)
            return 2;
        rc = mwref_likelihood_files(pfile, sfile, theta, n_theta, given, &psum, &nz, &logl);
        if (rc)
            return rc;
        printf("prob_sum %.17g\nnum_zero %d\nsearch_likelihood %.17g\n", psum, nz, logl);
        free_parameters(&probe);
        return 0;
    }
    rc = mwref_evaluate_files(pfile, sfile, theta, n_theta, rank, nranks, repeats,
                              &bg, st, areas, &psum, &nz, &logl, &secs);
    if (rc)
        return rc;
    printf("background_integral %.17g\n", bg);
    for (i = 0; i < probe.number_streams; ++i)
        printf("stream_integral %d %.17g\n", i, st[i]);
    for (rc = 0; rc < probe.number_integrals; ++rc)
        for (i = 0; i <= probe.number_streams; ++i)
            printf("area_integral %d %d %.17g\n", rc, i, areas[rc * (1 + probe.number_streams) + i]);
    printf("prob_sum %.17g\n", psum);
    printf("num_zero %d\n", nz);
    printf("search_likelihood %.17g\n", logl);
    if (timing)
        printf("seconds %.6f\n", secs);
    free_parameters(&probe);
    return 0;
}
#endif
