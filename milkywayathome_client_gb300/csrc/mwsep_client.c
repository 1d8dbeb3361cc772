/* mwsep_client.c -- command-line separation client on libmwsep_gb300.
 *
 * The flow of worker() in the reference (src/milkyway_client_app.c:197-288)
 * with the GPU evaluator registered in the EvalFunc slot:
 *
 *   read_astronomy_parameters, read_star_points, initialize_state,
 *   parameter-count check, set_astronomy_parameters,
 *   evaluate(parameters, &ap, &es, &sp) - 3.0
 *
 * and the reference's result lines on stderr.  Without BOINC or popt: flags
 * are parsed by hand.
 *
 *   mwsep_client -a astronomy_parameters.txt -p stars.txt [--mixed | --df] [-k N] theta...
 *     --mixed   compensated-FP32 evaluator (default: plain FP64)
 *     --df      double-float evaluator (the plain form's bounds on the FP32 pipes)
 *     -k N      evaluate N times (timing; prints seconds per evaluation)
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "milkyway_separation_gb300.h"

static double now_s(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* The library's binary files start with an 8-byte magic; anything else is
 * read as the reference's text format. */
static int has_magic(const char* path, const char* magic)
{
    char buf[8];
    FILE* f = fopen(path, "rb");
    size_t got;
    if (!f) return 0;
    got = fread(buf, 1, 8, f);
    fclose(f);
    return got == 8 && memcmp(buf, magic, 8) == 0;
}

int main(int argc, char** argv)
{
    const char* pfile = NULL;
    const char* sfile = NULL;
    int mixed = 0, repeats = 1, n = 0, i, rc;
    double* params = (double*)calloc((size_t)argc, sizeof(double));
    ASTRONOMY_PARAMETERS ap;
    STAR_POINTS sp;
    EVALUATION_STATE es;
    EvalFunc evaluate;
    double likelihood = 0.0, t0, t1;

    for (i = 1; i < argc; ++i)
    {
        if (!strcmp(argv[i], "-a") && i + 1 < argc) pfile = argv[++i];
        else if (!strcmp(argv[i], "-p") && i + 1 < argc) sfile = argv[++i];
        else if (!strcmp(argv[i], "-k") && i + 1 < argc) repeats = atoi(argv[++i]);
        else if (!strcmp(argv[i], "--mixed")) mixed = 1;
        else if (!strcmp(argv[i], "--df")) mixed = 2;
        else params[n++] = strtod(argv[i], NULL);
    }
    if (!pfile || !sfile)
    {
        fprintf(stderr, "usage: %s -a params -p stars [--mixed | --df] [-k N] theta...\n", argv[0]);
        return 2;
    }
    memset(&ap, 0, sizeof(ap));
    memset(&sp, 0, sizeof(sp));
    rc = has_magic(pfile, "MWSEPPAR") ? mwsep_read_astronomy_parameters_binary(pfile, &ap)
                                      : mwsep_read_astronomy_parameters(pfile, &ap);
    if (rc)
    {
        fprintf(stderr, "APP: error reading astronomy parameters from file %s: %s\n", pfile,
                mwsep_status_string(rc));
        return 1;
    }
    rc = has_magic(sfile, "MWSEPCAT") ? mwsep_read_star_points_binary(sfile, &sp) : mwsep_read_star_points(sfile, &sp);
    if (rc)
    {
        fprintf(stderr, "APP: error reading star points from file %s: %s\n", sfile, mwsep_status_string(rc));
        return 1;
    }
    if (mwsep_initialize_state(&ap, &sp, &es))
        return 1;
    if (n < 1 || n != mwsep_get_optimized_parameter_count(&ap))
    {
        fprintf(stderr,
                "Error reading parameters: number of parameters from the command line (%d) does not match "
                "the number of parameters to be optimized in %s (%d)\n",
                n, pfile, mwsep_get_optimized_parameter_count(&ap));
        return 1;
    }
    mwsep_set_astronomy_parameters(&ap, params);

    evaluate = mixed == 1 ? mwsep_evaluate_mixed : mixed == 2 ? mwsep_evaluate_df : mwsep_evaluate;
    if (repeats < 1)
        repeats = 1;
    t0 = now_s();
    for (i = 0; i < repeats; ++i)
        likelihood = evaluate(params, &ap, &es, &sp) - 3.0;
    t1 = now_s();
    if (likelihood != likelihood)
    {
        fprintf(stderr, "APP: evaluation failed: %s\n", mwsep_status_string(mwsep_last_error()));
        return 1;
    }

    fprintf(stderr, "<background_integral> %.20lf </background_integral>\n", es.background_integral);
    fprintf(stderr, "<stream_integrals>");
    for (i = 0; i < ap.number_streams; ++i)
        fprintf(stderr, " %.20lf", es.stream_integrals[i]);
    fprintf(stderr, " </stream_integrals>\n");
    fprintf(stderr, "<search_likelihood> %0.20f </search_likelihood>\n", likelihood);
    fprintf(stderr, "<search_application> %s %s </search_application>\n", mwsep_version(),
            mixed == 1 ? "mixed" : mixed == 2 ? "double-float" : "double");
    if (repeats > 1)
        fprintf(stderr, "<seconds_per_evaluation> %.6f </seconds_per_evaluation>\n", (t1 - t0) / repeats);

    free(params);
    mwsep_free_state(&es);
    mwsep_free_star_points(&sp);
    mwsep_free_parameters(&ap);
    return 0;
}
