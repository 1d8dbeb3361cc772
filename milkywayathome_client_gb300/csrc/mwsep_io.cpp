/* mwsep_io.cpp -- the reference's problem files and structs, host side.
 *
 * Same text formats and semantics as the reference (cpu/parameters.c,
 * cpu/star_points.c, cpu/evaluation_state.c, util/io_util.c), so the
 * reference's own input files load unchanged and the structs can be handed
 * to reference code.  Differences: errors are returned as MWSEP_ERR_* codes
 * instead of exit(-1), and split_astronomy_parameters does not print.
 */
#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "milkyway_separation_gb300.h"
#include "mwsep_params.h"
#include "mwsep_status.h"

namespace {

/* Non-blank lines of a file with surrounding blanks removed. */
struct Lines
{
    std::vector<std::string> v;
    size_t pos = 0;

    bool load(const char* path)
    {
        FILE* f = fopen(path, "r");
        if (!f) return false;
        std::string cur;
        int ch;
        while ((ch = fgetc(f)) != EOF)
        {
            if (ch == '\n' || ch == '\r')
            {
                push(cur);
                cur.clear();
            }
            else
                cur.push_back((char)ch);
        }
        push(cur);
        fclose(f);
        return true;
    }
    void push(const std::string& s)
    {
        size_t a = 0, b = s.size();
        while (a < b && isspace((unsigned char)s[a])) ++a;
        while (b > a && isspace((unsigned char)s[b - 1])) --b;
        if (b > a) v.push_back(s.substr(a, b - a));
    }
    /* Text after the first ':' when the current line starts with key. */
    const char* take(const char* key)
    {
        if (pos >= v.size()) return nullptr;
        const std::string& s = v[pos];
        if (s.compare(0, strlen(key), key) != 0) return nullptr;
        const size_t colon = s.find(':');
        if (colon == std::string::npos) return nullptr;
        ++pos;
        return s.c_str() + colon + 1;
    }
    /* "key[N]: a, b, c" with exactly N values. */
    bool take_array(const char* key, std::vector<double>& out)
    {
        if (pos >= v.size()) return false;
        const std::string& s = v[pos];
        const size_t klen = strlen(key);
        if (s.compare(0, klen, key) != 0 || s.size() <= klen || s[klen] != '[') return false;
        const long declared = strtol(s.c_str() + klen + 1, nullptr, 10);
        const char* rest = take(key);
        if (!rest || declared < 0 || declared > 4096) return false;
        out.clear();
        if (!numbers(rest, out)) return false;
        return (long)out.size() == declared;
    }
    static bool numbers(const char* p, std::vector<double>& out)
    {
        while (*p)
        {
            while (*p && (isspace((unsigned char)*p) || *p == ',')) ++p;
            if (!*p) break;
            char* end = nullptr;
            const double x = strtod(p, &end);
            if (end == p) return false;
            out.push_back(x);
            p = end;
        }
        return true;
    }
};

template <typename T>
T* dup_array(const std::vector<double>& v)
{
    T* p = (T*)calloc(v.empty() ? 1 : v.size(), sizeof(T));
    if (!p) return nullptr;
    for (size_t i = 0; i < v.size(); ++i) p[i] = (T)v[i];
    return p;
}

bool parse_triplet(const char* s, double& a, double& b, int& n)
{
    std::vector<double> v;
    if (!s || !Lines::numbers(s, v) || v.size() != 3) return false;
    a = v[0];
    b = v[1];
    n = (int)v[2];
    return true;
}

/* parameters.c:185-189, 221-225 */
void finish_integral(INTEGRAL* in)
{
    in->r_step_size = (in->r_max - in->r_min) / (double)in->r_steps;
    in->mu_step_size = (in->mu_max - in->mu_min) / (double)in->mu_steps;
    in->nu_step_size = (in->nu_max - in->nu_min) / (double)in->nu_steps;
    in->min_calculation = 0;
    in->max_calculation = (long)in->r_steps * in->mu_steps * in->nu_steps;
}

void fwrite_doubles(FILE* f, const char* name, int n, const double* a)
{
    /* util/io_util.c fwrite_double_array */
    fprintf(f, "%s[%d]: ", name, n);
    for (int i = 0; i < n; ++i)
    {
        fprintf(f, "%.20lf", a[i]);
        if (i < n - 1) fprintf(f, ", ");
    }
    fprintf(f, "\n");
}

void fwrite_ints(FILE* f, const char* name, int n, const int* a)
{
    /* util/io_util.c fwrite_int_array */
    fprintf(f, "%s[%d]: ", name, n);
    for (int i = 0; i < n; ++i)
    {
        if (i == 0) fprintf(f, " %d", a[i]);
        else fprintf(f, ", %d", a[i]);
    }
    fprintf(f, "\n");
}

} // namespace

extern "C" void mwsep_free_parameters(ASTRONOMY_PARAMETERS* ap)
{
    if (!ap) return;
    free(ap->background_parameters);
    free(ap->background_step);
    free(ap->background_min);
    free(ap->background_max);
    free(ap->background_optimize);
    free(ap->stream_weights);
    free(ap->stream_weight_step);
    free(ap->stream_weight_min);
    free(ap->stream_weight_max);
    free(ap->stream_weight_optimize);
    for (int i = 0; i < ap->number_streams; ++i)
    {
        if (ap->stream_parameters) free(ap->stream_parameters[i]);
        if (ap->stream_step) free(ap->stream_step[i]);
        if (ap->stream_min) free(ap->stream_min[i]);
        if (ap->stream_max) free(ap->stream_max[i]);
        if (ap->stream_optimize) free(ap->stream_optimize[i]);
    }
    free(ap->stream_parameters);
    free(ap->stream_step);
    free(ap->stream_min);
    free(ap->stream_max);
    free(ap->stream_optimize);
    for (int i = 0; i < ap->number_integrals; ++i)
        if (ap->integral) free(ap->integral[i]);
    free(ap->integral);
    memset(ap, 0, sizeof(*ap));
}

/* cpu/parameters.c:61-91 and :107-228 */
extern "C" int mwsep_read_astronomy_parameters(const char* path, ASTRONOMY_PARAMETERS* ap)
{
    if (!path || !ap) return mwsep_fail(MWSEP_ERR_ARG);
    memset(ap, 0, sizeof(*ap));
    Lines L;
    if (!L.load(path)) return mwsep_fail(MWSEP_ERR_IO);

    std::vector<double> v;
    const char* s;
    int rc = MWSEP_ERR_IO;
    size_t n_bg_values = 0;

    s = L.take("parameters_version");
    ap->parameters_version = s ? strtod(s, nullptr) : 0.01;

    if (!(s = L.take("number_parameters"))) goto fail;
    ap->number_background_parameters = atoi(s);
    if (!(s = L.take("background_weight"))) goto fail;
    ap->background_weight = strtod(s, nullptr);

    /* Each array is as long as its own bracket says (util/io_util.c:55-71);
     * number_parameters counts the leading values the search maps.  One of
     * the reference's test files (astronomy_parameters-79-aux.txt) lists
     * seven background values, the aux profile's three among them, under
     * number_parameters 4. */
    if (ap->number_background_parameters < 0) goto fail;
    if (!L.take_array("background_parameters", v)) goto fail;
    if (v.size() < (size_t)ap->number_background_parameters) goto fail;
    n_bg_values = v.size();
    ap->background_parameters = dup_array<double>(v);
    if (!L.take_array("background_step", v) || v.size() < (size_t)ap->number_background_parameters) goto fail;
    ap->background_step = dup_array<double>(v);
    if (!L.take_array("background_min", v) || v.size() < (size_t)ap->number_background_parameters) goto fail;
    ap->background_min = dup_array<double>(v);
    if (!L.take_array("background_max", v) || v.size() < (size_t)ap->number_background_parameters) goto fail;
    ap->background_max = dup_array<double>(v);
    if (!L.take_array("optimize_parameter", v) || v.size() < (size_t)ap->number_background_parameters) goto fail;
    ap->background_optimize = dup_array<int>(v);

    {
        if (!(s = L.take("number_streams"))) goto fail;
        std::vector<double> ns;
        if (!Lines::numbers(s, ns) || ns.size() != 2) goto fail;
        const int S = (int)ns[0];
        const int P = (int)ns[1];
        if (S < 0 || S > 1024 || P < 0 || P > 1024) goto fail;
        ap->number_stream_parameters = P;
        ap->stream_weights = (double*)calloc(S ? S : 1, sizeof(double));
        ap->stream_weight_step = (double*)calloc(S ? S : 1, sizeof(double));
        ap->stream_weight_min = (double*)calloc(S ? S : 1, sizeof(double));
        ap->stream_weight_max = (double*)calloc(S ? S : 1, sizeof(double));
        ap->stream_weight_optimize = (int*)calloc(S ? S : 1, sizeof(int));
        ap->stream_parameters = (double**)calloc(S ? S : 1, sizeof(double*));
        ap->stream_step = (double**)calloc(S ? S : 1, sizeof(double*));
        ap->stream_min = (double**)calloc(S ? S : 1, sizeof(double*));
        ap->stream_max = (double**)calloc(S ? S : 1, sizeof(double*));
        ap->stream_optimize = (int**)calloc(S ? S : 1, sizeof(int*));
        ap->number_streams = S; /* set after the arrays so free() is safe */
        for (int i = 0; i < S; ++i)
        {
            /* matched with its colon: "stream_weight" prefixes the _step keys */
            if (!(s = L.take("stream_weight:"))) goto fail;
            ap->stream_weights[i] = strtod(s, nullptr);
            if (!(s = L.take("stream_weight_step"))) goto fail;
            ap->stream_weight_step[i] = strtod(s, nullptr);
            if (!(s = L.take("stream_weight_min"))) goto fail;
            ap->stream_weight_min[i] = strtod(s, nullptr);
            if (!(s = L.take("stream_weight_max"))) goto fail;
            ap->stream_weight_max[i] = strtod(s, nullptr);
            if (!(s = L.take("optimize_weight"))) goto fail;
            ap->stream_weight_optimize[i] = atoi(s);
            if (!L.take_array("stream_parameters", v) || (int)v.size() != P) goto fail;
            ap->stream_parameters[i] = dup_array<double>(v);
            if (!L.take_array("stream_step", v)) goto fail;
            ap->stream_step[i] = dup_array<double>(v);
            if (!L.take_array("stream_min", v)) goto fail;
            ap->stream_min[i] = dup_array<double>(v);
            if (!L.take_array("stream_max", v)) goto fail;
            ap->stream_max[i] = dup_array<double>(v);
            if (!L.take_array("optimize_parameter", v) || (int)v.size() != P) goto fail;
            ap->stream_optimize[i] = dup_array<int>(v);
        }
    }

    if (!(s = L.take("convolve"))) goto fail;
    ap->convolve = atoi(s);
    if (!(s = L.take("sgr_coordinates"))) goto fail;
    ap->sgr_coordinates = atoi(s);
    if (ap->parameters_version > 0.01) /* parameters.c:158-161 */
    {
        if (!(s = L.take("aux_bg_profile"))) goto fail;
        ap->aux_bg_profile = atoi(s);
    }
    /* the aux profile reads background values 4..6 (init_constants,
     * cpu/evaluation_optimized.c:72-77) */
    if (ap->aux_bg_profile == 1 && n_bg_values < 7) goto fail;
    if (!(s = L.take("wedge"))) goto fail;
    ap->wedge = atoi(s);

    {
        ap->integral = (INTEGRAL**)calloc(1, sizeof(INTEGRAL*));
        ap->integral[0] = (INTEGRAL*)calloc(1, sizeof(INTEGRAL));
        ap->number_integrals = 1;
        INTEGRAL* in = ap->integral[0];
        if (!parse_triplet(L.take("r["), in->r_min, in->r_max, in->r_steps)) goto fail;
        if (!parse_triplet(L.take("mu["), in->mu_min, in->mu_max, in->mu_steps)) goto fail;
        if (!parse_triplet(L.take("nu["), in->nu_min, in->nu_max, in->nu_steps)) goto fail;
        finish_integral(in);
        if (!(s = L.take("number_cuts"))) goto fail;
        const int cuts = atoi(s);
        if (cuts < 0 || cuts > 1024) goto fail;
        INTEGRAL** grown = (INTEGRAL**)realloc(ap->integral, sizeof(INTEGRAL*) * (size_t)(cuts + 1));
        if (!grown) goto fail;
        ap->integral = grown;
        for (int i = 1; i <= cuts; ++i)
        {
            ap->integral[i] = (INTEGRAL*)calloc(1, sizeof(INTEGRAL));
            ap->number_integrals = i + 1;
            INTEGRAL* c = ap->integral[i];
            if (!parse_triplet(L.take("r_cut["), c->r_min, c->r_max, c->r_steps)) goto fail;
            if (!parse_triplet(L.take("mu_cut["), c->mu_min, c->mu_max, c->mu_steps)) goto fail;
            if (!parse_triplet(L.take("nu_cut["), c->nu_min, c->nu_max, c->nu_steps)) goto fail;
            finish_integral(c);
        }
    }
    return MWSEP_OK;

fail:
    mwsep_free_parameters(ap);
    return mwsep_fail(rc);
}

/* cpu/parameters.c:230-305 */
extern "C" int mwsep_write_astronomy_parameters(const char* path, const ASTRONOMY_PARAMETERS* ap)
{
    if (!path || !ap) return mwsep_fail(MWSEP_ERR_ARG);
    FILE* f = fopen(path, "w");
    if (!f) return mwsep_fail(MWSEP_ERR_IO);
    fprintf(f, "parameters_version: %lf\n", ap->parameters_version);
    fprintf(f, "number_parameters: %d\n", ap->number_background_parameters);
    fprintf(f, "background_weight: %lf\n", ap->background_weight);
    /* the aux profile's values 4..6 are written even where
     * number_parameters counts fewer (the reader's file form) */
    fwrite_doubles(f, "background_parameters", mwsep_background_values(ap), ap->background_parameters);
    fwrite_doubles(f, "background_step", ap->number_background_parameters, ap->background_step);
    fwrite_doubles(f, "background_min", ap->number_background_parameters, ap->background_min);
    fwrite_doubles(f, "background_max", ap->number_background_parameters, ap->background_max);
    fwrite_ints(f, "optimize_parameter", ap->number_background_parameters, ap->background_optimize);
    fprintf(f, "number_streams: %d, %d\n", ap->number_streams, ap->number_stream_parameters);
    for (int i = 0; i < ap->number_streams; ++i)
    {
        fprintf(f, "stream_weight: %lf\n", ap->stream_weights[i]);
        fprintf(f, "stream_weight_step: %lf\n", ap->stream_weight_step[i]);
        fprintf(f, "stream_weight_min: %lf\n", ap->stream_weight_min[i]);
        fprintf(f, "stream_weight_max: %lf\n", ap->stream_weight_max[i]);
        fprintf(f, "optimize_weight: %d\n", ap->stream_weight_optimize[i]);
        fwrite_doubles(f, "stream_parameters", ap->number_stream_parameters, ap->stream_parameters[i]);
        fwrite_doubles(f, "stream_step", ap->number_stream_parameters, ap->stream_step[i]);
        fwrite_doubles(f, "stream_min", ap->number_stream_parameters, ap->stream_min[i]);
        fwrite_doubles(f, "stream_max", ap->number_stream_parameters, ap->stream_max[i]);
        fwrite_ints(f, "optimize_parameter", ap->number_stream_parameters, ap->stream_optimize[i]);
    }
    fprintf(f, "convolve: %d\n", ap->convolve);
    fprintf(f, "sgr_coordinates: %d\n", ap->sgr_coordinates);
    fprintf(f, "aux_bg_profile: %d\n", ap->aux_bg_profile);
    fprintf(f, "wedge: %d\n", ap->wedge);
    const INTEGRAL* in = ap->integral[0];
    fprintf(f, "r[min,max,steps]: %lf, %lf, %d\n", in->r_min, in->r_max, in->r_steps);
    fprintf(f, "mu[min,max,steps]: %lf, %lf, %d\n", in->mu_min, in->mu_max, in->mu_steps);
    fprintf(f, "nu[min,max,steps]: %lf, %lf, %d\n", in->nu_min, in->nu_max, in->nu_steps);
    fprintf(f, "number_cuts: %d\n", ap->number_integrals - 1);
    for (int i = 1; i < ap->number_integrals; ++i)
    {
        const INTEGRAL* c = ap->integral[i];
        fprintf(f, "r_cut[min,max,steps][3]: %lf, %lf, %d\n", c->r_min, c->r_max, c->r_steps);
        fprintf(f, "mu_cut[min,max,steps][3]: %lf, %lf, %d\n", c->mu_min, c->mu_max, c->mu_steps);
        fprintf(f, "nu_cut[min,max,steps][3]: %lf, %lf, %d\n", c->nu_min, c->nu_max, c->nu_steps);
    }
    if (fclose(f) != 0) return mwsep_fail(MWSEP_ERR_IO);
    return MWSEP_OK;
}

/* cpu/parameters.c:307-330 */
extern "C" int mwsep_get_optimized_parameter_count(const ASTRONOMY_PARAMETERS* ap)
{
    if (!ap) return -mwsep_fail(MWSEP_ERR_ARG);
    int n = 0;
    for (int i = 0; i < ap->number_background_parameters; ++i)
        if (ap->background_optimize[i]) ++n;
    for (int i = 0; i < ap->number_streams; ++i)
    {
        if (ap->stream_weight_optimize[i]) ++n;
        for (int j = 0; j < ap->number_stream_parameters; ++j)
            if (ap->stream_optimize[i][j]) ++n;
    }
    return n;
}

/* cpu/parameters.c:332-363 */
extern "C" int mwsep_set_astronomy_parameters(ASTRONOMY_PARAMETERS* ap, const double* p)
{
    if (!ap || !p) return mwsep_fail(MWSEP_ERR_ARG);
    int k = 0;
    for (int i = 0; i < ap->number_background_parameters; ++i)
        if (ap->background_optimize[i]) ap->background_parameters[i] = p[k++];
    for (int i = 0; i < ap->number_streams; ++i)
    {
        if (ap->stream_weight_optimize[i]) ap->stream_weights[i] = p[k++];
        for (int j = 0; j < ap->number_stream_parameters; ++j)
            if (ap->stream_optimize[i][j]) ap->stream_parameters[i][j] = p[k++];
    }
    return MWSEP_OK;
}

/* cpu/parameters.c:365-397 */
extern "C" int mwsep_get_search_parameters(const ASTRONOMY_PARAMETERS* ap, double* out)
{
    if (!ap || !out) return mwsep_fail(MWSEP_ERR_ARG);
    int k = 0;
    for (int i = 0; i < ap->number_background_parameters; ++i)
        if (ap->background_optimize[i]) out[k++] = ap->background_parameters[i];
    for (int i = 0; i < ap->number_streams; ++i)
    {
        if (ap->stream_weight_optimize[i]) out[k++] = ap->stream_weights[i];
        for (int j = 0; j < ap->number_stream_parameters; ++j)
            if (ap->stream_optimize[i][j]) out[k++] = ap->stream_parameters[i][j];
    }
    return MWSEP_OK;
}

namespace {

/* The optimised entries of one per-parameter array family, in theta order
 * (the walk of get_search_parameters). */
int gather_optimised(const ASTRONOMY_PARAMETERS* ap, const double* bg, const double* sw, double* const* st,
                     double* out)
{
    if (!ap || !out || !bg || !sw || !st) return mwsep_fail(MWSEP_ERR_ARG);
    int k = 0;
    for (int i = 0; i < ap->number_background_parameters; ++i)
        if (ap->background_optimize[i]) out[k++] = bg[i];
    for (int i = 0; i < ap->number_streams; ++i)
    {
        if (ap->stream_weight_optimize[i]) out[k++] = sw[i];
        for (int j = 0; j < ap->number_stream_parameters; ++j)
            if (ap->stream_optimize[i][j]) out[k++] = st[i][j];
    }
    return MWSEP_OK;
}

} // namespace

/* cpu/parameters.c:399-432 */
extern "C" int mwsep_get_step(const ASTRONOMY_PARAMETERS* ap, double* out)
{
    if (!ap) return mwsep_fail(MWSEP_ERR_ARG);
    return gather_optimised(ap, ap->background_step, ap->stream_weight_step, ap->stream_step, out);
}

/* cpu/parameters.c:434-466 */
extern "C" int mwsep_get_min_parameters(const ASTRONOMY_PARAMETERS* ap, double* out)
{
    if (!ap) return mwsep_fail(MWSEP_ERR_ARG);
    return gather_optimised(ap, ap->background_min, ap->stream_weight_min, ap->stream_min, out);
}

/* cpu/parameters.c:468-500 */
extern "C" int mwsep_get_max_parameters(const ASTRONOMY_PARAMETERS* ap, double* out)
{
    if (!ap) return mwsep_fail(MWSEP_ERR_ARG);
    return gather_optimised(ap, ap->background_max, ap->stream_weight_max, ap->stream_max, out);
}

/* cpu/parameters.c:502-522 */
extern "C" int mwsep_split_astronomy_parameters(ASTRONOMY_PARAMETERS* ap, int rank, int max_rank)
{
    if (!ap || max_rank <= 0 || rank < 0 || rank >= max_rank) return mwsep_fail(MWSEP_ERR_ARG);
    for (int i = 0; i < ap->number_integrals; ++i)
    {
        INTEGRAL* in = ap->integral[i];
        const long total = (long)in->r_steps * in->nu_steps * in->mu_steps;
        in->min_calculation = (long)(total * ((double)rank / (double)max_rank));
        in->max_calculation = (long)(total * ((double)(rank + 1) / (double)max_rank));
    }
    return MWSEP_OK;
}

/* cpu/star_points.c:26-52, 69-81 */
extern "C" int mwsep_read_star_points(const char* path, STAR_POINTS* sp)
{
    if (!path || !sp) return mwsep_fail(MWSEP_ERR_ARG);
    sp->number_stars = 0;
    sp->stars = nullptr;
    FILE* f = fopen(path, "r");
    if (!f) return mwsep_fail(MWSEP_ERR_IO);
    int n = 0;
    if (fscanf(f, "%d", &n) != 1 || n < 0)
    {
        fclose(f);
        return mwsep_fail(MWSEP_ERR_IO);
    }
    double** rows = (double**)calloc(n ? n : 1, sizeof(double*));
    if (!rows)
    {
        fclose(f);
        return mwsep_fail(MWSEP_ERR_NOMEM);
    }
    for (int i = 0; i < n; ++i)
    {
        rows[i] = (double*)malloc(3 * sizeof(double));
        if (!rows[i] || fscanf(f, "%lf %lf %lf", &rows[i][0], &rows[i][1], &rows[i][2]) != 3)
        {
            for (int j = 0; j <= i; ++j) free(rows[j]);
            free(rows);
            fclose(f);
            return mwsep_fail(MWSEP_ERR_IO);
        }
    }
    fclose(f);
    sp->number_stars = n;
    sp->stars = rows;
    return MWSEP_OK;
}

/* cpu/star_points.c:54-67, 83-93 */
extern "C" int mwsep_write_star_points(const char* path, const STAR_POINTS* sp)
{
    if (!path || !sp) return mwsep_fail(MWSEP_ERR_ARG);
    FILE* f = fopen(path, "w");
    if (!f) return mwsep_fail(MWSEP_ERR_IO);
    fprintf(f, "%d\n", sp->number_stars);
    for (int i = 0; i < sp->number_stars; ++i)
        fprintf(f, "%lf %lf %lf\n", sp->stars[i][0], sp->stars[i][1], sp->stars[i][2]);
    if (fclose(f) != 0) return mwsep_fail(MWSEP_ERR_IO);
    return MWSEP_OK;
}

/* The per-star lines of separation()'s output file
 * (cpu/separation.c:229): "<stream> <x> <y> <z>" in the stripe frame,
 * stream 0 for the background. */
extern "C" int mwsep_write_separation(const char* path, int n, const int* assignment, const double* xyz)
{
    if (!path || n < 0 || (n > 0 && (!assignment || !xyz))) return mwsep_fail(MWSEP_ERR_ARG);
    FILE* f = fopen(path, "w");
    if (!f) return mwsep_fail(MWSEP_ERR_IO);
    for (int i = 0; i < n; ++i)
        fprintf(f, "%d %lf %lf %lf\n", assignment[i], xyz[3 * (size_t)i], xyz[3 * (size_t)i + 1],
                xyz[3 * (size_t)i + 2]);
    if (fclose(f) != 0) return mwsep_fail(MWSEP_ERR_IO);
    return MWSEP_OK;
}

/* cpu/star_points.c:95-103 */
extern "C" void mwsep_free_star_points(STAR_POINTS* sp)
{
    if (!sp) return;
    for (int i = 0; i < sp->number_stars; ++i)
        if (sp->stars) free(sp->stars[i]);
    free(sp->stars);
    sp->stars = nullptr;
    sp->number_stars = 0;
}

/* cpu/star_points.c:105-131 */
extern "C" int mwsep_split_star_points(STAR_POINTS* sp, int rank, int max_rank)
{
    if (!sp) return mwsep_fail(MWSEP_ERR_ARG);
    if (rank == 0 && max_rank == 0) return MWSEP_OK;
    if (max_rank <= 0 || rank < 0 || rank >= max_rank) return mwsep_fail(MWSEP_ERR_ARG);
    const int first = (int)(((double)sp->number_stars) * (((double)rank) / ((double)max_rank)));
    const int last = (int)(((double)sp->number_stars) * (((double)rank + 1.0) / ((double)max_rank)));
    const int n = last - first;
    double** rows = (double**)calloc(n > 0 ? n : 1, sizeof(double*));
    if (!rows) return mwsep_fail(MWSEP_ERR_NOMEM);
    for (int i = 0; i < n; ++i)
    {
        rows[i] = (double*)malloc(3 * sizeof(double));
        if (!rows[i])
        {
            for (int j = 0; j < i; ++j) free(rows[j]);
            free(rows);
            return mwsep_fail(MWSEP_ERR_NOMEM);
        }
        memcpy(rows[i], sp->stars[first + i], 3 * sizeof(double));
    }
    mwsep_free_star_points(sp);
    sp->stars = rows;
    sp->number_stars = n;
    return MWSEP_OK;
}

/* cpu/evaluation_state.c:229-259 (initialize_integral_area) and :285-308
 * (initialize_state). */
extern "C" int mwsep_initialize_state(const ASTRONOMY_PARAMETERS* ap, const STAR_POINTS* sp,
                                      EVALUATION_STATE* es)
{
    if (!ap || !sp || !es) return mwsep_fail(MWSEP_ERR_ARG);
    memset(es, 0, sizeof(*es));
    es->stream_integrals = (double*)calloc(ap->number_streams ? ap->number_streams : 1, sizeof(double));
    es->number_streams = ap->number_streams;
    es->total_stars = sp->number_stars;
    es->number_integrals = ap->number_integrals;
    es->integral = (INTEGRAL_AREA**)calloc(ap->number_integrals ? ap->number_integrals : 1,
                                           sizeof(INTEGRAL_AREA*));
    if (!es->stream_integrals || !es->integral) return mwsep_fail(MWSEP_ERR_NOMEM);
    for (int i = 0; i < ap->number_integrals; ++i)
    {
        INTEGRAL_AREA* ia = (INTEGRAL_AREA*)calloc(1, sizeof(INTEGRAL_AREA));
        if (!ia) return mwsep_fail(MWSEP_ERR_NOMEM);
        const INTEGRAL* in = ap->integral[i];
        ia->mu_min = in->mu_min;
        ia->mu_max = in->mu_max;
        ia->mu_steps = in->mu_steps;
        ia->nu_min = in->nu_min;
        ia->nu_max = in->nu_max;
        ia->nu_steps = in->nu_steps;
        ia->r_min = in->r_min;
        ia->r_max = in->r_max;
        ia->r_steps = in->r_steps;
        ia->min_calculation = in->min_calculation;
        ia->max_calculation = in->max_calculation;
        ia->current_calculation = in->min_calculation;
        ia->mu_step_size = (ia->mu_max - ia->mu_min) / ia->mu_steps;
        ia->nu_step_size = (ia->nu_max - ia->nu_min) / ia->nu_steps;
        ia->r_step_size = (ia->r_max - ia->r_min) / ia->r_steps;
        ia->number_streams = ap->number_streams;
        ia->stream_integrals = (double*)calloc(ap->number_streams ? ap->number_streams : 1, sizeof(double));
        if (!ia->stream_integrals) return mwsep_fail(MWSEP_ERR_NOMEM);
        es->integral[i] = ia;
    }
    return MWSEP_OK;
}

/* cpu/evaluation_state.c:333-343 (also frees the areas themselves). */
extern "C" void mwsep_free_state(EVALUATION_STATE* es)
{
    if (!es) return;
    free(es->stream_integrals);
    for (int i = 0; i < es->number_integrals; ++i)
    {
        if (es->integral && es->integral[i])
        {
            free(es->integral[i]->stream_integrals);
            free(es->integral[i]);
        }
    }
    free(es->integral);
    memset(es, 0, sizeof(*es));
}
