/* sep_oracle.c -- CPU restatement of the reference separation likelihood.
 *
 * TEST INFRASTRUCTURE ONLY (see sep_oracle.h).  Never part of the product.
 *
 * Every function cites the reference file:line it restates.  Arithmetic is
 * written in the reference's association order; compiled with
 * -ffp-contract=off it reproduces the reference's IEEE doubles, which the
 * tests check against the reference compiled from its own sources.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <ctype.h>

#include "sep_oracle.h"

#define SO_MAX_STREAMS 16
#define SO_MAX_SPARAMS 8
#define SO_MAX_BG 16
#define SO_MAX_AREAS 16

/* include/milkyway.h:46-57 -- pi is M_PI on glibc; deg = 180/pi */
#define SO_PI 3.1415926535897932384626433832795028841971693993751
#define SO_DEG (180.0 / SO_PI)
#define SO_DPI SO_PI
#define SO_D2PI 6.2831853071795864769252867665590057683943387987502
#define SO_GL_EPS 3.0e-11

/* evaluation_optimized.c:41-46 */
#define SO_STDEV 0.6
#define SO_LBR_R 8.5
#define SO_ABSM 4.2
static const double so_sigmoid[3] = {0.9402, 1.6171, 23.5877};

typedef struct
{
    double r_min, r_max, r_step;
    double mu_min, mu_max, mu_step;
    double nu_min, nu_max, nu_step;
    int r_steps, mu_steps, nu_steps;
} so_area;

struct so_problem
{
    double version;
    int n_bg;
    double bg_weight;
    double bg[SO_MAX_BG];
    int bg_opt[SO_MAX_BG];
    int n_streams, n_sparams;
    double st_weight[SO_MAX_STREAMS];
    int st_weight_opt[SO_MAX_STREAMS];
    double st[SO_MAX_STREAMS][SO_MAX_SPARAMS];
    int st_opt[SO_MAX_STREAMS][SO_MAX_SPARAMS];
    int convolve, sgr, aux, wedge;
    int n_areas;
    so_area area[SO_MAX_AREAS];
    int n_stars;
    double* stars; /* [n_stars][3] l, b, r_kpc */
};

/* Parameter-dependent constants: init_constants, evaluation_optimized.c:54-133 */
typedef struct
{
    double alpha, q, r0, delta, bg_a, bg_b, bg_c, coeff, alpha_delta3;
    double sigma[SO_MAX_STREAMS], sigma_sq2[SO_MAX_STREAMS];
    double a[SO_MAX_STREAMS][3], c[SO_MAX_STREAMS][3];
    double* gl_x;
    double* gl_w;
    double* dx;
    double* xyz; /* [convolve][3] scratch, as the reference's global xyz */
} so_consts;

/* ------------------------------------------------------------------ parse */

typedef struct
{
    char** lines;
    int n, pos;
} so_lines;

static void so_free_lines(so_lines* L)
{
    int i;
    for (i = 0; i < L->n; ++i)
        free(L->lines[i]);
    free(L->lines);
}

static int so_read_lines(const char* path, so_lines* L)
{
    FILE* f = fopen(path, "r");
    char buf[8192];
    int cap = 64;
    if (!f)
        return 1;
    L->lines = (char**)malloc(sizeof(char*) * (size_t)cap);
    L->n = 0;
    L->pos = 0;
    while (fgets(buf, sizeof buf, f))
    {
        char* s = buf;
        size_t len;
        while (*s && isspace((unsigned char)*s))
            ++s;
        len = strlen(s);
        while (len && isspace((unsigned char)s[len - 1]))
            s[--len] = '\0';
        if (!len)
            continue;
        if (L->n == cap)
        {
            cap *= 2;
            L->lines = (char**)realloc(L->lines, sizeof(char*) * (size_t)cap);
        }
        L->lines[L->n] = (char*)malloc(len + 1);
        memcpy(L->lines[L->n], s, len + 1);
        L->n++;
    }
    fclose(f);
    return 0;
}

/* Return the text after "<key>...:" on the current line and advance, or NULL
 * when the line does not start with key. */
static const char* so_take(so_lines* L, const char* key)
{
    const char* s;
    const char* colon;
    if (L->pos >= L->n)
        return NULL;
    s = L->lines[L->pos];
    if (strncmp(s, key, strlen(key)) != 0)
        return NULL;
    colon = strchr(s, ':');
    if (!colon)
        return NULL;
    L->pos++;
    return colon + 1;
}

/* Parse up to max numbers separated by commas / blanks. */
static int so_numbers(const char* s, double* out, int max)
{
    int n = 0;
    char* end;
    while (s && *s && n < max)
    {
        while (*s && (isspace((unsigned char)*s) || *s == ','))
            ++s;
        if (!*s)
            break;
        out[n] = strtod(s, &end);
        if (end == s)
            return -1;
        ++n;
        s = end;
    }
    return n;
}

/* "name[N]: v0, v1, ..."  (util/io_util.c fread_double_array) */
static int so_array(so_lines* L, const char* key, double* out, int max)
{
    const char* line;
    const char* br;
    int declared, got;
    if (L->pos >= L->n)
        return -1;
    line = L->lines[L->pos];
    if (strncmp(line, key, strlen(key)) != 0)
        return -1;
    br = line + strlen(key);
    if (*br != '[')
        return -1;
    declared = atoi(br + 1);
    if (declared < 0 || declared > max)
        return -1;
    {
        const char* rest = so_take(L, key);
        got = so_numbers(rest, out, max);
    }
    if (got != declared)
        return -1;
    return declared;
}

static int so_parse_params(const char* path, so_problem* p)
{
    so_lines L;
    const char* s;
    double v[64];
    int i, j, n, rc = 1;

    if (so_read_lines(path, &L))
        return 1;

    /* parameters.c:111-117: a missing version line means 0.01 */
    s = so_take(&L, "parameters_version");
    p->version = s ? strtod(s, NULL) : 0.01;

    if (!(s = so_take(&L, "number_parameters"))) goto out;
    p->n_bg = atoi(s);
    if (!(s = so_take(&L, "background_weight"))) goto out;
    p->bg_weight = strtod(s, NULL);

    n = so_array(&L, "background_parameters", v, SO_MAX_BG);
    if (n < 0) goto out;
    for (i = 0; i < n; ++i) p->bg[i] = v[i];
    if (so_array(&L, "background_step", v, SO_MAX_BG) < 0) goto out;
    if (so_array(&L, "background_min", v, SO_MAX_BG) < 0) goto out;
    if (so_array(&L, "background_max", v, SO_MAX_BG) < 0) goto out;
    n = so_array(&L, "optimize_parameter", v, SO_MAX_BG);
    if (n < 0) goto out;
    for (i = 0; i < n; ++i) p->bg_opt[i] = (int)v[i];

    if (!(s = so_take(&L, "number_streams"))) goto out;
    if (so_numbers(s, v, 2) != 2) goto out;
    p->n_streams = (int)v[0];
    p->n_sparams = (int)v[1];
    if (p->n_streams < 0 || p->n_streams > SO_MAX_STREAMS || p->n_sparams < 5 ||
        p->n_sparams > SO_MAX_SPARAMS)
        goto out;

    for (i = 0; i < p->n_streams; ++i)
    {
        /* matched with its colon: "stream_weight" prefixes the _step/_min/_max keys */
        if (!(s = so_take(&L, "stream_weight:")))
            goto out;
        p->st_weight[i] = strtod(s, NULL);
        if (!so_take(&L, "stream_weight_step")) goto out;
        if (!so_take(&L, "stream_weight_min")) goto out;
        if (!so_take(&L, "stream_weight_max")) goto out;
        if (!(s = so_take(&L, "optimize_weight"))) goto out;
        p->st_weight_opt[i] = atoi(s);
        n = so_array(&L, "stream_parameters", v, SO_MAX_SPARAMS);
        if (n < 0) goto out;
        for (j = 0; j < n; ++j) p->st[i][j] = v[j];
        if (so_array(&L, "stream_step", v, SO_MAX_SPARAMS) < 0) goto out;
        if (so_array(&L, "stream_min", v, SO_MAX_SPARAMS) < 0) goto out;
        if (so_array(&L, "stream_max", v, SO_MAX_SPARAMS) < 0) goto out;
        n = so_array(&L, "optimize_parameter", v, SO_MAX_SPARAMS);
        if (n < 0) goto out;
        for (j = 0; j < n; ++j) p->st_opt[i][j] = (int)v[j];
    }

    if (!(s = so_take(&L, "convolve"))) goto out;
    p->convolve = atoi(s);
    if (!(s = so_take(&L, "sgr_coordinates"))) goto out;
    p->sgr = atoi(s);
    p->aux = 0;
    if (p->version > 0.01) /* parameters.c:158-161 */
    {
        if (!(s = so_take(&L, "aux_bg_profile"))) goto out;
        p->aux = atoi(s);
    }
    if (!(s = so_take(&L, "wedge"))) goto out;
    p->wedge = atoi(s);

    {
        static const char* keys[3] = {"r[", "mu[", "nu["};
        static const char* cut_keys[3] = {"r_cut[", "mu_cut[", "nu_cut["};
        int a, k;
        for (k = 0; k < 3; ++k)
        {
            double t[3];
            if (!(s = so_take(&L, keys[k]))) goto out;
            if (so_numbers(s, t, 3) != 3) goto out;
            if (k == 0) { p->area[0].r_min = t[0]; p->area[0].r_max = t[1]; p->area[0].r_steps = (int)t[2]; }
            if (k == 1) { p->area[0].mu_min = t[0]; p->area[0].mu_max = t[1]; p->area[0].mu_steps = (int)t[2]; }
            if (k == 2) { p->area[0].nu_min = t[0]; p->area[0].nu_max = t[1]; p->area[0].nu_steps = (int)t[2]; }
        }
        if (!(s = so_take(&L, "number_cuts"))) goto out;
        p->n_areas = atoi(s) + 1;
        if (p->n_areas < 1 || p->n_areas > SO_MAX_AREAS) goto out;
        for (a = 1; a < p->n_areas; ++a)
        {
            for (k = 0; k < 3; ++k)
            {
                double t[3];
                const char* after;
                if (!(s = so_take(&L, cut_keys[k]))) goto out;
                /* the "[%d]" index sits before the colon; s is after it */
                after = s;
                if (so_numbers(after, t, 3) != 3) goto out;
                if (k == 0) { p->area[a].r_min = t[0]; p->area[a].r_max = t[1]; p->area[a].r_steps = (int)t[2]; }
                if (k == 1) { p->area[a].mu_min = t[0]; p->area[a].mu_max = t[1]; p->area[a].mu_steps = (int)t[2]; }
                if (k == 2) { p->area[a].nu_min = t[0]; p->area[a].nu_max = t[1]; p->area[a].nu_steps = (int)t[2]; }
            }
        }
        for (a = 0; a < p->n_areas; ++a)
        {
            so_area* A = &p->area[a];
            if (A->r_steps <= 0 || A->mu_steps <= 0 || A->nu_steps <= 0) goto out;
            /* evaluation_state.c:247-249 (step sizes of INTEGRAL_AREA) */
            A->mu_step = (A->mu_max - A->mu_min) / A->mu_steps;
            A->nu_step = (A->nu_max - A->nu_min) / A->nu_steps;
            A->r_step = (A->r_max - A->r_min) / A->r_steps;
        }
    }
    if (p->convolve <= 0) goto out;
    rc = 0;
out:
    so_free_lines(&L);
    return rc;
}

/* cpu/star_points.c:69-81 */
static int so_parse_stars(const char* path, so_problem* p)
{
    FILE* f = fopen(path, "r");
    int i, n;
    if (!f)
        return 1;
    if (fscanf(f, "%d", &n) != 1 || n < 0)
    {
        fclose(f);
        return 1;
    }
    p->stars = (double*)malloc(sizeof(double) * 3 * (size_t)(n ? n : 1));
    for (i = 0; i < n; ++i)
    {
        if (fscanf(f, "%lf %lf %lf", &p->stars[3 * i], &p->stars[3 * i + 1], &p->stars[3 * i + 2]) != 3)
        {
            fclose(f);
            return 1;
        }
    }
    p->n_stars = n;
    fclose(f);
    return 0;
}

so_problem* so_open(const char* param_path, const char* star_path)
{
    so_problem* p = (so_problem*)calloc(1, sizeof(so_problem));
    if (!p)
        return NULL;
    if (so_parse_params(param_path, p) || (star_path && so_parse_stars(star_path, p)))
    {
        so_close(p);
        return NULL;
    }
    return p;
}

void so_close(so_problem* p)
{
    if (!p)
        return;
    free(p->stars);
    free(p);
}

int so_n_theta(const so_problem* p)
{
    /* parameters.c:307-330 */
    int i, j, n = 0;
    for (i = 0; i < p->n_bg; ++i)
        n += p->bg_opt[i] ? 1 : 0;
    for (i = 0; i < p->n_streams; ++i)
    {
        n += p->st_weight_opt[i] ? 1 : 0;
        for (j = 0; j < p->n_sparams; ++j)
            n += p->st_opt[i][j] ? 1 : 0;
    }
    return n;
}
int so_n_streams(const so_problem* p) { return p->n_streams; }
int so_n_areas(const so_problem* p) { return p->n_areas; }
int so_n_stars(const so_problem* p) { return p->n_stars; }
int so_convolve(const so_problem* p) { return p->convolve; }
int so_area_dims(const so_problem* p, int a, int* out)
{
    if (a < 0 || a >= p->n_areas)
        return 1;
    out[0] = p->area[a].mu_steps;
    out[1] = p->area[a].nu_steps;
    out[2] = p->area[a].r_steps;
    return 0;
}

/* parameters.c:332-363: scatter theta into the optimised slots */
static void so_set_theta(so_problem* p, const double* theta)
{
    int i, j, k = 0;
    for (i = 0; i < p->n_bg; ++i)
        if (p->bg_opt[i])
            p->bg[i] = theta[k++];
    for (i = 0; i < p->n_streams; ++i)
    {
        if (p->st_weight_opt[i])
            p->st_weight[i] = theta[k++];
        for (j = 0; j < p->n_sparams; ++j)
            if (p->st_opt[i][j])
                p->st[i][j] = theta[k++];
    }
}

/* -------------------------------------------------------------- geometry */

/* atSurveyGeometry.c:87-102 */
static void so_bound(double* angle, double lo, double hi)
{
    while (*angle < lo)
        *angle += 360.0;
    while (*angle >= hi)
        *angle -= 360.0;
}

/* atSurveyGeometry.c:104-119 */
static void so_bound2(double* theta, double* phi)
{
    so_bound(theta, -180.0, 180.0);
    if (fabs(*theta) > 90.0)
    {
        *theta = 180.0 - *theta;
        *phi += 180;
    }
    so_bound(theta, -180.0, 180.0);
    so_bound(phi, 0.0, 360.0);
    if (fabs(*theta) == 90.0)
        *phi = 0.;
}

/* atSurveyGeometry.h:27-29 dmod / dsign */
static double so_dmod(double a, double b)
{
    if (b == 0.0)
        return a;
    return (a * b > 0.0) ? a - b * floor(a / b) : a + b * floor(-a / b);
}

/* atSurveyGeometry.c:26-64.  The reference's degree<->radian macros carry a
 * trailing expression "DPI/180.0", so x*deg2rad evaluates as (x*DPI)/180.0. */
static void so_gc_to_eq(double amu, double anu, double* ra, double* dec, double anode, double ainc)
{
    double x1, y1, z1, x2, y2, z2;
    amu = amu * SO_DPI / 180.0;
    anu = anu * SO_DPI / 180.0;
    anode = anode * SO_DPI / 180.0;
    ainc = ainc * SO_DPI / 180.0;
    x2 = cos(amu - anode) * cos(anu);
    y2 = sin(amu - anode) * cos(anu);
    z2 = sin(anu);
    x1 = x2;
    y1 = y2 * cos(ainc) - z2 * sin(ainc);
    z1 = y2 * sin(ainc) + z2 * cos(ainc);
    *ra = atan2(y1, x1) + anode;
    *dec = asin(z1);
    *ra = *ra * 180.0 / SO_DPI;
    *dec = *dec * 180.0 / SO_DPI;
    so_bound2(dec, ra);
}

/* atSurveyGeometry.c:212-240 (SLALIB slaEqgal: fixed FK4/galactic matrix,
 * spherical->Cartesian, rotate, Cartesian->spherical, range-normalise) */
static void so_eqgal(double dr, double dd, double* dl, double* db)
{
    static const double m[3][3] = {
        {-0.054875539726, -0.873437108010, -0.483834985808},
        {0.494109453312, -0.444829589425, 0.746982251810},
        {-0.867666135858, -0.198076386122, 0.455983795705}};
    double v1[3], v2[3], cosb, x, y, z, r, w;
    int i, j;

    cosb = cos(dd);
    v1[0] = cos(dr) * cosb;
    v1[1] = sin(dr) * cosb;
    v1[2] = sin(dd);
    for (j = 0; j < 3; ++j)
    {
        w = 0.0;
        for (i = 0; i < 3; ++i)
            w += m[j][i] * v1[i];
        v2[j] = w;
    }
    x = v2[0];
    y = v2[1];
    z = v2[2];
    r = sqrt(x * x + y * y);
    *dl = (r != 0.0) ? atan2(y, x) : 0.0;
    *db = (z != 0.0) ? atan2(z, r) : 0.0;
    /* slaDranrm */
    w = so_dmod(*dl, SO_D2PI);
    *dl = (w >= 0.0) ? w : w + SO_D2PI;
    /* slaDrange */
    w = so_dmod(*db, SO_D2PI);
    *db = (fabs(w) < SO_DPI) ? w : w - ((*db < 0.0) ? -SO_D2PI : SO_D2PI);
}

/* atSurveyGeometry.c:66-83 */
static void so_eq_to_gal(double ra, double dec, double* glong, double* glat)
{
    ra = ra * SO_DPI / 180.0;
    dec = dec * SO_DPI / 180.0;
    so_eqgal(ra, dec, glong, glat);
    *glong = *glong * 180.0 / SO_DPI;
    *glat = *glat * 180.0 / SO_DPI;
    so_bound2(glat, glong);
}

/* stCoords.c:108-130 (stripe separation 2.5 deg, survey centre RA 185,
 * Dec 32.5; node = RA centre - 90) */
static double so_wedge_incl(int wedge)
{
    double d = 2.5;
    double eta = wedge * d - 57.5 - (wedge > 46 ? 180.0 : 0.0);
    return eta + 32.5;
}
static double so_node(void) { return 185.0 - 90.0; }

/* atSurveyGeometry.c:247-272 */
static void so_gc_to_sgr(double mu, double nu, int wedge, double* lamda, double* beta)
{
    double radpdeg = 3.141592653589793 / 180;
    double x, y, z;
    mu = mu * radpdeg;
    nu = nu * radpdeg;
    x = cos(mu) * cos(nu);
    y = -sin(nu);
    z = sin(mu) * cos(nu);
    *lamda = atan2(y, x);
    *lamda = *lamda / radpdeg;
    *lamda = *lamda + 2.5 * wedge;
    if (*lamda < 0)
        *lamda = *lamda + 360;
    *beta = asin(z);
    *beta = *beta / radpdeg;
}

/* atSurveyGeometry.c:276-412.  The reference writes each entry of the
 * Sgr->Galactic rotation as a ratio whose denominator is identically 1
 * (sums of cos^2+sin^2 products); this restatement uses the simplified
 * Euler-angle entries, which agree to a few ulp. */
/* The Sgr -> Galactic rotation of atSurveyGeometry.c:278-290: Euler angles
 * phi = 183.75, theta = 76.54, psi = 194.111534 degrees, each entry written
 * as a ratio of sums of squared sines and cosines (identically one in exact
 * arithmetic, not in doubles).  The terms are formed and summed in the
 * reference's order so the entries carry its rounding. */
static void so_sgr_rotation(double* r)
{
    const double radpdeg = 3.141592653589793 / 180;
    const double phi = (180 + 3.75) * radpdeg;
    const double theta = (90 - 13.46) * radpdeg;
    const double psi = (180 + 14.111534) * radpdeg;
    const double ct = cos(theta), st = sin(theta), cf = cos(phi), sf = sin(phi), cp = cos(psi), sp = sin(psi);
    const double ct2 = pow(ct, 2), st2 = pow(st, 2), cf2 = pow(cf, 2), sf2 = pow(sf, 2), cp2 = pow(cp, 2),
                 sp2 = pow(sp, 2);
    /* the shared denominators of the 2x2 block, of r13/r23, of r31/r32 */
    double d4 = cp2 * cf2 * ct2;
    d4 += cp2 * cf2 * st2;
    d4 += ct2 * sp2 * sf2;
    d4 += sp2 * cf2 * ct2;
    d4 += sp2 * cf2 * st2;
    d4 += ct2 * cp2 * sf2;
    d4 += st2 * sf2 * cp2;
    d4 += st2 * sf2 * sp2;
    const double d3a = ct2 * sf2 + cf2 * ct2 + cf2 * st2 + st2 * sf2;
    const double d3b = cp2 * ct2 + sp2 * st2 + cp2 * st2 + sp2 * ct2;
    r[0] = -(ct * sf * sp - ct2 * cf * cp - cp * st2 * cf) / d4;
    r[1] = -(ct * sf * cp + ct2 * cf * sp + sp * st2 * cf) / d4;
    r[2] = (st * sf) / d3a;
    r[3] = (ct * cf * sp + ct2 * cp * sf + cp * st2 * sf) / d4;
    r[4] = -(-ct * cf * cp + ct2 * sp * sf + sp * st2 * sf) / d4;
    r[5] = -(st * cf) / d3a;
    r[6] = (sp * st) / d3b;
    r[7] = (cp * st) / d3b;
    r[8] = ct / (ct2 + st2);
}

static void so_sgr_to_gal(double lamda, double beta, double* l, double* b)
{
    double radpdeg = 3.141592653589793 / 180;
    double rot[9];
    double x2 = 0.0, y2 = 0.0, z2, x1, y1, z1;
    double r11, r12, r13, r21, r22, r23, r31, r32, r33;
    so_sgr_rotation(rot);
    r11 = rot[0], r12 = rot[1], r13 = rot[2], r21 = rot[3], r22 = rot[4], r23 = rot[5], r31 = rot[6],
    r32 = rot[7], r33 = rot[8];

    if (beta > 90)
    {
        beta = 90 - (beta - 90);
        lamda = lamda + 180;
        if (lamda > 360)
            lamda = lamda - 360;
    }
    if (beta < -90)
    {
        beta = -90 - (beta + 90);
        lamda = lamda + 180;
        if (lamda > 360)
            lamda = lamda - 360;
    }
    if (lamda < 0)
        lamda = lamda + 360;
    beta = beta + 90;
    beta = beta * radpdeg;
    z2 = cos(beta);
    if (lamda == 0)
    {
        x2 = sin(beta);
        y2 = 0;
    }
    else if (lamda < 90)
    {
        lamda = lamda * radpdeg;
        x2 = sqrt((1 - cos(beta) * cos(beta)) / (1 + tan(lamda) * tan(lamda)));
        y2 = x2 * tan(lamda);
    }
    else if (lamda == 90)
    {
        x2 = 0;
        y2 = sin(beta);
    }
    else if (lamda < 180)
    {
        lamda = lamda * radpdeg;
        y2 = sqrt((1 - cos(beta) * cos(beta)) / (1 / (tan(lamda) * tan(lamda)) + 1));
        x2 = y2 / tan(lamda);
    }
    else if (lamda == 180)
    {
        x2 = -sin(beta);
        y2 = 0;
    }
    else if (lamda < 270)
    {
        lamda = lamda * radpdeg;
        x2 = sqrt((1 - cos(beta) * cos(beta)) / (1 + tan(lamda) * tan(lamda)));
        y2 = x2 * tan(lamda);
        x2 = -x2;
        y2 = -y2;
    }
    else if (lamda == 270)
    {
        x2 = 0;
        y2 = -sin(beta);
    }
    else if (lamda < 360)
    {
        lamda = lamda * radpdeg;
        x2 = sqrt((1 - cos(beta) * cos(beta)) / (1 + tan(lamda) * tan(lamda)));
        y2 = x2 * tan(lamda);
    }
    else if (lamda == 360)
    {
        x2 = sin(beta);
        y2 = 0;
    }
    x1 = r11 * x2 + r12 * y2 + r13 * z2;
    y1 = r21 * x2 + r22 * y2 + r23 * z2;
    z1 = r31 * x2 + r32 * y2 + r33 * z2;
    if (z1 > 1)
    {
        *l = 0;
        *b = 90;
    }
    else
    {
        *b = asin(z1);
        *b = *b / radpdeg;
        *l = atan2(y1, x1);
        *l = *l / radpdeg;
        if (*l < 0)
            *l = *l + 360;
    }
}

/* (mu, nu) of a wedge -> Galactic (l, b): evaluation_optimized.c:480-491 and
 * :96-105 (same pair of transforms for the stream centres). */
static void so_wedge_point_lb(const so_problem* p, double mu, double nu, double* l, double* b)
{
    if (p->sgr == 0)
    {
        double ra, dec;
        so_gc_to_eq(mu, nu, &ra, &dec, so_node(), so_wedge_incl(p->wedge));
        so_eq_to_gal(ra, dec, l, b);
    }
    else
    {
        double lamda, beta;
        so_gc_to_sgr(mu, nu, p->wedge, &lamda, &beta);
        so_sgr_to_gal(lamda, beta, l, b);
    }
}

void so_gc_to_lb(int wedge, double mu, double nu, double* l, double* b)
{
    double ra, dec;
    so_gc_to_eq(mu, nu, &ra, &dec, so_node(), so_wedge_incl(wedge));
    so_eq_to_gal(ra, dec, l, b);
}

/* stCoords.c:33-48: law-of-cosines form with the Sun at 8.5 kpc */
void so_lbr_to_xyz(double l, double b, double r, double* xyz)
{
    const double r0 = 8.5;
    double bsin = sin(b / SO_DEG), lsin = sin(l / SO_DEG);
    double bcos = cos(b / SO_DEG), lcos = cos(l / SO_DEG);
    double zp, d;
    xyz[2] = r * bsin;
    zp = r * bcos;
    d = sqrt(r0 * r0 + zp * zp - 2 * r0 * zp * lcos);
    xyz[0] = (zp * zp - r0 * r0 - d * d) / (2 * r0);
    xyz[1] = zp * lsin;
}

/* numericalIntegration.c:67-104 (Newton iteration on the Legendre
 * recurrence, Numerical Recipes gauleg) on [-1, 1] */
void so_gauss_legendre(int n, double* x, double* w)
{
    const double x1 = -1.0, x2 = 1.0;
    int m = (n + 1) / 2, i, j;
    double xm = 0.5 * (x2 + x1), xl = 0.5 * (x2 - x1);
    double z, z1, pp, p1, p2, p3;
    for (i = 1; i <= m; ++i)
    {
        z = cos(SO_PI * (i - 0.25) / (n + 0.5));
        do
        {
            p1 = 1.0;
            p2 = 0.0;
            for (j = 1; j <= n; ++j)
            {
                p3 = p2;
                p2 = p1;
                p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
            }
            pp = n * (z * p1 - p2) / (z * z - 1.0);
            z1 = z;
            z = z1 - p1 / pp;
        } while (fabs(z - z1) > SO_GL_EPS);
        x[i - 1] = xm - xl * z;
        x[n - i] = xm + xl * z;
        w[i - 1] = 2.0 * xl / ((1.0 - z * z) * pp * pp);
        w[n - i] = w[i - 1];
    }
}

/* ------------------------------------------------------------- constants */

/* evaluation_optimized.c:54-133 */
static void so_init_consts(const so_problem* p, so_consts* k)
{
    int i;
    k->alpha = p->bg[0];
    k->q = p->bg[1];
    k->r0 = p->bg[2];
    k->delta = p->bg[3];
    k->bg_a = k->bg_b = k->bg_c = 0.0;
    if (p->aux == 1)
    {
        k->bg_a = p->bg[4];
        k->bg_b = p->bg[5];
        k->bg_c = p->bg[6];
    }
    k->coeff = 1 / (SO_STDEV * sqrt(2 * SO_PI));
    k->alpha_delta3 = 3 - k->alpha + k->delta;
    for (i = 0; i < p->n_streams; ++i)
    {
        double l, b;
        k->sigma[i] = p->st[i][4];
        k->sigma_sq2[i] = 2.0 * k->sigma[i] * k->sigma[i];
        so_wedge_point_lb(p, p->st[i][0], 0, &l, &b);
        so_lbr_to_xyz(l, b, p->st[i][1], k->c[i]);
        k->a[i][0] = sin(p->st[i][2]) * cos(p->st[i][3]);
        k->a[i][1] = sin(p->st[i][2]) * sin(p->st[i][3]);
        k->a[i][2] = cos(p->st[i][2]);
    }
    k->gl_x = (double*)malloc(sizeof(double) * (size_t)p->convolve);
    k->gl_w = (double*)malloc(sizeof(double) * (size_t)p->convolve);
    k->dx = (double*)malloc(sizeof(double) * (size_t)p->convolve);
    k->xyz = (double*)calloc(3 * (size_t)p->convolve, sizeof(double));
    so_gauss_legendre(p->convolve, k->gl_x, k->gl_w);
    for (i = 0; i < p->convolve; ++i)
        k->dx[i] = 3 * SO_STDEV * k->gl_x[i];
}

static void so_free_consts(so_consts* k)
{
    free(k->gl_x);
    free(k->gl_w);
    free(k->dx);
    free(k->xyz);
}

/* evaluation_optimized.c:159-188 (r in kpc -> convolved magnitude tables) */
static void so_prob_consts(const so_problem* p, const so_consts* k, double coords,
                           double* r_point, double* r_in_mag, double* r_in_mag2,
                           double* qw_r3_N, double* reff_xr_rp3)
{
    double gPrime, exp_result, g, exponent, r3, N, reff_value, rPrime3;
    int i;
    gPrime = 5.0 * (log10(coords * 1000) - 1.0) + SO_ABSM;
    exp_result = exp(so_sigmoid[1] * (gPrime - so_sigmoid[2]));
    reff_value = so_sigmoid[0] / (exp_result + 1);
    rPrime3 = coords * coords * coords;
    /* "xr" expands to 3 * stdev inside the product */
    *reff_xr_rp3 = reff_value * 3 * SO_STDEV / rPrime3;
    for (i = 0; i < p->convolve; ++i)
    {
        g = gPrime + k->dx[i];
        r_in_mag[i] = g;
        r_in_mag2[i] = g * g;
        r_point[i] = pow(10.0, (g - SO_ABSM) / 5.0 + 1.0) / 1000.0;
        r3 = r_point[i] * r_point[i] * r_point[i];
        exponent = (g - gPrime) * (g - gPrime) / (2 * SO_STDEV * SO_STDEV);
        N = k->coeff * exp(-exponent);
        qw_r3_N[i] = k->gl_w[i] * r3 * N;
    }
}

/* evaluation_optimized.c:190-299.  lb = (l, b) in degrees. */
static void so_probabilities(const so_problem* p, so_consts* k, const double* r_point,
                             const double* r_in_mag, const double* r_in_mag2,
                             const double* qw_r3_N, double reff_xr_rp3, const double* lb,
                             double* bg_prob, double* st_prob)
{
    double bsin, lsin, bcos, lcos, zp, rg, rs, xyzs[3], dotted, xyz_norm;
    double* xyz = k->xyz;
    int i, j;
    const int C = p->convolve;

    bsin = sin(lb[1] / SO_DEG);
    lsin = sin(lb[0] / SO_DEG);
    bcos = cos(lb[1] / SO_DEG);
    lcos = cos(lb[0] / SO_DEG);

    if (k->q == 0)
    {
        /* The reference leaves xyz as the previous point left it here; this
         * restatement refreshes it so the stream terms stay defined. */
        *bg_prob = -1;
        for (i = 0; i < C; ++i)
        {
            xyz[3 * i + 2] = r_point[i] * bsin;
            zp = r_point[i] * bcos;
            xyz[3 * i + 0] = zp * lcos - SO_LBR_R;
            xyz[3 * i + 1] = zp * lsin;
        }
    }
    else
    {
        *bg_prob = 0;
        if (k->alpha == 1 && k->delta == 1)
        {
            for (i = 0; i < C; ++i)
            {
                xyz[3 * i + 2] = r_point[i] * bsin;
                zp = r_point[i] * bcos;
                xyz[3 * i + 0] = zp * lcos - SO_LBR_R;
                xyz[3 * i + 1] = zp * lsin;
                rg = sqrt(xyz[3 * i] * xyz[3 * i] + xyz[3 * i + 1] * xyz[3 * i + 1] +
                          (xyz[3 * i + 2] * xyz[3 * i + 2]) / (k->q * k->q));
                rs = rg + k->r0;
                if (p->aux == 1)
                {
                    double h_prob = qw_r3_N[i] / (rg * rs * rs * rs);
                    double aux_prob = qw_r3_N[i] * (k->bg_a * r_in_mag2[i] + k->bg_b * r_in_mag[i] + k->bg_c);
                    *bg_prob += h_prob + aux_prob;
                }
                else
                {
                    *bg_prob += qw_r3_N[i] / (rg * rs * rs * rs);
                }
            }
        }
        else
        {
            for (i = 0; i < C; ++i)
            {
                xyz[3 * i + 2] = r_point[i] * bsin;
                zp = r_point[i] * bcos;
                xyz[3 * i + 0] = zp * lcos - SO_LBR_R;
                xyz[3 * i + 1] = zp * lsin;
                rg = sqrt(xyz[3 * i] * xyz[3 * i] + xyz[3 * i + 1] * xyz[3 * i + 1] +
                          (xyz[3 * i + 2] * xyz[3 * i + 2]) / (k->q * k->q));
                *bg_prob += qw_r3_N[i] / (pow(rg, k->alpha) * pow(rg + k->r0, k->alpha_delta3));
            }
        }
        *bg_prob *= reff_xr_rp3;
    }

    for (i = 0; i < p->n_streams; ++i)
    {
        st_prob[i] = 0;
        if (k->sigma[i] > -0.0001 && k->sigma[i] < 0.0001)
            continue;
        for (j = 0; j < C; ++j)
        {
            xyzs[0] = xyz[3 * j + 0] - k->c[i][0];
            xyzs[1] = xyz[3 * j + 1] - k->c[i][1];
            xyzs[2] = xyz[3 * j + 2] - k->c[i][2];
            dotted = k->a[i][0] * xyzs[0] + k->a[i][1] * xyzs[1] + k->a[i][2] * xyzs[2];
            xyzs[0] = xyzs[0] - dotted * k->a[i][0];
            xyzs[1] = xyzs[1] - dotted * k->a[i][1];
            xyzs[2] = xyzs[2] - dotted * k->a[i][2];
            xyz_norm = xyzs[0] * xyzs[0] + xyzs[1] * xyzs[1] + xyzs[2] * xyzs[2];
            st_prob[i] += qw_r3_N[j] * exp(-xyz_norm / k->sigma_sq2[i]);
        }
        st_prob[i] *= reff_xr_rp3;
    }
}

/* ------------------------------------------------------------- integrals */

typedef struct
{
    int R, C, NU;
    double *irv, *reff, *r_point, *r_in_mag, *r_in_mag2, *qw, *ids, *nus;
} so_rtab;

/* evaluation_optimized.c:360-422 */
static void so_build_rtab(const so_problem* p, const so_consts* k, const so_area* A, so_rtab* t)
{
    int i;
    double r, next_r, rPrime;
    t->R = A->r_steps;
    t->C = p->convolve;
    t->NU = A->nu_steps;
    t->irv = (double*)malloc(sizeof(double) * (size_t)t->R);
    t->reff = (double*)malloc(sizeof(double) * (size_t)t->R);
    t->r_point = (double*)malloc(sizeof(double) * (size_t)t->R * (size_t)t->C);
    t->r_in_mag = (double*)malloc(sizeof(double) * (size_t)t->R * (size_t)t->C);
    t->r_in_mag2 = (double*)malloc(sizeof(double) * (size_t)t->R * (size_t)t->C);
    t->qw = (double*)malloc(sizeof(double) * (size_t)t->R * (size_t)t->C);
    t->ids = (double*)malloc(sizeof(double) * (size_t)t->NU);
    t->nus = (double*)malloc(sizeof(double) * (size_t)t->NU);
    for (i = 0; i < t->R; ++i)
    {
        double log_r = A->r_min + (i * A->r_step);
        r = pow(10.0, (log_r - 14.2) / 5.0);
        next_r = pow(10.0, (log_r + A->r_step - 14.2) / 5.0);
        t->irv[i] = (((next_r * next_r * next_r) - (r * r * r)) / 3.0) * A->mu_step / SO_DEG;
        rPrime = (next_r + r) / 2.0;
        so_prob_consts(p, k, rPrime, t->r_point + (size_t)i * t->C, t->r_in_mag + (size_t)i * t->C,
                       t->r_in_mag2 + (size_t)i * t->C, t->qw + (size_t)i * t->C, &t->reff[i]);
    }
    for (i = 0; i < t->NU; ++i)
    {
        t->nus[i] = A->nu_min + (i * A->nu_step);
        t->ids[i] = cos((90 - t->nus[i] - A->nu_step) / SO_DEG) - cos((90 - t->nus[i]) / SO_DEG);
        t->nus[i] += 0.5 * A->nu_step;
    }
}

static void so_free_rtab(so_rtab* t)
{
    free(t->irv);
    free(t->reff);
    free(t->r_point);
    free(t->r_in_mag);
    free(t->r_in_mag2);
    free(t->qw);
    free(t->ids);
    free(t->nus);
}

/* evaluation_optimized.c:424-562.  Processes linear cell indices
 * [lo, hi) in the reference's order (mu outer, nu, r inner) with Kahan
 * summation; out gets (1+S) values; cells (optional) gets per-cell values. */
static void so_integral_area(const so_problem* p, so_consts* k, const so_area* A, long lo, long hi,
                             double* out, double* cells)
{
    so_rtab t;
    const int S = p->n_streams;
    double bg_int = 0.0, bg_c = 0.0, tmp, bg, V;
    double st[SO_MAX_STREAMS], st_int[SO_MAX_STREAMS], st_c[SO_MAX_STREAMS];
    double lb[2];
    long idx;
    int i, cur_mu = -1, cur_nu = -1;

    so_build_rtab(p, k, A, &t);
    for (i = 0; i < S; ++i)
        st_int[i] = st_c[i] = 0.0;

    for (idx = lo; idx < hi; ++idx)
    {
        /* evaluation_state.c:261-283 (get_steps) */
        int r_step = (int)(idx % A->r_steps);
        int nu_step = (int)((idx / A->r_steps) % A->nu_steps);
        int mu_step = (int)(idx / ((long)A->r_steps * A->nu_steps));
        if (mu_step != cur_mu || nu_step != cur_nu)
        {
            double mu = A->mu_min + (mu_step * A->mu_step);
            so_wedge_point_lb(p, mu + 0.5 * A->mu_step, t.nus[nu_step], &lb[0], &lb[1]);
            cur_mu = mu_step;
            cur_nu = nu_step;
        }
        V = t.irv[r_step] * t.ids[nu_step];
        so_probabilities(p, k, t.r_point + (size_t)r_step * t.C, t.r_in_mag + (size_t)r_step * t.C,
                         t.r_in_mag2 + (size_t)r_step * t.C, t.qw + (size_t)r_step * t.C,
                         t.reff[r_step], lb, &bg, st);
        bg *= V;
        tmp = bg_int;
        bg_int += bg;
        bg_c += bg - (bg_int - tmp);
        if (cells)
            cells[(size_t)(idx - lo) * (1 + S)] = bg;
        for (i = 0; i < S; ++i)
        {
            st[i] *= V;
            tmp = st_int[i];
            st_int[i] += st[i];
            st_c[i] += st[i] - (st_int[i] - tmp);
            if (cells)
                cells[(size_t)(idx - lo) * (1 + S) + 1 + i] = st[i];
        }
    }
    out[0] = bg_int + bg_c;
    for (i = 0; i < S; ++i)
        out[1 + i] = st_int[i] + st_c[i];
    so_free_rtab(&t);
}

/* evaluation_optimized.c:564-611 (+ the slice bounds of parameters.c:502-522) */
static void so_all_integrals(const so_problem* p, so_consts* k, int rank, int nranks,
                             double* areas, double* integrals)
{
    const int S = p->n_streams;
    int a, i;
    for (a = 0; a < p->n_areas; ++a)
    {
        const so_area* A = &p->area[a];
        long total = (long)A->r_steps * A->nu_steps * A->mu_steps;
        long lo = 0, hi = total;
        if (nranks > 1)
        {
            lo = (long)(total * ((double)rank / (double)nranks));
            hi = (long)(total * ((double)(rank + 1) / (double)nranks));
        }
        so_integral_area(p, k, A, lo, hi, areas + (size_t)a * (1 + S), NULL);
    }
    for (i = 0; i <= S; ++i)
        integrals[i] = areas[i];
    for (a = 1; a < p->n_areas; ++a)
        for (i = 0; i <= S; ++i)
            integrals[i] -= areas[(size_t)a * (1 + S) + i];
}

/* evaluation_optimized.c:613-753 over stars [s0, s1) */
static void so_likelihood_range(const so_problem* p, so_consts* k, const double* integrals, int s0, int s1,
                                double* prob_sum_out, int* num_zero_out, double* bg_only_out, double* st_only_out)
{
    const int S = p->n_streams;
    const int C = p->convolve;
    double* r_point = (double*)malloc(sizeof(double) * (size_t)C);
    double* r_in_mag = (double*)malloc(sizeof(double) * (size_t)C);
    double* r_in_mag2 = (double*)malloc(sizeof(double) * (size_t)C);
    double* qw = (double*)malloc(sizeof(double) * (size_t)C);
    double reff, bg_prob, st_prob[SO_MAX_STREAMS], exp_st[SO_MAX_STREAMS];
    double exp_bg, sum_exp, prob_sum = 0, prob_c = 0, tmp;
    double bg_only, bg_sum = 0, bg_c = 0, st_only, st_sum[SO_MAX_STREAMS], st_c[SO_MAX_STREAMS];
    int i, s, num_zero = 0;

    exp_bg = exp(p->bg_weight);
    sum_exp = exp_bg;
    for (i = 0; i < S; ++i)
    {
        exp_st[i] = exp(p->st_weight[i]);
        sum_exp += exp(p->st_weight[i]);
        st_sum[i] = st_c[i] = 0.0;
    }
    sum_exp *= 0.001;

    for (s = s0; s < s1; ++s)
    {
        const double* star = p->stars + 3 * (size_t)s;
        double star_prob;
        so_prob_consts(p, k, star[2], r_point, r_in_mag, r_in_mag2, qw, &reff);
        so_probabilities(p, k, r_point, r_in_mag, r_in_mag2, qw, reff, star, &bg_prob, st_prob);

        bg_only = (bg_prob / integrals[0]) * exp_bg;
        star_prob = bg_only;
        if (bg_only == 0.0)
            bg_only = -238;
        else
            bg_only = log10(bg_only / sum_exp);
        tmp = bg_sum;
        bg_sum += bg_only;
        bg_c += bg_only - (bg_sum - tmp);

        for (i = 0; i < S; ++i)
        {
            st_only = st_prob[i] / integrals[1 + i] * exp_st[i];
            star_prob += st_only;
            if (st_only == 0.0)
                st_only = -238;
            else
                st_only = log10(st_only / sum_exp);
            tmp = st_sum[i];
            st_sum[i] += st_only;
            st_c[i] += st_only - (st_sum[i] - tmp);
        }
        star_prob /= sum_exp;
        if (star_prob != 0.0)
        {
            star_prob = log10(star_prob);
            tmp = prob_sum;
            prob_sum += star_prob;
            prob_c += star_prob - (prob_sum - tmp);
        }
        else
        {
            num_zero++;
            prob_sum -= 238.0;
        }
    }
    *prob_sum_out = prob_sum + prob_c;
    *num_zero_out = num_zero;
    if (bg_only_out)
        *bg_only_out = (bg_sum + bg_c) / (s1 - s0) - 3.0;
    if (st_only_out)
        for (i = 0; i < S; ++i)
            st_only_out[i] = (st_sum[i] + st_c[i]) / (s1 - s0) - 3.0;
    free(r_point);
    free(r_in_mag);
    free(r_in_mag2);
    free(qw);
}

int so_integrals(so_problem* p, const double* theta, int rank, int nranks, double* area_integrals,
                 double* integrals)
{
    so_consts k;
    double areas[SO_MAX_AREAS * (SO_MAX_STREAMS + 1)], ints[SO_MAX_STREAMS + 1];
    int i;
    so_set_theta(p, theta);
    so_init_consts(p, &k);
    so_all_integrals(p, &k, rank, nranks, areas, ints);
    if (area_integrals)
        for (i = 0; i < p->n_areas * (1 + p->n_streams); ++i)
            area_integrals[i] = areas[i];
    if (integrals)
        for (i = 0; i <= p->n_streams; ++i)
            integrals[i] = ints[i];
    so_free_consts(&k);
    return 0;
}

int so_likelihood(so_problem* p, const double* theta, const double* integrals, double* prob_sum,
                  int* num_zero, double* likelihood, double* bg_only, double* st_only)
{
    so_consts k;
    double ps;
    int nz;
    if (p->n_stars <= 0)
        return 1;
    so_set_theta(p, theta);
    so_init_consts(p, &k);
    so_likelihood_range(p, &k, integrals, 0, p->n_stars, &ps, &nz, bg_only, st_only);
    if (prob_sum)
        *prob_sum = ps;
    if (num_zero)
        *num_zero = nz;
    if (likelihood)
        *likelihood = ps / p->n_stars - 3.0;
    so_free_consts(&k);
    return 0;
}

int so_evaluate(so_problem* p, const double* theta, int rank, int nranks, double* area_integrals,
                double* integrals, double* prob_sum, int* num_zero, double* likelihood, double* bg_only,
                double* st_only)
{
    so_consts k;
    double areas[SO_MAX_AREAS * (SO_MAX_STREAMS + 1)], ints[SO_MAX_STREAMS + 1], ps;
    int i, nz, s0 = 0, s1 = p->n_stars;
    if (p->n_stars <= 0)
        return 1;
    so_set_theta(p, theta);
    so_init_consts(p, &k);
    so_all_integrals(p, &k, rank, nranks, areas, ints);
    if (nranks > 1)
    {
        /* star_points.c:113-114 */
        s0 = (int)(((double)p->n_stars) * (((double)rank) / ((double)nranks)));
        s1 = (int)(((double)p->n_stars) * (((double)rank + 1.0) / ((double)nranks)));
        if (s1 <= s0)
        {
            so_free_consts(&k);
            return 1;
        }
    }
    so_likelihood_range(p, &k, ints, s0, s1, &ps, &nz, bg_only, st_only);
    if (area_integrals)
        for (i = 0; i < p->n_areas * (1 + p->n_streams); ++i)
            area_integrals[i] = areas[i];
    if (integrals)
        for (i = 0; i <= p->n_streams; ++i)
            integrals[i] = ints[i];
    if (prob_sum)
        *prob_sum = ps;
    if (num_zero)
        *num_zero = nz;
    if (likelihood)
        *likelihood = ps / (s1 - s0) - 3.0; /* cpu_evaluate :783, app :278 */
    so_free_consts(&k);
    return 0;
}

int so_cell_values(so_problem* p, const double* theta, int area, double* out)
{
    so_consts k;
    double acc[SO_MAX_STREAMS + 1];
    const so_area* A;
    if (area < 0 || area >= p->n_areas)
        return 1;
    A = &p->area[area];
    so_set_theta(p, theta);
    so_init_consts(p, &k);
    so_integral_area(p, &k, A, 0, (long)A->mu_steps * A->nu_steps * A->r_steps, acc, out);
    so_free_consts(&k);
    return 0;
}

int so_cell_lb(so_problem* p, int area, double* out)
{
    const so_area* A;
    int i, j;
    if (area < 0 || area >= p->n_areas)
        return 1;
    A = &p->area[area];
    for (i = 0; i < A->mu_steps; ++i)
    {
        double mu = A->mu_min + (i * A->mu_step);
        for (j = 0; j < A->nu_steps; ++j)
        {
            double nu = A->nu_min + (j * A->nu_step);
            nu += 0.5 * A->nu_step;
            so_wedge_point_lb(p, mu + 0.5 * A->mu_step, nu, &out[2 * ((size_t)i * A->nu_steps + j)],
                              &out[2 * ((size_t)i * A->nu_steps + j) + 1]);
        }
    }
    return 0;
}

int so_r_tables(so_problem* p, int area, double* irv, double* reff, double* r_point, double* qw, double* ids,
                double* nus)
{
    so_consts k;
    so_rtab t;
    if (area < 0 || area >= p->n_areas)
        return 1;
    so_init_consts(p, &k);
    so_build_rtab(p, &k, &p->area[area], &t);
    memcpy(irv, t.irv, sizeof(double) * (size_t)t.R);
    memcpy(reff, t.reff, sizeof(double) * (size_t)t.R);
    memcpy(r_point, t.r_point, sizeof(double) * (size_t)t.R * t.C);
    memcpy(qw, t.qw, sizeof(double) * (size_t)t.R * t.C);
    memcpy(ids, t.ids, sizeof(double) * (size_t)t.NU);
    memcpy(nus, t.nus, sizeof(double) * (size_t)t.NU);
    so_free_rtab(&t);
    so_free_consts(&k);
    return 0;
}

int so_r_mag_tables(so_problem* p, int area, double* r_in_mag, double* r_in_mag2)
{
    so_consts k;
    so_rtab t;
    if (area < 0 || area >= p->n_areas)
        return 1;
    so_init_consts(p, &k);
    so_build_rtab(p, &k, &p->area[area], &t);
    memcpy(r_in_mag, t.r_in_mag, sizeof(double) * (size_t)t.R * t.C);
    memcpy(r_in_mag2, t.r_in_mag2, sizeof(double) * (size_t)t.R * t.C);
    so_free_rtab(&t);
    so_free_consts(&k);
    return 0;
}

int so_star_densities(so_problem* p, const double* theta, double* bg, double* st)
{
    so_consts k;
    const int C = p->convolve, S = p->n_streams;
    double *r_point, *r_in_mag, *r_in_mag2, *qw, reff, sp[SO_MAX_STREAMS];
    int s, i;
    so_set_theta(p, theta);
    so_init_consts(p, &k);
    r_point = (double*)malloc(sizeof(double) * (size_t)C);
    r_in_mag = (double*)malloc(sizeof(double) * (size_t)C);
    r_in_mag2 = (double*)malloc(sizeof(double) * (size_t)C);
    qw = (double*)malloc(sizeof(double) * (size_t)C);
    for (s = 0; s < p->n_stars; ++s)
    {
        const double* star = p->stars + 3 * (size_t)s;
        so_prob_consts(p, &k, star[2], r_point, r_in_mag, r_in_mag2, qw, &reff);
        so_probabilities(p, &k, r_point, r_in_mag, r_in_mag2, qw, reff, star, &bg[s], sp);
        for (i = 0; i < S; ++i)
            st[(size_t)s * S + i] = sp[i];
    }
    free(r_point);
    free(r_in_mag);
    free(r_in_mag2);
    free(qw);
    so_free_consts(&k);
    return 0;
}


/* ------------------------------------------------------------ separation */

/* stVector.c:56-103 */
static double so_norm3(const double* v) { return sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }
static double so_dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

/* stCoords.c:177-185 */
static void so_lb_to_xyz(double l, double b, double* xyz)
{
    l = l / SO_DEG;
    b = b / SO_DEG;
    xyz[0] = cos(l) * cos(b);
    xyz[1] = sin(l) * cos(b);
    xyz[2] = sin(b);
}

/* atSurveyGeometry.c:415-441 (survey centre RA 185, Dec 32.5) */
static void so_survey_to_eq(double slong, double slat, double* ra, double* dec)
{
    double anode, etaPole, x1, y1, z1;
    slong = slong * SO_DPI / 180.0;
    slat = slat * SO_DPI / 180.0;
    anode = 185.0 - 90.0;
    anode = anode * SO_DPI / 180.0;
    etaPole = 32.5 * SO_DPI / 180.0;
    x1 = -sin(slong);
    y1 = cos(slat + etaPole) * cos(slong);
    z1 = sin(slat + etaPole) * cos(slong);
    *ra = atan2(y1, x1) + anode;
    *dec = asin(z1);
    *ra = *ra * 180.0 / SO_DPI;
    *dec = *dec * 180.0 / SO_DPI;
    so_bound2(dec, ra);
}

void so_stripe_transform(int sgr, int wedge, double* m)
{
    double n[3], axis[3], t[3] = {0.0, 0.0, 1.0}, angle, sin_a, x, y, z, w, an;
    if (sgr == 0)
    {
        /* stCoords.c:142-150, atSurveyGeometry.c:444-459 */
        double eta = (wedge <= 46) ? wedge * 2.5 - 57.5 : wedge * 2.5 - 57.5 - 180.0;
        double ra, dec, l, b;
        so_survey_to_eq(0, 90.0 + eta, &ra, &dec);
        so_eq_to_gal(ra, dec, &l, &b);
        so_lb_to_xyz(l, b, n);
    }
    else
    {
        /* stCoords.c:153-174 */
        double l1, b1, l2, b2, a1[3], a2[3];
        so_sgr_to_gal(wedge * 2.5, 0, &l1, &b1);
        so_sgr_to_gal(wedge * 2.5, 90, &l2, &b2);
        so_lb_to_xyz(l1, b1, a1);
        so_lb_to_xyz(l2, b2, a2);
        n[0] = a1[1] * a2[2] - a1[2] * a2[1];
        n[1] = a1[2] * a2[0] - a1[0] * a2[2];
        n[2] = a1[0] * a2[1] - a1[1] * a2[0];
    }
    /* stVector.c:109-137: rotation taking n onto the z axis */
    axis[0] = n[1] * t[2] - n[2] * t[1];
    axis[1] = n[2] * t[0] - n[0] * t[2];
    axis[2] = n[0] * t[1] - n[1] * t[0];
    an = so_norm3(axis);
    axis[0] /= an;
    axis[1] /= an;
    axis[2] /= an;
    angle = acos(so_dot3(n, t) / (so_norm3(n) * so_norm3(t)));
    sin_a = sin(angle / 2);
    x = axis[0] * sin_a;
    y = axis[1] * sin_a;
    z = axis[2] * sin_a;
    w = cos(angle / 2);
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

/* stVector.c:155-169 with stCoords.c:52-65 (xyz2lbr), :188-201 (xyz_mag,
 * xyz2lbg): back to (l, b, r), replace r by the magnitude minus 11, to
 * Galactic xyz again, shift by the Sun, rotate. */
void so_transform_point(const double* point, const double* m, double* out)
{
    const double r0 = 8.5;
    double lbg[3], v[3], temp, xsun;
    xsun = point[0] + r0;
    temp = xsun * xsun + point[1] * point[1];
    lbg[0] = atan2(point[1], xsun) * SO_DEG;
    lbg[1] = atan2(point[2], sqrt(temp)) * SO_DEG;
    lbg[2] = sqrt(temp + point[2] * point[2]);
    if (lbg[0] < 0)
        lbg[0] += 360;
    lbg[2] = 5.0 * (log(100.0 * lbg[2]) / log(10.0)) + 4.2 - 11.0;
    so_lbr_to_xyz(lbg[0], lbg[1], lbg[2], v);
    v[0] = v[0] - (-8.5);
    v[1] = v[1] - 0.0;
    v[2] = v[2] - 0.0;
    out[0] = m[0] * v[0] + m[1] * v[1] + m[2] * v[2];
    out[1] = m[3] * v[0] + m[4] * v[1] + m[5] * v[2];
    out[2] = m[6] * v[0] + m[7] * v[1] + m[8] * v[2];
}

int so_separation(so_problem* p, const double* theta, const double* integrals, double* sprob, double* xyz,
                  double* expected)
{
    so_consts k;
    const int C = p->convolve, S = p->n_streams;
    double *r_point, *r_in_mag, *r_in_mag2, *qw, reff, pb, ps[SO_MAX_STREAMS], eps_s[SO_MAX_STREAMS], eps_b,
        denom, nst[SO_MAX_STREAMS], m[9];
    int s, j;
    so_set_theta(p, theta);
    so_init_consts(p, &k);
    so_stripe_transform(p->sgr, p->wedge, m);
    /* separation.c:128-140 */
    denom = 1.0;
    for (j = 0; j < S; ++j)
        denom += exp(p->st_weight[j]);
    for (j = 0; j < S; ++j)
    {
        eps_s[j] = exp(p->st_weight[j]) / denom;
        nst[j] = 0;
    }
    eps_b = 1.0 / denom;
    r_point = (double*)malloc(sizeof(double) * (size_t)C);
    r_in_mag = (double*)malloc(sizeof(double) * (size_t)C);
    r_in_mag2 = (double*)malloc(sizeof(double) * (size_t)C);
    qw = (double*)malloc(sizeof(double) * (size_t)C);
    for (s = 0; s < p->n_stars; ++s)
    {
        const double* star = p->stars + 3 * (size_t)s;
        double pbx, psg[SO_MAX_STREAMS], psg_sum = 0, starxyz[3];
        so_prob_consts(p, &k, star[2], r_point, r_in_mag, r_in_mag2, qw, &reff);
        so_probabilities(p, &k, r_point, r_in_mag, r_in_mag2, qw, reff, star, &pb, ps);
        /* :170-196 */
        pbx = eps_b * pb / integrals[0];
        for (j = 0; j < S; ++j)
            psg[j] = eps_s[j] * ps[j] / integrals[1 + j];
        for (j = 0; j < S; ++j)
            psg_sum += psg[j];
        for (j = 0; j < S; ++j)
        {
            const double sp = psg[j] / (psg_sum + pbx);
            if (sprob)
                sprob[(size_t)s * S + j] = sp;
            nst[j] += sp;
        }
        /* :226-227 */
        if (xyz)
        {
            so_lbr_to_xyz(star[0], star[1], star[2], starxyz);
            so_transform_point(starxyz, m, xyz + 3 * (size_t)s);
        }
    }
    if (expected)
        for (j = 0; j < S; ++j)
            expected[j] = nst[j];
    free(r_point);
    free(r_in_mag);
    free(r_in_mag2);
    free(qw);
    so_free_consts(&k);
    return 0;
}

#ifdef SEP_ORACLE_MAIN
#include <time.h>
/* sep_oracle -a params -p stars [-r rank -n nranks] [-t] theta... */
int main(int argc, char** argv)
{
    const char *pf = NULL, *sf = NULL;
    int rank = 0, nranks = 1, timing = 0, n = 0, i, nz = 0;
    double theta[256], ints[SO_MAX_STREAMS + 1], areas[SO_MAX_AREAS * (SO_MAX_STREAMS + 1)], ps = 0, ll = 0;
    struct timespec t0, t1;
    so_problem* p;
    for (i = 1; i < argc; ++i)
    {
        if (!strcmp(argv[i], "-a") && i + 1 < argc) pf = argv[++i];
        else if (!strcmp(argv[i], "-p") && i + 1 < argc) sf = argv[++i];
        else if (!strcmp(argv[i], "-r") && i + 1 < argc) rank = atoi(argv[++i]);
        else if (!strcmp(argv[i], "-n") && i + 1 < argc) nranks = atoi(argv[++i]);
        else if (!strcmp(argv[i], "-t")) timing = 1;
        else if (n < 256) theta[n++] = strtod(argv[i], NULL);
    }
    if (!pf || !sf)
        return 2;
    p = so_open(pf, sf);
    if (!p || n != so_n_theta(p))
        return 1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    if (so_evaluate(p, theta, rank, nranks, areas, ints, &ps, &nz, &ll, NULL, NULL))
        return 1;
    clock_gettime(CLOCK_MONOTONIC, &t1);
    printf("background_integral %.17g\n", ints[0]);
    for (i = 0; i < so_n_streams(p); ++i)
        printf("stream_integral %d %.17g\n", i, ints[1 + i]);
    printf("prob_sum %.17g\nnum_zero %d\nsearch_likelihood %.17g\n", ps, nz, ll);
    if (timing)
        printf("seconds %.6f\n", (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec));
    so_close(p);
    return 0;
}
#endif
