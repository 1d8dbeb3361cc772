/* sanitize_harness.cpp -- drives the library's host-only translation units
 * (parameter and star-file I/O, binary formats, the finite-difference
 * consumers and the matrix inversion) under AddressSanitizer and
 * UndefinedBehaviorSanitizer, with no GPU.  Test infrastructure: built and run
 * by tests/test_sanitizers.py.
 *
 * The device-facing context calls that these units reach are replaced by a
 * fake context whose "evaluation" is the quadratic
 *     f(theta) = -1/2 theta' A theta + g' theta,
 * so the finite-difference Hessian must come out as -A and the gradient at
 * theta as g - A theta (central differences are exact on a quadratic up to
 * rounding).
 *
 *     sanitize_harness TMPDIR params.txt stars.txt [params.txt stars.txt ...]
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "milkyway_separation_gb300.h"

static int g_status = 0;
#define CHECK(cond)                                                                                 \
    do                                                                                              \
    {                                                                                               \
        if (!(cond))                                                                                \
        {                                                                                           \
            fprintf(stderr, "check failed: %s (%s:%d)\n", #cond, __FILE__, __LINE__);               \
            g_status = 1;                                                                           \
        }                                                                                           \
    } while (0)

/* ---- the status functions the units call ---- */
extern "C" int mwsep_fail(int status) { return status; }

/* ---- a fake context: a quadratic in theta ---- */
struct mwsep_ctx
{
    int P;
    std::vector<double> A, g;
};

extern "C" int mwsep_ctx_wedge_theta_count(const mwsep_ctx* c, int wedge)
{
    return (c && wedge == 0) ? c->P : -1;
}

extern "C" int mwsep_ctx_evaluate_requests(mwsep_ctx* c, int n, const mwsep_request* reqs, int precision,
                                           mwsep_result* out)
{
    (void)precision;
    if (!c || n < 1 || !reqs || !out) return MWSEP_ERR_ARG;
    for (int r = 0; r < n; ++r)
    {
        const double* t = reqs[r].theta;
        double f = 0.0;
        for (int i = 0; i < c->P; ++i)
        {
            double row = 0.0;
            for (int j = 0; j < c->P; ++j) row += c->A[(size_t)i * c->P + j] * t[j];
            f += -0.5 * t[i] * row + c->g[(size_t)i] * t[i];
        }
        memset(&out[r], 0, sizeof(out[r]));
        out[r].likelihood = f;
    }
    return MWSEP_OK;
}

extern "C" int mwsep_ctx_set_stars_soa(mwsep_ctx*, int, const double*, const double*, const double*)
{
    return MWSEP_OK;
}
extern "C" int mwsep_ctx_set_stars(mwsep_ctx*, const STAR_POINTS*) { return MWSEP_OK; }

static bool same_params(const ASTRONOMY_PARAMETERS& a, const ASTRONOMY_PARAMETERS& b)
{
    if (a.parameters_version != b.parameters_version || a.number_background_parameters != b.number_background_parameters ||
        a.background_weight != b.background_weight || a.number_streams != b.number_streams ||
        a.number_stream_parameters != b.number_stream_parameters || a.convolve != b.convolve ||
        a.sgr_coordinates != b.sgr_coordinates || a.aux_bg_profile != b.aux_bg_profile || a.wedge != b.wedge ||
        a.number_integrals != b.number_integrals)
        return false;
    for (int i = 0; i < a.number_background_parameters; ++i)
        if (a.background_parameters[i] != b.background_parameters[i] || a.background_step[i] != b.background_step[i] ||
            a.background_min[i] != b.background_min[i] || a.background_max[i] != b.background_max[i] ||
            a.background_optimize[i] != b.background_optimize[i])
            return false;
    for (int s = 0; s < a.number_streams; ++s)
    {
        if (a.stream_weights[s] != b.stream_weights[s] || a.stream_weight_optimize[s] != b.stream_weight_optimize[s])
            return false;
        for (int j = 0; j < a.number_stream_parameters; ++j)
            if (a.stream_parameters[s][j] != b.stream_parameters[s][j] || a.stream_optimize[s][j] != b.stream_optimize[s][j])
                return false;
    }
    for (int i = 0; i < a.number_integrals; ++i)
        if (memcmp(a.integral[i], b.integral[i], sizeof(INTEGRAL)) != 0) return false;
    return true;
}

static void params_case(const std::string& dir, const char* path)
{
    ASTRONOMY_PARAMETERS ap, back, bin;
    CHECK(mwsep_read_astronomy_parameters(path, &ap) == MWSEP_OK);
    const int P = mwsep_get_optimized_parameter_count(&ap);
    CHECK(P > 0);
    std::vector<double> theta((size_t)P), step((size_t)P), lo((size_t)P), hi((size_t)P);
    CHECK(mwsep_get_search_parameters(&ap, theta.data()) == MWSEP_OK);
    CHECK(mwsep_get_step(&ap, step.data()) == MWSEP_OK);
    CHECK(mwsep_get_min_parameters(&ap, lo.data()) == MWSEP_OK);
    CHECK(mwsep_get_max_parameters(&ap, hi.data()) == MWSEP_OK);
    CHECK(mwsep_set_astronomy_parameters(&ap, theta.data()) == MWSEP_OK);
    const std::string txt = dir + "/p.txt", binp = dir + "/p.mwsp";
    CHECK(mwsep_write_astronomy_parameters(txt.c_str(), &ap) == MWSEP_OK);
    CHECK(mwsep_read_astronomy_parameters(txt.c_str(), &back) == MWSEP_OK);
    CHECK(mwsep_write_astronomy_parameters_binary(binp.c_str(), &ap) == MWSEP_OK);
    CHECK(mwsep_read_astronomy_parameters_binary(binp.c_str(), &bin) == MWSEP_OK);
    CHECK(same_params(ap, bin));
    /* corrupt the binary file byte by byte: every read must fail cleanly */
    {
        FILE* f = fopen(binp.c_str(), "rb");
        std::vector<unsigned char> raw;
        int ch;
        while (f && (ch = fgetc(f)) != EOF) raw.push_back((unsigned char)ch);
        if (f) fclose(f);
        const std::string bad = dir + "/bad.mwsp";
        for (size_t at = 0; at < raw.size(); at += 7)
        {
            std::vector<unsigned char> r = raw;
            r[at] ^= 0x5a;
            FILE* g = fopen(bad.c_str(), "wb");
            fwrite(r.data(), 1, r.size(), g);
            fclose(g);
            ASTRONOMY_PARAMETERS x;
            if (mwsep_read_astronomy_parameters_binary(bad.c_str(), &x) == MWSEP_OK) mwsep_free_parameters(&x);
        }
        for (size_t cut = 0; cut < raw.size(); cut += 13)
        {
            FILE* g = fopen(bad.c_str(), "wb");
            fwrite(raw.data(), 1, cut, g);
            fclose(g);
            ASTRONOMY_PARAMETERS x;
            CHECK(mwsep_read_astronomy_parameters_binary(bad.c_str(), &x) != MWSEP_OK);
        }
    }
    CHECK(mwsep_split_astronomy_parameters(&back, 1, 3) == MWSEP_OK);
    mwsep_free_parameters(&back);
    mwsep_free_parameters(&bin);
    mwsep_free_parameters(&ap);
}

static void stars_case(const std::string& dir, const char* path)
{
    STAR_POINTS sp, back;
    CHECK(mwsep_read_star_points(path, &sp) == MWSEP_OK);
    const std::string cat = dir + "/s.mwsb";
    CHECK(mwsep_write_star_points_binary(cat.c_str(), &sp) == MWSEP_OK);
    CHECK(mwsep_read_star_points_binary(cat.c_str(), &back) == MWSEP_OK);
    CHECK(back.number_stars == sp.number_stars);
    for (int i = 0; i < sp.number_stars; ++i)
        CHECK(memcmp(back.stars[i], sp.stars[i], 3 * sizeof(double)) == 0);
    mwsep_star_catalogue m;
    CHECK(mwsep_map_star_catalogue(cat.c_str(), &m) == MWSEP_OK);
    double sum = 0.0;
    for (int i = 0; i < m.number_stars; ++i) sum += m.l[i] + m.b[i] + m.r[i];
    CHECK(isfinite(sum));
    CHECK(mwsep_unmap_star_catalogue(&m) == MWSEP_OK);
    mwsep_ctx fake{};
    CHECK(mwsep_ctx_set_stars_file(&fake, cat.c_str()) == MWSEP_OK);
    CHECK(mwsep_ctx_set_stars_file(&fake, path) == MWSEP_OK);
    /* truncations of the catalogue are rejected */
    {
        FILE* f = fopen(cat.c_str(), "rb");
        std::vector<unsigned char> raw;
        int ch;
        while (f && (ch = fgetc(f)) != EOF) raw.push_back((unsigned char)ch);
        if (f) fclose(f);
        const std::string bad = dir + "/bad.mwsb";
        for (size_t cut : {(size_t)0, (size_t)8, (size_t)63, (size_t)64, raw.size() / 2, raw.size() - 1})
        {
            FILE* g = fopen(bad.c_str(), "wb");
            fwrite(raw.data(), 1, cut, g);
            fclose(g);
            CHECK(mwsep_map_star_catalogue(bad.c_str(), &m) != MWSEP_OK);
        }
    }
    std::vector<int> assign((size_t)sp.number_stars);
    std::vector<double> xyz((size_t)sp.number_stars * 3, 1.0);
    for (int i = 0; i < sp.number_stars; ++i) assign[(size_t)i] = i % 3;
    CHECK(mwsep_write_separation((dir + "/sep.txt").c_str(), sp.number_stars, assign.data(), xyz.data()) == MWSEP_OK);
    CHECK(mwsep_split_star_points(&back, 2, 5) == MWSEP_OK);
    mwsep_free_star_points(&back);
    mwsep_free_star_points(&sp);
}

static void optimiser_case(const std::string& dir)
{
    for (int P : {1, 2, 5, 9})
    {
        mwsep_ctx c;
        c.P = P;
        c.A.assign((size_t)P * P, 0.0);
        c.g.assign((size_t)P, 0.0);
        unsigned s = 12345u + (unsigned)P;
        auto rnd = [&]() {
            s = s * 1103515245u + 12345u;
            return ((s >> 8) & 0xffff) / 65536.0 - 0.5;
        };
        for (int i = 0; i < P; ++i)
        {
            c.g[(size_t)i] = rnd();
            for (int j = 0; j <= i; ++j)
            {
                const double v = rnd() + (i == j ? 2.0 * P : 0.0);
                c.A[(size_t)i * P + j] = v;
                c.A[(size_t)j * P + i] = v;
            }
        }
        std::vector<double> theta((size_t)P), step((size_t)P, 0.125), grad((size_t)P), H((size_t)P * P);
        for (int i = 0; i < P; ++i) theta[(size_t)i] = rnd();
        double f0 = 0.0;
        CHECK(mwsep_ctx_hessian(&c, 0, theta.data(), step.data(), MWSEP_PLAIN_F64, &f0, grad.data(), H.data()) ==
              MWSEP_OK);
        for (int i = 0; i < P; ++i)
        {
            double want = c.g[(size_t)i];
            for (int j = 0; j < P; ++j) want -= c.A[(size_t)i * P + j] * theta[(size_t)j];
            CHECK(fabs(grad[(size_t)i] - want) <= 1e-9 * (1.0 + fabs(want)));
            for (int j = 0; j < P; ++j)
                CHECK(fabs(H[(size_t)i * P + j] + c.A[(size_t)i * P + j]) <= 1e-8 * (1.0 + fabs(c.A[(size_t)i * P + j])));
        }
        std::vector<double> g2((size_t)P);
        double f1 = 0.0;
        CHECK(mwsep_ctx_gradient(&c, 0, theta.data(), step.data(), MWSEP_MIXED_F32, &f1, g2.data()) == MWSEP_OK);
        CHECK(f1 == f0);
        for (int i = 0; i < P; ++i) CHECK(g2[(size_t)i] == grad[(size_t)i]);
        std::vector<double> sigma((size_t)P * P), sd((size_t)P), inv((size_t)P * P);
        CHECK(mwsep_errors_from_hessian(P, H.data(), 1000, sigma.data(), sd.data()) == MWSEP_OK);
        CHECK(mwsep_invert_matrix(P, c.A.data(), inv.data()) == MWSEP_OK);
        for (int i = 0; i < P; ++i)
            for (int j = 0; j < P; ++j)
            {
                double e = 0.0;
                for (int k = 0; k < P; ++k) e += c.A[(size_t)i * P + k] * inv[(size_t)k * P + j];
                CHECK(fabs(e - (i == j ? 1.0 : 0.0)) <= 1e-12);
            }
        CHECK(mwsep_write_errors((dir + "/errors.txt").c_str(), P, H.data(), sigma.data(), sd.data()) == MWSEP_OK);
        step[0] = 0.0;
        CHECK(mwsep_ctx_hessian(&c, 0, theta.data(), step.data(), MWSEP_PLAIN_F64, &f0, grad.data(), H.data()) ==
              MWSEP_ERR_ARG);
    }
    std::vector<double> z(9, 0.0), out(9);
    CHECK(mwsep_invert_matrix(3, z.data(), out.data()) == MWSEP_ERR_ARG);
}

int main(int argc, char** argv)
{
    if (argc < 4 || (argc - 2) % 2 != 0)
    {
        fprintf(stderr, "usage: %s TMPDIR params stars [params stars ...]\n", argv[0]);
        return 2;
    }
    const std::string dir = argv[1];
    for (int i = 2; i + 1 < argc; i += 2)
    {
        params_case(dir, argv[i]);
        stars_case(dir, argv[i + 1]);
    }
    optimiser_case(dir);
    if (g_status == 0) printf("sanitize harness: ok\n");
    return g_status;
}
