/* mwsep_binary.cpp -- binary star catalogues and parameter files.
 *
 * The reference reads both as text (cpu/star_points.c:26-52, 69-81;
 * cpu/parameters.c:61-91, 107-228).  At 10^5 - 10^6 stars the text parse
 * costs more than a GPU evaluation, and a serving process wants to map a
 * catalogue instead of parsing it, so the library adds:
 *
 * Star catalogue, little-endian, 64-byte header:
 *     char     magic[8]      "MWSEPCAT"
 *     uint32   version       1
 *     uint32   header_bytes  64
 *     uint64   number_stars  n
 *     uint64   offset_l      byte offset of double l[n]   (degrees)
 *     uint64   offset_b      byte offset of double b[n]   (degrees)
 *     uint64   offset_r      byte offset of double r[n]   (kpc, as in the text file)
 *     uint64   file_bytes    total size
 *     uint64   reserved      0
 * with each array starting on a 64-byte boundary, so a mapped file hands
 * out SoA columns that are uploaded as they lie (mwsep_ctx_set_stars_soa).
 *
 * Parameter file, little-endian: magic "MWSEPPAR", uint32 version 1,
 * uint32 body_bytes, the fields of ASTRONOMY_PARAMETERS in declaration order
 * (arrays by their lengths; each INTEGRAL as its 9 doubles, 3 ints and 2
 * int64), then a 64-bit FNV-1a checksum of the body.  A round trip gives the
 * same struct, bit for bit, as the text file it was made from.
 */
#include <fcntl.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <limits.h>
#include <vector>

#include "milkyway_separation_gb300.h"
#include "mwsep_params.h"
#include "mwsep_status.h"

namespace {

const char kCatMagic[8] = {'M', 'W', 'S', 'E', 'P', 'C', 'A', 'T'};
const char kParMagic[8] = {'M', 'W', 'S', 'E', 'P', 'P', 'A', 'R'};
constexpr uint32_t kVersion = 1;
/* parameter files: 1 stored number_background_parameters values of each
 * background array; 2 also the count of background values (the aux
 * profile's 4..6 kept where number_parameters counts fewer) */
constexpr uint32_t kParVersion = 2;
constexpr uint64_t kAlign = 64;

struct CatHeader
{
    char magic[8];
    uint32_t version;
    uint32_t header_bytes;
    uint64_t n;
    uint64_t off_l, off_b, off_r;
    uint64_t file_bytes;
    uint64_t reserved;
};
static_assert(sizeof(CatHeader) == 64, "catalogue header is 64 bytes");

bool little_endian()
{
    const uint32_t one = 1;
    unsigned char c;
    memcpy(&c, &one, 1);
    return c == 1;
}

uint64_t align_up(uint64_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

bool write_all(FILE* f, const void* p, size_t n) { return n == 0 || fwrite(p, 1, n, f) == n; }

uint64_t fnv1a(const unsigned char* p, size_t n)
{
    uint64_t h = 1469598103934665603ULL;
    for (size_t i = 0; i < n; ++i)
    {
        h ^= p[i];
        h *= 1099511628211ULL;
    }
    return h;
}

/* Append-only byte buffer for the parameter body. */
struct Out
{
    std::vector<unsigned char> b;
    template <typename T> void put(const T& v)
    {
        const unsigned char* p = (const unsigned char*)&v;
        b.insert(b.end(), p, p + sizeof(T));
    }
    template <typename T> void put_n(const T* a, int n)
    {
        for (int i = 0; i < n; ++i) put(a[i]);
    }
};

/* Bounds-checked reader over the parameter body. */
struct In
{
    const unsigned char* p;
    size_t n, at = 0;
    bool ok = true;
    template <typename T> T get()
    {
        T v{};
        if (!ok || at + sizeof(T) > n)
        {
            ok = false;
            return v;
        }
        memcpy(&v, p + at, sizeof(T));
        at += sizeof(T);
        return v;
    }
    template <typename T> T* get_n(int count)
    {
        if (count < 0 || count > (1 << 20)) ok = false;
        if (!ok) return nullptr;
        T* a = (T*)calloc(count ? (size_t)count : 1, sizeof(T));
        if (!a)
        {
            ok = false;
            return nullptr;
        }
        for (int i = 0; i < count; ++i) a[i] = get<T>();
        return a;
    }
};

} // namespace

extern "C" int mwsep_write_star_catalogue(const char* path, int n, const double* l, const double* b, const double* r)
{
    if (!path || n < 0 || (n > 0 && (!l || !b || !r))) return mwsep_fail(MWSEP_ERR_ARG);
    if (!little_endian()) return mwsep_fail(MWSEP_ERR_UNSUPPORTED);
    const uint64_t col = 8ULL * (uint64_t)n;
    CatHeader h;
    memset(&h, 0, sizeof(h));
    memcpy(h.magic, kCatMagic, 8);
    h.version = kVersion;
    h.header_bytes = sizeof(CatHeader);
    h.n = (uint64_t)n;
    h.off_l = align_up(sizeof(CatHeader));
    h.off_b = align_up(h.off_l + col);
    h.off_r = align_up(h.off_b + col);
    h.file_bytes = h.off_r + col;
    FILE* f = fopen(path, "wb");
    if (!f) return mwsep_fail(MWSEP_ERR_IO);
    static const unsigned char zeros[kAlign] = {};
    bool ok = write_all(f, &h, sizeof(h));
    ok = ok && write_all(f, zeros, h.off_l - sizeof(h));
    ok = ok && write_all(f, l, col) && write_all(f, zeros, h.off_b - (h.off_l + col));
    ok = ok && write_all(f, b, col) && write_all(f, zeros, h.off_r - (h.off_b + col));
    ok = ok && write_all(f, r, col);
    if (fclose(f) != 0) ok = false;
    return ok ? MWSEP_OK : mwsep_fail(MWSEP_ERR_IO);
}

extern "C" int mwsep_write_star_points_binary(const char* path, const STAR_POINTS* sp)
{
    if (!path || !sp || sp->number_stars < 0) return mwsep_fail(MWSEP_ERR_ARG);
    const int n = sp->number_stars;
    std::vector<double> l((size_t)n), b((size_t)n), r((size_t)n);
    for (int i = 0; i < n; ++i)
    {
        l[(size_t)i] = sp->stars[i][0];
        b[(size_t)i] = sp->stars[i][1];
        r[(size_t)i] = sp->stars[i][2];
    }
    return mwsep_write_star_catalogue(path, n, l.data(), b.data(), r.data());
}

extern "C" int mwsep_map_star_catalogue(const char* path, mwsep_star_catalogue* out)
{
    if (!path || !out) return mwsep_fail(MWSEP_ERR_ARG);
    memset(out, 0, sizeof(*out));
    if (!little_endian()) return mwsep_fail(MWSEP_ERR_UNSUPPORTED);
    const int fd = open(path, O_RDONLY);
    if (fd < 0) return mwsep_fail(MWSEP_ERR_IO);
    struct stat st;
    if (fstat(fd, &st) != 0 || st.st_size < (off_t)sizeof(CatHeader))
    {
        close(fd);
        return mwsep_fail(MWSEP_ERR_IO);
    }
    const size_t bytes = (size_t)st.st_size;
    void* m = mmap(nullptr, bytes, PROT_READ, MAP_PRIVATE, fd, 0);
    close(fd);
    if (m == MAP_FAILED) return mwsep_fail(MWSEP_ERR_IO);
    CatHeader h;
    memcpy(&h, m, sizeof(h));
    const uint64_t col = 8ULL * h.n;
    auto column_fits = [&](uint64_t off) {
        return off % 8 == 0 && off >= sizeof(CatHeader) && off <= bytes && col <= bytes - off;
    };
    const bool ok = memcmp(h.magic, kCatMagic, 8) == 0 && h.version == kVersion &&
                    h.header_bytes == sizeof(CatHeader) && h.n <= (uint64_t)INT_MAX && h.file_bytes == bytes &&
                    column_fits(h.off_l) && column_fits(h.off_b) && column_fits(h.off_r);
    if (!ok)
    {
        munmap(m, bytes);
        return mwsep_fail(MWSEP_ERR_IO);
    }
    const char* base = (const char*)m;
    out->number_stars = (int)h.n;
    out->l = (const double*)(base + h.off_l);
    out->b = (const double*)(base + h.off_b);
    out->r = (const double*)(base + h.off_r);
    out->map = m;
    out->map_bytes = bytes;
    return MWSEP_OK;
}

extern "C" int mwsep_unmap_star_catalogue(mwsep_star_catalogue* cat)
{
    if (!cat) return mwsep_fail(MWSEP_ERR_ARG);
    if (cat->map) munmap(cat->map, cat->map_bytes);
    memset(cat, 0, sizeof(*cat));
    return MWSEP_OK;
}

extern "C" int mwsep_read_star_points_binary(const char* path, STAR_POINTS* sp)
{
    if (!path || !sp) return mwsep_fail(MWSEP_ERR_ARG);
    sp->number_stars = 0;
    sp->stars = nullptr;
    mwsep_star_catalogue cat;
    int rc = mwsep_map_star_catalogue(path, &cat);
    if (rc) return rc;
    const int n = cat.number_stars;
    double** rows = (double**)calloc(n ? (size_t)n : 1, sizeof(double*));
    if (!rows)
    {
        mwsep_unmap_star_catalogue(&cat);
        return mwsep_fail(MWSEP_ERR_NOMEM);
    }
    for (int i = 0; i < n; ++i)
    {
        rows[i] = (double*)malloc(3 * sizeof(double));
        if (!rows[i])
        {
            for (int j = 0; j < i; ++j) free(rows[j]);
            free(rows);
            mwsep_unmap_star_catalogue(&cat);
            return mwsep_fail(MWSEP_ERR_NOMEM);
        }
        rows[i][0] = cat.l[i];
        rows[i][1] = cat.b[i];
        rows[i][2] = cat.r[i];
    }
    mwsep_unmap_star_catalogue(&cat);
    sp->number_stars = n;
    sp->stars = rows;
    return MWSEP_OK;
}

extern "C" int mwsep_ctx_set_stars_file(mwsep_ctx* ctx, const char* path)
{
    if (!ctx || !path) return mwsep_fail(MWSEP_ERR_ARG);
    char magic[8] = {};
    FILE* f = fopen(path, "rb");
    if (!f) return mwsep_fail(MWSEP_ERR_IO);
    const size_t got = fread(magic, 1, 8, f);
    fclose(f);
    if (got == 8 && memcmp(magic, kCatMagic, 8) == 0)
    {
        mwsep_star_catalogue cat;
        int rc = mwsep_map_star_catalogue(path, &cat);
        if (rc) return rc;
        rc = mwsep_ctx_set_stars_soa(ctx, cat.number_stars, cat.l, cat.b, cat.r);
        mwsep_unmap_star_catalogue(&cat);
        return rc;
    }
    STAR_POINTS sp;
    int rc = mwsep_read_star_points(path, &sp);
    if (rc) return rc;
    rc = mwsep_ctx_set_stars(ctx, &sp);
    mwsep_free_star_points(&sp);
    return rc;
}

extern "C" int mwsep_write_astronomy_parameters_binary(const char* path, const ASTRONOMY_PARAMETERS* ap)
{
    if (!path || !ap) return mwsep_fail(MWSEP_ERR_ARG);
    if (!little_endian()) return mwsep_fail(MWSEP_ERR_UNSUPPORTED);
    const int nb = ap->number_background_parameters, S = ap->number_streams, P = ap->number_stream_parameters;
    if (nb < 0 || S < 0 || P < 0 || ap->number_integrals < 0) return mwsep_fail(MWSEP_ERR_ARG);
    const int nv = mwsep_background_values(ap);
    Out o;
    o.put(ap->parameters_version);
    o.put(nb);
    o.put(nv);
    o.put(ap->background_weight);
    o.put_n(ap->background_parameters, nv);
    o.put_n(ap->background_step, nb);
    o.put_n(ap->background_min, nb);
    o.put_n(ap->background_max, nb);
    o.put_n(ap->background_optimize, nb);
    o.put(S);
    o.put(P);
    for (int i = 0; i < S; ++i)
    {
        o.put(ap->stream_weights[i]);
        o.put(ap->stream_weight_step[i]);
        o.put(ap->stream_weight_min[i]);
        o.put(ap->stream_weight_max[i]);
        o.put(ap->stream_weight_optimize[i]);
        o.put_n(ap->stream_parameters[i], P);
        o.put_n(ap->stream_step[i], P);
        o.put_n(ap->stream_min[i], P);
        o.put_n(ap->stream_max[i], P);
        o.put_n(ap->stream_optimize[i], P);
    }
    o.put(ap->convolve);
    o.put(ap->sgr_coordinates);
    o.put(ap->aux_bg_profile);
    o.put(ap->wedge);
    o.put(ap->number_integrals);
    for (int i = 0; i < ap->number_integrals; ++i)
    {
        const INTEGRAL* in = ap->integral[i];
        o.put(in->r_min), o.put(in->r_max), o.put(in->r_step_size);
        o.put(in->nu_min), o.put(in->nu_max), o.put(in->nu_step_size);
        o.put(in->mu_min), o.put(in->mu_max), o.put(in->mu_step_size);
        o.put(in->r_steps), o.put(in->nu_steps), o.put(in->mu_steps);
        o.put((int64_t)in->min_calculation), o.put((int64_t)in->max_calculation);
    }
    const uint32_t body = (uint32_t)o.b.size();
    const uint64_t sum = fnv1a(o.b.data(), o.b.size());
    FILE* f = fopen(path, "wb");
    if (!f) return mwsep_fail(MWSEP_ERR_IO);
    bool ok = write_all(f, kParMagic, 8) && write_all(f, &kParVersion, 4) && write_all(f, &body, 4) &&
              write_all(f, o.b.data(), o.b.size()) && write_all(f, &sum, 8);
    if (fclose(f) != 0) ok = false;
    return ok ? MWSEP_OK : mwsep_fail(MWSEP_ERR_IO);
}

extern "C" int mwsep_read_astronomy_parameters_binary(const char* path, ASTRONOMY_PARAMETERS* ap)
{
    if (!path || !ap) return mwsep_fail(MWSEP_ERR_ARG);
    memset(ap, 0, sizeof(*ap));
    if (!little_endian()) return mwsep_fail(MWSEP_ERR_UNSUPPORTED);
    FILE* f = fopen(path, "rb");
    if (!f) return mwsep_fail(MWSEP_ERR_IO);
    char magic[8];
    uint32_t version = 0, body = 0;
    bool ok = fread(magic, 1, 8, f) == 8 && fread(&version, 4, 1, f) == 1 && fread(&body, 4, 1, f) == 1 &&
              memcmp(magic, kParMagic, 8) == 0 && (version == 1 || version == kParVersion) && body <= (1u << 26);
    std::vector<unsigned char> buf;
    uint64_t sum = 0;
    if (ok)
    {
        buf.resize(body);
        ok = (body == 0 || fread(buf.data(), 1, body, f) == body) && fread(&sum, 8, 1, f) == 1 &&
             fnv1a(buf.data(), buf.size()) == sum;
    }
    fclose(f);
    if (!ok) return mwsep_fail(MWSEP_ERR_IO);

    In in{buf.data(), buf.size()};
    ap->parameters_version = in.get<double>();
    const int nb = in.get<int>();
    const int nv = version >= 2 ? in.get<int>() : nb;
    ap->background_weight = in.get<double>();
    if (nb < 0 || nb > 1024 || nv < nb || nv > 1024) in.ok = false;
    ap->background_parameters = in.get_n<double>(nv);
    ap->background_step = in.get_n<double>(nb);
    ap->background_min = in.get_n<double>(nb);
    ap->background_max = in.get_n<double>(nb);
    ap->background_optimize = in.get_n<int>(nb);
    ap->number_background_parameters = nb;
    const int S = in.get<int>();
    const int P = in.get<int>();
    if (S < 0 || S > 1024 || P < 0 || P > 1024) in.ok = false;
    if (in.ok)
    {
        const size_t ns = S ? (size_t)S : 1;
        ap->stream_weights = (double*)calloc(ns, sizeof(double));
        ap->stream_weight_step = (double*)calloc(ns, sizeof(double));
        ap->stream_weight_min = (double*)calloc(ns, sizeof(double));
        ap->stream_weight_max = (double*)calloc(ns, sizeof(double));
        ap->stream_weight_optimize = (int*)calloc(ns, sizeof(int));
        ap->stream_parameters = (double**)calloc(ns, sizeof(double*));
        ap->stream_step = (double**)calloc(ns, sizeof(double*));
        ap->stream_min = (double**)calloc(ns, sizeof(double*));
        ap->stream_max = (double**)calloc(ns, sizeof(double*));
        ap->stream_optimize = (int**)calloc(ns, sizeof(int*));
        ap->number_stream_parameters = P;
        ap->number_streams = S; /* after the arrays, so free is safe */
        if (!ap->stream_weights || !ap->stream_weight_step || !ap->stream_weight_min || !ap->stream_weight_max ||
            !ap->stream_weight_optimize || !ap->stream_parameters || !ap->stream_step || !ap->stream_min ||
            !ap->stream_max || !ap->stream_optimize)
            in.ok = false;
    }
    for (int i = 0; i < S && in.ok; ++i)
    {
        ap->stream_weights[i] = in.get<double>();
        ap->stream_weight_step[i] = in.get<double>();
        ap->stream_weight_min[i] = in.get<double>();
        ap->stream_weight_max[i] = in.get<double>();
        ap->stream_weight_optimize[i] = in.get<int>();
        ap->stream_parameters[i] = in.get_n<double>(P);
        ap->stream_step[i] = in.get_n<double>(P);
        ap->stream_min[i] = in.get_n<double>(P);
        ap->stream_max[i] = in.get_n<double>(P);
        ap->stream_optimize[i] = in.get_n<int>(P);
    }
    ap->convolve = in.get<int>();
    ap->sgr_coordinates = in.get<int>();
    ap->aux_bg_profile = in.get<int>();
    if (ap->aux_bg_profile == 1 && nv < 7) in.ok = false;
    ap->wedge = in.get<int>();
    const int ni = in.get<int>();
    if (ni < 0 || ni > 1025) in.ok = false;
    if (in.ok)
    {
        ap->integral = (INTEGRAL**)calloc(ni ? (size_t)ni : 1, sizeof(INTEGRAL*));
        if (!ap->integral) in.ok = false;
        for (int i = 0; i < ni && in.ok; ++i)
        {
            INTEGRAL* g = (INTEGRAL*)calloc(1, sizeof(INTEGRAL));
            if (!g)
            {
                in.ok = false;
                break;
            }
            ap->integral[i] = g;
            ap->number_integrals = i + 1;
            g->r_min = in.get<double>(), g->r_max = in.get<double>(), g->r_step_size = in.get<double>();
            g->nu_min = in.get<double>(), g->nu_max = in.get<double>(), g->nu_step_size = in.get<double>();
            g->mu_min = in.get<double>(), g->mu_max = in.get<double>(), g->mu_step_size = in.get<double>();
            g->r_steps = in.get<int>(), g->nu_steps = in.get<int>(), g->mu_steps = in.get<int>();
            g->min_calculation = (long)in.get<int64_t>();
            g->max_calculation = (long)in.get<int64_t>();
        }
    }
    if (!in.ok || in.at != in.n)
    {
        mwsep_free_parameters(ap);
        return mwsep_fail(MWSEP_ERR_IO);
    }
    return MWSEP_OK;
}
