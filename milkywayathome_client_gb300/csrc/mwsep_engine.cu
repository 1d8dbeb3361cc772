/* mwsep_engine.cu -- host side of the tiled engine.
 *
 * Evaluates a batch of requests, each naming a resident wedge and a
 * parameter vector, with one persistent launch per phase (integrals, then
 * likelihood) for all requests of a stream-count group:
 *
 *   H2D counters, constants, requests, tile lists
 *   -> integral tiles (persistent, dynamic tile counter)
 *   -> per-request integral reduction (+ cut subtraction)
 *   -> likelihood tiles -> per-request likelihood reduction
 *   -> one D2H of every request's results.
 *
 * The sequence is captured once as a CUDA graph and replayed: tile and
 * request counts live in device memory, copies are of the buffers' full
 * capacity, so any batch that fits the current capacities replays the same
 * graph (re-captured only when a buffer grows or the set of kernel groups
 * changes).
 *
 * Tiles are cut from each request's items by its wedge's tile shape
 * (k_chunk r-bins per item, tile_items items per tile, tile_stars stars per
 * likelihood tile); the shape depends on the wedge alone, so a request's
 * bits are the same alone and in any batch.  mwsep_ctx_autotune picks the
 * shape per wedge by timing candidates.
 */
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <vector>

#include "milkyway_separation_gb300.h"
#include "mwsep_ctx.h"
#include "mwsep_internal.h"
#include "mwsep_status.h"

using namespace mwsep;

namespace {

constexpr int NG = MWSEP_ENG_GROUPS;

/* The kernel group of a stream count: S itself up to 4, 5 for 5..8. */
int stream_group(int S) { return S <= 4 ? S : 5; }

/* Grow-only capacity with headroom. */
size_t grow(size_t need) { return need + need / 2 + 64; }

int blocks_per_sm(int precision, int phase, int group)
{
    return precision == MWSEP_PLAIN_F64 ? mwsep_engine_f64_blocks_per_sm(phase, group)
                                        : mwsep_engine_f32_blocks_per_sm(phase, group);
}

void invalidate_graph(EngineState& e)
{
    if (e.graph) cudaGraphExecDestroy(e.graph);
    e.graph = nullptr;
    for (long long& k : e.graph_key) k = -1;
}

/* Device descriptors of every wedge's areas (one per precision, with that
 * precision's k_chunk applied) and catalogues. */
int ensure_descriptors(mwsep_ctx* c)
{
    EngineState& e = c->eng;
    const int W = (int)c->wedges.size();
    if (!e.desc_dirty && (int)e.seen_gen.size() == W)
        for (int w = 0; w < W; ++w)
            if (e.seen_gen[w] != c->wedges[w]->tune_gen) e.desc_dirty = true;
    if (!e.desc_dirty && (int)e.seen_gen.size() == W) return MWSEP_OK;
    e.area_base.assign(W, 0);
    int na = 0;
    for (int w = 0; w < W; ++w)
    {
        e.area_base[w] = na;
        na += 2 * (c->wedges[w]->has_problem ? c->wedges[w]->prob.n_areas : 0);
    }
    const size_t abytes = sizeof(mwsep_area_dev) * (size_t)std::max(na, 1);
    const size_t sbytes = sizeof(mwsep_stars_dev) * (size_t)std::max(W, 1);
    const void* old_a = e.d_areas.p;
    const void* old_s = e.d_stars.p;
    if (e.d_areas.ensure(abytes, c->dev_bytes) || e.d_stars.ensure(sbytes, c->dev_bytes) ||
        e.h_areas.ensure(abytes) || e.h_stars.ensure(sbytes))
        return mwsep_fail(MWSEP_ERR_NOMEM);
    if (old_a != e.d_areas.p || old_s != e.d_stars.p) invalidate_graph(e);
    mwsep_area_dev* ha = e.h_areas.as<mwsep_area_dev>();
    mwsep_stars_dev* hs = e.h_stars.as<mwsep_stars_dev>();
    for (int w = 0; w < W; ++w)
    {
        const Wedge& wd = *c->wedges[w];
        memset(&hs[w], 0, sizeof(hs[w]));
        if (wd.has_stars) hs[w] = wd.stars_view;
        if (!wd.has_problem) continue;
        for (int a = 0; a < wd.prob.n_areas; ++a)
            for (int p = 0; p < 2; ++p)
            {
                mwsep_area_dev v = wd.areas[a].view;
                set_chunking(v, wd.tune[p].k_chunk, wd.tune[p].warp_items);
                ha[e.area_base[w] + 2 * a + p] = v;
            }
    }
    CU(h2d(c, e.d_areas.p, ha, abytes));
    CU(h2d(c, e.d_stars.p, hs, sbytes));
    /* the pinned staging is rewritten next time: finish these copies */
    CU(cudaStreamSynchronize(c->stream));
    e.n_area_desc = na;
    e.n_star_desc = W;
    e.seen_gen.assign(W, 0);
    for (int w = 0; w < W; ++w) e.seen_gen[w] = c->wedges[w]->tune_gen;
    e.desc_dirty = false;
    return MWSEP_OK;
}

/* Tile ranges of one batch, per kernel group: [begin, end) in the tile
 * arrays (group 0 first). */
struct BatchShape
{
    int n_req = 0;
    int it_begin[NG] = {}, it_end[NG] = {};
    int lt_begin[NG] = {}, lt_end[NG] = {};
};

/* Build the host side of one batch into the pinned staging buffers.
 * max_itiles >= 0 truncates the integral tile list (autotuner timing runs);
 * with_likelihood = false leaves the likelihood tile lists empty. */
int build_batch(mwsep_ctx* c, int n, const mwsep_request* reqs, int precision, long long max_itiles,
                bool with_likelihood, BatchShape& shape)
{
    EngineState& e = c->eng;
    /* count tiles first */
    long long nit[NG] = {}, nlt[NG] = {};
    for (int i = 0; i < n; ++i)
    {
        const Wedge& w = *c->wedges[reqs[i].wedge];
        const Tune& t = w.tune[precision];
        const int cls = stream_group(w.prob.n_streams);
        for (int a = 0; a < w.prob.n_areas; ++a)
        {
            mwsep_area_dev v = w.areas[a].view;
            set_chunking(v, t.k_chunk, t.warp_items);
            nit[cls] += (v.n_items + t.tile_items - 1) / t.tile_items;
        }
        if (with_likelihood) nlt[cls] += (w.n_stars + t.tile_stars - 1) / t.tile_stars;
    }
    long long total_it = 0, total_lt = 0;
    for (int g = 0; g < NG; ++g)
    {
        total_it += nit[g];
        total_lt += nlt[g];
    }
    total_lt = std::max<long long>(1, total_lt);
    if (total_it > (1LL << 30) || total_lt > (1LL << 30)) return mwsep_fail(MWSEP_ERR_UNSUPPORTED);

    /* capacities (grow-only); any reallocation invalidates the graph.  The
     * HBM budget is checked before anything grows. */
    const size_t req_cap = std::max(e.d_reqs.bytes / sizeof(mwsep_req_dev), (size_t)n);
    struct Need
    {
        DevBuf* d;
        HostPinned* h;
        size_t bytes;
    } needs[] = {
        {&e.d_theta, &e.h_theta, sizeof(mwsep_theta_consts) * req_cap},
        {&e.d_reqs, &e.h_reqs, sizeof(mwsep_req_dev) * req_cap},
        {&e.d_itiles, &e.h_itiles, sizeof(mwsep_itile) * (size_t)std::max<long long>(total_it, 1)},
        {&e.d_ltiles, &e.h_ltiles, sizeof(mwsep_ltile) * (size_t)total_lt},
        {&e.d_ipart, nullptr, sizeof(double2) * MWSEP_ENG_ICOMP * (size_t)std::max<long long>(total_it, 1)},
        {&e.d_lpart, nullptr, sizeof(double2) * MWSEP_ENG_LCOMP * (size_t)total_lt},
        {&e.d_out, &e.h_out, sizeof(double) * MWSEP_ENG_OUT_STRIDE * req_cap},
        {&e.d_counters, &e.h_counters, sizeof(int) * MWSEP_ENG_COUNTERS},
    };
    size_t extra = 0;
    for (const Need& q : needs)
        if (q.d->bytes < q.bytes) extra += grow(q.bytes) - q.d->bytes;
    if (c->hbm_budget && c->dev_bytes + extra > c->hbm_budget) return mwsep_fail(MWSEP_ERR_BUDGET);
    bool moved = false;
    for (const Need& q : needs)
    {
        if (q.d->bytes < q.bytes)
        {
            if (q.d->ensure(grow(q.bytes), c->dev_bytes)) return mwsep_fail(MWSEP_ERR_NOMEM);
            moved = true;
        }
        if (q.h && q.h->bytes < q.d->bytes && q.h->ensure(q.d->bytes)) return mwsep_fail(MWSEP_ERR_NOMEM);
    }
    if (moved) invalidate_graph(e);

    mwsep_theta_consts* hth = e.h_theta.as<mwsep_theta_consts>();
    mwsep_req_dev* hq = e.h_reqs.as<mwsep_req_dev>();
    mwsep_itile* hit = e.h_itiles.as<mwsep_itile>();
    mwsep_ltile* hlt = e.h_ltiles.as<mwsep_ltile>();
    long long it_pos[NG], lt_pos[NG];
    it_pos[0] = lt_pos[0] = 0;
    for (int g = 1; g < NG; ++g)
    {
        it_pos[g] = it_pos[g - 1] + nit[g - 1];
        lt_pos[g] = lt_pos[g - 1] + nlt[g - 1];
    }
    for (int i = 0; i < n; ++i)
    {
        const int wi = reqs[i].wedge;
        const Wedge& w = *c->wedges[wi];
        const Tune& t = w.tune[precision];
        const int cls = stream_group(w.prob.n_streams);
        theta_consts(w.prob, reqs[i].theta, hth[i]);
        mwsep_req_dev& q = hq[i];
        memset(&q, 0, sizeof(q));
        q.n_streams = w.prob.n_streams;
        q.n_areas = w.prob.n_areas;
        q.stars = wi;
        for (int a = 0; a < w.prob.n_areas; ++a)
        {
            mwsep_area_dev v = w.areas[a].view;
            set_chunking(v, t.k_chunk, t.warp_items);
            q.area_slot[a] = (int)it_pos[cls];
            for (long long b = 0; b < v.n_items; b += t.tile_items)
            {
                mwsep_itile& tl = hit[it_pos[cls]++];
                tl.req = i;
                tl.area_desc = e.area_base[wi] + 2 * a + precision;
                tl.item_begin = b;
                tl.item_end = std::min<long long>(b + t.tile_items, v.n_items);
            }
            q.area_slot[a + 1] = (int)it_pos[cls];
        }
        q.lk_slot0 = (int)lt_pos[cls];
        if (with_likelihood)
            for (int s = 0; s < w.n_stars; s += t.tile_stars)
            {
                mwsep_ltile& tl = hlt[lt_pos[cls]++];
                tl.req = i;
                tl.star_begin = s;
                tl.star_end = std::min(s + t.tile_stars, w.n_stars);
                tl.pad0 = 0;
            }
        q.lk_slot1 = (int)lt_pos[cls];
    }
    shape.n_req = n;
    long long ib = 0, lb = 0;
    for (int g = 0; g < NG; ++g)
    {
        shape.it_begin[g] = (int)ib;
        shape.it_end[g] = (int)(ib + nit[g]);
        shape.lt_begin[g] = (int)lb;
        shape.lt_end[g] = (int)(lb + nlt[g]);
        ib += nit[g];
        lb += nlt[g];
    }
    if (max_itiles >= 0)
        /* timing runs: keep only the first tiles of each group */
        for (int k = 0; k < NG; ++k)
            shape.it_end[k] = (int)std::min<long long>(shape.it_end[k], shape.it_begin[k] + max_itiles);
    return MWSEP_OK;
}

mwsep_engine_args engine_args(mwsep_ctx* c)
{
    EngineState& e = c->eng;
    mwsep_engine_args a;
    a.areas = e.d_areas.as<mwsep_area_dev>();
    a.stars = e.d_stars.as<mwsep_stars_dev>();
    a.reqs = e.d_reqs.as<mwsep_req_dev>();
    a.thetas = e.d_theta.as<mwsep_theta_consts>();
    a.itiles = e.d_itiles.as<mwsep_itile>();
    a.ltiles = e.d_ltiles.as<mwsep_ltile>();
    a.ipart = e.d_ipart.as<double2>();
    a.lpart = e.d_lpart.as<double2>();
    a.out = e.d_out.as<double>();
    a.counters = e.d_counters.as<int>();
    a.n_area_desc = e.n_area_desc;
    a.n_star_desc = e.n_star_desc;
    return a;
}

/* Issue (or capture) the launch sequence of one batch. */
int issue(mwsep_ctx* c, int precision, const bool* has_i, const bool* has_l, bool with_likelihood, int* launches)
{
    EngineState& e = c->eng;
    cudaStream_t st = c->stream;
    const mwsep_engine_args a = engine_args(c);
    CU(h2d(c, e.d_counters.p, e.h_counters.p, sizeof(int) * MWSEP_ENG_COUNTERS));
    CU(h2d(c, e.d_theta.p, e.h_theta.p, e.d_theta.bytes));
    CU(h2d(c, e.d_reqs.p, e.h_reqs.p, e.d_reqs.bytes));
    CU(h2d(c, e.d_itiles.p, e.h_itiles.p, e.d_itiles.bytes));
    if (with_likelihood) CU(h2d(c, e.d_ltiles.p, e.h_ltiles.p, e.d_ltiles.bytes));
    int n = 0;
    for (int cls = 0; cls < NG; ++cls)
    {
        if (!has_i[cls]) continue;
        const int g = c->sm_count * blocks_per_sm(precision, 0, cls);
        CK(precision == MWSEP_PLAIN_F64 ? mwsep_engine_f64_launch(0, cls, &a, g, st)
                                        : mwsep_engine_f32_launch(0, cls, &a, g, st));
        ++n;
    }
    const int rg = c->sm_count * 4;
    CK(mwsep_engine_reduce(0, &a, rg, st));
    ++n;
    if (with_likelihood)
    {
        for (int cls = 0; cls < NG; ++cls)
        {
            if (!has_l[cls]) continue;
            const int g = c->sm_count * blocks_per_sm(precision, 1, cls);
            CK(precision == MWSEP_PLAIN_F64 ? mwsep_engine_f64_launch(1, cls, &a, g, st)
                                            : mwsep_engine_f32_launch(1, cls, &a, g, st));
            ++n;
        }
        CK(mwsep_engine_reduce(1, &a, rg, st));
        ++n;
    }
    CU(d2h(c, e.h_out.p, e.d_out.p, e.d_out.bytes));
    *launches = n;
    return MWSEP_OK;
}

/* Run a built batch: replay the captured graph when the shape group
 * matches, otherwise capture a new one. */
int run_batch(mwsep_ctx* c, int precision, const BatchShape& shape, bool with_likelihood, bool use_graph)
{
    mwsep::Range nvtx_range("mwsep.engine_batch");
    EngineState& e = c->eng;
    /* counters: per group next/end for integral and likelihood tiles */
    int* cnt = e.h_counters.as<int>();
    memset(cnt, 0, sizeof(int) * MWSEP_ENG_COUNTERS);
    for (int k = 0; k < NG; ++k)
    {
        cnt[4 * k + 0] = shape.it_begin[k];
        cnt[4 * k + 1] = shape.lt_begin[k];
        cnt[4 * k + 2] = shape.it_end[k];
        cnt[4 * k + 3] = shape.lt_end[k];
    }
    cnt[MWSEP_ENG_NREQ] = shape.n_req;
    bool has_i[NG], has_l[NG];
    long long imask = 0, lmask = 0;
    for (int k = 0; k < NG; ++k)
    {
        has_i[k] = shape.it_end[k] > shape.it_begin[k];
        has_l[k] = with_likelihood && shape.lt_end[k] > shape.lt_begin[k];
        imask |= (long long)has_i[k] << k;
        lmask |= (long long)has_l[k] << k;
    }

    cudaStream_t st = c->stream;
    int launches = 0;
    CU(cudaEventRecord(c->ev[0], st));
    if (use_graph)
    {
        const long long key[5] = {precision, imask, lmask, (long long)with_likelihood,
                                  (long long)e.d_ipart.bytes};
        if (!e.graph || memcmp(key, e.graph_key, sizeof(key)) != 0)
        {
            invalidate_graph(e);
            cudaGraph_t g = nullptr;
            CU(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            const int rc = issue(c, precision, has_i, has_l, with_likelihood, &launches);
            const cudaError_t ce = cudaStreamEndCapture(st, &g);
            if (rc || ce != cudaSuccess)
            {
                if (g) cudaGraphDestroy(g);
                cudaGetLastError();
                return mwsep_fail(rc ? rc : MWSEP_ERR_CUDA);
            }
            const cudaError_t ie = cudaGraphInstantiate(&e.graph, g, 0);
            cudaGraphDestroy(g);
            if (ie != cudaSuccess)
            {
                e.graph = nullptr;
                cudaGetLastError();
                return mwsep_fail(MWSEP_ERR_CUDA);
            }
            memcpy(e.graph_key, key, sizeof(key));
            e.graph_launches = launches;
        }
        CU(cudaGraphLaunch(e.graph, st));
        launches = e.graph_launches;
    }
    else
    {
        int rc = issue(c, precision, has_i, has_l, with_likelihood, &launches);
        if (rc) return rc;
    }
    CU(cudaEventRecord(c->ev[5], st));
    CU(cudaStreamSynchronize(st));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev[0], c->ev[5]);
    for (int i = 0; i < 4; ++i) c->last_ms[i] = 0.0;
    c->last_ms[4] = ms;
    c->last_launches = launches;
    return MWSEP_OK;
}

int check_requests(mwsep_ctx* c, int n, const mwsep_request* reqs)
{
    if (n < 1 || !reqs) return MWSEP_ERR_ARG;
    for (int i = 0; i < n; ++i)
    {
        const int w = reqs[i].wedge;
        if (w < 0 || w >= (int)c->wedges.size() || !reqs[i].theta) return MWSEP_ERR_ARG;
        if (!c->wedges[w]->has_problem || !c->wedges[w]->has_stars) return MWSEP_ERR_STATE;
    }
    return MWSEP_OK;
}

/* The double-float form: requests grouped by wedge, each group one batch
 * through the single-wedge path (its warp-tile kernel takes a batch of
 * parameter vectors as blockIdx.y); the timings are the groups' sums. */
int evaluate_requests_df(mwsep_ctx* c, int n, const mwsep_request* reqs, mwsep_result* out)
{
    std::vector<char> done((size_t)n, 0);
    std::vector<int> idx;
    std::vector<double> th;
    std::vector<mwsep_result> res;
    double ms[5] = {};
    int launches = 0;
    for (int i = 0; i < n; ++i)
    {
        if (done[(size_t)i]) continue;
        const int wid = reqs[i].wedge;
        const int P = c->wedges[wid]->prob.n_theta;
        idx.clear();
        th.clear();
        for (int j = i; j < n; ++j)
            if (!done[(size_t)j] && reqs[j].wedge == wid)
            {
                done[(size_t)j] = 1;
                idx.push_back(j);
                th.insert(th.end(), reqs[j].theta, reqs[j].theta + P);
            }
        res.resize(idx.size());
        for (size_t b = 0; b < idx.size(); b += 65535)
        {
            const int m = (int)std::min<size_t>(65535, idx.size() - b);
            const double* tp = P > 0 ? th.data() + b * (size_t)P : reqs[i].theta;
            const int rc = mwsep::evaluate_wedge(c, wid, m, tp, MWSEP_PLAIN_DF, res.data() + b);
            if (rc) return rc;
            for (int k = 0; k < 5; ++k) ms[k] += c->last_ms[k];
            launches += c->last_launches;
        }
        for (size_t k = 0; k < idx.size(); ++k) out[idx[k]] = res[k];
    }
    for (int k = 0; k < 5; ++k) c->last_ms[k] = ms[k];
    c->last_launches = launches;
    return MWSEP_OK;
}

/* Estimated device bytes of a wedge before building it. */
size_t wedge_bytes_estimate(const ASTRONOMY_PARAMETERS* ap, const STAR_POINTS* sp)
{
    size_t b = 0;
    for (int a = 0; a < ap->number_integrals; ++a)
    {
        const INTEGRAL* in = ap->integral[a];
        const size_t cols = (size_t)in->mu_steps * in->nu_steps, rc = (size_t)in->r_steps * ap->convolve;
        b += cols * 32 + rc * (4 * 8 + 16) + (size_t)in->r_steps * 16 + (size_t)in->nu_steps * 16;
    }
    const size_t n = sp ? (size_t)sp->number_stars : 0;
    b += n * (3 * 8 + 32 + 8) + n * (size_t)ap->convolve * (4 * 8 + 16);
    return b;
}

} // namespace

extern "C" void mwsep_engine_release(mwsep_ctx* c)
{
    EngineState& e = c->eng;
    invalidate_graph(e);
    DevBuf* bufs[] = {&e.d_areas, &e.d_stars, &e.d_reqs, &e.d_itiles, &e.d_ltiles, &e.d_theta,
                      &e.d_ipart, &e.d_lpart, &e.d_out, &e.d_counters};
    for (DevBuf* b : bufs) b->release(c->dev_bytes);
    HostPinned* hb[] = {&e.h_areas, &e.h_stars, &e.h_reqs, &e.h_itiles, &e.h_ltiles, &e.h_theta, &e.h_out,
                        &e.h_counters};
    for (HostPinned* h : hb) h->release();
}

extern "C" int mwsep_ctx_set_hbm_budget(mwsep_ctx* c, size_t bytes)
{
    if (!c) return mwsep_fail(MWSEP_ERR_ARG);
    c->hbm_budget = bytes;
    return MWSEP_OK;
}

extern "C" int mwsep_ctx_add_wedge(mwsep_ctx* c, const ASTRONOMY_PARAMETERS* ap, const STAR_POINTS* sp, int* id)
{
    if (!c || !ap || !sp || !id) return mwsep_fail(MWSEP_ERR_ARG);
    int rc = check_problem(ap);
    if (rc) return mwsep_fail(rc);
    if (c->hbm_budget && c->dev_bytes + wedge_bytes_estimate(ap, sp) > c->hbm_budget)
        return mwsep_fail(MWSEP_ERR_BUDGET);
    CU(cudaSetDevice(c->device));
    Wedge* w = new (std::nothrow) Wedge();
    if (!w) return mwsep_fail(MWSEP_ERR_NOMEM);
    rc = wedge_set_problem(c, *w, ap);
    if (!rc) rc = wedge_set_stars_rows(c, *w, sp, false);
    if (rc)
    {
        wedge_release(c, *w);
        delete w;
        return rc;
    }
    default_tune(c, *w); /* now that the catalogue size is known */
    c->wedges.push_back(w);
    c->eng.desc_dirty = true;
    *id = (int)c->wedges.size() - 1;
    return MWSEP_OK;
}

extern "C" int mwsep_ctx_wedge_theta_count(const mwsep_ctx* c, int id)
{
    if (!c || id < 0 || id >= (int)c->wedges.size() || !c->wedges[id]->has_problem)
        return -mwsep_fail(MWSEP_ERR_ARG);
    return c->wedges[id]->prob.n_theta;
}

extern "C" int mwsep_ctx_wedge_bytes(const mwsep_ctx* c, int id, size_t* out)
{
    if (!c || !out || id < 0 || id >= (int)c->wedges.size()) return mwsep_fail(MWSEP_ERR_ARG);
    *out = c->wedges[id]->bytes;
    return MWSEP_OK;
}

extern "C" int mwsep_ctx_wedge_points(const mwsep_ctx* c, int id, double* out)
{
    if (!c || !out || id < 0 || id >= (int)c->wedges.size()) return mwsep_fail(MWSEP_ERR_ARG);
    const Wedge& w = *c->wedges[id];
    if (!w.has_problem) return mwsep_fail(MWSEP_ERR_STATE);
    double cells = 0.0;
    for (int a = 0; a < w.prob.n_areas; ++a)
        cells += (double)(w.prob.area[a].cell_end - w.prob.area[a].cell_begin);
    *out = (cells + (w.has_stars ? (double)w.n_stars : 0.0)) * (double)w.prob.convolve;
    return MWSEP_OK;
}

extern "C" int mwsep_ctx_evaluate_requests(mwsep_ctx* c, int n, const mwsep_request* reqs, int precision,
                                           mwsep_result* out)
{
    if (!c || !out) return mwsep_fail(MWSEP_ERR_ARG);
    if (precision != MWSEP_PLAIN_F64 && precision != MWSEP_MIXED_F32 && precision != MWSEP_PLAIN_DF)
        return mwsep_fail(MWSEP_ERR_ARG);
    int rc = check_requests(c, n, reqs);
    if (rc) return mwsep_fail(rc);
    CU(cudaSetDevice(c->device));
    if (precision == MWSEP_PLAIN_DF) return evaluate_requests_df(c, n, reqs, out);
    if (precision == MWSEP_PLAIN_F64)
    {
        /* the plain likelihood reads the FP64 star tables */
        rc = wait_stars(c, c->stream);
        for (int i = 0; i < n && !rc; ++i) rc = ensure_star_f64(c, *c->wedges[reqs[i].wedge], c->stream);
        if (rc) return rc;
    }
    rc = ensure_descriptors(c);
    if (rc) return rc;
    BatchShape shape;
    rc = build_batch(c, n, reqs, precision, -1, true, shape);
    if (rc) return rc;
    rc = run_batch(c, precision, shape, true, env_long("MWSEP_ENGINE_GRAPH", 1) != 0);
    if (rc) return rc;
    const double* ho = c->eng.h_out.as<double>();
    for (int i = 0; i < n; ++i)
    {
        const Wedge& w = *c->wedges[reqs[i].wedge];
        const int S = w.prob.n_streams, A = w.prob.n_areas;
        const double* o = ho + (size_t)i * MWSEP_ENG_OUT_STRIDE;
        mwsep_result& r = out[i];
        memset(&r, 0, sizeof(r));
        r.number_streams = S;
        r.number_integrals = A;
        for (int a = 0; a < A; ++a)
            for (int k = 0; k <= S; ++k) r.area_integrals[a][k] = o[MWSEP_ENG_OUT_AREAS + a * MWSEP_ENG_ICOMP + k];
        r.background_integral = o[MWSEP_ENG_OUT_INTS];
        for (int s = 0; s < S; ++s) r.stream_integrals[s] = o[MWSEP_ENG_OUT_INTS + 1 + s];
        const double* lk = o + MWSEP_ENG_OUT_LK;
        const double N = (double)w.n_stars;
        r.prob_sum = lk[0];
        r.num_zero = (int)llround(lk[1]);
        r.likelihood = lk[0] / N - 3.0;
        r.background_only_likelihood = lk[2] / N - 3.0;
        for (int s = 0; s < S; ++s) r.stream_only_likelihood[s] = lk[3 + s] / N - 3.0;
        r.status = MWSEP_OK;
    }
    return MWSEP_OK;
}

extern "C" int mwsep_ctx_wedge_tile_shape(const mwsep_ctx* c, int id, int precision, int* k_chunk, int* tile_items)
{
    if (!c || id < 0 || id >= (int)c->wedges.size() || precision < 0 || precision > 2 || !k_chunk ||
        !tile_items)
        return mwsep_fail(MWSEP_ERR_ARG);
    *k_chunk = c->wedges[id]->tune[precision].k_chunk;
    *tile_items = c->wedges[id]->tune[precision].tile_items;
    return MWSEP_OK;
}

namespace {

/* The double-float form runs its requests per wedge (evaluate_wedge), so
 * its tuner times whole single evaluations: r-chunks of whole lane groups
 * (1, 2, 3, 4, 6 or 8 of the chunk that fills them), the r range split
 * evenly in 1 to 4 chunks, and the current one; the integral's device time,
 * best of two, picks the chunk. */
int autotune_df(mwsep_ctx* c, int id, const double* theta, double* predicted_ms)
{
    Wedge& w = *c->wedges[id];
    int R = 1;
    for (int a = 0; a < w.prob.n_areas; ++a) R = std::max(R, w.prob.area[a].r_steps);
    const int group = 32 * mwsep_df_tile_p(w.prob.n_streams);
    int g = group;
    for (int b = std::max(w.prob.convolve, 1); b;)
    {
        const int t = g % b;
        g = b;
        b = t;
    }
    const int ks = group / g;
    const Tune saved = w.tune[MWSEP_PLAIN_DF];
    std::vector<int> kcs{saved.k_chunk};
    auto add = [&](int kc) {
        kc = std::max(1, std::min(R, kc));
        if (std::find(kcs.begin(), kcs.end(), kc) == kcs.end()) kcs.push_back(kc);
    };
    for (int m : {1, 2, 3, 4, 6, 8}) add(ks * m);
    for (int d = 1; d <= 4; ++d) add((R + d - 1) / d);
    double best = 1e300;
    Tune best_t = saved;
    mwsep_result r;
    for (int kc : kcs)
    {
        Tune& t = w.tune[MWSEP_PLAIN_DF];
        t = saved;
        t.k_chunk = kc;
        double ms = 1e300;
        for (int rep = 0; rep < 2; ++rep)
        {
            const int rc = mwsep::evaluate_wedge(c, id, 1, theta, MWSEP_PLAIN_DF, &r);
            if (rc)
            {
                w.tune[MWSEP_PLAIN_DF] = saved;
                return rc;
            }
            ms = std::min(ms, c->last_ms[0]);
        }
        if (ms < best)
        {
            best = ms;
            best_t = t;
        }
    }
    w.tune[MWSEP_PLAIN_DF] = best_t;
    w.tune[MWSEP_PLAIN_DF].tuned = true;
    ++w.tune_gen;
    if (predicted_ms) *predicted_ms = best < 1e299 ? best : -1.0;
    return MWSEP_OK;
}

} // namespace

/* The project autotuner: for one wedge and precision, time the integral
 * tiles of a truncated single request (the first few waves of tiles) for
 * candidate (k_chunk, tile_items) shapes, predict the full integral time per
 * evaluation from the time per convolution point, and keep the fastest. */
extern "C" int mwsep_ctx_autotune(mwsep_ctx* c, int id, int precision, double* predicted_ms)
{
    mwsep::Range nvtx_range("mwsep.autotune");
    if (!c || id < 0 || id >= (int)c->wedges.size()) return mwsep_fail(MWSEP_ERR_ARG);
    if (precision != MWSEP_PLAIN_F64 && precision != MWSEP_MIXED_F32 && precision != MWSEP_PLAIN_DF)
        return mwsep_fail(MWSEP_ERR_ARG);
    Wedge& w = *c->wedges[id];
    if (!w.has_problem || !w.has_stars) return mwsep_fail(MWSEP_ERR_STATE);
    CU(cudaSetDevice(c->device));
    /* the problem's own parameter values as the timing point */
    std::vector<double> theta(std::max(w.prob.n_theta, 1));
    {
        int k = 0;
        for (int i = 0; i < w.prob.n_bg; ++i)
            if (w.prob.bg_opt[i]) theta[k++] = w.prob.bg[i];
        for (int s = 0; s < w.prob.n_streams; ++s)
        {
            if (w.prob.st_weight_opt[s]) theta[k++] = w.prob.st_weight[s];
            for (int j = 0; j < w.prob.n_sparams; ++j)
                if (w.prob.st_opt[s][j]) theta[k++] = w.prob.st[s][j];
        }
    }
    if (precision == MWSEP_PLAIN_DF) return autotune_df(c, id, theta.data(), predicted_ms);
    mwsep_request rq;
    rq.wedge = id;
    rq.theta = theta.data();

    int R = 1;
    long long cols = 0;
    for (int a = 0; a < w.prob.n_areas; ++a)
    {
        R = std::max(R, w.prob.area[a].r_steps);
        cols = std::max<long long>(cols, (long long)w.prob.area[a].mu_steps * w.prob.area[a].nu_steps);
    }
    const int C = w.prob.convolve;
    const Tune saved = w.tune[precision];
    const int cls = stream_group(w.prob.n_streams);
    const int waves = 6;
    /* concurrent takers of integral tiles: warps for the compensated engine,
     * blocks for the plain one */
    const long long resident = (long long)c->sm_count * blocks_per_sm(precision, 0, cls) *
                               (precision == MWSEP_MIXED_F32 ? saved.block / 32 : 1);
    std::vector<int> kcs;
    if (saved.warp_items)
    {
        /* warp tiles: r-chunks of whole lane groups, and the default */
        const int ks = warp_tile_kstep(C, w.prob.n_streams);
        for (int m : {1, 2, 3, 4, 6, 8})
        {
            const int kc = std::min(R, ks * m);
            if (std::find(kcs.begin(), kcs.end(), kc) == kcs.end()) kcs.push_back(kc);
        }
        if (std::find(kcs.begin(), kcs.end(), saved.k_chunk) == kcs.end()) kcs.push_back(saved.k_chunk);
    }
    else
        for (int d = 1; d <= 64 && (R + d - 1) / d >= 1; d *= 2)
        {
            const int kc = (R + d - 1) / d;
            if (kcs.empty() || kcs.back() != kc) kcs.push_back(kc);
            if (kc == 1) break;
        }
    /* items per engine tile: the compensated engine gives a tile to one
     * warp (warp tiles, or thread items per lane), the plain engine to a
     * block (thread items per thread) */
    const int tile_mult[3] = {2, 8, 32};
    const int warp_tiles[3] = {2, 4, 8};
    const int tile_threads = precision == MWSEP_MIXED_F32 ? 32 : saved.block;
    double best = 1e300;
    Tune best_t = saved;
    for (int kc : kcs)
    {
        for (int mi = 0; mi < 3; ++mi)
        {
            Tune& t = w.tune[precision];
            t = saved;
            t.k_chunk = kc;
            t.tile_items = saved.warp_items ? warp_tiles[mi] : tile_threads * tile_mult[mi];
            ++w.tune_gen;
            c->eng.desc_dirty = true;
            int rc = ensure_descriptors(c);
            if (rc) return rc;
            BatchShape shape;
            rc = build_batch(c, 1, &rq, precision, resident * waves, false, shape);
            if (rc) return rc;
            /* items in the timed prefix (of the first area) and the
             * columns an item covers */
            mwsep_area_dev v0 = w.areas[0].view;
            set_chunking(v0, t.k_chunk, t.warp_items);
            const long long items = std::min<long long>(
                (long long)(shape.it_end[cls] - shape.it_begin[cls]) * t.tile_items, v0.n_items);
            if (items <= 0) continue;
            const double cols_per_item = t.warp_items ? (double)cols / ((double)v0.n_items / v0.n_kchunks) : 1.0;
            double ms = 1e300;
            for (int rep = 0; rep < 2; ++rep)
            {
                rc = run_batch(c, precision, shape, false, false);
                if (rc) return rc;
                ms = std::min(ms, c->last_ms[4]);
            }
            /* ms per convolution point of the prefix -> a full evaluation */
            const double points = (double)items * cols_per_item * kc * C;
            const double full_points = 0.0 + (double)cols * R * C;
            const double pred = ms / points * full_points;
            if (pred < best)
            {
                best = pred;
                best_t = t;
            }
        }
    }
    w.tune[precision] = best_t;
    w.tune[precision].tuned = true;
    ++w.tune_gen;
    c->eng.desc_dirty = true;
    invalidate_graph(c->eng);
    if (predicted_ms) *predicted_ms = best < 1e299 ? best : -1.0;
    return MWSEP_OK;
}
